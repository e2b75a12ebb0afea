// Host mesh topology and the mesh-file readers.  See mesh.hpp for the reference
// functions each piece follows.
#include "mesh.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <unordered_map>

namespace gcfd {

static inline uint64_t edge_key(int a, int b) {
  const uint64_t lo = static_cast<uint64_t>(a < b ? a : b);
  const uint64_t hi = static_cast<uint64_t>(a < b ? b : a);
  return lo | (hi << 32);
}

namespace {

// The edges of one periodic half as a connected curve, as Curve.ReOrder does
// (types/elemental.go:141-199, AssembleCurve :201-240): start from the half's
// first edge (its last with `reverse`), which must sit at an open end of the
// curve, and walk the shared vertices.  Where the listed start is not an end
// edge, ReOrder starts at the end that Go's map iteration yields first; this
// restatement takes the end with the smaller vertex index instead.
std::string order_curve(const Topology& t, const std::vector<int>& edges, bool reverse, std::vector<int>* out) {
  std::unordered_map<int, std::vector<int>> at;  // vertex -> incident edges of the curve
  for (int en : edges) {
    at[static_cast<int>(t.key[en] & 0xffffffffULL)].push_back(en);
    at[static_cast<int>(t.key[en] >> 32)].push_back(en);
  }
  int nends = 0, endv = -1;
  for (const auto& kv : at) {
    if (kv.second.size() > 2) return "periodic boundary curve branches at a vertex";
    if (kv.second.size() == 1) {
      ++nends;
      if (endv < 0 || kv.first < endv) endv = kv.first;
    }
  }
  if (nends != 2) return "periodic boundary edges do not form one open curve";
  auto deg = [&](int v) { return static_cast<int>(at[v].size()); };
  int start = reverse ? edges.back() : edges.front();
  const int s0 = static_cast<int>(t.key[start] & 0xffffffffULL), s1 = static_cast<int>(t.key[start] >> 32);
  if (deg(s0) != 1 && deg(s1) != 1) start = at[endv][0];
  out->clear();
  out->push_back(start);
  const int a = static_cast<int>(t.key[start] & 0xffffffffULL), b = static_cast<int>(t.key[start] >> 32);
  int end = (deg(a) == 2) ? a : b;  // the open end to continue from
  int prev = start;
  while (deg(end) == 2) {
    const std::vector<int>& inc = at[end];
    const int next = (inc[0] == prev) ? inc[1] : inc[0];
    out->push_back(next);
    const int na = static_cast<int>(t.key[next] & 0xffffffffULL), nb = static_cast<int>(t.key[next] >> 32);
    end = (na == end) ? nb : na;
    prev = next;
    if (out->size() > edges.size()) return "periodic boundary curve is closed";
  }
  if (out->size() != edges.size()) return "periodic boundary edges do not form one open curve";
  return "";
}

}  // namespace

// Periodic pairs, as NewTriangulation does (triangulation.go:63-99): each
// tag's edge list is split into halves, each half is ordered as a connected
// curve (the second starting from its last edge for PeriodicReversed), and the
// i-th edges of the two curves become one shared edge: the first curve's
// element is the left side, the second curve's element the right side (its
// face points reversed like any shared edge's).  The reference keeps the
// second edge as a one-sided edge whose flux is a no-op (edges.go:436-437) and
// lets the order of Go's map iteration decide which of the two records the
// second element's edge uses (dfr_startup.go:289-310); here the second edge is
// removed and the element's edge is the shared one.  Each side keeps its own
// geometry (normal, ||n||) from its own edge (keyR).
std::string pair_periodic(const std::vector<std::pair<int, std::vector<int>>>& groups, Topology* t) {
  if (groups.empty()) return "";
  std::vector<char> dead(t->nEdges, 0);
  for (const auto& g : groups) {
    const std::vector<int>& L = g.second;
    const bool reversed = (g.first & 0xff) == BC_PeriodicReversed;
    if (L.size() % 2 != 0)
      return "periodic boundaries must be present in pairs, have dimension " + std::to_string(L.size()) +
             ", not even";
    const size_t l2 = L.size() / 2;
    std::vector<int> c0, c1;
    std::string msg = order_curve(*t, std::vector<int>(L.begin(), L.begin() + l2), false, &c0);
    if (msg.empty()) msg = order_curve(*t, std::vector<int>(L.begin() + l2, L.end()), reversed, &c1);
    if (!msg.empty()) return msg;
    for (size_t i = 0; i < l2; ++i) {
      const int e1 = c0[i], e2 = c1[i];
      if (t->kR[e1] >= 0 || t->kR[e2] >= 0 || dead[e1] || dead[e2] || e1 == e2)
        return "periodic boundary edge is not a free boundary edge";
      t->kR[e1] = t->kL[e2];
      t->eR[e1] = t->eL[e2];
      t->revR[e1] = t->revL[e2];
      t->keyR[e1] = t->key[e2];
      t->bc[e1] = BC_None;
      t->elemEdge[3 * t->kL[e2] + t->eL[e2]] = e1;
      dead[e2] = 1;
    }
  }
  // Drop the absorbed edges and renumber.
  std::vector<int> newIndex(t->nEdges, -1);
  int n = 0;
  for (int en = 0; en < t->nEdges; ++en)
    if (!dead[en]) newIndex[en] = n++;
  auto compact = [&](auto& v) {
    for (int en = 0; en < t->nEdges; ++en)
      if (!dead[en]) v[newIndex[en]] = v[en];
    v.resize(n);
  };
  compact(t->key);
  compact(t->keyR);
  compact(t->kL);
  compact(t->eL);
  compact(t->kR);
  compact(t->eR);
  compact(t->revL);
  compact(t->revR);
  compact(t->bc);
  for (int& e : t->elemEdge) e = newIndex[e];
  t->nEdges = n;
  return "";
}

std::string build_topology(int Nv, int K, const int32_t* etov, int nbc, const int32_t* bc_v1,
                           const int32_t* bc_v2, const int32_t* bc_flag, Topology* t) {
  t->K = K;
  t->Nv = Nv;
  t->elemEdge.assign(static_cast<size_t>(K) * 3, -1);
  std::unordered_map<uint64_t, int> index;
  index.reserve(static_cast<size_t>(K) * 2);
  for (int k = 0; k < K; ++k) {
    for (int ed = 0; ed < 3; ++ed) {
      const int a = etov[3 * k + ed], b = etov[3 * k + (ed + 1) % 3];
      if (a < 0 || b < 0 || a >= Nv || b >= Nv) return "element vertex index out of range";
      if (a == b) return "degenerate element edge";
      const uint64_t key = edge_key(a, b);
      const uint8_t rev = (a > b) ? 1 : 0;
      auto it = index.find(key);
      if (it == index.end()) {
        const int en = static_cast<int>(t->key.size());
        index.emplace(key, en);
        t->key.push_back(key);
        t->kL.push_back(k);
        t->eL.push_back(ed);
        t->revL.push_back(rev);
        t->kR.push_back(-1);
        t->eR.push_back(-1);
        t->revR.push_back(0);
        t->bc.push_back(BC_None);
        t->elemEdge[3 * k + ed] = en;
      } else {
        const int en = it->second;
        if (t->kR[en] >= 0) return "edge shared by more than two triangles";
        t->kR[en] = k;
        t->eR[en] = ed;
        t->revR[en] = rev;
        t->elemEdge[3 * k + ed] = en;
      }
    }
  }
  t->nEdges = static_cast<int>(t->key.size());
  t->keyR = t->key;
  // Periodic tags: the edges of each (group, flag) in input order.
  std::vector<std::pair<int, std::vector<int>>> periodic;
  for (int i = 0; i < nbc; ++i) {
    const int flag = bc_flag[i] & 0xff, group = bc_flag[i] >> 8;
    auto it = index.find(edge_key(bc_v1[i], bc_v2[i]));
    if (it == index.end()) return "boundary condition names an edge that is not in the mesh";
    switch (flag) {
      case BC_Far: case BC_IVortex: case BC_Wall: case BC_In: case BC_Out: case BC_Cyl:
        if (group != 0) return "boundary flag " + std::to_string(bc_flag[i]) + ": group bits on a non-periodic BC";
        t->bc[it->second] = flag;
        break;
      case BC_Periodic: case BC_PeriodicReversed: {
        const int gk = (group << 8) | flag;
        auto g = std::find_if(periodic.begin(), periodic.end(), [&](const auto& x) { return x.first == gk; });
        if (g == periodic.end()) {
          periodic.emplace_back(gk, std::vector<int>());
          g = periodic.end() - 1;
        }
        g->second.push_back(it->second);
        break;
      }
      default:
        return "boundary condition type not implemented: " + std::to_string(flag);
    }
  }
  return pair_periodic(periodic, t);
}

// ---------------------------------------------------------------------------
// Mesh files.

int bc_flag_of_tag(const std::string& tag) {
  std::string base;
  for (char ch : tag) base.push_back(static_cast<char>(std::tolower(static_cast<unsigned char>(ch))));
  const auto b = base.find_first_not_of(" \t"), e = base.find_last_not_of(" \t");
  base = (b == std::string::npos) ? std::string() : base.substr(b, e - b + 1);
  const auto dash = base.find('-');
  if (dash != std::string::npos && dash > 0) base = base.substr(0, dash);
  static const std::unordered_map<std::string, int> flags = {
      {"inflow", 1}, {"in", 1}, {"dirichlet", 2}, {"slip", 3}, {"far", 4}, {"wall", 5}, {"cyl", 6},
      {"neuman", 7}, {"out", 8}, {"outflow", 8}, {"ivortex", 9}, {"periodic", 10}, {"periodicreversed", 11}};
  const auto it = flags.find(base);
  return it == flags.end() ? -1 : it->second;
}

namespace {

std::vector<std::string> split_ws(const std::string& line) {
  std::istringstream is(line);
  std::vector<std::string> t;
  std::string w;
  while (is >> w) t.push_back(w);
  return t;
}

// Throws std::runtime_error on malformed input; the caller turns it into a status.
struct Lines {
  std::vector<std::string> v;
  const std::string& at(size_t i) const {
    if (i >= v.size()) throw std::runtime_error("unexpected end of file");
    return v[i];
  }
  std::vector<std::string> tok(size_t i, size_t need) const {
    auto t = split_ws(at(i));
    if (t.size() < need) throw std::runtime_error("malformed line " + std::to_string(i + 1) + ": [" + v[i] + "]");
    return t;
  }
};

void add_bc(MeshFile* m, const std::string& tag, int a, int b) {
  int f = bc_flag_of_tag(tag);
  if (f < 0) throw std::runtime_error("unable to find BC with base name, full tag: [" + tag + "]");
  if (f == BC_Periodic || f == BC_PeriodicReversed) {
    // one group per periodic tag (BCMAP keys it by the full tag, types/cfd.go:43)
    std::string low;
    for (char ch : tag) low.push_back(static_cast<char>(std::tolower(static_cast<unsigned char>(ch))));
    auto it = std::find(m->periodicTags.begin(), m->periodicTags.end(), low);
    const int g = static_cast<int>(it - m->periodicTags.begin());
    if (it == m->periodicTags.end()) m->periodicTags.push_back(low);
    f |= g << 8;
  }
  m->bc_v1.push_back(a);
  m->bc_v2.push_back(b);
  m->bc_flag.push_back(f);
}

void read_gambit(const Lines& L, MeshFile* m) {
  size_t pos = 6;
  auto h = L.tok(pos, 5);
  const int Nv = std::stoi(h[0]), K = std::stoi(h[1]), Nmats = std::stoi(h[2]), Nbcs = std::stoi(h[3]);
  if (std::stoi(h[4]) != 2) throw std::runtime_error("only 2D Gambit meshes are supported");
  pos += 3;
  m->vx.assign(Nv, 0.0);
  m->vy.assign(Nv, 0.0);
  for (int i = 0; i < Nv; ++i) {
    auto t = L.tok(pos + i, 3);
    const int ind = std::stoi(t[0]) - 1;
    if (ind < 0 || ind >= Nv) throw std::runtime_error("vertex index out of range");
    m->vx[ind] = std::stod(t[1]);
    m->vy[ind] = std::stod(t[2]);
  }
  pos += Nv + 2;
  m->etov.assign(static_cast<size_t>(K) * 3, 0);
  for (int i = 0; i < K; ++i) {
    auto t = L.tok(pos + i, 6);
    const int k = std::stoi(t[0]) - 1;
    if (k < 0 || k >= K) throw std::runtime_error("element index out of range");
    for (int c = 0; c < 3; ++c) m->etov[3 * k + c] = std::stoi(t[3 + c]) - 1;
  }
  pos += K + 2;
  for (int g = 0; g < Nmats; ++g) {
    const std::string& ln = L.at(pos);
    const auto at = ln.find("ELEMENTS:");
    if (at == std::string::npos) throw std::runtime_error("malformed element group header");
    const int nel = std::stoi(split_ws(ln.substr(at + 9)).at(0));
    pos += 3 + (nel + 9) / 10 + 2;
  }
  for (int b = 0; b < Nbcs; ++b) {
    if (b != 0) ++pos;
    auto head = L.tok(pos, 3);
    const std::string& tag = head[0];
    std::string low;
    for (char ch : tag) low.push_back(static_cast<char>(std::tolower(static_cast<unsigned char>(ch))));
    const int nfaces = (low == "cyl" && head.size() > 3) ? std::stoi(head[3]) : std::stoi(head[2]);
    ++pos;
    for (int i = 0; i < nfaces; ++i) {
      auto t = L.tok(pos + i, 3);
      const int k = std::stoi(t[0]) - 1, face = std::stoi(t[2]);
      if (k < 0 || k >= K || face < 1 || face > 3) throw std::runtime_error("boundary face out of range");
      const int32_t* v = &m->etov[3 * k];
      const int a = v[face - 1], c = v[face % 3];
      add_bc(m, tag, a, c);
    }
    pos += nfaces + 1;
  }
}

void read_su2(const Lines& raw, MeshFile* m) {
  Lines L;
  for (const auto& ln : raw.v) {
    const auto b = ln.find_first_not_of(" \t\r");
    if (b == std::string::npos || ln[b] == '%') continue;
    const auto e = ln.find_last_not_of(" \t\r");
    L.v.push_back(ln.substr(b, e - b + 1));
  }
  size_t pos = 0;
  auto token = [&]() {
    const std::string& ln = L.at(pos++);
    const auto eq = ln.find('=');
    if (eq == std::string::npos) throw std::runtime_error("badly formed input line [" + ln + "], should have an =");
    auto v = ln.substr(eq + 1);
    const auto b = v.find_first_not_of(" \t");
    return b == std::string::npos ? std::string() : v.substr(b);
  };
  if (std::stoi(token()) != 2) throw std::runtime_error("only 2D SU2 meshes are supported");
  const int K = std::stoi(token());
  m->etov.assign(static_cast<size_t>(K) * 3, 0);
  for (int k = 0; k < K; ++k) {
    auto t = L.tok(pos + k, 4);
    if (std::stoi(t[0]) != 5) throw std::runtime_error("unable to deal with non-triangular elements right now");
    for (int c = 0; c < 3; ++c) m->etov[3 * k + c] = std::stoi(t[1 + c]);
  }
  pos += K;
  const int Nv = std::stoi(token());
  m->vx.assign(Nv, 0.0);
  m->vy.assign(Nv, 0.0);
  for (int i = 0; i < Nv; ++i) {
    auto t = L.tok(pos + i, 2);
    m->vx[i] = std::stod(t[0]);
    m->vy[i] = std::stod(t[1]);
  }
  pos += Nv;
  const int nmark = std::stoi(token());
  for (int b = 0; b < nmark; ++b) {
    const std::string tag = split_ws(token()).at(0);
    const int ne = std::stoi(token());
    for (int i = 0; i < ne; ++i) {
      auto t = L.tok(pos + i, 3);
      if (std::stoi(t[0]) != 3) throw std::runtime_error("BCs should only contain line elements in 2D");
      add_bc(m, tag, std::stoi(t[1]), std::stoi(t[2]));
    }
    pos += ne;
  }
}

bool ends_with(const std::string& s, const std::string& suf) {
  return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

}  // namespace

std::string read_mesh_file(const std::string& path, MeshFile* out) {
  std::string p = path;
  while (!p.empty() && std::isspace(static_cast<unsigned char>(p.back()))) p.pop_back();
  const bool neu = ends_with(p, ".neu"), su2 = ends_with(p, ".su2");
  if (!neu && !su2) return "unsupported file type: " + path;
  std::ifstream f(p);
  if (!f) return "cannot open " + p;
  Lines L;
  std::string ln;
  while (std::getline(f, ln)) {
    if (!ln.empty() && ln.back() == '\r') ln.pop_back();
    L.v.push_back(ln);
  }
  MeshFile m;
  try {
    if (neu) read_gambit(L, &m);
    else read_su2(L, &m);
  } catch (const std::exception& e) {
    return p + ": " + e.what();
  }
  const int Nv = static_cast<int>(m.vx.size());
  for (int32_t v : m.etov)
    if (v < 0 || v >= Nv) return p + ": element vertex out of range";
  *out = std::move(m);
  return std::string();
}

}  // namespace gcfd
