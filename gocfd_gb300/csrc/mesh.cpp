// Host mesh topology and geometry.  See mesh.hpp for the reference functions
// each piece follows.
#include "mesh.hpp"

#include <cmath>
#include <unordered_map>

namespace gcfd {

static inline uint64_t edge_key(int a, int b) {
  const uint64_t lo = static_cast<uint64_t>(a < b ? a : b);
  const uint64_t hi = static_cast<uint64_t>(a < b ? b : a);
  return lo | (hi << 32);
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
  for (int i = 0; i < nbc; ++i) {
    const int flag = bc_flag[i];
    auto it = index.find(edge_key(bc_v1[i], bc_v2[i]));
    if (it == index.end()) return "boundary condition names an edge that is not in the mesh";
    switch (flag) {
      case BC_Far: case BC_IVortex: case BC_Wall: case BC_In: case BC_Out: case BC_Cyl:
        t->bc[it->second] = flag;
        break;
      default:
        return "boundary condition type not implemented: " + std::to_string(flag);
    }
  }
  return "";
}

void build_geometry(const DFRElement& el, const Topology& t, const double* vx, const double* vy,
                    const int32_t* etov, Geometry* g) {
  const int K = t.K;
  g->J.assign(4 * static_cast<size_t>(K), 0.0);
  g->Jinv.assign(4 * static_cast<size_t>(K), 0.0);
  g->Jdet.assign(K, 0.0);
  for (int k = 0; k < K; ++k) {
    const int v1 = etov[3 * k], v2 = etov[3 * k + 1], v3 = etov[3 * k + 2];
    const double xr = 0.5 * (vx[v2] - vx[v1]), yr = 0.5 * (vy[v2] - vy[v1]);
    const double xs = 0.5 * (vx[v3] - vx[v1]), ys = 0.5 * (vy[v3] - vy[v1]);
    const double det = xr * ys - xs * yr;
    double* J = &g->J[4 * k];
    double* Ji = &g->Jinv[4 * k];
    J[0] = xr; J[1] = xs; J[2] = yr; J[3] = ys;
    g->Jdet[k] = det;
    Ji[0] = ys / det; Ji[1] = -xs / det; Ji[2] = -yr / det; Ji[3] = xr / det;
  }
  g->nx.assign(3 * static_cast<size_t>(K), 0.0);
  g->ny.assign(3 * static_cast<size_t>(K), 0.0);
  g->IInII.assign(3 * static_cast<size_t>(K), 0.0);
  for (int en = 0; en < t.nEdges; ++en) {
    const int lo = static_cast<int>(t.key[en] & 0xffffffffULL);
    const int hi = static_cast<int>(t.key[en] >> 32);
    for (int c = 0; c < 2; ++c) {
      const int k = c == 0 ? t.kL[en] : t.kR[en];
      if (k < 0) continue;
      const int ed = c == 0 ? t.eL[en] : t.eR[en];
      const bool rev = (c == 0 ? t.revL[en] : t.revR[en]) != 0;
      // Vertices ordered opposite to the element's traversal: (-dy, dx) points out.
      const int a = rev ? lo : hi, b = rev ? hi : lo;
      const double dx = vx[b] - vx[a], dy = vy[b] - vy[a];
      const double len = std::sqrt(dx * dx + dy * dy);
      const size_t ind = static_cast<size_t>(ed) * K + k;
      g->nx[ind] = -dy / len;
      g->ny[ind] = dx / len;
      g->IInII[ind] = (ed == 1) ? len / (2.0 * std::sqrt(2.0)) : len / 2.0;
    }
  }
  g->edgeLenMax.assign(K, 0.0);
  g->hK.assign(K, 0.0);
  const double np12 = double(el.N + 1) * double(el.N + 1);
  for (int k = 0; k < K; ++k) {
    double mx = -1.0;
    for (int ed = 0; ed < 3; ++ed) mx = std::max(mx, g->IInII[static_cast<size_t>(ed) * K + k]);
    g->edgeLenMax[k] = g->Jdet[k] / mx;
    g->hK[k] = g->edgeLenMax[k] / np12;
  }
  auto local = [&](const std::vector<double>& R, const std::vector<double>& S,
                   std::vector<double>* X, std::vector<double>* Y) {
    const int n = static_cast<int>(R.size());
    X->assign(static_cast<size_t>(n) * K, 0.0);
    Y->assign(static_cast<size_t>(n) * K, 0.0);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < K; ++k) {
        const int va = etov[3 * k], vb = etov[3 * k + 1], vc = etov[3 * k + 2];
        const double a = -(R[i] + S[i]), b = R[i] + 1.0, c = S[i] + 1.0;
        (*X)[static_cast<size_t>(i) * K + k] = 0.5 * (a * vx[va] + b * vx[vb] + c * vx[vc]);
        (*Y)[static_cast<size_t>(i) * K + k] = 0.5 * (a * vy[va] + b * vy[vb] + c * vy[vc]);
      }
  };
  local(el.rFlux, el.sFlux, &g->xFlux, &g->yFlux);
  local(el.r, el.s, &g->xSol, &g->ySol);
}

}  // namespace gcfd
