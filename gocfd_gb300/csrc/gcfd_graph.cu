// libgcfd: the solution output's graph mesh and fields — what the reference
// streams to meshfile.gobcfd / solutionfile.gobcfd (CreateAVSGraphMesh and
// AVSFieldWriter, DG2D/graphics_support.go:43-128,173-230; GetPlotField,
// model_problems/Euler2D/plot.go:14-85; written per step by Solve,
// euler.go:190-215) — as arrays for the caller's own writer.
//
// Graph points of an element (lenElement = 3 (NpEdge + 1) + Np of them, in the
// reference's order): for each edge n = 0..2 its starting vertex, then the
// edge's NpEdge flux points counter-clockwise; then the Np interior RT points,
// which are the solution points.  A field is a flow function of fluids.go
// evaluated at the solution points, taken to the graph points by the solution
// basis (GraphInterp, dfr_startup.go:62-63), and each vertex value replaced by
// the mean of the two edge points beside it (AverageGraphFieldVertices,
// DG2D/graphics_support2.go:184-199); stored element-major in FP32.
//
// The element's sub-triangles: the reference triangulates the reference
// element's graph points with the Triangle library, constrained to the element
// edges and without Steiner points (geometry2D/triangulate.go:34-93, a
// constrained Delaunay triangulation).  All the constraint segments lie on the
// convex hull, so that is the Delaunay triangulation of the points; it is built
// here by Bowyer-Watson insertion.  Where four or more points are co-circular
// the Delaunay triangulation is not unique and the choice may differ from
// Triangle's.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <string>
#include <vector>

#include "gcfd_ctx.hpp"

namespace gcfd_host {
namespace {

struct GraphElement {
  int L = 0;                              // graph points per element
  std::vector<double> r, s;               // reference coordinates, L each
  std::vector<std::array<int, 3>> tris;   // counter-clockwise, local point indices
};

// Reference-element graph points (GetRSForGraphMesh, graphics_support.go:130-159).
void graph_points(const DFRElement& el, std::vector<double>* r, std::vector<double>* s) {
  const double vr[3] = {-1.0, 1.0, -1.0}, vs[3] = {-1.0, -1.0, 1.0};
  r->clear();
  s->clear();
  for (int n = 0; n < 3; ++n) {
    r->push_back(vr[n]);
    s->push_back(vs[n]);
    for (int i = 0; i < el.NpEdge; ++i) {
      r->push_back(el.rFlux[2 * el.Np + n * el.NpEdge + i]);
      s->push_back(el.sFlux[2 * el.Np + n * el.NpEdge + i]);
    }
  }
  for (int i = 0; i < el.Np; ++i) {
    r->push_back(el.rFlux[i]);
    s->push_back(el.sFlux[i]);
  }
}

double orient(double ax, double ay, double bx, double by, double cx, double cy) {
  return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}

// > 0 when d lies inside the circumcircle of the counter-clockwise triangle abc.
double incircle(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy) {
  const double adx = ax - dx, ady = ay - dy, bdx = bx - dx, bdy = by - dy, cdx = cx - dx, cdy = cy - dy;
  const double ad = adx * adx + ady * ady, bd = bdx * bdx + bdy * bdy, cd = cdx * cdx + cdy * cdy;
  return adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx);
}

// Delaunay triangulation of the points by Bowyer-Watson insertion inside a
// large enclosing triangle; the triangles touching it are dropped at the end.
std::vector<std::array<int, 3>> delaunay(const std::vector<double>& x, const std::vector<double>& y) {
  const int n = static_cast<int>(x.size());
  std::vector<double> px(x), py(y);
  px.push_back(-1e4); py.push_back(-1e4);
  px.push_back(1e4);  py.push_back(-1e4);
  px.push_back(0.0);  py.push_back(1e4);
  std::vector<std::array<int, 3>> tris{{n, n + 1, n + 2}};
  const double eps = 1e-12;
  for (int p = 0; p < n; ++p) {
    std::vector<std::array<int, 3>> keep, bad;
    for (const auto& t : tris) {
      if (incircle(px[t[0]], py[t[0]], px[t[1]], py[t[1]], px[t[2]], py[t[2]], px[p], py[p]) > eps)
        bad.push_back(t);
      else
        keep.push_back(t);
    }
    // the cavity's boundary: edges of exactly one bad triangle
    std::vector<std::array<int, 2>> edges;
    for (const auto& t : bad)
      for (int e = 0; e < 3; ++e) edges.push_back({t[e], t[(e + 1) % 3]});
    for (const auto& e : edges) {
      bool shared = false;
      for (const auto& f : edges)
        if (f[0] == e[1] && f[1] == e[0]) shared = true;
      if (shared) continue;
      std::array<int, 3> t{e[0], e[1], p};
      if (orient(px[t[0]], py[t[0]], px[t[1]], py[t[1]], px[t[2]], py[t[2]]) < 0) std::swap(t[0], t[1]);
      keep.push_back(t);
    }
    tris.swap(keep);
  }
  std::vector<std::array<int, 3>> out;
  for (const auto& t : tris)
    if (t[0] < n && t[1] < n && t[2] < n &&
        orient(px[t[0]], py[t[0]], px[t[1]], py[t[1]], px[t[2]], py[t[2]]) > eps)
      out.push_back(t);
  std::sort(out.begin(), out.end());
  return out;
}

GraphElement graph_element(const DFRElement& el) {
  GraphElement g;
  graph_points(el, &g.r, &g.s);
  g.L = static_cast<int>(g.r.size());
  g.tris = delaunay(g.r, g.s);
  return g;
}

// GraphInterp rows: the solution basis (orthonormal modes times Vinv) at each
// graph point, L x Np.
std::vector<double> graph_interp(const DFRElement& el, const GraphElement& g) {
  std::vector<double> G(static_cast<size_t>(g.L) * el.Np, 0.0);
  int nm = 0;
  std::vector<std::array<int, 2>> modes;
  for (int i = 0; i <= el.N; ++i)
    for (int j = 0; j <= el.N - i; ++j) modes.push_back({i, j}), ++nm;
  for (int p = 0; p < g.L; ++p) {
    std::vector<double> phi(nm);
    for (int m = 0; m < nm; ++m) phi[m] = simplex2d_p(g.r[p], g.s[p], modes[m][0], modes[m][1]);
    for (int c = 0; c < el.Np; ++c) {
      double v = 0.0;
      for (int m = 0; m < nm; ++m) v += phi[m] * el.Vinv(m, c);
      G[static_cast<size_t>(p) * el.Np + c] = v;
    }
  }
  return G;
}

struct GraphState {
  GraphElement g;
  double* G = nullptr;   // device GraphInterp, L x Np
  float* out = nullptr;  // device field, K x L
};

// Flow functions of GetFlowFunctionBase (fluids.go:289-336), kinds 0..13.
__device__ double flow_function(int kind, double rho, double ru, double rv, double E, double gamma, double pinf,
                                double qqinf) {
  const double gm1 = gamma - 1.0, oorho = 1.0 / rho;
  switch (kind) {
    case 0: return rho;
    case 1: return ru;
    case 2: return rv;
    case 3: return E;
    case 10: return ru * oorho;
    case 11: return rv * oorho;
    default: break;
  }
  const double u = ru * oorho, v = rv * oorho, U2 = u * u + v * v;
  const double q = 0.5 * rho * U2, p = gm1 * (E - q);
  switch (kind) {
    case 9: return sqrt(U2);
    case 6: return q;
    case 5: return p;
    case 7: return (p - pinf) / qqinf;
    case 8: return sqrt(fabs(gamma * p * oorho));
    case 12: return (E + p) / rho;
    case 13: return log(p) - gamma * log(rho);
    default: return sqrt(U2) / sqrt(fabs(gamma * p * oorho));  // 4: Mach
  }
}

// One thread per element: the flow function at the Np solution points, the
// graph values by GraphInterp, then the vertex means.
__global__ void k_graph_field(const double* __restrict__ Q, const double* __restrict__ G, int K, int Np, int NE,
                              int L, int kind, double gamma, double pinf, double qqinf, float* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const size_t sK = static_cast<size_t>(K);
  double f[36];  // Np <= 36 for N <= 7
  for (int i = 0; i < Np; ++i) {
    const size_t ind = static_cast<size_t>(i) * sK + k;
    f[i] = flow_function(kind, Q[ind], Q[static_cast<size_t>(Np) * sK + ind], Q[2 * static_cast<size_t>(Np) * sK + ind],
                         Q[3 * static_cast<size_t>(Np) * sK + ind], gamma, pinf, qqinf);
  }
  float* o = out + static_cast<size_t>(k) * L;
  for (int p = 0; p < L; ++p) {
    double v = 0.0;
    for (int i = 0; i < Np; ++i) v += G[static_cast<size_t>(p) * Np + i] * f[i];
    o[p] = static_cast<float>(v);
  }
  // vertex n sits at n (NE + 1): the mean of the next point and of the point
  // before it (cyclically), in FP64 as the reference does before its FP32 copy
  const int E1 = NE + 1;
  double vv[3];
  for (int n = 0; n < 3; ++n) {
    const int iV = n * E1, iVp = iV + 1, iVm = (n == 0) ? 3 * E1 - 1 : iV - 1;
    double a = 0.0, b = 0.0;
    for (int i = 0; i < Np; ++i) {
      a += G[static_cast<size_t>(iVp) * Np + i] * f[i];
      b += G[static_cast<size_t>(iVm) * Np + i] * f[i];
    }
    vv[n] = 0.5 * (a + b);
  }
  for (int n = 0; n < 3; ++n) o[n * E1] = static_cast<float>(vv[n]);
}

GraphState* graph_state(gcfd_ctx* c, int* rc) {
  *rc = GCFD_OK;
  if (!c->graphOut) {
    auto gs = std::make_shared<GraphState>();
    gs->g = graph_element(c->el);
    const std::vector<double> G = graph_interp(c->el, gs->g);
    double* dG = nullptr;
    if ((*rc = upload(c, &dG, G))) return nullptr;
    gs->G = dG;
    float* o = nullptr;
    if ((*rc = dalloc(c, &o, static_cast<size_t>(c->K) * gs->g.L))) return nullptr;
    gs->out = o;
    c->graphOut = gs;
  }
  return static_cast<GraphState*>(c->graphOut.get());
}

}  // namespace
}  // namespace gcfd_host

using namespace gcfd_host;

extern "C" {

int gcfd_host_graph_element(int32_t N, int32_t* len_element, int32_t* ntri, double* rs, int32_t* tris) {
  DFRElement e;
  try {
    e = build_dfr_element(N);
  } catch (const std::exception& ex) {
    return fail(nullptr, GCFD_ERR_UNSUPPORTED, ex.what());
  }
  const GraphElement g = graph_element(e);
  if (len_element) *len_element = g.L;
  if (ntri) *ntri = static_cast<int32_t>(g.tris.size());
  if (rs)
    for (int p = 0; p < g.L; ++p) {
      rs[2 * p] = g.r[p];
      rs[2 * p + 1] = g.s[p];
    }
  if (tris)
    for (size_t t = 0; t < g.tris.size(); ++t)
      for (int v = 0; v < 3; ++v) tris[3 * t + v] = g.tris[t][v];
  return GCFD_OK;
}

int gcfd_graph_mesh(gcfd_ctx* c, int32_t* len_element, int32_t* ntri_per_element, float* xy, int64_t* tris) {
  if (!c) return GCFD_ERR_ARG;
  int rc;
  GraphState* gs = graph_state(c, &rc);
  if (!gs) return rc;
  const GraphElement& g = gs->g;
  if (len_element) *len_element = g.L;
  if (ntri_per_element) *ntri_per_element = static_cast<int32_t>(g.tris.size());
  const int K = c->K;
  if (xy) {
    const int32_t* ev = c->meshEToV.data();
    for (int k = 0; k < K; ++k)
      for (int p = 0; p < g.L; ++p) {
        double x, y;
        element_point(ev, c->meshVX.data(), c->meshVY.data(), k, g.r[p], g.s[p], &x, &y);
        // the vertices exactly as the mesh gives them
        const int E1 = c->NE + 1;
        if (p < 3 * E1 && p % E1 == 0) {
          const int v = ev[3 * static_cast<size_t>(k) + p / E1];
          x = c->meshVX[v];
          y = c->meshVY[v];
        }
        xy[2 * (static_cast<size_t>(k) * g.L + p)] = static_cast<float>(x);
        xy[2 * (static_cast<size_t>(k) * g.L + p) + 1] = static_cast<float>(y);
      }
  }
  if (tris) {
    const size_t nt = g.tris.size();
    for (int k = 0; k < K; ++k)
      for (size_t t = 0; t < nt; ++t)
        for (int v = 0; v < 3; ++v)
          tris[3 * (static_cast<size_t>(k) * nt + t) + v] = static_cast<int64_t>(k) * g.L + g.tris[t][v];
  }
  return GCFD_OK;
}

int gcfd_graph_fields(gcfd_ctx* c, int32_t nfields, const int32_t* kinds, float* out) {
  if (!c || (nfields > 0 && (!kinds || !out))) return c ? fail(c, GCFD_ERR_ARG, "null fields") : GCFD_ERR_ARG;
  for (int f = 0; f < nfields; ++f)
    if (kinds[f] < 0 || kinds[f] > 13)
      return fail(c, GCFD_ERR_ARG, "flow function kinds are 0..13 (Density .. Entropy)");
  int rc;
  GraphState* gs = graph_state(c, &rc);
  if (!gs) return rc;
  if ((rc = sync_fp64_state(c))) return rc;
  const double gamma = c->fsFar.gamma;
  const double* qi = c->fsFar.qinf;
  const double qq = 0.5 * (qi[1] * qi[1] + qi[2] * qi[2]) / qi[0];  // QQinf: dynamic pressure of Qinf
  const size_t n = static_cast<size_t>(c->K) * gs->g.L;
  for (int f = 0; f < nfields; ++f) {
    k_graph_field<<<(c->K + 127) / 128, 128, 0, c->stream>>>(c->Q[0], gs->G, c->K, c->Np, c->NE, gs->g.L, kinds[f],
                                                             gamma, c->fsFar.pinf, qq, gs->out);
    GCFD_CUDA(c, cudaGetLastError());
    GCFD_CUDA(c, cudaMemcpyAsync(out + n * f, gs->out, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  }
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  return GCFD_OK;
}

}  // extern "C"
