// libgcfd: post-processing of the solution on the device — the solution
// interpolated at arbitrary points (the sampled lines of the Sod validation,
// NewSODShockTube / InterpolateFields, sod_shock_tube/shock_tube.go:27-142)
// and the state and pressure at the wall edge points (the wall data of
// OutputFinal, model_problems/Euler2D/euler.go:251-316).
//
// Both evaluate, per output point p, sum_i W[p][i] Q[n][i][k_p] for the four
// variables: W is a row of FluxEdgeInterp for an edge point, or the Lagrange
// basis of the solution points at the point's reference coordinates for an
// arbitrary point.  The weights and element indices are set up on the host,
// the sums run on the device against the FP64 state.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "gcfd_ctx.hpp"

namespace gcfd_host {
namespace {

// out[n][p] = sum_i W[p][i] Q[n][i][elem[p]], one thread per (point, variable).
__global__ void k_sample(const double* __restrict__ Q, int K, int Np, int npts, const int* __restrict__ elem,
                         const double* __restrict__ W, double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * npts) return;
  const int n = t / npts, p = t - n * npts;
  const int k = elem[p];
  const double* q = Q + static_cast<size_t>(n) * Np * K + k;
  const double* w = W + static_cast<size_t>(p) * Np;
  double s = 0.0;
  for (int i = 0; i < Np; ++i) s += w[i] * q[static_cast<size_t>(i) * K];
  out[t] = s;
}

// Uniform grid over the mesh's bounding box; each cell lists the elements
// whose bounding boxes touch it.  Built once per context on first use.
struct PointLocator {
  double x0 = 0, y0 = 0, hx = 1, hy = 1;
  int nx = 1, ny = 1;
  std::vector<int> start, items;
};

struct PostState {
  PointLocator loc;
  bool ready = false;
  std::vector<double> vx, vy;
  std::vector<int> etov;
};

// Reference coordinates (r, s) of (x, y) in element k: the inverse of
// x = 0.5 (-(r+s) xa + (r+1) xb + (s+1) xc) (element_utils.go:163-175).
void ref_coords(const PostState& ps, int k, double x, double y, double* r, double* s) {
  const int a = ps.etov[3 * k], b = ps.etov[3 * k + 1], c = ps.etov[3 * k + 2];
  const double xr = 0.5 * (ps.vx[b] - ps.vx[a]), xs = 0.5 * (ps.vx[c] - ps.vx[a]);
  const double yr = 0.5 * (ps.vy[b] - ps.vy[a]), ys = 0.5 * (ps.vy[c] - ps.vy[a]);
  const double det = xr * ys - xs * yr;
  // (x, y) - vertex a = J (r + 1, s + 1)
  const double dx = x - ps.vx[a], dy = y - ps.vy[a];
  *r = (ys * dx - xs * dy) / det - 1.0;
  *s = (-yr * dx + xr * dy) / det - 1.0;
}

void build_locator(const gcfd_ctx* c, PostState* ps) {
  PointLocator& L = ps->loc;
  const int K = c->K;
  double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
  for (double v : ps->vx) { xmin = std::min(xmin, v); xmax = std::max(xmax, v); }
  for (double v : ps->vy) { ymin = std::min(ymin, v); ymax = std::max(ymax, v); }
  const double w = std::max(xmax - xmin, 1e-300), h = std::max(ymax - ymin, 1e-300);
  const double cells = std::max(1.0, static_cast<double>(K) / 2.0);
  L.nx = std::max(1, std::min(1 << 14, static_cast<int>(std::sqrt(cells * w / h))));
  L.ny = std::max(1, std::min(1 << 14, static_cast<int>(cells / L.nx)));
  L.x0 = xmin;
  L.y0 = ymin;
  L.hx = w / L.nx;
  L.hy = h / L.ny;
  auto cell_range = [&](int k, int* i0, int* i1, int* j0, int* j1) {
    double ax = 1e300, bx = -1e300, ay = 1e300, by = -1e300;
    for (int v = 0; v < 3; ++v) {
      const int q = ps->etov[3 * k + v];
      ax = std::min(ax, ps->vx[q]); bx = std::max(bx, ps->vx[q]);
      ay = std::min(ay, ps->vy[q]); by = std::max(by, ps->vy[q]);
    }
    *i0 = std::clamp(static_cast<int>((ax - L.x0) / L.hx), 0, L.nx - 1);
    *i1 = std::clamp(static_cast<int>((bx - L.x0) / L.hx), 0, L.nx - 1);
    *j0 = std::clamp(static_cast<int>((ay - L.y0) / L.hy), 0, L.ny - 1);
    *j1 = std::clamp(static_cast<int>((by - L.y0) / L.hy), 0, L.ny - 1);
  };
  std::vector<int> count(static_cast<size_t>(L.nx) * L.ny + 1, 0);
  for (int k = 0; k < K; ++k) {
    int i0, i1, j0, j1;
    cell_range(k, &i0, &i1, &j0, &j1);
    for (int j = j0; j <= j1; ++j)
      for (int i = i0; i <= i1; ++i) ++count[static_cast<size_t>(j) * L.nx + i + 1];
  }
  for (size_t q = 1; q < count.size(); ++q) count[q] += count[q - 1];
  L.start = count;
  L.items.assign(count.back(), 0);
  std::vector<int> fill(count.begin(), count.end() - 1);
  for (int k = 0; k < K; ++k) {
    int i0, i1, j0, j1;
    cell_range(k, &i0, &i1, &j0, &j1);
    for (int j = j0; j <= j1; ++j)
      for (int i = i0; i <= i1; ++i) L.items[fill[static_cast<size_t>(j) * L.nx + i]++] = k;
  }
}

// The element containing (x, y) (barycentric test with a round-off margin; the
// lowest element index wins on shared edges and vertices), or -1.
int locate(const PostState& ps, double x, double y, double* r, double* s) {
  const PointLocator& L = ps.loc;
  const int i = static_cast<int>(std::floor((x - L.x0) / L.hx)), j = static_cast<int>(std::floor((y - L.y0) / L.hy));
  const double tol = 1e-12;
  int best = -1;
  for (int jj = std::max(0, j - 1); jj <= std::min(L.ny - 1, j + 1); ++jj)
    for (int ii = std::max(0, i - 1); ii <= std::min(L.nx - 1, i + 1); ++ii) {
      const size_t cell = static_cast<size_t>(jj) * L.nx + ii;
      for (int q = L.start[cell]; q < L.start[cell + 1]; ++q) {
        const int k = L.items[q];
        if (best >= 0 && k >= best) continue;
        double rr, ss;
        ref_coords(ps, k, x, y, &rr, &ss);
        if (rr >= -1.0 - tol && ss >= -1.0 - tol && rr + ss <= tol) {
          best = k;
          *r = rr;
          *s = ss;
        }
      }
    }
  return best;
}

// Lagrange basis of the solution points at (r, s): l_i = sum_m psi_m(r, s) Vinv[m][i].
void lagrange_at(const DFRElement& el, double r, double s, double* w) {
  const int Np = el.Np;
  std::vector<double> psi(Np);
  int m = 0;
  for (int i = 0; i <= el.N; ++i)
    for (int j = 0; j <= el.N - i; ++j, ++m) psi[m] = simplex2d_p(r, s, i, j);
  for (int p = 0; p < Np; ++p) {
    double v = 0.0;
    for (int q = 0; q < Np; ++q) v += psi[q] * el.Vinv(q, p);
    w[p] = v;
  }
}

// Device sums for npts points with their elements and weight rows.
int run_sample(gcfd_ctx* c, const std::vector<int>& elem, const std::vector<double>& W, double* q4) {
  const int npts = static_cast<int>(elem.size());
  if (npts == 0) return GCFD_OK;
  int rc = sync_fp64_state(c);
  if (rc) return rc;
  int* de = nullptr;
  double *dw = nullptr, *dout = nullptr;
  cudaError_t e = cudaMalloc(&de, sizeof(int) * npts);
  if (e == cudaSuccess) e = cudaMalloc(&dw, sizeof(double) * W.size());
  if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(double) * 4 * npts);
  if (e == cudaSuccess) e = cudaMemcpyAsync(de, elem.data(), sizeof(int) * npts, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dw, W.data(), sizeof(double) * W.size(), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    k_sample<<<(4 * npts + 127) / 128, 128, 0, c->stream>>>(c->Q[0], c->K, c->Np, npts, de, dw, dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(q4, dout, sizeof(double) * 4 * npts, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(de);
  cudaFree(dw);
  cudaFree(dout);
  if (e != cudaSuccess)
    return fail(c, e == cudaErrorMemoryAllocation ? GCFD_ERR_OOM : GCFD_ERR_CUDA,
                std::string("sampling: ") + cudaGetErrorString(e));
  return GCFD_OK;
}

PostState* post_state(gcfd_ctx* c) {
  if (!c->post) {
    auto* ps = new PostState();
    ps->vx = c->meshVX;
    ps->vy = c->meshVY;
    ps->etov = c->meshEToV;
    c->post = std::shared_ptr<void>(ps, [](void* p) { delete static_cast<PostState*>(p); });
  }
  return static_cast<PostState*>(c->post.get());
}

}  // namespace
}  // namespace gcfd_host

using namespace gcfd_host;

extern "C" {

int gcfd_sample_points(gcfd_ctx* c, int32_t npts, const double* x, const double* y, double* q4, int32_t* elem) {
  if (!c) return GCFD_ERR_ARG;
  if (npts < 0 || (npts > 0 && (!x || !y || !q4))) return fail(c, GCFD_ERR_ARG, "sample points: null argument");
  PostState* ps = post_state(c);
  if (!ps->ready) {
    build_locator(c, ps);
    ps->ready = true;
  }
  const int Np = c->Np;
  std::vector<int> ek(npts, 0);
  std::vector<double> W(static_cast<size_t>(npts) * Np, 0.0);
  int missing = -1;
  for (int p = 0; p < npts; ++p) {
    double r = 0, s = 0;
    const int k = locate(*ps, x[p], y[p], &r, &s);
    if (elem) elem[p] = k;
    if (k < 0) {
      if (missing < 0) missing = p;
      continue;
    }
    ek[p] = k;
    lagrange_at(c->el, r, s, &W[static_cast<size_t>(p) * Np]);
  }
  if (missing >= 0)
    return fail(c, GCFD_ERR_ARG, "sample point " + std::to_string(missing) + " (" + std::to_string(x[missing]) +
                                     ", " + std::to_string(y[missing]) + ") lies in no element");
  return run_sample(c, ek, W, q4);
}

int gcfd_wall_points(gcfd_ctx* c, int32_t* npts, double* x, double* y, double* q4, double* p) {
  if (!c || !npts) return c ? fail(c, GCFD_ERR_ARG, "wall points: null count") : GCFD_ERR_ARG;
  const int NE = c->NE, Np = c->Np, K = c->K;
  const int per = (c->N == 0) ? 1 : NE;  // N = 0: one point per edge, as OutputFinal writes
  std::vector<int> edges;
  for (int b = 0; b < c->nBC; ++b) {
    const int en = c->edgeOrder[c->nInt + b];
    if (c->topo.bc[en] == BC_Wall || c->topo.bc[en] == BC_Cyl) edges.push_back(en);
  }
  const int n = static_cast<int>(edges.size()) * per;
  if (!x && !y && !q4 && !p) {
    *npts = n;
    return GCFD_OK;
  }
  if (*npts < n) return fail(c, GCFD_ERR_SHAPE, "wall points: " + std::to_string(n) + " points, room for " +
                                                    std::to_string(*npts));
  std::vector<int> ek(n);
  std::vector<double> W(static_cast<size_t>(n) * Np);
  for (size_t q = 0; q < edges.size(); ++q) {
    const int en = edges[q];
    const int k = c->topo.kL[en], e = c->topo.eL[en];
    for (int i = 0; i < per; ++i) {
      const int row = e * NE + i;
      const size_t o = q * per + i;
      ek[o] = k;
      for (int j = 0; j < Np; ++j) W[o * Np + j] = c->el.FluxEdgeInterp(row, j);
      const int fr = 2 * Np + row;  // the edge point among the RT flux points
      double px, py;
      element_point(c->meshEToV.data(), c->meshVX.data(), c->meshVY.data(), k, c->el.rFlux[fr], c->el.sFlux[fr],
                    &px, &py);
      if (x) x[o] = px;
      if (y) y[o] = py;
    }
  }
  std::vector<double> qv(static_cast<size_t>(4) * n);
  int rc = run_sample(c, ek, W, qv.data());
  if (rc) return rc;
  const double g = c->fsFar.gamma;
  for (int o = 0; o < n; ++o) {
    const double rho = qv[o], mu = qv[n + o], mv = qv[2 * n + o], E = qv[3 * n + o];
    if (q4)
      for (int v = 0; v < 4; ++v) q4[static_cast<size_t>(v) * n + o] = qv[static_cast<size_t>(v) * n + o];
    if (p) p[o] = (g - 1.0) * (E - 0.5 * (mu * mu + mv * mv) / rho);
  }
  *npts = n;
  (void)K;
  return GCFD_OK;
}

}  // extern "C"
