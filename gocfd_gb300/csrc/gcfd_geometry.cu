// libgcfd: the mesh geometry and the initial state built on the device.
//
// The host builds only the topology (edge hashing and periodic pairing,
// mesh.cpp); the per-element geometry of ProcessGeometry (DG2D/dfr_startup.go:
// 125-175,256-314: Jacobian, its inverse and determinant, the outward unit
// normal and the ||n|| scale IInII of each element edge, hK), the per-edge
// tables the edge kernels read, the mixed path's FP32 copies, the solution
// points' coordinates (CalculateElementLocalGeometry, element_utils.go:163-175)
// and the initial state (InitializeSolution, euler.go:728-794) are computed
// here from the vertex and element arrays, one thread per element or edge.
//
// Element k's edge e runs from vertex e to vertex e + 1 (mod 3) of its row of
// EToV (triangulation.go:19-171); its outward normal is (-dy, dx) / |d| for
// d = x(v_e) - x(v_{e+1}), the vertices taken against the element's
// counter-clockwise traversal (GetEdgeCoordinates, triangulation.go:230-235).
// Products and sums are explicitly rounded (no FMA contraction), so every
// platform gets the same bits.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "gcfd_ctx.hpp"

namespace gcfd_host {
namespace {

struct ElemGeoArgs {
  int K, N;
  const double* vx;
  const double* vy;
  const int32_t* etov;  // [3 k + v]
  double* Jdet;         // [K]
  double* Jinv;         // [4][K]: ys, -xs, -yr, xr over |J|
  double* nxE;          // [3][K]
  double* nyE;
  double* IIE;
  double* hK;           // [K]
  int* bad;             // [2]: count of elements with |J| <= 0, the first of them
};

__global__ void k_geo_elements(ElemGeoArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const size_t sK = static_cast<size_t>(a.K);
  int v[3];
  double x[3], y[3];
  for (int i = 0; i < 3; ++i) {
    v[i] = a.etov[3 * static_cast<size_t>(k) + i];
    x[i] = a.vx[v[i]];
    y[i] = a.vy[v[i]];
  }
  const double xr = __dmul_rn(0.5, __dsub_rn(x[1], x[0])), yr = __dmul_rn(0.5, __dsub_rn(y[1], y[0]));
  const double xs = __dmul_rn(0.5, __dsub_rn(x[2], x[0])), ys = __dmul_rn(0.5, __dsub_rn(y[2], y[0]));
  const double det = __dsub_rn(__dmul_rn(xr, ys), __dmul_rn(xs, yr));
  a.Jdet[k] = det;
  a.Jinv[k] = __ddiv_rn(ys, det);
  a.Jinv[sK + k] = __ddiv_rn(-xs, det);
  a.Jinv[2 * sK + k] = __ddiv_rn(-yr, det);
  a.Jinv[3 * sK + k] = __ddiv_rn(xr, det);
  if (!(det > 0.0)) {
    atomicAdd(&a.bad[0], 1);
    atomicMin(&a.bad[1], k);
  }
  double mx = -1.0;
  for (int e = 0; e < 3; ++e) {
    const int e1 = (e + 1) % 3;
    const double dx = __dsub_rn(x[e], x[e1]), dy = __dsub_rn(y[e], y[e1]);
    const double len = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    a.nxE[e * sK + k] = __ddiv_rn(-dy, len);
    a.nyE[e * sK + k] = __ddiv_rn(dx, len);
    const double ii = (e == 1) ? __ddiv_rn(len, __dmul_rn(2.0, sqrt(2.0))) : __ddiv_rn(len, 2.0);
    a.IIE[e * sK + k] = ii;
    mx = fmax(mx, ii);
  }
  const double np1 = static_cast<double>(a.N + 1);
  a.hK[k] = __ddiv_rn(__ddiv_rn(det, mx), __dmul_rn(np1, np1));
}

// Per device edge (interior first, then boundary): the left element's normal
// and scale, the right side's scale, 1 / hK of the left element.
__global__ void k_geo_edges(int nEdges, int nInt, int K, const int* kL, const int* kR, const int* eLR,
                            const double* nxE, const double* nyE, const double* IIE, const double* hK, double* nx,
                            double* ny, double* IIL, double* IIR, double* oohK) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nEdges) return;
  const size_t sK = static_cast<size_t>(K);
  const int l = kL[i], el = eLR[i] & 3;
  const size_t fl = el * sK + l;
  nx[i] = nxE[fl];
  ny[i] = nyE[fl];
  IIL[i] = IIE[fl];
  IIR[i] = (i < nInt) ? IIE[(eLR[i] >> 2) * sK + kR[i]] : 0.0;
  oohK[i] = 1.0 / hK[l];
}

// The mixed path's FP32 copies: [6][K] Jdet, Jinv0..3, 1/Jdet; [3][K] IInII;
// per edge nx, ny, 1/hK.
__global__ void k_geo_mixed(int K, int nEdges, const double* Jdet, const double* Jinv, const double* IIE,
                            const double* nx, const double* ny, const double* oohK, float* mgeo, float* mII,
                            float* mnx, float* mny, float* moohK) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t sK = static_cast<size_t>(K);
  if (t < K) {
    mgeo[t] = static_cast<float>(Jdet[t]);
    for (int q = 0; q < 4; ++q) mgeo[(q + 1) * sK + t] = static_cast<float>(Jinv[q * sK + t]);
    mgeo[5 * sK + t] = static_cast<float>(1.0 / Jdet[t]);
    for (int e = 0; e < 3; ++e) mII[e * sK + t] = static_cast<float>(IIE[e * sK + t]);
  }
  if (t < nEdges) {
    mnx[t] = static_cast<float>(nx[t]);
    mny[t] = static_cast<float>(ny[t]);
    moohK[t] = static_cast<float>(oohK[t]);
  }
}

// Physical coordinates of reference point (r, s) of element k (element_utils.go:163-175).
__device__ __forceinline__ void element_point_dev(const double* vx, const double* vy, const int32_t* etov, int k,
                                                  double r, double s, double* x, double* y) {
  const int va = etov[3 * static_cast<size_t>(k)], vb = etov[3 * static_cast<size_t>(k) + 1],
            vc = etov[3 * static_cast<size_t>(k) + 2];
  const double A = -(r + s), B = r + 1.0, Cc = s + 1.0;
  *x = __dmul_rn(0.5, __dadd_rn(__dadd_rn(__dmul_rn(A, vx[va]), __dmul_rn(B, vx[vb])), __dmul_rn(Cc, vx[vc])));
  *y = __dmul_rn(0.5, __dadd_rn(__dadd_rn(__dmul_rn(A, vy[va]), __dmul_rn(B, vy[vb])), __dmul_rn(Cc, vy[vc])));
}

__global__ void k_solution_points(int K, int Np, const double* vx, const double* vy, const int32_t* etov,
                                  const double* rs, double* X, double* Y) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  for (int i = 0; i < Np; ++i)
    element_point_dev(vx, vy, etov, k, rs[2 * i], rs[2 * i + 1], &X[static_cast<size_t>(i) * K + k],
                      &Y[static_cast<size_t>(i) * K + k]);
}

struct InitArgs {
  int K, Np, init;
  const double* vx;
  const double* vy;
  const int32_t* etov;
  const double* rs;
  double vx0, vy0, vbeta, vgamma;
  double qFar[4], qIn[4], qOut[4];
  double* Q;  // [4][Np][K]
};

// InitializeSolution (euler.go:728-794): the isentropic vortex at t = 0
// (analytic_vortex.go:31-82), the Sod states split at x = 0.5, or the far field.
__global__ void k_initial_state(InitArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const size_t sK = static_cast<size_t>(a.K);
  for (int i = 0; i < a.Np; ++i) {
    double q[4];
    double x, y;
    element_point_dev(a.vx, a.vy, a.etov, k, a.rs[2 * i], a.rs[2 * i + 1], &x, &y);
    if (a.init == GCFD_INIT_IVORTEX) {
      const double pi = 3.14159265358979323846, g = a.vgamma, GM1 = g - 1.0;
      double u = 1.0, v = 0.0;
      const double r2 = (x - a.vx0) * (x - a.vx0) + (y - a.vy0) * (y - a.vy0);
      const double ex1r = exp(1.0 - r2);
      const double tv1 = 1.0 - (GM1 * a.vbeta * a.vbeta * exp(2.0 * (1.0 - r2)) / (16.0 * g * pi * pi));
      u -= a.vbeta * ex1r * (y - a.vy0) * (0.5 / pi);
      v += a.vbeta * ex1r * (x - a.vx0) * (0.5 / pi);
      const double rho = pow(tv1, 1.0 / GM1), p = pow(rho, g);
      q[0] = rho;
      q[1] = rho * u;
      q[2] = rho * v;
      q[3] = p * (1.0 / GM1) + 0.5 * rho * (u * u + v * v);
    } else if (a.init == GCFD_INIT_SHOCKTUBE) {
      const double* src = (x < 0.5) ? a.qIn : a.qOut;
      for (int n = 0; n < 4; ++n) q[n] = src[n];
    } else {
      for (int n = 0; n < 4; ++n) q[n] = a.qFar[n];
    }
    for (int n = 0; n < 4; ++n) a.Q[(static_cast<size_t>(n) * a.Np + i) * sK + k] = q[n];
  }
}

int grid(int n) { return (n + 127) / 128; }

}  // namespace

int device_geometry(gcfd_ctx* c, const gcfd_mesh* m, const std::vector<int>& kL, const std::vector<int>& kR,
                    const std::vector<int>& eLR) {
  const int K = c->K, nE = c->nEdges;
  int rc;
  std::vector<double> vx(m->vx, m->vx + m->nverts), vy(m->vy, m->vy + m->nverts);
  std::vector<int32_t> ev(m->etov, m->etov + 3 * static_cast<size_t>(K));
  std::vector<double> rs(2 * static_cast<size_t>(c->Np));
  for (int i = 0; i < c->Np; ++i) {
    rs[2 * i] = c->el.r[i];
    rs[2 * i + 1] = c->el.s[i];
  }
  if ((rc = upload(c, &c->dVX, vx))) return rc;
  if ((rc = upload(c, &c->dVY, vy))) return rc;
  if ((rc = upload(c, &c->dEToV, ev))) return rc;
  if ((rc = upload(c, &c->dRS, rs))) return rc;
  for (double** p : {&c->Jdet, &c->dhK})
    if ((rc = dalloc(c, p, static_cast<size_t>(K)))) return rc;
  if ((rc = dalloc(c, &c->Jinv, 4 * static_cast<size_t>(K)))) return rc;
  for (double** p : {&c->dnxE, &c->dnyE, &c->dIIE})
    if ((rc = dalloc(c, p, 3 * static_cast<size_t>(K)))) return rc;
  int* bad = nullptr;
  if ((rc = dalloc(c, &bad, 2))) return rc;
  const int bad0[2] = {0, K};
  GCFD_CUDA(c, cudaMemcpyAsync(bad, bad0, sizeof(bad0), cudaMemcpyHostToDevice, c->stream));
  ElemGeoArgs a{K, c->N, c->dVX, c->dVY, c->dEToV, c->Jdet, c->Jinv, c->dnxE, c->dnyE, c->dIIE, c->dhK, bad};
  k_geo_elements<<<grid(K), 128, 0, c->stream>>>(a);
  GCFD_CUDA(c, cudaGetLastError());
  int hb[2];
  GCFD_CUDA(c, cudaMemcpyAsync(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, c->stream));
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  if (hb[0] > 0)
    return fail(c, GCFD_ERR_ARG, "element " + std::to_string(hb[1]) + " is not counter-clockwise (|J| <= 0)");
  if ((rc = upload(c, &c->ekL, kL))) return rc;
  if ((rc = upload(c, &c->ekR, kR))) return rc;
  if ((rc = upload(c, &c->eLR, eLR))) return rc;
  for (double** p : {&c->enx, &c->eny, &c->eIIL, &c->eIIR, &c->eoohK})
    if ((rc = dalloc(c, p, static_cast<size_t>(nE)))) return rc;
  k_geo_edges<<<grid(nE), 128, 0, c->stream>>>(nE, c->nInt, K, c->ekL, c->ekR, c->eLR, c->dnxE, c->dnyE, c->dIIE,
                                               c->dhK, c->enx, c->eny, c->eIIL, c->eIIR, c->eoohK);
  GCFD_CUDA(c, cudaGetLastError());
  return GCFD_OK;
}

int device_geometry_mixed(gcfd_ctx* c) {
  const int K = c->K, nE = c->nEdges;
  int rc;
  if ((rc = dalloc(c, &c->mgeo, 6 * static_cast<size_t>(K)))) return rc;
  if ((rc = dalloc(c, &c->mII, 3 * static_cast<size_t>(K)))) return rc;
  for (float** p : {&c->mnx, &c->mny, &c->moohK})
    if ((rc = dalloc(c, p, static_cast<size_t>(nE)))) return rc;
  k_geo_mixed<<<grid(std::max(K, nE)), 128, 0, c->stream>>>(K, nE, c->Jdet, c->Jinv, c->dIIE, c->enx, c->eny,
                                                             c->eoohK, c->mgeo, c->mII, c->mnx, c->mny, c->moohK);
  GCFD_CUDA(c, cudaGetLastError());
  return GCFD_OK;
}

int device_solution_points(gcfd_ctx* c, double** X, double** Y) {
  int rc;
  const size_t n = static_cast<size_t>(c->Np) * c->K;
  if ((rc = dalloc(c, X, n))) return rc;
  if ((rc = dalloc(c, Y, n))) return rc;
  k_solution_points<<<grid(c->K), 128, 0, c->stream>>>(c->K, c->Np, c->dVX, c->dVY, c->dEToV, c->dRS, *X, *Y);
  GCFD_CUDA(c, cudaGetLastError());
  return GCFD_OK;
}

int device_initial_state(gcfd_ctx* c) {
  InitArgs a;
  a.K = c->K;
  a.Np = c->Np;
  a.init = c->prm.init_type;
  a.vx = c->dVX;
  a.vy = c->dVY;
  a.etov = c->dEToV;
  a.rs = c->dRS;
  a.vx0 = c->vx0;
  a.vy0 = c->vy0;
  a.vbeta = c->vbeta;
  a.vgamma = c->vgamma;
  for (int n = 0; n < 4; ++n) {
    a.qFar[n] = c->fsFar.qinf[n];
    a.qIn[n] = c->fsIn.qinf[n];
    a.qOut[n] = c->fsOut.qinf[n];
  }
  a.Q = c->Q[0];
  k_initial_state<<<grid(c->K), 128, 0, c->stream>>>(a);
  GCFD_CUDA(c, cudaGetLastError());
  return GCFD_OK;
}

}  // namespace gcfd_host
