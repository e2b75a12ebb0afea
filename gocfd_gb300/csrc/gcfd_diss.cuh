// (d) Persson shock sensor, C0 artificial viscosity and the RT-gradient
// dissipation of the FP64 path ("PerssonC0" limiter):
//   UpdateSeMoment                 DG2D/dfr_shock_capturing.go:142-166
//   UpdateShockFinderSigma         model_problems/Euler2D/dissipation.go:491-518
//   CalculateElementViscosity      dissipation.go:397-412
//   MergeElementScalarToVertices   euler.go:1048-1065 (max), MergeVertexScalarToElement
//                                  euler.go:1067-1086 (sum / 3), InterpolateEpsilonSigma
//                                  dissipation.go:219-242 (barycentric stencil :414-449)
//   limitAndFilterSolution         dissipation.go:606-622 (stage state at rkStep 2, RHS every stage)
//   CalculateEpsilonGradient       dissipation.go:244-272, GetSolutionGradientUsingRTElement
//                                  euler.go:864-918, metrics dfr_startup.go:213-254
//   StoreEdgeViscousFlux           edges.go:151-244 (left normal on both sides; the penalty
//                                  jump pairs the stored left face states with themselves reversed)
//   StoreEdgeAggregates (viscous)  edges.go:274-286
//   AddDissipation                 dissipation.go:274-346
//   limitAndFilterSolution on RHSQ dissipation.go:606-622 (every stage)
// One thread per element (sensor, preparation, gradient) or per mesh edge.
// Vertex maxima use atomicMax on the bit patterns of non-negative doubles.
#pragma once
#include "gcfd_kernels.cuh"

namespace gcfd {

struct DissArgs {
  int K, nInt, nBC, stage;
  const double* Qs;           // stage state (rho block used by the sensor)
  double* Qlim;               // stage state to limit in place (rkStep 2)
  double* QF;                 // faces [n][j][k], written here (FP64 path layout)
  const double* Iop;          // FluxEdgeInterp
  const int* etov;            // [3][K]
  const double* hK;           // K
  const double* SensP;        // Np x Np
  const double* Mass;
  const double* SensD;
  const double* V;            // Np x Np
  const double* Vinv;
  const double* mf;           // Np modal filter
  const double* Div;          // NpFlux x NpFlux
  const double* Bary;         // NpFlux x 3
  const double* Jinv;         // [4][K]
  const double* Jdet;         // K
  const double* nxE;          // element-edge outward normals [3][K]
  const double* nyE;
  const double* IIE;          // element-edge IInII [3][K]
  const int* elemEdge;        // [3][K] device edge index
  const int* ekL;             // per device edge
  const int* ekR;
  const int* eLR;
  const double* enx;
  const double* eny;
  const double* eIIL;
  const double* eoohK;
  unsigned long long* sigV;   // per vertex (double bits)
  unsigned long long* epsV;
  double* DissX;              // [4][NR][K], NR = Np + 3 NpEdge (interior rows, then edge rows)
  double* DissY;
  double* VF;                 // [edge][4][NpEdge] viscous normal flux, left order
  double* viscSpeed;          // per edge
  unsigned long long* gvisc;  // per stage max viscous speed
  double kappa, eps0, S0, omega;
  double* sigE;               // optional (adjoint recompute): element sigma, eps and Se
  double* epsE;
  double* SeE;
  // Mixed path: edge-major FP32 face deltas [edge][side][n][NEP] and their
  // reference states [k][n] (hi, lo) stand in for QF.
  const float* faces32;
  const float2* base32;
  const int* eslot32;         // [3][K] edge * 2 + side
  // Mixed path: the gradient rows and viscous fluxes in FP32 (in the FP64 arrays' memory).
  float* DissX32;
  float* DissY32;
  float* VF32;
};

template <int N>
struct DissDims {
  static constexpr int NP = Dims<N>::NP, NE = Dims<N>::NE, NE3 = Dims<N>::NE3, NF = Dims<N>::NF;
  static constexpr int NR = NP + NE3;
};

// Stage 1: sensor moment, sigma ramp, element viscosity, vertex maxima.
template <int N>
__global__ void __launch_bounds__(128) k_diss_sensor(DissArgs a) {
  constexpr int NP = DissDims<N>::NP;
  __shared__ double sP[NP * NP], sM[NP * NP], sDq[NP * NP];
  stage_operator(sP, a.SensP, NP * NP);
  stage_operator(sM, a.Mass, NP * NP);
  stage_operator(sDq, a.SensD, NP * NP);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const size_t sK = static_cast<size_t>(a.K);
  double rho[NP];
#pragma unroll
  for (int j = 0; j < NP; ++j) rho[j] = a.Qs[j * sK + k];
  double num = 0.0, den = 0.0;
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    double x = 0.0, y = 0.0, dq = 0.0;
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      x += sP[i * NP + j] * rho[j];
      y += sM[i * NP + j] * rho[j];
      dq += sDq[i * NP + j] * rho[j];
    }
    num += dq * x;
    den += rho[i] * y;
  }
  const double se = log10(num / den);
  const double left = a.S0 - a.kappa, right = a.S0 + a.kappa;
  double sigma = 0.0;  // a NaN moment (round-off in num) keeps sigma = 0
  if (se < left) sigma = 0.0;
  else if (se >= left && se <= right) sigma = 0.5 * (1.0 + sin(3.14159265358979323846 * (0.5 / a.kappa) * (se - a.S0)));
  else if (se > right) sigma = 1.0;
  const double eps = a.eps0 * a.hK[k] * sigma;
  if (a.sigE) {
    a.sigE[k] = sigma;
    a.epsE[k] = eps;
    a.SeE[k] = se;
  }
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const int vert = a.etov[v * sK + k];
    atomicMax(&a.sigV[vert], static_cast<unsigned long long>(__double_as_longlong(sigma)));
    atomicMax(&a.epsV[vert], static_cast<unsigned long long>(__double_as_longlong(eps)));
  }
}

__device__ __forceinline__ double vdouble(const unsigned long long* p, int i) {
  return __longlong_as_double(static_cast<long long>(p[i]));
}

// Modal limiter/filter of one element's variable: u <- V diag(mf (1 - sin(pi sigma / 2))) Vinv u
// for modes >= 1 (limitAndFilterSolution).
template <int NP>
__device__ __forceinline__ void limit_filter_modal(double u[NP], const double* sV, const double* sVi,
                                                   const double* mf, double alpha) {
  double m[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < NP; ++j) acc += sVi[i * NP + j] * u[j];
    m[i] = acc;
  }
#pragma unroll
  for (int i = 1; i < NP; ++i) m[i] *= mf[i] * (1.0 - alpha);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < NP; ++j) acc += sV[i * NP + j] * m[j];
    u[i] = acc;
  }
}

// Vertex-averaged sigma of element k (MergeVertexScalarToElement, euler.go:1067-1086).
__device__ __forceinline__ double element_sigma(const DissArgs& a, int k, size_t sK) {
  double acc = 0.0;
#pragma unroll
  for (int v = 0; v < 3; ++v) acc = acc + vdouble(a.sigV, a.etov[v * sK + k]);
  return acc / 3.0;
}

// Stage 2 (rkStep 2 only): the modal limiter applied in place to the stage
// state before its faces are interpolated.  One thread per (variable, element).
template <int N>
__global__ void __launch_bounds__(128) k_diss_limit(DissArgs a) {
  constexpr int NP = DissDims<N>::NP;
  __shared__ double sV[NP * NP], sVi[NP * NP], smf[NP];
  stage_operator(sV, a.V, NP * NP);
  stage_operator(sVi, a.Vinv, NP * NP);
  stage_operator(smf, a.mf, NP);
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * a.K) return;
  const int n = t / a.K, k = t - n * a.K;
  const size_t sK = static_cast<size_t>(a.K);
  const double alpha = sin(0.5 * 3.14159265358979323846 * element_sigma(a, k, sK));
  double q[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) q[i] = a.Qlim[(n * NP + i) * sK + k];
  limit_filter_modal<NP>(q, sV, sVi, smf, alpha);
#pragma unroll
  for (int i = 0; i < NP; ++i) a.Qlim[(n * NP + i) * sK + k] = q[i];
}

// Stage 4: eps * grad(Q) at the interior and edge flux points.  With
// DX_j = metric_j U_j (interior: Jinv0 / Jinv2, edges: nx IInII / |J|), the x
// and y gradients share A = Div[:, 0:Np] U, B = Div[:, Np:2Np] U and the edge
// sums C_e, so both come from one pass over Div.
template <int N>
__global__ void __launch_bounds__(128) k_diss_grad(DissArgs a) {
  constexpr int NP = DissDims<N>::NP, NE = DissDims<N>::NE, NE3 = DissDims<N>::NE3;
  constexpr int NF = DissDims<N>::NF, NR = DissDims<N>::NR;
  extern __shared__ double smem[];
  double* sDiv = smem;                 // NF x NF
  double* sB = smem + NF * NF;         // NF x 3
  stage_operator(sDiv, a.Div, NF * NF);
  stage_operator(sB, a.Bary, NF * 3);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const size_t sK = static_cast<size_t>(a.K);
  const double J0 = a.Jinv[k], J1 = a.Jinv[sK + k], J2 = a.Jinv[2 * sK + k], J3 = a.Jinv[3 * sK + k];
  const double ooJd = 1.0 / a.Jdet[k];
  double ev[3], mx[3], my[3];
  int eg[3];
  bool own[3];
  int eLn[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) ev[v] = vdouble(a.epsV, a.etov[v * sK + k]);
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    eg[e] = a.elemEdge[e * sK + k];
    own[e] = a.ekL[eg[e]] == k && (a.eLR[eg[e]] & 3) == e;
    eLn[e] = a.eLR[eg[e]] & 3;
    const double ii = a.IIE[e * sK + k];
    mx[e] = ooJd * a.nxE[e * sK + k] * ii;
    my[e] = ooJd * a.nyE[e * sK + k] * ii;
  }
#pragma unroll 1
  for (int n = 0; n < 4; ++n) {
    double U[NP], Ue[NE3];
#pragma unroll
    for (int i = 0; i < NP; ++i) U[i] = a.Qs[(n * NP + i) * sK + k];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const int kl = a.ekL[eg[e]];
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const int ii = own[e] ? p : NE - 1 - p;  // stored left states, this element's order
        Ue[e * NE + p] = a.QF[(n * NE3 + eLn[e] * NE + ii) * sK + kl];
      }
    }
#pragma unroll 1
    for (int rr = 0; rr < NR; ++rr) {
      const int r = rr < NP ? rr : 2 * NP + (rr - NP);
      const double* row = sDiv + r * NF;
      double A = 0.0, B = 0.0, C[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int j = 0; j < NP; ++j) {
        A += row[j] * U[j];
        B += row[NP + j] * U[j];
      }
#pragma unroll
      for (int e = 0; e < 3; ++e)
#pragma unroll
        for (int p = 0; p < NE; ++p) C[e] += row[2 * NP + e * NE + p] * Ue[e * NE + p];
      const double gx = J0 * A + J2 * B + mx[0] * C[0] + mx[1] * C[1] + mx[2] * C[2];
      const double gy = J1 * A + J3 * B + my[0] * C[0] + my[1] * C[1] + my[2] * C[2];
      const double epsr = sB[r * 3] * ev[0] + sB[r * 3 + 1] * ev[1] + sB[r * 3 + 2] * ev[2];
      a.DissX[(n * NR + rr) * sK + k] = gx * epsr;
      a.DissY[(n * NR + rr) * sK + k] = gy * epsr;
    }
  }
}

// Stage 5: viscous normal flux and viscous wave speed per mesh edge.
template <int N>
__global__ void __launch_bounds__(128) k_diss_edge(DissArgs a) {
  constexpr int NP = DissDims<N>::NP, NE = DissDims<N>::NE, NE3 = DissDims<N>::NE3;
  constexpr int NF = DissDims<N>::NF, NR = DissDims<N>::NR;
  __shared__ double sB[NF * 3];
  stage_operator(sB, a.Bary, NF * 3);
  __syncthreads();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  double vmax = 0.0;
  if (g < a.nInt + a.nBC) {
    const size_t sK = static_cast<size_t>(a.K);
    const int kL = a.ekL[g], eL = a.eLR[g] & 3;
    const double nx = a.enx[g], ny = a.eny[g];
    const double oohK = a.eoohK[g];
    double evL[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) evL[v] = vdouble(a.epsV, a.etov[v * sK + kL]);
    double epsL[NE];
    double vm = -1.7976931348623157e308;
#pragma unroll
    for (int p = 0; p < NE; ++p) {
      const int r = 2 * NP + eL * NE + p;
      epsL[p] = sB[r * 3] * evL[0] + sB[r * 3 + 1] * evL[1] + sB[r * 3 + 2] * evL[2];
      vm = fmax(oohK * oohK * epsL[p], vm);
    }
    vmax = vm;
    a.viscSpeed[g] = vm;
    double* vf = a.VF + static_cast<size_t>(g) * 4 * NE;
    if (g >= a.nInt) {
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          const size_t ind = (n * NR + NP + eL * NE + p) * sK + kL;
          vf[n * NE + p] = nx * a.DissX[ind] + ny * a.DissY[ind];
        }
    } else {
      const int kR = a.ekR[g], eR = a.eLR[g] >> 2;
      double evR[3];
#pragma unroll
      for (int v = 0; v < 3; ++v) evR[v] = vdouble(a.epsV, a.etov[v * sK + kR]);
      const double len = (eL == 1) ? 2.0 * sqrt(2.0) * a.eIIL[g] : 2.0 * a.eIIL[g];
      const double ooLen = 1.0 / len;
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          const size_t indL = (n * NR + NP + eL * NE + p) * sK + kL;
          const size_t indR = (n * NR + NP + eR * NE + (NE - 1 - p)) * sK + kR;
          const double vFL = nx * a.DissX[indL] + ny * a.DissY[indL];
          const double vFR = nx * a.DissX[indR] + ny * a.DissY[indR];
          double v = 0.5 * (vFL + vFR);
          const int rR = 2 * NP + eR * NE + (NE - 1 - p);
          const double epsR = sB[rR * 3] * evR[0] + sB[rR * 3 + 1] * evR[1] + sB[rR * 3 + 2] * evR[2];
          const double lam = 0.5 * (epsL[p] + epsR);
          const double qa = a.QF[(n * NE3 + eL * NE + p) * sK + kL];
          const double qb = a.QF[(n * NE3 + eL * NE + (NE - 1 - p)) * sK + kL];
          v -= (a.omega * lam * ooLen) * (qa - qb);
          vf[n * NE + p] = v;
        }
    }
  }
  vmax = warp_max(vmax);
  if ((threadIdx.x & 31) == 0)
    atomicMax(a.gvisc, static_cast<unsigned long long>(__double_as_longlong(fmax(vmax, 0.0))));
}

// Stage 6: AddDissipation on the Euler RHS that k_div_update left in rhsOut,
// the modal filter of the RHS (limitAndFilterSolution on RHSQ every stage),
// this stage's time step with the viscous limit (CalcElementMaxWaveSpeed +
// calculateGlobalDT / CalculateLocalDT, euler.go:945-1002) and the SSP stage
// update.  One thread per element, one conserved variable at a time.
// stage -1 writes the dissipated, filtered RHS back into rhsOut.
template <int N>
__global__ void __launch_bounds__(128) k_diss_update(UpdateArgs<double> a) {
  constexpr int NP = DissDims<N>::NP, NE = DissDims<N>::NE, NF = DissDims<N>::NF, NR = DissDims<N>::NR;
  __shared__ double sD[NP * NF], sV[NP * NP], sVi[NP * NP], smf[NP];
  stage_operator(sD, a.Div, NP * NF);
  stage_operator(sV, a.V, NP * NP);
  stage_operator(sVi, a.Vinv, NP * NP);
  stage_operator(smf, a.mf, NP);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = k < a.K;
  const size_t sK = static_cast<size_t>(a.K);
  double rloc_max[4], rloc_abs[4], rloc_s2[4];
#pragma unroll
  for (int n = 0; n < 4; ++n) { rloc_max[n] = -1.7976931348623157e308; rloc_abs[n] = 0.0; rloc_s2[n] = 0.0; }
  if (active) {
    const double Jd = a.Jdet[k], oojd = 1.0 / Jd;
    const double J0 = a.Jinv[k], J1 = a.Jinv[sK + k], J2 = a.Jinv[2 * sK + k], J3 = a.Jinv[3 * sK + k];
    double sig = 0.0;
#pragma unroll
    for (int v = 0; v < 3; ++v) sig = sig + __longlong_as_double(static_cast<long long>(a.sigV[a.etov[v * sK + k]]));
    const double alpha = sin(0.5 * 3.14159265358979323846 * (sig / 3.0));
    int eg[3];
    double esg[3];
    bool own[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      eg[e] = a.elemEdge[e * sK + k];
      own[e] = a.ekL[eg[e]] == k && (a.eLR[eg[e]] & 3) == e;
      esg[e] = (own[e] ? 1.0 : -1.0) * a.IIE[e * sK + k];
    }
    double dtk = 0.0;
    if (a.stage >= 0) {
      if (a.localDT) {
        double v = (a.stage == 0) ? -100.0 : a.DT[k];
        double dv = a.DTVisc[k];
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          v = fmax(v, a.edgeSpeed[eg[e]]);
          dv = fmax(dv, a.viscSpeed[eg[e]]);
        }
        dtk = a.cfl / v;
        if (dv > 1.e-9) {
          dv = a.cdiff / dv;
          dtk = fmin(dtk, dv);
        }
        a.DTVisc[k] = dv;
        a.DT[k] = dtk;
      } else {
        const double gm = __longlong_as_double(static_cast<long long>(a.sc->gmax[a.stage]));
        const double gv = __longlong_as_double(static_cast<long long>(a.gvisc[a.stage]));
        dtk = fmin(a.cfl / gm, a.cdiff / gv);
        const double t = a.sc->time;
        if (t + dtk > a.finalTime) dtk = a.finalTime - t;
        if (k == 0) a.sc->dt[a.stage] = dtk;
      }
    }
#pragma unroll 1
    for (int n = 0; n < 4; ++n) {
      double u[NP];
#pragma unroll
      for (int r = 0; r < NP; ++r) u[r] = 0.0;
#pragma unroll 1
      for (int j = 0; j < NP; ++j) {
        const size_t ind = (n * NR + j) * sK + k;
        const double dx = a.DissX[ind], dy = a.DissY[ind];
        const double fr = Jd * (J0 * dx + J1 * dy), fs = Jd * (J2 * dx + J3 * dy);
#pragma unroll
        for (int r = 0; r < NP; ++r) u[r] += sD[r * NF + j] * fr + sD[r * NF + NP + j] * fs;
      }
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        const double* vf = a.VF + (static_cast<size_t>(eg[e]) * 4 + n) * NE;
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          const double f = vf[own[e] ? p : NE - 1 - p] * esg[e];
#pragma unroll
          for (int r = 0; r < NP; ++r) u[r] += sD[r * NF + 2 * NP + e * NE + p] * f;
        }
      }
#pragma unroll
      for (int r = 0; r < NP; ++r) u[r] = a.rhsOut[(n * NP + r) * sK + k] + oojd * u[r];
      if (a.tapeRHSpre) {
#pragma unroll
        for (int r = 0; r < NP; ++r) a.tapeRHSpre[(n * NP + r) * sK + k] = u[r];
      }
      limit_filter_modal<NP>(u, sV, sVi, smf, alpha);
      if (a.stage < 0) {
#pragma unroll
        for (int r = 0; r < NP; ++r) a.rhsOut[(n * NP + r) * sK + k] = u[r];
      } else {
#pragma unroll
        for (int r = 0; r < NP; ++r) {
          if (a.tapeRHS) a.tapeRHS[(n * NP + r) * sK + k] = u[r];
          ssp_stage_update(a, (n * NP + r) * sK + k, u[r], dtk, rloc_max[n], rloc_abs[n], rloc_s2[n]);
        }
      }
    }
  }
  if (a.stage == 4) residual_reduce(a.sc, rloc_max, rloc_abs, rloc_s2);
}

}  // namespace gcfd
