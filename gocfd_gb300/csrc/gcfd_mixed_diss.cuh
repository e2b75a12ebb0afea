// PerssonC0 shock capturing on the mixed path, on the compensated FP32 state
// itself (no FP64 stage state): the Euler RHS stays in the FP32 delta form
// (k_mixed_stage with rhsOnly); the sensor's products (on the stage density),
// the rkStep-2 limiter and the RT gradient work on the element deltas
// dq = dQ0 + D_s - D_s(point 0); the viscous edge fluxes, AddDissipation and
// the modal RHS filter run in FP32; the sensor's log10 and sine ramp and the
// vertex maxima stay FP64.  k_mixed_diss_update adds the dissipation, filters,
// applies the viscous time-step limit and performs the mixed stage update
// (stage_tail).
#pragma once
#include "gcfd_diss.cuh"
#include "gcfd_mixed.cuh"

namespace gcfd {

// The modal filter's operators (V, V^-1, the mode filter) in constant memory,
// one copy per order N, for the same reason as the divergence operator.
static __constant__ float cV0[Dims<0>::NP * Dims<0>::NP], cV1[Dims<1>::NP * Dims<1>::NP],
    cV2[Dims<2>::NP * Dims<2>::NP], cV3[Dims<3>::NP * Dims<3>::NP], cV4[Dims<4>::NP * Dims<4>::NP];
static __constant__ float cVi0[Dims<0>::NP * Dims<0>::NP], cVi1[Dims<1>::NP * Dims<1>::NP],
    cVi2[Dims<2>::NP * Dims<2>::NP], cVi3[Dims<3>::NP * Dims<3>::NP], cVi4[Dims<4>::NP * Dims<4>::NP];
static __constant__ float cMf0[Dims<0>::NP], cMf1[Dims<1>::NP], cMf2[Dims<2>::NP], cMf3[Dims<3>::NP],
    cMf4[Dims<4>::NP];
template <int N>
__device__ __forceinline__ float v_op(int i) {
  if constexpr (N == 0) return cV0[i];
  else if constexpr (N == 1) return cV1[i];
  else if constexpr (N == 2) return cV2[i];
  else if constexpr (N == 3) return cV3[i];
  else return cV4[i];
}
template <int N>
__device__ __forceinline__ float vi_op(int i) {
  if constexpr (N == 0) return cVi0[i];
  else if constexpr (N == 1) return cVi1[i];
  else if constexpr (N == 2) return cVi2[i];
  else if constexpr (N == 3) return cVi3[i];
  else return cVi4[i];
}
template <int N>
__device__ __forceinline__ float mf_op(int i) {
  if constexpr (N == 0) return cMf0[i];
  else if constexpr (N == 1) return cMf1[i];
  else if constexpr (N == 2) return cMf2[i];
  else if constexpr (N == 3) return cMf3[i];
  else return cMf4[i];
}
// limitAndFilterSolution's filter u <- V diag(mf (1 - alpha)) V^-1 u for
// modes >= 1, in FP32 with constant-bank operators.
template <int N>
__device__ __forceinline__ void limit_filter_modal_c(float u[Dims<N>::NP], float alpha) {
  constexpr int NP = Dims<N>::NP;
  float m[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < NP; ++j) acc = fmaf(vi_op<N>(i * NP + j), u[j], acc);
    m[i] = acc;
  }
#pragma unroll
  for (int i = 1; i < NP; ++i) m[i] *= mf_op<N>(i) * (1.0f - alpha);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < NP; ++j) acc = fmaf(v_op<N>(i * NP + j), m[j], acc);
    u[i] = acc;
  }
}

// The stage-s deltas of variable n of element k relative to its stage state
// at solution point 0: dQ0 + (D_s - D_s(point 0)), as the stage kernel forms
// them (stage <= 0: dQ0).
template <int N>
__device__ __forceinline__ void stage_deltas(const MixedArgs& a, int n, int k, size_t sK,
                                             float dq[MixedDims<N>::NP]) {
  constexpr int NP = MixedDims<N>::NP;
  const size_t off = static_cast<size_t>(n) * NP * sK + k;
  const float* ds = (a.stage >= 1) ? a.D[a.stage] + off : nullptr;
  const float d0 = ds ? ds[0] : 0.0f;
#pragma unroll
  for (int i = 0; i < NP; ++i) dq[i] = a.dQ0[off + i * sK] + (ds ? ds[i * sK] - d0 : 0.0f);
}

// The shock sensor (k_diss_sensor: UpdateSeMoment, UpdateShockFinderSigma,
// CalculateElementViscosity) with its three Np x Np products in FP32; the
// moment's log10 and the sigma ramp stay in FP64.  FP32 rounding perturbs the
// high-mode energy by ~1e-7 of the density's, i.e. only moments far below the
// ramp (sigma = 0 there either way).
template <int N>
__global__ void __launch_bounds__(128) k_diss_sensor_mixed(DissArgs a, MixedArgs m) {
  constexpr int NP = DissDims<N>::NP;
  __shared__ float sP[NP * NP], sM[NP * NP], sDq[NP * NP];
  stage_operator(sP, a.SensP, NP * NP);
  stage_operator(sM, a.Mass, NP * NP);
  stage_operator(sDq, a.SensD, NP * NP);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const size_t sK = static_cast<size_t>(a.K);
  // The stage density from the mixed state: reference state plus deltas.
  float dq[NP], rho[NP];
  stage_deltas<N>(m, 0, k, sK, dq);
  const float2 b0 = m.base[static_cast<size_t>(k) * 4];
#pragma unroll
  for (int j = 0; j < NP; ++j) rho[j] = b0.x + (b0.y + dq[j]);
  float num = 0.0f, den = 0.0f;
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    float x = 0.0f, y = 0.0f, dq = 0.0f;
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      x = fmaf(sP[i * NP + j], rho[j], x);
      y = fmaf(sM[i * NP + j], rho[j], y);
      dq = fmaf(sDq[i * NP + j], rho[j], dq);
    }
    num = fmaf(dq, x, num);
    den = fmaf(rho[i], y, den);
  }
  const double se = log10(static_cast<double>(num) / static_cast<double>(den));
  const double left = a.S0 - a.kappa, right = a.S0 + a.kappa;
  double sigma = 0.0;  // a NaN moment keeps sigma = 0
  if (se < left) sigma = 0.0;
  else if (se >= left && se <= right) sigma = 0.5 * (1.0 + sin(3.14159265358979323846 * (0.5 / a.kappa) * (se - a.S0)));
  else if (se > right) sigma = 1.0;
  const double eps = a.eps0 * a.hK[k] * sigma;
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const int vert = a.etov[v * sK + k];
    atomicMax(&a.sigV[vert], static_cast<unsigned long long>(__double_as_longlong(sigma)));
    atomicMax(&a.epsV[vert], static_cast<unsigned long long>(__double_as_longlong(eps)));
  }
}

// The rkStep-2 modal limiter (k_diss_limit, limitAndFilterSolution) on the
// mixed stage state, in FP32 on the deltas dq = U - U_0: the filter keeps mode
// 0 (the constant), so filter(U) = U_0 + filter(dq).  The limited state goes
// back into the stage-2 increment, D2'_i = D2_0 + dq'_i - dQ0_i, with the
// faces and reference state rebuilt from it.  One thread per (element,
// variable), 32 x 4 per CTA.
template <int N>
__global__ void __launch_bounds__(128) k_mixed_limit(DissArgs d, MixedArgs a) {
  constexpr int NP = DissDims<N>::NP, NPP = MixedDims<N>::NPP;
  const int n = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + (threadIdx.x & 31);
  if (k >= a.K) return;
  const size_t sK = static_cast<size_t>(a.K);
  const size_t off = static_cast<size_t>(n) * NP * sK + k;
  const float alpha = static_cast<float>(sin(0.5 * 3.14159265358979323846 * element_sigma(d, k, sK)));
  float dq[NP];
  stage_deltas<N>(a, n, k, sK, dq);
  limit_filter_modal_c<N>(dq, alpha);
  const float d20 = a.D[2][off];
  float dqn[NPP];
#pragma unroll
  for (int r = 0; r < NPP; ++r) dqn[r] = 0.0f;
#pragma unroll
  for (int r = 0; r < NP; ++r) {
    a.D[2][off + r * sK] = d20 + (dq[r] - a.dQ0[off + r * sK]);
    dqn[r] = dq[r] - dq[0];
  }
  int es[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) es[e] = a.eslot[e * sK + k];
  write_faces<N>(a, es, n, dqn);
  float h = a.Qhi[off], l = a.Qlo[off];
  df_add(h, l, d20 + (dq[0] - a.dQ0[off]));
  a.base[static_cast<size_t>(k) * 4 + n] = make_float2(h, l);
}

// eps * grad(Q) at the interior and edge flux points (k_diss_grad,
// CalculateEpsilonGradient, dissipation.go:244-272) in FP32.  The RT gradient
// of a constant field is zero, so it is taken of U - U_0 (U_0 the element's
// value at solution point 0, subtracted in FP64): the rounding then scales with
// the variation of U across the element, not with U; the deltas are the mixed
// state's own (dQ0 + D_s - D_s(point 0)).  FP32 rows out (DissX32 / DissY32).
template <int N>
__global__ void __launch_bounds__(128) k_diss_grad_mixed(DissArgs a, MixedArgs m) {
  constexpr int NP = DissDims<N>::NP, NE = DissDims<N>::NE, NE3 = DissDims<N>::NE3;
  constexpr int NF = DissDims<N>::NF, NR = DissDims<N>::NR;
  extern __shared__ float smf32[];
  float* sDiv = smf32;          // NF x NF
  float* sB = smf32 + NF * NF;  // NF x 3
  stage_operator(sDiv, a.Div, NF * NF);
  stage_operator(sB, a.Bary, NF * 3);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const size_t sK = static_cast<size_t>(a.K);
  const float J0 = static_cast<float>(a.Jinv[k]), J1 = static_cast<float>(a.Jinv[sK + k]);
  const float J2 = static_cast<float>(a.Jinv[2 * sK + k]), J3 = static_cast<float>(a.Jinv[3 * sK + k]);
  const double ooJd = 1.0 / a.Jdet[k];
  constexpr int NEP = (NE + 1) & ~1;
  float ev[3], mx[3], my[3];
  int eg[3], kl[3];
  bool own[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) ev[v] = static_cast<float>(vdouble(a.epsV, a.etov[v * sK + k]));
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int slot = a.eslot32[e * sK + k];
    eg[e] = slot >> 1;
    own[e] = (slot & 1) == 0;
    kl[e] = a.ekL[eg[e]];
    const double ii = a.IIE[e * sK + k];
    mx[e] = static_cast<float>(ooJd * a.nxE[e * sK + k] * ii);
    my[e] = static_cast<float>(ooJd * a.nyE[e * sK + k] * ii);
  }
#pragma unroll 1
  for (int n = 0; n < 4; ++n) {
    const float2 b0 = m.base[static_cast<size_t>(k) * 4 + n];
    const double u0 = static_cast<double>(b0.x) + static_cast<double>(b0.y);
    float U[NP], Ue[NE3];
    stage_deltas<N>(m, n, k, sK, U);
    // The stored left states (the left element's faces, this element's order):
    // its reference state plus its FP32 face deltas.
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const float2 bl = a.base32[static_cast<size_t>(kl[e]) * 4 + n];
      const float shift = static_cast<float>((static_cast<double>(bl.x) + static_cast<double>(bl.y)) - u0);
      const float* fl = a.faces32 + (static_cast<size_t>(eg[e]) * 8 + n) * NEP;
#pragma unroll
      for (int p = 0; p < NE; ++p) Ue[e * NE + p] = shift + fl[own[e] ? p : NE - 1 - p];
    }
#pragma unroll 1
    for (int rr = 0; rr < NR; ++rr) {
      const int r = rr < NP ? rr : 2 * NP + (rr - NP);
      const float* row = sDiv + r * NF;
      float A = 0.0f, B = 0.0f, C[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int j = 0; j < NP; ++j) {
        A = fmaf(row[j], U[j], A);
        B = fmaf(row[NP + j], U[j], B);
      }
#pragma unroll
      for (int e = 0; e < 3; ++e)
#pragma unroll
        for (int p = 0; p < NE; ++p) C[e] = fmaf(row[2 * NP + e * NE + p], Ue[e * NE + p], C[e]);
      const float gx = J0 * A + J2 * B + mx[0] * C[0] + mx[1] * C[1] + mx[2] * C[2];
      const float gy = J1 * A + J3 * B + my[0] * C[0] + my[1] * C[1] + my[2] * C[2];
      const float epsr = sB[r * 3] * ev[0] + sB[r * 3 + 1] * ev[1] + sB[r * 3 + 2] * ev[2];
      a.DissX32[(n * NR + rr) * sK + k] = gx * epsr;
      a.DissY32[(n * NR + rr) * sK + k] = gy * epsr;
    }
  }
}

// Viscous normal flux and viscous wave speed per mesh edge (k_diss_edge,
// StoreEdgeViscousFlux edges.go:151-244) in FP32 from the FP32 gradient rows;
// the penalty's jump comes from the FP32 face deltas of the left element (its
// reference state cancels).  The wave-speed maximum is stored as FP64.
template <int N>
__global__ void __launch_bounds__(128) k_diss_edge_mixed(DissArgs a) {
  constexpr int NP = DissDims<N>::NP, NE = DissDims<N>::NE;
  constexpr int NF = DissDims<N>::NF, NR = DissDims<N>::NR, NEP = (NE + 1) & ~1;
  __shared__ float sB[NF * 3];
  stage_operator(sB, a.Bary, NF * 3);
  __syncthreads();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  float vmax = 0.0f;
  if (g < a.nInt + a.nBC) {
    const size_t sK = static_cast<size_t>(a.K);
    const int kL = a.ekL[g], eL = a.eLR[g] & 3;
    const float nx = static_cast<float>(a.enx[g]), ny = static_cast<float>(a.eny[g]);
    const float oohK = static_cast<float>(a.eoohK[g]);
    float evL[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) evL[v] = static_cast<float>(vdouble(a.epsV, a.etov[v * sK + kL]));
    float epsL[NE];
    float vm = -3.4028235e38f;
#pragma unroll
    for (int p = 0; p < NE; ++p) {
      const int r = 2 * NP + eL * NE + p;
      epsL[p] = sB[r * 3] * evL[0] + sB[r * 3 + 1] * evL[1] + sB[r * 3 + 2] * evL[2];
      vm = fmaxf(oohK * oohK * epsL[p], vm);
    }
    vmax = vm;
    a.viscSpeed[g] = static_cast<double>(vm);
    float* vf = a.VF32 + static_cast<size_t>(g) * 4 * NE;
    if (g >= a.nInt) {
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          const size_t ind = (n * NR + NP + eL * NE + p) * sK + kL;
          vf[n * NE + p] = nx * a.DissX32[ind] + ny * a.DissY32[ind];
        }
    } else {
      const int kR = a.ekR[g], eR = a.eLR[g] >> 2;
      float evR[3];
#pragma unroll
      for (int v = 0; v < 3; ++v) evR[v] = static_cast<float>(vdouble(a.epsV, a.etov[v * sK + kR]));
      const double len = (eL == 1) ? 2.0 * sqrt(2.0) * a.eIIL[g] : 2.0 * a.eIIL[g];
      const float pen = static_cast<float>(a.omega / len);
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const float* fl = a.faces32 + (static_cast<size_t>(g) * 8 + n) * NEP;  // side 0: left element
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          const size_t indL = (n * NR + NP + eL * NE + p) * sK + kL;
          const size_t indR = (n * NR + NP + eR * NE + (NE - 1 - p)) * sK + kR;
          const float vFL = nx * a.DissX32[indL] + ny * a.DissY32[indL];
          const float vFR = nx * a.DissX32[indR] + ny * a.DissY32[indR];
          const int rR = 2 * NP + eR * NE + (NE - 1 - p);
          const float epsR = sB[rR * 3] * evR[0] + sB[rR * 3 + 1] * evR[1] + sB[rR * 3 + 2] * evR[2];
          const float lam = 0.5f * (epsL[p] + epsR);
          vf[n * NE + p] = 0.5f * (vFL + vFR) - (pen * lam) * (fl[p] - fl[NE - 1 - p]);
        }
      }
    }
  }
  vmax = warp_max(vmax);
  if ((threadIdx.x & 31) == 0)
    atomicMax(a.gvisc,
              static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(fmaxf(vmax, 0.0f)))));
}

// RHS = F(a) (RHS_Euler + DivInt DOF(DissX, DissY, VF) / |J|), the viscous
// time-step limit, then the mixed stage update.  One thread per (element,
// variable); stage -1 writes the dissipated, filtered RHS to rhsOut.
template <int N>
__global__ void __launch_bounds__(128, N >= 4 ? 3 : 5) k_mixed_diss_update(MixedArgs a, UpdateArgs<double> u) {
  constexpr int NP = MixedDims<N>::NP, NE = MixedDims<N>::NE, NE3 = MixedDims<N>::NE3;
  constexpr int NR = NP + NE3;
  __shared__ double sdt;
  const int n = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * 32 + lane;
  const bool active = k < a.K;
  const size_t sK = static_cast<size_t>(a.K);
  const size_t off = static_cast<size_t>(n) * NP * sK + k;
  const int s = a.stage;
  // Local dt with the viscous limit (CalculateLocalDT; DT and DTVisc persist):
  // every variable's thread reads them before the barrier, one writes after.
  double dtLocal = 0.0, dvNew = 0.0;
  if (active && a.localDT && s >= 0) {
    double v = (s == 0) ? -100.0 : a.DT[k];
    double dv = u.DTVisc[k];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const int g = u.elemEdge[e * sK + k];
      v = fmax(v, a.edgeSpeed[g]);
      dv = fmax(dv, u.viscSpeed[g]);
    }
    dtLocal = a.cfl / v;
    if (dv > 1.e-9) {
      dv = u.cdiff / dv;
      dtLocal = fmin(dtLocal, dv);
    }
    dvNew = dv;
  }
  if (threadIdx.x == 0 && needs_global_dt(a, s)) sdt = global_stage_dt(a, s);
  __syncthreads();
  if (needs_global_dt(a, s)) dtLocal = sdt;
  float rmax = -3.4028235e38f, rabs = 0.0f;
  float2 rs2 = make_float2(0.0f, 0.0f);
  if (active) {
    const double Jdd = u.Jdet[k];
    const float Jd = static_cast<float>(Jdd), oojd = static_cast<float>(1.0 / Jdd);
    const float J0 = static_cast<float>(u.Jinv[k]), J1 = static_cast<float>(u.Jinv[sK + k]);
    const float J2 = static_cast<float>(u.Jinv[2 * sK + k]), J3 = static_cast<float>(u.Jinv[3 * sK + k]);
    double sig = 0.0;
#pragma unroll
    for (int v = 0; v < 3; ++v) sig = sig + __longlong_as_double(static_cast<long long>(u.sigV[u.etov[v * sK + k]]));
    const float alpha = static_cast<float>(sin(0.5 * 3.14159265358979323846 * (sig / 3.0)));
    int eg[3], eslot[3];
    float esg[3];
    bool own[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      eg[e] = u.elemEdge[e * sK + k];
      own[e] = u.ekL[eg[e]] == k && (u.eLR[eg[e]] & 3) == e;
      esg[e] = static_cast<float>((own[e] ? 1.0 : -1.0) * u.IIE[e * sK + k]);
      eslot[e] = a.eslot[e * sK + k];
    }
    // AddDissipation (dissipation.go:274-346) in FP32.
    float w[NP];
#pragma unroll
    for (int r = 0; r < NP; ++r) w[r] = 0.0f;
    constexpr int NPP = MixedDims<N>::NPP;  // DivInt[r][j] = div_op<N>(j * NPP + r)
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      const size_t ind = (n * NR + j) * sK + k;
      const float dx = a.DissX32[ind], dy = a.DissY32[ind];
      const float fr = Jd * (J0 * dx + J1 * dy), fs = Jd * (J2 * dx + J3 * dy);
#pragma unroll
      for (int r = 0; r < NP; ++r)
        w[r] = fmaf(div_op<N>(j * NPP + r), fr, fmaf(div_op<N>((NP + j) * NPP + r), fs, w[r]));
    }
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const float* vf = a.VF32 + (static_cast<size_t>(eg[e]) * 4 + n) * NE;
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const float f = vf[own[e] ? p : NE - 1 - p] * esg[e];
#pragma unroll
        for (int r = 0; r < NP; ++r) w[r] = fmaf(div_op<N>((2 * NP + e * NE + p) * NPP + r), f, w[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < NP; ++r) w[r] = static_cast<float>(a.rhsOut[off + r * sK]) + oojd * w[r];
    limit_filter_modal_c<N>(w, alpha);
    float rhs[NP];
#pragma unroll
    for (int r = 0; r < NP; ++r) rhs[r] = w[r];
    if (a.localDT && s >= 0 && n == 0) u.DTVisc[k] = dvNew;
    float dq0[NP], ds[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      dq0[i] = a.dQ0[off + i * sK];
      ds[i] = (s >= 1) ? a.D[s][off + i * sK] : 0.0f;
    }
    stage_tail<N>(a, eslot, n, k, off, sK, s, rhs, dq0, ds, dtLocal, rmax, rabs, rs2);
  }
  if (s == 4) {
    residual_commit(a.sc, n, lane, rmax, rabs, rs2);
  }
}

}  // namespace gcfd
