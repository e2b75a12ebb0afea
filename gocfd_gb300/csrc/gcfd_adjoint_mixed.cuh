// Reverse-sweep kernels of the mixed path's adjoint (FP32), in the layout of
// the mixed forward's stage kernel: a block is 32 elements x 4 variables, warp
// n owns variable n, so every row access is a 128-byte coalesced transaction,
// and the operators (DivInt, FluxEdgeInterp) are constant-memory arrays read as
// immediate FMA operands.
//
// k_adj_div32 is k_adj_div (gcfd_adjoint.cuh) for this layout, with two more
// pieces of the stage folded in: the face transpose of the stage after it (the
// adjoint of stage s+1's state, Qb[s+1], still lacks FluxEdgeInterp^T of that
// stage's face adjoints when the kernel of stage s reads it as the stage
// output's adjoint, and Qb[s+1] is read nowhere else, so the sum is formed in
// registers and never stored), and the stage state's faces for the edge
// adjoints (FluxEdgeInterp of Q0 + D_s, from the rows the block reads anyway).
#pragma once
#include "gcfd_adjoint.cuh"
#include "gcfd_mixed.cuh"

namespace gcfd {

// Operators of the order this translation unit is built for (one order per
// unit), set by AdjLaunch::mixed_consts, as packed pairs for fma.rn.f32x2
// (ffma2): one instruction updates two outputs, each lane rounding like fmaf.
//   cAdjDivFS[r][i]   (DivInt[r][i], DivInt[r][NP + i]): the r- and s-flux adjoints of point i
//   cAdjDivE[r][q]    (DivInt[r][2NP + 2q], DivInt[r][2NP + 2q + 1]): edge DOFs 2q, 2q + 1
//   cAdjCSFS, cAdjCSE the same pairs of DivInt's column sums (FP64, rounded)
//   cAdjIopT[j][h]    (FluxEdgeInterp[j][2h], FluxEdgeInterp[j][2h + 1]): FluxEdgeInterp^T
//   cAdjIop[i][q]     (FluxEdgeInterp[2q][i], FluxEdgeInterp[2q + 1][i]): the faces
// (zero past the last row or column).
template <int N>
struct AdjDims {
  static constexpr int NP = Dims<N>::NP, NE3 = Dims<N>::NE3, NF = Dims<N>::NF;
  static constexpr int NEH = (NE3 + 1) / 2, NPH = (NP + 1) / 2;
};
static __constant__ float2 cAdjDivFS[AdjDims<4>::NP * AdjDims<4>::NP];
static __constant__ float2 cAdjDivE[AdjDims<4>::NP * AdjDims<4>::NEH];
static __constant__ float2 cAdjCSFS[AdjDims<4>::NP];
static __constant__ float2 cAdjCSE[AdjDims<4>::NEH];
static __constant__ float2 cAdjIopT[AdjDims<4>::NE3 * AdjDims<4>::NPH];
static __constant__ float2 cAdjIop[AdjDims<4>::NP * AdjDims<4>::NEH];

// SSP(5,4) weights on the stage states (rkAdvance, euler.go:511-564) for the
// FP32 reverse sweep.  The transpose carries the step's final-state adjoint to
// its initial state along the weights' "identity" paths, whose sum is exactly
// one in real arithmetic (alpha_s + beta_s = 1, A2 + A3 + A4 = 1).  Rounded to
// FP32 one by one the sum is 1 - 2.3e-8, a drift of 4.6e-6 over 200 steps; these
// are multiples of 2^-24 within 3e-8 of the FP64 weights whose sums are one
// exactly (each pair's member in [0.5, 1] rounded, the other 1 minus it; A3, A4
// rounded, A2 = 1 - A3 - A4).
constexpr float kAdjQ = 1.0f / 16777216.0f;
__device__ constexpr float kAdjAl[4] = {1.0f, 7455300.0f * kAdjQ, 10403583.0f * kAdjQ, 2987686.0f * kAdjQ};
__device__ constexpr float kAdjBe[4] = {0.0f, 9321916.0f * kAdjQ, 6373633.0f * kAdjQ, 13789530.0f * kAdjQ};
constexpr float kAdjA2 = 8677707.0f * kAdjQ, kAdjA3 = 1611615.0f * kAdjQ, kAdjA4 = 6487894.0f * kAdjQ;

// faces (when not null) receives the stage state's FP32 faces, FluxEdgeInterp
// applied to Q0 + Ds per variable: the linearisation point of the edge
// adjoints that follow.
//
// qbF is the adjoint of the step's final state, which feeds stages 2, 3 and 4
// directly (rkAdvance's A2 Q2 + A3 Q3 + ... + W3 dt R3).  Stage 4 completes it
// in place (its own input, plus the face transpose of the next step's stage 0
// when that is pending), and stages 3 and 2 read it for their shares, so no
// A2 / A3 / W3 dt4 products are stored between the stages; dtK4 is stage 4's
// local dt (local time stepping).
template <int N>
__global__ void __launch_bounds__(128, 7) k_adj_div32(AdjArgs<float> a, const float* __restrict__ geo,
                                                   const float* __restrict__ QFbNext, float* __restrict__ faces,
                                                   float* qbF, const double* __restrict__ dtK4) {
  constexpr int NP = Dims<N>::NP, NE3 = Dims<N>::NE3;
  constexpr int NEH = AdjDims<N>::NEH, NPH = AdjDims<N>::NPH;
  __shared__ float sFx[4][NP][32], sFy[4][NP][32], sC[4][NP][32];
  __shared__ float sDt[4][32];
  const int n = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * 32 + lane;
  const bool active = k < a.K;
  const size_t sK = static_cast<size_t>(a.K);
  const int s = a.stage;
  const size_t off = static_cast<size_t>(n) * NP * sK + k;
  // Qbs is Qb0 at stage 0: its alpha term then joins the point update below
  const bool alias0 = (a.Qbs == a.Qb0);
  float dtb = 0.0f;
  float Jd = 1.0f, J0 = 0.0f, J1 = 0.0f, J2 = 0.0f, J3 = 0.0f, mooj = 0.0f;
  if (active) {
    Jd = geo[k];
    J0 = geo[sK + k];
    J1 = geo[2 * sK + k];
    J2 = geo[3 * sK + k];
    J3 = geo[4 * sK + k];
    mooj = -geo[5 * sK + k];
    float qb[NP];
#pragma unroll
    for (int r = 0; r < NP; ++r) qb[r] = a.Qbn[off + r * sK];
    if (QFbNext) {  // + FluxEdgeInterp^T of the later stage's face adjoints
      float f[NE3];
#pragma unroll
      for (int j = 0; j < NE3; ++j) f[j] = QFbNext[(static_cast<size_t>(n) * NE3 + j) * sK + k];
#pragma unroll
      for (int h = 0; h < NPH; ++h) {
        float2 acc = make_float2(qb[2 * h], 2 * h + 1 < NP ? qb[2 * h + 1] : 0.0f);
#pragma unroll
        for (int j = 0; j < NE3; ++j) acc = ffma2(cAdjIopT[j * NPH + h], make_float2(f[j], f[j]), acc);
        qb[2 * h] = acc.x;
        if (2 * h + 1 < NP) qb[2 * h + 1] = acc.y;
      }
    }
    // the SSP stage combination in reverse (k_adj_div's first part)
    float Rb[NP];
    if (s < 0) {
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        Rb[r] = qb[r];
        sC[n][r][lane] = 0.0f;
      }
    } else if (s == 4) {
      const float dt4 = static_cast<float>(a.localDT ? a.dtK[k] : a.dtS[4]);
      const float A4 = kAdjA4, W3 = kSSP[4][3], C4 = kSSP[4][4];
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        const size_t ind = off + r * sK;
        Rb[r] = C4 * dt4 * qb[r];
        if (QFbNext) qbF[ind] = qb[r];  // completed (otherwise it is qbF already)
        dtb += qb[r] * (W3 * a.rhs3[ind] + C4 * a.rhs[ind]);
        sC[n][r][lane] = A4 * qb[r];
      }
    } else {
      double ald, bed, gad;
      stage_coeffs(s, ald, bed, gad);
      const float al = kAdjAl[s], be = kAdjBe[s], ga = static_cast<float>(gad);
      const float dt = static_cast<float>(a.localDT ? a.dtK[k] : a.dtS[s]);
      const float W3dt4 = (s == 3) ? kSSP[4][3] * static_cast<float>(a.localDT ? dtK4[k] : a.dtS[4]) : 0.0f;
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        const size_t ind = off + r * sK;
        Rb[r] = ga * dt * qb[r] + (s == 3 ? W3dt4 * qbF[ind] : 0.0f);
        dtb += ga * qb[r] * a.rhs[ind];
        if (!alias0) {
          if (s == 3) a.Qb0[ind] = al * qb[r];
          else a.Qb0[ind] += al * qb[r];
        }
        sC[n][r][lane] = be * qb[r] + (alias0 ? al * qb[r] : 0.0f);
      }
    }
    // DivInt^T in delta form: with b = Rb[0],
    //   sum_r D[r][j] Rb[r] = sum_r D[r][j] (Rb[r] - b) + b colsum_j,
    // the column sums exact in FP64 (zero for the interior RT functions, whose
    // divergence integrates to zero).  DivInt's entries reach |D| ~ 4e2 (N = 4)
    // and 1.2e3 (N = 1) while a smooth Rb's products cancel to ~h |grad Rb|;
    // in delta form the FP32 rounding scales with Rb - b instead of Rb.
    const float b0 = Rb[0];
#pragma unroll
    for (int r = 1; r < NP; ++r) Rb[r] -= b0;
    // the edge-DOF adjoints of this variable, and its interior transformed-flux
    // adjoints (to the point phase through shared memory)
#pragma unroll
    for (int q = 0; q < NEH; ++q) {
      float2 e = make_float2(b0 * cAdjCSE[q].x, b0 * cAdjCSE[q].y);
#pragma unroll
      for (int r = 1; r < NP; ++r) e = ffma2(cAdjDivE[r * NEH + q], make_float2(Rb[r], Rb[r]), e);
      a.FEb[(static_cast<size_t>(n) * NE3 + 2 * q) * sK + k] = mooj * e.x;
      if (2 * q + 1 < NE3) a.FEb[(static_cast<size_t>(n) * NE3 + 2 * q + 1) * sK + k] = mooj * e.y;
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      float2 f = make_float2(b0 * cAdjCSFS[i].x, b0 * cAdjCSFS[i].y);
#pragma unroll
      for (int r = 1; r < NP; ++r) f = ffma2(cAdjDivFS[r * NP + i], make_float2(Rb[r], Rb[r]), f);
      const float fr = f.x * mooj, fs = f.y * mooj;
      sFx[n][i][lane] = Jd * (J0 * fr + J2 * fs);
      sFy[n][i][lane] = Jd * (J1 * fr + J3 * fs);
    }
    if (faces) {
      float q[NP];
#pragma unroll
      for (int i = 0; i < NP; ++i) q[i] = stage_value(a, off + i * sK);
#pragma unroll
      for (int h = 0; h < NEH; ++h) {
        float2 fc = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int i = 0; i < NP; ++i) fc = ffma2(cAdjIop[i * NEH + h], make_float2(q[i], q[i]), fc);
        faces[(static_cast<size_t>(n) * NE3 + 2 * h) * sK + k] = fc.x;
        if (2 * h + 1 < NE3) faces[(static_cast<size_t>(n) * NE3 + 2 * h + 1) * sK + k] = fc.y;
      }
    }
  }
  sDt[n][lane] = dtb;
  __syncthreads();
  if (s >= 0 && a.localDT) {
    if (n == 0 && active) a.dtOwnK[k] = static_cast<double>((sDt[0][lane] + sDt[1][lane]) + (sDt[2][lane] + sDt[3][lane]));
  } else if (s >= 0) {
    const double t = warp_sum(active ? static_cast<double>(dtb) : 0.0);
    if (lane == 0) atomicAdd(&a.dtbarG[s], t);
  }
  if (!active) return;
  // point phase: warp w takes points w, w + 4, ...; the interior flux Jacobian^T
  // needs all four variables of a point
  const bool first = (s == 1 || s == 4);  // first writers of Qbs
  // stages 2 and 3 start from their share of the final state's adjoint
  const float Aw = (s == 2) ? kAdjA2 : kAdjA3;
  const bool fromF = (s == 2 || s == 3);
  for (int i = n; i < NP; i += 4) {
    float q[4], Fxb[4], Fyb[4], qbp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const size_t ind = (static_cast<size_t>(m) * NP + i) * sK + k;
      q[m] = stage_value(a, ind);
      Fxb[m] = sFx[m][i][lane];
      Fyb[m] = sFy[m][i][lane];
    }
    euler_flux_vjp(a.gas, q, Fxb, Fyb, qbp);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const size_t ind = (static_cast<size_t>(m) * NP + i) * sK + k;
      const float v = sC[m][i][lane] + qbp[m];
      a.Qbs[ind] = first ? v : (fromF ? Aw * qbF[ind] : a.Qbs[ind]) + v;
    }
  }
}

}  // namespace gcfd
