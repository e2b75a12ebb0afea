// Mixed-precision ("delta form") DFR right-hand side and SSP(5,4) step.
//
// Arithmetic: every element carries a reference state Qb = the stage state at
// its solution point 0 (a compensated FP32 pair).  The RT divergence of a
// constant flux is zero
// (DivInt * dofs(const) = 0), so the RHS is computed from
//     dF = F(Q) - F(Qb)          at the interior points, and
//     fhat - n.F(Qb)             at the edge points,
// with exact delta-flux algebra in FP32 on dQ = Q - Qb.  Rounding errors then
// scale with |dQ| ~ h |grad Q| instead of |Q|, which is what keeps FP32 GEMMs
// against the reference's ill-conditioned DivInt within the FP64 result.
//
// State: the conserved state Q0 is accumulated in compensated FP32 (a hi/lo
// float pair per value, ~48 significant bits), which keeps the step free of
// FP64 instructions - GB300's FP64 pipe runs at 1/64 of the FP32 rate.  The
// FP64 copy of Q0 is rebuilt from hi + lo whenever the caller reads it.
// SSP(5,4) stage k is stored as the FP32 increment D_k = Q_k - Q0: the stage
// weights on (Q0, Q_k) sum to one (euler.go:511-564), so Q_{k+1} = Q0 + b D_k +
// c dt RHS exactly, and the final increment R = a2 D2 + a3 D3 + a4 D4 + ... is
// added to Q0 once per step.
//
// Layouts (HBM):
//   Qhi/Qlo[n][i][k] FP32 pair (state), dQ0[n][i][k] = Q0 - Q0(point 0) FP32,
//   D1..D4, R3 FP32 stage increments / stage-3 RHS,
//   P23 = A2 D2 + A3 D3 FP32 (formed at stage 2, read at stage 4)
//   faces[g][side][n][p]  FP32 dQ at edge points, side 0 = left element's CCW
//                         order, side 1 = right element's CCW order; p padded
//                         to NEP = NpEdge rounded up to even
//   fhat[g][n][p]         FP32 fhat - n_L.F(Qb_L), left order, p padded to NEP
//   corr[g][n]            FP32 n_L.(F(Qb_R) - F(Qb_L))
//   base[k][n]            float2 (hi, lo) Qb of the current stage, gathered by the
//                         edge kernels
// Element kernels run one thread per (element, variable): a block is 32
// elements x 4 variables, warp w owns variable w, so every row access is a
// 128-byte coalesced transaction.  The operators (DivInt^T, FluxEdgeInterp^T)
// are constant-memory arrays per order N, read as immediate operands.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gcfd_kernels.cuh"

namespace gcfd {

// Base-state primitives in FP32.  They only ever multiply deltas, so their own
// FP32 rounding enters the result at second order; no FP64 division needed.
struct BasePrim {
  float rho, m, n, E, u, v, p, H;
};

__device__ __forceinline__ BasePrim base_prim(const float b[4], float gm1) {
  BasePrim s;
  s.rho = b[0];
  s.m = b[1];
  s.n = b[2];
  s.E = b[3];
  const float ir = 1.0f / s.rho;
  s.u = s.m * ir;
  s.v = s.n * ir;
  s.p = gm1 * (s.E - 0.5f * (s.m * s.u + s.n * s.v));
  s.H = s.E + s.p;
  return s;
}

// Velocity and pressure deltas of state Qb + d relative to Qb.
struct DeltaPrim {
  float du, dv, dp;
  float ir;  // 1 / (rho_b + d_rho)
};
__device__ __forceinline__ DeltaPrim delta_prim(const BasePrim& b, const float d[4], float gm1) {
  DeltaPrim r;
  const float ir = __fdividef(1.0f, b.rho + d[0]);  // ~1 ulp; it only scales deltas
  r.ir = ir;
  r.du = (d[1] - b.u * d[0]) * ir;
  r.dv = (d[2] - b.v * d[0]) * ir;
  r.dp = gm1 * (d[3] - 0.5f * (b.m * r.du + d[1] * b.u + d[1] * r.du + b.n * r.dv + d[2] * b.v +
                               d[2] * r.dv));
  return r;
}

// Component c of F_x(Qb + d) - F_x(Qb) and F_y(...) - F_y(Qb) (exact algebra).
__device__ __forceinline__ void delta_flux_c(int c, const BasePrim& b, const float d[4],
                                             const DeltaPrim& q, float* dFx, float* dFy) {
  switch (c) {
    case 0:
      *dFx = d[1];
      *dFy = d[2];
      break;
    case 1:
      *dFx = b.m * q.du + d[1] * b.u + d[1] * q.du + q.dp;
      *dFy = b.n * q.du + d[2] * b.u + d[2] * q.du;
      break;
    case 2:
      *dFx = b.m * q.dv + d[1] * b.v + d[1] * q.dv;
      *dFy = b.n * q.dv + d[2] * b.v + d[2] * q.dv + q.dp;
      break;
    default: {
      const float dH = d[3] + q.dp;
      *dFx = b.u * dH + q.du * (b.H + dH);
      *dFy = b.v * dH + q.dv * (b.H + dH);
    }
  }
}

// n . (F(Qb + d) - F(Qb)) for all four components.
__device__ __forceinline__ void delta_normal_flux(const BasePrim& b, const float d[4], float nx,
                                                  float ny, float gm1, float out[4]) {
  const DeltaPrim q = delta_prim(b, d, gm1);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float fx, fy;
    delta_flux_c(c, b, d, q, &fx, &fy);
    out[c] = nx * fx + ny * fy;
  }
}

// Riemann flux minus n.F(Qb), from the two sides' deltas relative to Qb
// (AvgFlux / LaxFlux / RoeFlux of fluxes.go:135-190,284-413 in delta form).
__device__ __forceinline__ void riemann_delta(int kind, const BasePrim& b, const float dL[4],
                                              const float dR[4], float nx, float ny, float gamma,
                                              float f[4]) {
  const float gm1 = gamma - 1.0f;
  float cL[4], cR[4];
  delta_normal_flux(b, dL, nx, ny, gm1, cL);
  delta_normal_flux(b, dR, nx, ny, gm1, cR);
#pragma unroll
  for (int c = 0; c < 4; ++c) f[c] = 0.5f * (cL[c] + cR[c]);
  if (kind == kFluxAverage) return;
  float QL[4], QR[4];
  const float bq[4] = {b.rho, b.m, b.n, b.E};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    QL[c] = bq[c] + dL[c];
    QR[c] = bq[c] + dR[c];
  }
  const Gas<float> g{gamma, gm1, 1.0f / gm1};
  if (kind == kFluxLax) {
    const float uL = QL[1] / QL[0], vL = QL[2] / QL[0], uR = QR[1] / QR[0], vR = QR[2] / QR[0];
    const float CL = sound_speed(g, QL[0], QL[1], QL[2], QL[3]);
    const float CR = sound_speed(g, QR[0], QR[1], QR[2], QR[3]);
    const float maxV = fmaxf(sqrtf(uL * uL + vL * vL) + CL, sqrtf(uR * uR + vR * vR) + CR);
#pragma unroll
    for (int c = 0; c < 4; ++c) f[c] += 0.5f * maxV * (dL[c] - dR[c]);
    return;
  }
  // Roe: averages from the full states, jumps from the deltas.
  const DeltaPrim qL = delta_prim(b, dL, gm1), qR = delta_prim(b, dR, gm1);
  const float rhoL = QL[0], rhoR = QR[0];
  const float uxL = b.u + qL.du, uyL = b.v + qL.dv, uxR = b.u + qR.du, uyR = b.v + qR.dv;
  const float uL = uxL * nx + uyL * ny, vL = -uxL * ny + uyL * nx;
  const float uR = uxR * nx + uyR * ny, vR = -uxR * ny + uyR * nx;
  const float pL = b.p + qL.dp, pR = b.p + qR.dp;
  const float hL = (QL[3] + pL) / rhoL, hR = (QR[3] + pR) / rhoR;
  const float rLs = sqrtf(rhoL), rRs = sqrtf(rhoR), rs = rLs + rRs;
  const float rho = rLs * rRs;
  const float u = (rLs * uL + rRs * uR) / rs;
  const float v = (rLs * vL + rRs * vR) / rs;
  const float h = (rLs * hL + rRs * hR) / rs;
  const float c2 = gm1 * (h - 0.5f * (u * u + v * v));
  const float C = sqrtf(c2);
  const float dun = (qR.du - qL.du) * nx + (qR.dv - qL.dv) * ny;     // uR - uL
  const float dvt = -(qR.du - qL.du) * ny + (qR.dv - qL.dv) * nx;    // vR - vL
  const float dpj = qR.dp - qL.dp;                                    // pR - pL
  const float drj = dR[0] - dL[0];                                    // rhoR - rhoL
  float dW1 = -0.5f * (rho * dun) / C + 0.5f * dpj / c2;
  float dW2 = drj - dpj / c2;
  float dW3 = rho * dvt;
  float dW4 = 0.5f * (rho * dun) / C + 0.5f * dpj / c2;
  dW1 = fabsf(u - C) * dW1;
  dW2 = fabsf(u) * dW2;
  dW3 = fabsf(u) * dW3;
  dW4 = fabsf(u + C) * dW4;
  const float d0 = -0.5f * (dW1 + dW2 + dW4);
  const float d1 = -0.5f * (dW1 * (u - C) + dW2 * u + dW4 * (u + C));
  const float d2 = -0.5f * (dW1 * v + dW2 * v + dW3 + dW4 * v);
  const float d3 = -0.5f * (dW1 * (h - u * C) + 0.5f * dW2 * (u * u + v * v) + dW3 * v + dW4 * (h + u * C));
  f[0] += d0;
  f[1] += nx * d1 - ny * d2;
  f[2] += ny * d1 + nx * d2;
  f[3] += d3;
}

// RoeFlux (fluxes.go:284-413) in delta form, as riemann_delta's Roe branch,
// with one reciprocal per quantity instead of a division per use (the Roe
// averages, 1/C and 1/C^2 each once), plus the left state's wave speed
// |u| + c for the time step from the same primitives.
__device__ __forceinline__ void roe_delta_fast(const BasePrim& b, const float dL[4], const float dR[4],
                                               float nx, float ny, float gamma, float f[4], float* waveL) {
  const float gm1 = gamma - 1.0f;
  const DeltaPrim qL = delta_prim(b, dL, gm1), qR = delta_prim(b, dR, gm1);
  float cL[4], cR[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float fx, fy;
    delta_flux_c(c, b, dL, qL, &fx, &fy);
    cL[c] = nx * fx + ny * fy;
    delta_flux_c(c, b, dR, qR, &fx, &fy);
    cR[c] = nx * fx + ny * fy;
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) f[c] = 0.5f * (cL[c] + cR[c]);
  const float rhoL = b.rho + dL[0], rhoR = b.rho + dR[0];
  const float uxL = b.u + qL.du, uyL = b.v + qL.dv, uxR = b.u + qR.du, uyR = b.v + qR.dv;
  const float uL = uxL * nx + uyL * ny, vL = -uxL * ny + uyL * nx;
  const float uR = uxR * nx + uyR * ny, vR = -uxR * ny + uyR * nx;
  const float pL = b.p + qL.dp, pR = b.p + qR.dp;
  const float hL = (b.E + dL[3] + pL) * qL.ir, hR = (b.E + dR[3] + pR) * qR.ir;
  const float rLs = sqrtf(rhoL), rRs = sqrtf(rhoR);
  const float irs = __fdividef(1.0f, rLs + rRs);
  const float rho = rLs * rRs;
  const float u = (rLs * uL + rRs * uR) * irs;
  const float v = (rLs * vL + rRs * vR) * irs;
  const float h = (rLs * hL + rRs * hR) * irs;
  const float c2 = gm1 * (h - 0.5f * (u * u + v * v));
  const float C = sqrtf(c2);
  const float iC = __fdividef(1.0f, C), ic2 = iC * iC;
  const float dun = (qR.du - qL.du) * nx + (qR.dv - qL.dv) * ny;     // uR - uL
  const float dvt = -(qR.du - qL.du) * ny + (qR.dv - qL.dv) * nx;    // vR - vL
  const float dpj = qR.dp - qL.dp;                                    // pR - pL
  const float drj = dR[0] - dL[0];                                    // rhoR - rhoL
  const float t1 = 0.5f * (rho * dun) * iC, t2 = 0.5f * dpj * ic2;
  float dW1 = t2 - t1;
  float dW2 = drj - dpj * ic2;
  float dW3 = rho * dvt;
  float dW4 = t1 + t2;
  dW1 = fabsf(u - C) * dW1;
  dW2 = fabsf(u) * dW2;
  dW3 = fabsf(u) * dW3;
  dW4 = fabsf(u + C) * dW4;
  const float d0 = -0.5f * (dW1 + dW2 + dW4);
  const float d1 = -0.5f * (dW1 * (u - C) + dW2 * u + dW4 * (u + C));
  const float d2 = -0.5f * (dW1 * v + dW2 * v + dW3 + dW4 * v);
  const float d3 = -0.5f * (dW1 * (h - u * C) + 0.5f * dW2 * (u * u + v * v) + dW3 * v + dW4 * (h + u * C));
  f[0] += d0;
  f[1] += nx * d1 - ny * d2;
  f[2] += ny * d1 + nx * d2;
  f[3] += d3;
  *waveL = sqrtf(uxL * uxL + uyL * uyL) + sqrtf(fabsf(gamma * pL * qL.ir));
}

// ---------------------------------------------------------------------------
// Compensated FP32 arithmetic (Knuth two-sum, Dekker fast-two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
// (hi, lo) += x
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
  float s, e;
  two_sum(hi, x, s, e);
  e += lo;
  fast_two_sum(s, e, hi, lo);
}
// (ah, al) - (bh, bl) rounded to FP32; exact in the leading part whenever the
// two values are within a factor of two (Sterbenz).
__device__ __forceinline__ float df_diff(float ah, float al, float bh, float bl) {
  return (ah - bh) + (al - bl);
}

struct MixedArgs {
  int K, nInt, nBC;
  int stage;
  double* Q0;                 // FP64 state (source after set_state, target of to_fp64)
  float* Qhi;                 // compensated FP32 state
  float* Qlo;
  float* dQ0;                 // Q0 - Q0(point 0)
  float* D[5];                // D[1..4] stage increments (D[0] unused)
  float* R3;                  // stage-3 RHS
  float* P23;                 // A2 D2 + A3 D3 of rkAdvance's last stage, formed at stage 2 for stage 4
  float* faces;               // [g][2][4][NE]
  float* fhat;                // [g][4][NE]
  float* corr;                // [g][4]
  float2* base;               // [k][4] (hi, lo) reference state; updated in place per stage
  const float* geo;           // [6][K]: Jdet, Jinv0..3, 1/Jdet
  const float* II;            // [3][K] IInII
  const int* eslot;           // [3][K] edge id * 2 + side
  // edge kernels
  const int* ekL;
  const int* ekR;
  const float* enx;
  const float* eny;
  const float* eoohK;
  const int* bcFlag;
  const double* bx;
  const double* by;
  double* exBC;               // [nBC][NE][4] exact boundary states of the current step
  double* edgeSpeed;
  unsigned long long* gmax;
  const double* time;
  Scalars* sc;
  double cfl, finalTime;
  int localDT;
  double* DT;
  int flux;
  float gamma;
  double gammaD;
  FreeStreamT<double> fsFar, fsIn, fsOut;
  double vbeta, vx0, vy0, vgamma;
  double* rhsOut;             // stage -1 (or rhsOnly): RHS in FP64 [n][i][k]
  int rhsOnly;                // write the RHS of stage `stage` to rhsOut instead of updating
  const unsigned long long* gviscS;  // per-stage max viscous speed when the dissipation limits dt
  double cdiff;
  const float* Btc;           // tensor-core path: DivInt split hi / lo in the shared-memory operand layout
  const float* BtcF;          // tensor-core path: FluxEdgeInterp split hi / lo, the same layout
  const float* DissX32;       // PerssonC0: FP32 eps-gradient rows [4][NR][K] and viscous fluxes [edge][4][NE]
  const float* DissY32;
  const float* VF32;
  unsigned int* err;          // error flags (bit 0: a tensor-core wait ran out)
  float* tapeRHS;             // adjoint tape: the stage's RHS [n][i][k] (nullptr: not taped)
  float* tapeQ0;              // adjoint tape, stage 4: the step's starting Qhi [n][i][k] (nullptr: not taped)
};

// SSP(5,4) weights of rkAdvance (euler.go:511-564) in increment form:
// D1 = C0 dtR, D_{k+1} = B_k D_k + C_k dtR, R = A2 D2 + A3 D3 + A4 D4 + R3W dtR3 + C4 dtR.
constexpr float kSspC0 = 0.391752226571890f;
constexpr float kSspB1 = 0.555629506348765f, kSspC1 = 0.368410593050371f;
constexpr float kSspB2 = 0.379898148511597f, kSspC2 = 0.251891774271694f;
constexpr float kSspB3 = 0.821920045606868f, kSspC3 = 0.544974750228521f;
constexpr float kSspA2 = 0.517231671970585f, kSspA3 = 0.096059710526146f;
constexpr float kSspA4 = 0.386708617503269f, kSspR3 = 0.063692468666290f;
constexpr float kSspC4 = 0.226007483236906f;

template <int N>
struct MixedDims {
  static constexpr int NP = Dims<N>::NP, NE = Dims<N>::NE, NE3 = Dims<N>::NE3, NF = Dims<N>::NF;
  static constexpr int NPP = (NP + 3) & ~3;  // padded to float4
  // Edge-major stride per (slot, variable): NpEdge rounded up to even, so every
  // (slot, variable) run starts 8-byte aligned and moves as float2.
  static constexpr int NEP = (NE + 1) & ~1;
  // Face interpolation operator, transposed: [NPP][NE3P], face points padded to float4.
  static constexpr int NE3P = (NE3 + 3) & ~3;
  static constexpr int ISZ = NPP * NE3P;
  static constexpr int DSZ = NF * NPP;
};

// The FP32 operators of the mixed path live in constant memory, one copy per
// order N (they depend on N only): DivInt^T [NF][NPP] and FluxEdgeInterp^T
// [NPP][NE3P].  Every warp reads the same entry at the same time, so with the
// loops unrolled each entry is an immediate constant-bank operand of its FMA
// and the element kernels issue no shared-memory loads for them.
static __constant__ float cDivT0[MixedDims<0>::DSZ], cDivT1[MixedDims<1>::DSZ], cDivT2[MixedDims<2>::DSZ],
    cDivT3[MixedDims<3>::DSZ], cDivT4[MixedDims<4>::DSZ];
static __constant__ float cIopT0[MixedDims<0>::ISZ], cIopT1[MixedDims<1>::ISZ], cIopT2[MixedDims<2>::ISZ],
    cIopT3[MixedDims<3>::ISZ], cIopT4[MixedDims<4>::ISZ];

// DivInt[r][j] = div_op<N>(j * NPP + r).
template <int N>
__device__ __forceinline__ float div_op(int idx) {
  if constexpr (N == 0) return cDivT0[idx];
  else if constexpr (N == 1) return cDivT1[idx];
  else if constexpr (N == 2) return cDivT2[idx];
  else if constexpr (N == 3) return cDivT3[idx];
  else return cDivT4[idx];
}
// FluxEdgeInterp[q][i] = iop_op<N>(i * NE3P + q).
template <int N>
__device__ __forceinline__ float iop_op(int idx) {
  if constexpr (N == 0) return cIopT0[idx];
  else if constexpr (N == 1) return cIopT1[idx];
  else if constexpr (N == 2) return cIopT2[idx];
  else if constexpr (N == 3) return cIopT3[idx];
  else return cIopT4[idx];
}

// Packed FP32 pairs: fma.rn.f32x2 (sm_100 and later) performs two independent
// round-to-nearest FMAs in one instruction, so an operator applied to one
// input value updates two outputs per instruction.  Each lane is an ordinary
// fmaf, so a product accumulated through ffma2 rounds exactly like the same
// chain of fmaf calls.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
// (DivInt[2h][j], DivInt[2h+1][j]) = div_pair<N>(j * NPP / 2 + h).
template <int N>
__device__ __forceinline__ float2 div_pair(int idx) {
  if constexpr (N == 0) return reinterpret_cast<const float2*>(cDivT0)[idx];
  else if constexpr (N == 1) return reinterpret_cast<const float2*>(cDivT1)[idx];
  else if constexpr (N == 2) return reinterpret_cast<const float2*>(cDivT2)[idx];
  else if constexpr (N == 3) return reinterpret_cast<const float2*>(cDivT3)[idx];
  else return reinterpret_cast<const float2*>(cDivT4)[idx];
}
// (FluxEdgeInterp[2h][i], FluxEdgeInterp[2h+1][i]) = iop_pair<N>(i * NE3P / 2 + h).
template <int N>
__device__ __forceinline__ float2 iop_pair(int idx) {
  if constexpr (N == 0) return reinterpret_cast<const float2*>(cIopT0)[idx];
  else if constexpr (N == 1) return reinterpret_cast<const float2*>(cIopT1)[idx];
  else if constexpr (N == 2) return reinterpret_cast<const float2*>(cIopT2)[idx];
  else if constexpr (N == 3) return reinterpret_cast<const float2*>(cIopT3)[idx];
  else return reinterpret_cast<const float2*>(cIopT4)[idx];
}
// acc[h] += (DivInt[2h][j], DivInt[2h+1][j]) * v for every output pair h.
template <int N>
__device__ __forceinline__ void div_column(int j, float v, float2 acc[]) {
  constexpr int NH = MixedDims<N>::NPP / 2;
  const float2 vv = make_float2(v, v);
#pragma unroll
  for (int h = 0; h < NH; ++h) acc[h] = ffma2(div_pair<N>(j * NH + h), vv, acc[h]);
}

// Writes the element's 3 edges of face deltas for variable n (face point
// q = e*NE + p): out_q = sum_i FluxEdgeInterp[q][i] dq[i], accumulated over i
// in order.
// Stores the element's 3 edges of face deltas for variable n from the face
// values out[q], q = e*NE + p.
template <int N>
__device__ __forceinline__ void store_faces(const MixedArgs& a, const int eslot[3], int n, const float out[]) {
  constexpr int NE = MixedDims<N>::NE, NEP = MixedDims<N>::NEP;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    float* dst = a.faces + (static_cast<size_t>(eslot[e]) * 4 + n) * NEP;
    // (slot*4 + n) * NEP floats with NEP even: 8-byte aligned, pairs go out as float2.
#pragma unroll
    for (int p = 0; p + 1 < NE; p += 2)
      reinterpret_cast<float2*>(dst)[p / 2] = make_float2(out[e * NE + p], out[e * NE + p + 1]);
    if (NE & 1) dst[NE - 1] = out[e * NE + NE - 1];
  }
}

template <int N>
__device__ __forceinline__ void write_faces(const MixedArgs& a, const int eslot[3], int n, const float dq[]) {
  constexpr int NP = MixedDims<N>::NP, NE3 = MixedDims<N>::NE3;
  constexpr int NE3P = MixedDims<N>::NE3P, NQ = NE3P / 2;
  float2 out[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) out[q] = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    const float2 v = make_float2(dq[i], dq[i]);
#pragma unroll
    for (int q = 0; q < NQ; ++q) out[q] = ffma2(iop_pair<N>(i * NQ + q), v, out[q]);
  }
  float f[NE3];
#pragma unroll
  for (int q = 0; q < NE3; ++q) f[q] = (q & 1) ? out[q >> 1].y : out[q >> 1].x;
  store_faces<N>(a, eslot, n, f);
}

// Stage-0 preparation from the FP64 state: hi/lo split, dQ0, faces, reference states.
// Elements [k0, k1).
template <int N>
__global__ void __launch_bounds__(128) k_mixed_prepare(MixedArgs a, int k0, int k1) {
  constexpr int NP = MixedDims<N>::NP, NPP = MixedDims<N>::NPP;
  const int n = threadIdx.x >> 5;
  const int k = k0 + blockIdx.x * 32 + (threadIdx.x & 31);
  if (k >= k1) return;
  const size_t sK = static_cast<size_t>(a.K);
  const size_t off = static_cast<size_t>(n) * NP * sK + k;
  const double q0 = a.Q0[off];
  float dq[NPP];
#pragma unroll
  for (int i = 0; i < NPP; ++i) dq[i] = 0.0f;
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    const double q = a.Q0[off + i * sK];
    const float hi = static_cast<float>(q);
    a.Qhi[off + i * sK] = hi;
    a.Qlo[off + i * sK] = static_cast<float>(q - static_cast<double>(hi));
    dq[i] = static_cast<float>(q - q0);
    a.dQ0[off + i * sK] = dq[i];
  }
  const float h0 = static_cast<float>(q0);
  a.base[static_cast<size_t>(k) * 4 + n] = make_float2(h0, static_cast<float>(q0 - static_cast<double>(h0)));
  int es[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) es[e] = a.eslot[e * sK + k];
  write_faces<N>(a, es, n, dq);
}

// FP64 copy of the compensated state, for gcfd_get_state.
// FP64 state = hi + lo for elements [k0, k1) of every [n][i] row (rows x K).
static __global__ void k_mixed_to_fp64(const float* __restrict__ hi, const float* __restrict__ lo,
                                double* __restrict__ q, int K, int rows, int k0, int k1) {
  const int w = k1 - k0;
  const size_t n = static_cast<size_t>(rows) * w;
  for (size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t r = t / w, i = r * K + k0 + (t - r * w);
    q[i] = static_cast<double>(hi[i]) + static_cast<double>(lo[i]);
  }
}

// (c) interior-edge fluxes in delta form, one thread per mesh edge, one
// instantiation per flux kind FK; Roe-ER runs in FP64 (fluxes.go:415-503 has
// no delta form).
// A block's 128 edges own a contiguous run of the edge-major face array, which
// is copied into shared memory with coalesced 16-byte cp.async (the copy
// overlaps the base-state loads); the fluxes leave the same way, through a
// shared-memory record per edge and coalesced 16-byte stores.
template <int N>
struct EdgeDims {
  static constexpr int NEP = MixedDims<N>::NEP;
  static constexpr int FW = 8 * NEP;                  // floats of one edge's faces (2 sides x 4 variables)
  static constexpr int FWP = FW + ((FW % 8) ? 0 : 4);  // record stride = 4 mod 8 words: no bank conflicts
  static constexpr int OW = 4 * NEP + 4;               // fhat (4 x NEP) and corr (4)
  static constexpr int OWP = OW + ((OW % 8) ? 0 : 4);
};

template <int N, int FK>
__global__ void __launch_bounds__(128, FK == kFluxRoeER ? 1 : 5) k_mixed_edge(MixedArgs a) {
  constexpr bool RoeER = (FK == kFluxRoeER);
  constexpr int NE = MixedDims<N>::NE, NEP = MixedDims<N>::NEP;
  constexpr int FW = EdgeDims<N>::FW, FWP = EdgeDims<N>::FWP, OWP = EdgeDims<N>::OWP;
  static_assert(FW % 4 == 0 && FWP % 4 == 0 && OWP % 4 == 0, "16-byte records");
  __shared__ __align__(16) float sf[128 * FWP];
  __shared__ __align__(16) float so[128 * OWP];
  const int g0 = blockIdx.x * 128;
  const int nE = min(128, a.nInt - g0);
  {
    const float* src = a.faces + static_cast<size_t>(g0) * FW;
    for (int i = threadIdx.x; i < nE * (FW / 4); i += 128) {
      const int e = i / (FW / 4), c = i - e * (FW / 4);
      const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(&sf[e * FWP + 4 * c]));
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src + 4 * i));
    }
    asm volatile("cp.async.commit_group;\n" ::);
  }
  const int g = g0 + threadIdx.x;
  const bool active = g < a.nInt;
  float smax = 0.0f;
  float bh[4] = {1.f, 0.f, 0.f, 1.f}, bl[4] = {0.f, 0.f, 0.f, 0.f}, dB[4] = {0.f, 0.f, 0.f, 0.f};
  float nx = 0.f, ny = 0.f, oohK = 0.f;
  if (active) {
    const int kL = a.ekL[g], kR = a.ekR[g];
    nx = a.enx[g];
    ny = a.eny[g];
    oohK = a.eoohK[g];
    const float4* pL = reinterpret_cast<const float4*>(a.base + static_cast<size_t>(kL) * 4);
    const float4* pR = reinterpret_cast<const float4*>(a.base + static_cast<size_t>(kR) * 4);
    const float4 L01 = pL[0], L23 = pL[1], R01 = pR[0], R23 = pR[1];
    bh[0] = L01.x; bl[0] = L01.y; bh[1] = L01.z; bl[1] = L01.w;
    bh[2] = L23.x; bl[2] = L23.y; bh[3] = L23.z; bl[3] = L23.w;
    dB[0] = df_diff(R01.x, R01.y, bh[0], bl[0]);
    dB[1] = df_diff(R01.z, R01.w, bh[1], bl[1]);
    dB[2] = df_diff(R23.x, R23.y, bh[2], bl[2]);
    dB[3] = df_diff(R23.z, R23.w, bh[3], bl[3]);
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();
  if (active) {
    const float gm1 = a.gamma - 1.0f;
    const BasePrim b = base_prim(bh, gm1);
    const Gas<float> gf{a.gamma, gm1, 1.0f / gm1};
    float fr[FW];  // [side][variable][NEP]
    const float4* rec = reinterpret_cast<const float4*>(&sf[threadIdx.x * FWP]);
#pragma unroll
    for (int c = 0; c < FW / 4; ++c) {
      const float4 v = rec[c];
      fr[4 * c] = v.x;
      fr[4 * c + 1] = v.y;
      fr[4 * c + 2] = v.z;
      fr[4 * c + 3] = v.w;
    }
    float fo[4][NE];
    float sm = 0.0f;
#pragma unroll
    for (int p = 0; p < NE; ++p) {
      float ql[4], qr[4], f[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        ql[c] = fr[c * NEP + p];
        qr[c] = fr[4 * NEP + c * NEP + NE - 1 - p] + dB[c];
      }
      if constexpr (RoeER) {
        double QLd[4], QRd[4], fd[4], Fx[4], Fy[4], bd[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          bd[c] = static_cast<double>(bh[c]) + static_cast<double>(bl[c]);
          QLd[c] = bd[c] + ql[c];
          QRd[c] = bd[c] + qr[c];
        }
        const double gm1d = a.gammaD - 1.0;
        const Gas<double> gd{a.gammaD, gm1d, 1.0 / gm1d};
        flux_roe_er(gd, QLd, QRd, static_cast<double>(nx), static_cast<double>(ny), fd);
        euler_flux(gd, bd, Fx, Fy);
#pragma unroll
        for (int c = 0; c < 4; ++c)
          f[c] = static_cast<float>(fd[c] - (static_cast<double>(nx) * Fx[c] + static_cast<double>(ny) * Fy[c]));
      } else if constexpr (FK == kFluxRoe) {
        float w;
        roe_delta_fast(b, ql, qr, nx, ny, a.gamma, f, &w);
        sm = fmaxf(sm, oohK * w);
      } else {
        riemann_delta(FK, b, ql, qr, nx, ny, a.gamma, f);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) fo[c][p] = f[c];
      if constexpr (FK != kFluxRoe) {
        const float QL[4] = {b.rho + ql[0], b.m + ql[1], b.n + ql[2], b.E + ql[3]};
        sm = fmaxf(sm, oohK * (speed(QL[0], QL[1], QL[2]) + sound_speed(gf, QL[0], QL[1], QL[2], QL[3])));
      }
    }
    float cr[4];
    delta_normal_flux(b, dB, nx, ny, gm1, cr);
    float* o = &so[threadIdx.x * OWP];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
#pragma unroll
      for (int p = 0; p < NEP; ++p) o[c * NEP + p] = (p < NE) ? fo[c][p < NE ? p : 0] : 0.0f;
      o[4 * NEP + c] = cr[c];
    }
    smax = sm;
    a.edgeSpeed[g] = static_cast<double>(sm);
  }
  __syncthreads();
  {
    float* fdst = a.fhat + static_cast<size_t>(g0) * 4 * NEP;
    for (int i = threadIdx.x; i < nE * NEP; i += 128) {
      const int e = i / NEP, c = i - e * NEP;
      reinterpret_cast<float4*>(fdst)[i] = *reinterpret_cast<const float4*>(&so[e * OWP + 4 * c]);
    }
    if (active)
      reinterpret_cast<float4*>(a.corr)[g] = *reinterpret_cast<const float4*>(&so[threadIdx.x * OWP + 4 * NEP]);
  }
  smax = warp_max(smax);  // wave speeds are >= 0: their FP64 bit patterns order like integers
  if ((threadIdx.x & 31) == 0)
    atomicMax(a.gmax, static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(smax))));
}

// (c) boundary edges: face state, characteristic / wall / exact-state BC and
// the physical normal flux in FP64 (bcs.go:11-133, edges.go:413-452), then the
// delta to FP32.  GB300's FP64 pipe is narrow and these points carry the
// transcendental work (exp/pow), so one thread owns one (edge, point): a block
// is 8 edges (threadIdx.x) x NpEdge points (threadIdx.y), spread over many SMs,
// and the kernel runs on a forked stream beside the interior-edge kernel.
template <int N>
__global__ void __launch_bounds__(8 * MixedDims<N>::NE) k_mixed_edge_bc(MixedArgs a) {
  constexpr int NE = MixedDims<N>::NE, NEP = MixedDims<N>::NEP;
  __shared__ double sspeed[NE][8];
  const int tx = threadIdx.x, p = threadIdx.y;
  const int bb = blockIdx.x * 8 + tx;
  double ws = 0.0;
  int g = -1;
  if (bb < a.nBC) {
    g = a.nInt + bb;
    const int kL = a.ekL[g];
    const double nxd = a.enx[g], nyd = a.eny[g];
    double bL[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float2 v = a.base[static_cast<size_t>(kL) * 4 + c];
      bL[c] = static_cast<double>(v.x) + static_cast<double>(v.y);
    }
    const double gm1d = a.gammaD - 1.0;
    const Gas<double> gd{a.gammaD, gm1d, 1.0 / gm1d};
    double Fx[4], Fy[4];
    euler_flux(gd, bL, Fx, Fy);
    const float* fL = a.faces + static_cast<size_t>(g) * 2 * 4 * NEP;
    double qi[4], qb[4], f[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) qi[c] = bL[c] + static_cast<double>(fL[c * NEP + p]);
    bool wall = false;
    switch (a.bcFlag[bb]) {
      case 4: riemann_bc<double, true>(a.fsFar, qi, a.fsFar.qinf, nxd, nyd, qb); break;
      case 1: riemann_bc<double, true>(a.fsIn, qi, a.fsIn.qinf, nxd, nyd, qb); break;
      case 8: riemann_bc<double, true>(a.fsOut, qi, a.fsOut.qinf, nxd, nyd, qb); break;
      case 9: {
        // The BC time is frozen for the 5 stages (euler.go:621): evaluate the
        // exact state once per step and reuse it.
        double ex[4];
        double* cache = a.exBC + (static_cast<size_t>(bb) * NE + p) * 4;
        if (a.stage <= 0) {
          ivortex_state(a.vbeta, a.vx0, a.vy0, a.vgamma, *a.time, a.bx[bb * NE + p], a.by[bb * NE + p], ex);
          if (a.stage == 0)
#pragma unroll
            for (int c = 0; c < 4; ++c) cache[c] = ex[c];
        } else {
#pragma unroll
          for (int c = 0; c < 4; ++c) ex[c] = cache[c];
        }
        riemann_bc<double, true>(a.fsFar, qi, ex, nxd, nyd, qb);
        break;
      }
      case 5: case 6:
        wall = true;
#pragma unroll
        for (int c = 0; c < 4; ++c) qb[c] = qi[c];
        break;
      default:
#pragma unroll
        for (int c = 0; c < 4; ++c) qb[c] = qi[c];
    }
    if (wall) {
      const double pw = pressure(gd, qi[0], qi[1], qi[2], qi[3]);
      f[0] = 0.0; f[1] = nxd * pw; f[2] = nyd * pw; f[3] = 0.0;
    } else {
      double Gx[4], Gy[4];
      euler_flux(gd, qb, Gx, Gy);
#pragma unroll
      for (int c = 0; c < 4; ++c) f[c] = nxd * Gx[c] + nyd * Gy[c];
    }
    float* fo = a.fhat + static_cast<size_t>(g) * 4 * NEP;
#pragma unroll
    for (int c = 0; c < 4; ++c) fo[c * NEP + p] = static_cast<float>(f[c] - (nxd * Fx[c] + nyd * Fy[c]));
    ws = static_cast<double>(a.eoohK[g]) * (speed(qb[0], qb[1], qb[2]) + sound_speed(gd, qb[0], qb[1], qb[2], qb[3]));
  }
  sspeed[p][tx] = ws;
  __syncthreads();
  if (p == 0) {
    double m = 0.0;
#pragma unroll
    for (int q = 0; q < NE; ++q) m = fmax(m, sspeed[q][tx]);
    if (g >= 0) a.edgeSpeed[g] = m;
    // lanes 0..7 of the p == 0 row hold all 8 edges of the block
    for (int o = 4; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0x000000ffu, m, o, 8));
    if (tx == 0) atomicMax(a.gmax, static_cast<unsigned long long>(__double_as_longlong(m)));
  }
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p));
}

// L2 prefetch of what stage_tail will read for block blk, issued by one warp
// per variable n: the compensated state at point 0 (stages 0-3), or the whole
// compensated state, the stage-2/3 combination P23 and the stage-3 RHS (stage 4).
// With K % 4 == 0 every row of the block is 128 contiguous, 16-byte aligned
// bytes and lane j bulk-prefetches rows j, j+32, ...; otherwise each thread
// prefetches its own element's lines.
__device__ __forceinline__ void bulk_prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(bytes) : "memory");
}
template <int N>
__device__ __forceinline__ void stage_tail_prefetch(const MixedArgs& a, int blk, int n, int lane, size_t sK, int s) {
  constexpr int NP = MixedDims<N>::NP;
  if (s < 0 || a.rhsOnly) return;
  const size_t base = static_cast<size_t>(n) * NP * sK + static_cast<size_t>(blk) * 32;
  const bool full = (a.K & 3) == 0 && blk * 32 + 32 <= a.K;
  if (!full) {
    const int k = blk * 32 + lane;
    if (k >= a.K) return;
    const int rows = (s < 4) ? 1 : NP;
    for (int r = 0; r < rows; ++r) {
      prefetch_l2(a.Qhi + base + lane + r * sK);
      prefetch_l2(a.Qlo + base + lane + r * sK);
      if (s == 4) {
        prefetch_l2(a.P23 + base + lane + r * sK);
        prefetch_l2(a.R3 + base + lane + r * sK);
      }
    }
    return;
  }
  if (s < 4) {
    if (lane < 2) bulk_prefetch_l2((lane ? a.Qlo : a.Qhi) + base, 128);
    return;
  }
  for (int it = lane; it < 4 * NP; it += 32) {
    const int arr = it / NP, r = it - arr * NP;
    const float* p = arr == 0 ? a.Qhi : arr == 1 ? a.Qlo : arr == 2 ? a.P23 : a.R3;
    bulk_prefetch_l2(p + base + r * sK, 128);
  }
}

// One warp's residual partials of the final stage: the maxima by atomics
// (order independent); the lanes' compensated FP32 sums of squares are summed
// over the warp by a fixed shuffle tree of compensated additions (no FP64
// arithmetic: GB300's FP64 pipe is narrow), and lane 0 stores hi + lo in FP64
// in the warp's slot of sc->rpart (unit = CTA, variable n), which k_resid_blocks
// and k_step_end sum in FP64 in a fixed order.
__device__ __forceinline__ void residual_commit(Scalars* sc, int n, int lane, float rmax, float rabs, float2 rs2) {
  rmax = warp_max(rmax);
  rabs = warp_max(rabs);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, rs2.x, o);
    const float ol = __shfl_xor_sync(0xffffffffu, rs2.y, o);
    float s, e;
    two_sum(rs2.x, oh, s, e);
    rs2.x = s;
    rs2.y = (rs2.y + ol) + e;
  }
  if (lane == 0) {
    atomicMax(&sc->rmax[n], order_key(static_cast<double>(rmax)));
    atomicMax(&sc->rabs[n], static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(rabs))));
    sc->rpart[static_cast<size_t>(blockIdx.x) * 4 + n] = static_cast<double>(rs2.x) + static_cast<double>(rs2.y);
  }
}

// rs2 += x * x in compensated FP32: the product's rounding error from an FMA,
// the sum's from a two-sum (about 48 significant bits).
__device__ __forceinline__ void sumsq_add(float2& rs2, float x) {
  const float p = x * x;
  const float pe = fmaf(x, x, -p);
  float s, e;
  two_sum(rs2.x, p, s, e);
  rs2.x = s;
  rs2.y += e + pe;
}

// The stage's global time step (calculateGlobalDT, euler.go:945-971, with the
// viscous cap and the FinalTime clip), computed once per CTA.
__device__ __forceinline__ double global_stage_dt(const MixedArgs& a, int s) {
  const double gm = __longlong_as_double(static_cast<long long>(a.sc->gmax[s]));
  double dtk = a.cfl / gm;
  if (a.gviscS) dtk = fmin(dtk, a.cdiff / __longlong_as_double(static_cast<long long>(a.gviscS[s])));
  const double t = a.sc->time;
  if (t + dtk > a.finalTime) dtk = a.finalTime - t;
  return dtk;
}
// Whether a stage kernel needs the global time step.
__device__ __forceinline__ bool needs_global_dt(const MixedArgs& a, int s) {
  return s >= 0 && !a.rhsOnly && !a.localDT;
}

// The stage update after the divergence (shared by the FMA and tensor-core
// stage kernels): the RHS goes to rhsOut (stage -1) or into the SSP increments,
// the next stage's faces and reference state, and at stage 4 the compensated
// state and the residual partials.  dtk is the element's time step: its local
// one with local time stepping, else the stage's global one.
//
// With DeferFaces the next stage's deltas are left in dqnOut instead of being
// interpolated to the faces here (the tensor-core kernel runs that GEMM on
// tcgen05 for the whole CTA afterwards).
template <int N, bool DeferFaces = false>
__device__ __forceinline__ void stage_tail(const MixedArgs& a, const int eslot[3], int n, int k,
                                           size_t off, size_t sK, int s, const float rhs[], const float dq0[],
                                           const float ds[], double dtk, float& rmax, float& rabs,
                                           float2& rs2, float* dqnOut = nullptr) {
  constexpr int NP = MixedDims<N>::NP, NPP = MixedDims<N>::NPP;
  if (s < 0 || a.rhsOnly) {
#pragma unroll
    for (int r = 0; r < NP; ++r) a.rhsOut[off + r * sK] = rhs[r];
  } else {
    if (a.localDT) {
      if (n == 0) a.DT[k] = dtk;
    } else {
      if (k == 0 && n == 0) a.sc->dt[s] = dtk;
    }
    const float dt = static_cast<float>(dtk);
    if (a.tapeRHS) {
#pragma unroll
      for (int r = 0; r < NP; ++r) a.tapeRHS[off + r * sK] = rhs[r];
    }
    float dn[NP];
    if (s == 0) {
#pragma unroll
      for (int r = 0; r < NP; ++r) dn[r] = kSspC0 * (dt * rhs[r]);
    } else if (s == 1) {
#pragma unroll
      for (int r = 0; r < NP; ++r) dn[r] = kSspB1 * ds[r] + kSspC1 * (dt * rhs[r]);
    } else if (s == 2) {
      // D3 is known here and D2 is ds: their share of the final combination is
      // formed now, so that stage 4 reads one array for both
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        dn[r] = kSspB2 * ds[r] + kSspC2 * (dt * rhs[r]);
        a.P23[off + r * sK] = fmaf(kSspA3, dn[r], kSspA2 * ds[r]);
      }
    } else if (s == 3) {
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        a.R3[off + r * sK] = rhs[r];
        dn[r] = kSspB3 * ds[r] + kSspC3 * (dt * rhs[r]);
      }
    }
    if (s < 4) {
      float* dst = a.D[s + 1] + off;
#pragma unroll
      for (int r = 0; r < NP; ++r) dst[r * sK] = dn[r];
      float dqn[NPP];
#pragma unroll
      for (int r = 0; r < NPP; ++r) dqn[r] = (r < NP) ? dq0[r] + (dn[r] - dn[0]) : 0.0f;
      if constexpr (DeferFaces) {
#pragma unroll
        for (int r = 0; r < NPP; ++r) dqnOut[r] = dqn[r];
      } else {
        write_faces<N>(a, eslot, n, dqn);
      }
      float h = a.Qhi[off], l = a.Qlo[off];
      df_add(h, l, dn[0]);
      a.base[static_cast<size_t>(k) * 4 + n] = make_float2(h, l);
    } else {
      // Final increment and the compensated accumulation (rkAdvance stage 4).
      float qh[NP], ql[NP];
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        const float inc =
            fmaf(kSspC4, dt * rhs[r], fmaf(kSspR3, dt * a.R3[off + r * sK], fmaf(kSspA4, ds[r], a.P23[off + r * sK])));
        qh[r] = a.Qhi[off + r * sK];
        ql[r] = a.Qlo[off + r * sK];
        if (a.tapeQ0) a.tapeQ0[off + r * sK] = qh[r];
        df_add(qh[r], ql[r], inc);
        a.Qhi[off + r * sK] = qh[r];
        a.Qlo[off + r * sK] = ql[r];
        rmax = fmaxf(rmax, inc);
        rabs = fmaxf(rabs, fabsf(inc));
        sumsq_add(rs2, inc);
        if (inc != inc) rabs = inc;
      }
      // Prepare the next step's stage 0 from the new state.
      float dqn[NPP];
#pragma unroll
      for (int r = 0; r < NPP; ++r) dqn[r] = 0.0f;
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        dqn[r] = df_diff(qh[r], ql[r], qh[0], ql[0]);
        a.dQ0[off + r * sK] = dqn[r];
      }
      if constexpr (DeferFaces) {
#pragma unroll
        for (int r = 0; r < NPP; ++r) dqnOut[r] = dqn[r];
      } else {
        write_faces<N>(a, eslot, n, dqn);
      }
      a.base[static_cast<size_t>(k) * 4 + n] = make_float2(qh[0], ql[0]);
    }
  }
}

// Interior transformed delta fluxes of variable n at every solution point and
// their divergence columns (DivInt columns 0..2NP-1), accumulated into the
// output pairs acc.  The stage delta at point i is d = dQ0 + (D_s - D_s(0))
// (from shared memory); its velocity and pressure deltas du, dv, dp come from
// shared memory (spr), computed once per element.  The four variables' delta
// fluxes share one form,
//     dFx = Px wx + sx (Bx + wx) + cx,   dFy = Py wy + sy (By + wy) + cy,
// with per-variable choices (n = 0: sx, sy = d1, d2 and w = P = 0, B = 1;
// n = 1: w = du, s = d1, d2, P = m_b, n_b, B = u_b, cx = dp; n = 2: w = dv,
// B = v_b, cy = dp; n = 3: s = d3 + dp, wx, wy = du, dv, P = H_b, B = u_b, v_b),
// so all four warps of a CTA run the same instructions on different operands
// (the exact algebra of delta_flux_c, regrouped).
template <int N>
__device__ __forceinline__ void interior_columns(int n, const BasePrim& b, const float (*sd)[MixedDims<N>::NP][32],
                                                 const float (*spr)[MixedDims<N>::NP][32], int lane,
                                                 float Jd, float J0, float J1, float J2, float J3, float2 acc[]) {
  constexpr int NP = MixedDims<N>::NP;
  const int ra = (n == 3) ? 3 : 1, rb = (n == 3) ? 3 : 2;  // rows of sx and sy
  const int wxr = (n == 2) ? 1 : 0, wyr = (n == 1) ? 0 : 1;  // du or dv
  const bool twoRows = n != 3, hasW = n != 0, twoW = n == 3;  // which reads the variable needs
  const float mw = (n == 0) ? 0.0f : 1.0f;                   // variable 0 has no velocity term
  const float ms = (n == 3) ? 1.0f : 0.0f;                   // energy: s = d3 + dp
  const float mcx = (n == 1) ? 1.0f : 0.0f, mcy = (n == 2) ? 1.0f : 0.0f;
  const float Px = (n == 3) ? b.H : ((n == 0) ? 0.0f : b.m);
  const float Py = (n == 3) ? b.H : ((n == 0) ? 0.0f : b.n);
  const float Bx = (n == 0) ? 1.0f : ((n == 2) ? b.v : b.u);
  const float By = (n == 0) ? 1.0f : ((n == 1) ? b.u : b.v);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    const float dp = spr[2][i][lane];
    const float xa = sd[ra][i][lane];
    float xb = xa, wxv = 0.0f, wyv = 0.0f;
    if (twoRows) xb = sd[rb][i][lane];
    if (hasW) {
      wxv = spr[wxr][i][lane];
      wyv = wxv;
      if (twoW) wyv = spr[wyr][i][lane];
    }
    const float sx = fmaf(ms, dp, xa);
    const float sy = fmaf(ms, dp, xb);
    const float wx = mw * wxv, wy = mw * wyv;
    const float fx = fmaf(Px, wx, fmaf(sx, Bx + wx, mcx * dp));
    const float fy = fmaf(Py, wy, fmaf(sy, By + wy, mcy * dp));
    const float Fr = Jd * (J0 * fx + J1 * fy);
    const float Fs = Jd * (J2 * fx + J3 * fy);
    div_column<N>(NP + i, Fs, acc);
    div_column<N>(i, Fr, acc);
  }
}

// (b)+(e): delta-form divergence, SSP stage update on the FP32 increments, and
// the next stage's faces / reference states.  stage -1 writes the RHS only.
//
// One CTA = 32 elements x 4 variables (warp n owns variable n, lane = element).
// The element's stage inputs (dQ0, D_s) are staged in shared memory by
// coalesced row loads; its three edge records (fhat, 4 x NEP floats, and
// corr, 4 floats, per edge) are gathered as 16-byte cp.async chunks shared
// out over the element's four threads and waited for after the interior flux
// work.  The velocity and pressure deltas of the NP points are computed once
// per element (warp n takes points n, n+4, ...) and shared through shared
// memory.  Both GEMMs (DivInt against the flux DOFs, FluxEdgeInterp against
// the next stage's deltas) run on packed FP32 pairs (two outputs per FMA
// instruction, constant-bank operator pairs).
template <int N>
struct StageDims {
  static constexpr int NEP = MixedDims<N>::NEP;
  static constexpr int CH = NEP + 1;    // 16-byte chunks per edge record
  static constexpr int RW = 3 * CH * 4;  // floats per element's three records
};

template <int N>
__global__ void __launch_bounds__(128, 7) k_mixed_stage(MixedArgs a) {
  constexpr int NP = MixedDims<N>::NP, NE = MixedDims<N>::NE, NPP = MixedDims<N>::NPP;
  constexpr int NEP = MixedDims<N>::NEP, CH = StageDims<N>::CH, RW = StageDims<N>::RW;
  constexpr int NH = NPP / 2;
  // Rows are indexed by lane, so a 32-float stride is free of bank conflicts.
  // sds: the stage increments D_s; sd: the conserved deltas against the stage
  // state (dQ0 + D_s - D_s[0]) and spr: the velocity and pressure deltas, both
  // per point for all four variables, so that each variable's interior flux
  // reads only the rows it uses (3 or 4 words per point).
  __shared__ float sds[4][NP][32];
  __shared__ float sd[4][NP][32];
  __shared__ float spr[3][NP][32];
  __shared__ __align__(16) float srec[32 * RW];
  __shared__ double sdt;
  const int n = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * 32 + lane;
  const bool active = k < a.K;
  const size_t sK = static_cast<size_t>(a.K);
  const size_t off = static_cast<size_t>(n) * NP * sK + k;
  const int s = a.stage;
  int eslot[3] = {0, 0, 0};
  float eII[3] = {0.f, 0.f, 0.f};
  if (active) {
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      eslot[e] = a.eslot[e * sK + k];
      eII[e] = a.II[e * sK + k];
    }
    // Chunks c = n, n+4, ... of the element's 3 x CH record chunks.
#pragma unroll
    for (int t = 0; t < (3 * CH + 3) / 4; ++t) {
      const int c = n + 4 * t;
      if (c < 3 * CH) {
        const int e = c / CH, j = c - e * CH;
        const size_t g = static_cast<size_t>((e == 0 ? eslot[0] : (e == 1 ? eslot[1] : eslot[2])) >> 1);
        const float* src = (j < NEP) ? a.fhat + g * 4 * NEP + 4 * j : a.corr + g * 4;
        const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(&srec[lane * RW + 4 * c]));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src));
      }
    }
  }
  asm volatile("cp.async.commit_group;\n" ::);
  stage_tail_prefetch<N>(a, blockIdx.x, n, lane, sK, s);
  float Jd = 0.f, J0 = 0.f, J1 = 0.f, J2 = 0.f, J3 = 0.f, ooJ = 0.f;
  // dQ0 of the points whose deltas this warp forms (n, n+4, ...), all four
  // variables, loaded before the barrier and used after it.
  constexpr int NT = (NP + 3) / 4;
  float q0p[NT][4];
#pragma unroll
  for (int t = 0; t < NT; ++t)
#pragma unroll
    for (int c = 0; c < 4; ++c) q0p[t][c] = 0.0f;
  if (active) {
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int i = n + 4 * t;
      if (i < NP) {
#pragma unroll
        for (int c = 0; c < 4; ++c) q0p[t][c] = a.dQ0[(static_cast<size_t>(c) * NP + i) * sK + k];
      }
    }
    if (s >= 1) {
#pragma unroll
      for (int i = 0; i < NP; ++i) sds[n][i][lane] = a.D[s][off + i * sK];
    }
    Jd = a.geo[k];
    J0 = a.geo[sK + k];
    J1 = a.geo[2 * sK + k];
    J2 = a.geo[3 * sK + k];
    J3 = a.geo[4 * sK + k];
    ooJ = a.geo[5 * sK + k];
  } else {
    // lanes past K: zero deltas for the shared work
#pragma unroll
    for (int i = 0; i < NP; ++i) sds[n][i][lane] = 0.0f;
  }
  // Local time step of this stage: DT persists across stages, so every thread
  // of the element reads it before the barrier and one writes it after.
  double dtk = 0.0;
  if (active && a.localDT && s >= 0 && !a.rhsOnly) {
    double v = (s == 0) ? -100.0 : a.DT[k];
#pragma unroll
    for (int e = 0; e < 3; ++e) v = fmax(v, a.edgeSpeed[eslot[e] >> 1]);
    dtk = a.cfl / v;
  }
  if (threadIdx.x == 0 && needs_global_dt(a, s)) sdt = global_stage_dt(a, s);
  __syncthreads();
  if (needs_global_dt(a, s)) dtk = sdt;
  const float gm1 = a.gamma - 1.0f;
  float bq[4] = {1.0f, 0.0f, 0.0f, 2.5f};  // lanes past K: a harmless reference state
  if (active) {
    const float4* pb = reinterpret_cast<const float4*>(a.base + static_cast<size_t>(k) * 4);
    const float4 b01 = pb[0], b23 = pb[1];
    bq[0] = b01.x;
    bq[1] = b01.z;
    bq[2] = b23.x;
    bq[3] = b23.z;
  }
  const BasePrim b = base_prim(bq, gm1);
  // Conserved, velocity and pressure deltas of points n, n+4, ... for the whole element.
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const int i = n + 4 * t;
    if (i < NP) {
      float d[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        d[c] = q0p[t][c] + ((s >= 1) ? sds[c][i][lane] - sds[c][0][lane] : 0.0f);
        sd[c][i][lane] = d[c];
      }
      const DeltaPrim q = delta_prim(b, d, gm1);
      spr[0][i][lane] = q.du;
      spr[1][i][lane] = q.dv;
      spr[2][i][lane] = q.dp;
    }
  }
  __syncthreads();
  float2 acc[NH];
#pragma unroll
  for (int h = 0; h < NH; ++h) acc[h] = make_float2(0.0f, 0.0f);
  interior_columns<N>(n, b, sd, spr, lane, Jd, J0, J1, J2, J3, acc);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();  // every thread's record chunks
  float rmax = -3.4028235e38f, rabs = 0.0f;
  float2 rs2 = make_float2(0.0f, 0.0f);
  if (active) {
    // Edge DOFs: IInII * (s fhat - n_e.F(Qb)), owner order / reversed for the right side.
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const float* rec = &srec[lane * RW + e * CH * 4];
      const bool right = eslot[e] & 1;
      const float ii = eII[e];
      const float cc = right ? rec[4 * NEP + n] : 0.0f;
      float v[NEP];
      const float2* rp = reinterpret_cast<const float2*>(rec + n * NEP);
#pragma unroll
      for (int q = 0; q < NEP / 2; ++q) {
        const float2 t = rp[q];
        v[2 * q] = t.x;
        v[2 * q + 1] = t.y;
      }
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const float dof = right ? -(v[NE - 1 - p] - cc) * ii : v[p] * ii;
        div_column<N>(2 * NP + e * NE + p, dof, acc);
      }
    }
    float rhs[NP], dq0[NP], ds[NP];
#pragma unroll
    for (int r = 0; r < NP; ++r) {
      rhs[r] = -((r & 1) ? acc[r >> 1].y : acc[r >> 1].x) * ooJ;
      // dQ0 back from the stage delta (exact at stage 0; at later stages to
      // the rounding of dQ0 + (D_s - D_s[0]))
      ds[r] = (s >= 1) ? sds[n][r][lane] : 0.0f;
      dq0[r] = (s >= 1) ? sd[n][r][lane] - (ds[r] - sds[n][0][lane]) : sd[n][r][lane];
    }
    stage_tail<N>(a, eslot, n, k, off, sK, s, rhs, dq0, ds, dtk, rmax, rabs, rs2);
  }
  if (s == 4 && !a.rhsOnly) {
    residual_commit(a.sc, n, lane, rmax, rabs, rs2);
  }
}

}  // namespace gcfd
