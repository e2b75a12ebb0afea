// The mixed path's stage kernel with the DFR divergence GEMM on the tensor
// cores (precision mode GCFD_PREC_TF32X3).
//
// A CTA is 32 elements x 4 variables = 128 threads, one per row of the GEMM
//     D[m][r] = sum_j DOF_m[j] * DivInt[r][j],   m = (variable, element), r < 16
// (RHSInternalPoints, euler.go:665-699, for 128 rows at once).  Each thread
// builds its row of delta-form RT DOFs (interior transformed fluxes and edge
// fluxes) in registers, splits it into TF32 hi and lo parts and stores both
// into Tensor Memory (tcgen05.st, lane = row); DivInt, split the same way on
// the host, sits in shared memory in the no-swizzle K-major core-matrix layout.
// One thread issues 3 x NFP/8 tcgen05.mma.kind::tf32 (M = 128, N = 16, K = 8):
// hi*hi + hi*lo + lo*hi ("3xTF32"), about FP32 accuracy, accumulated in FP32
// in Tensor Memory, then every thread reads its row back with tcgen05.ld and
// applies the same stage update as the FMA kernel (stage_tail).  The next
// stage's face deltas (InterpolateSolutionToEdges, edges.go:485-488) are a
// second GEMM on the tensor cores:
//     F[m][q] = sum_i dq_m[i] * FluxEdgeInterp[q][i],   q < 3 NpEdge,
// each thread's updated deltas (16 K columns, TF32 hi and lo) stored into the
// columns the divergence's A used, FluxEdgeInterp split the same way in shared
// memory, 3 x 2 MMAs (M = 128, N = 16 or 32, K = 8) into the divergence's D
// columns, read back and stored as the edge-major faces.
#pragma once
#include "gcfd_mixed.cuh"
#include "gcfd_tc.cuh"

namespace gcfd {

template <int N>
struct TcDims {
  static constexpr int NF = MixedDims<N>::NF;
  static constexpr int NFP = (NF + 15) & ~15;  // K padded to the 16-column TMEM stores
  static constexpr int NOUT = 16;              // GEMM N: output points, padded
  static constexpr int COL_LO = NFP;           // TMEM columns: A hi [0, NFP), A lo [NFP, 2 NFP), D after
  static constexpr int COL_D = 2 * NFP;
  static constexpr int NEED = 2 * NFP + NOUT;
  static constexpr int NCOLS = NEED <= 32 ? 32 : (NEED <= 64 ? 64 : (NEED <= 128 ? 128 : 256));
  static constexpr int BSZ = NOUT * NFP;       // floats per B split
  static_assert(MixedDims<N>::NP <= NOUT, "output points must fit the N = 16 tile");
  // Face GEMM (FluxEdgeInterp): K = 16 solution points (padded), N = the 3 NpEdge
  // face points rounded up to 16; A (hi, lo) reuses columns [0, 32), D the
  // columns of the divergence result from COL_D.
  static constexpr int KF = 16;
  static constexpr int NFACE = ((MixedDims<N>::NE3 + 15) / 16) * 16;
  static constexpr int BFSZ = NFACE * KF;      // floats per face-operand split
  static_assert(COL_D >= 2 * KF && COL_D + NFACE <= NCOLS, "face GEMM must fit the allocated columns");
  static_assert(NFACE <= 32 && MixedDims<N>::NPP <= KF, "face GEMM tile");
};

// Host-side layout of one B split: element (r, j) of the 16 x NFP operand at
// (r / 8) * SBO + (j / 4) * LBO + (r % 8) * 4 + (j % 4) floats, with LBO = 32
// floats (128 B, the next core matrix along K) and SBO = NFP / 4 * 32 floats.
inline int tc_b_index(int r, int j, int NFP) { return (r / 8) * (NFP / 4) * 32 + (j / 4) * 32 + (r % 8) * 4 + (j % 4); }

template <int N>
__global__ void __launch_bounds__(128, 4) k_mixed_stage_tc(MixedArgs a) {
  constexpr int NP = MixedDims<N>::NP, NE = MixedDims<N>::NE, NE3 = MixedDims<N>::NE3;
  constexpr int NEP = MixedDims<N>::NEP;
  constexpr int NFP = TcDims<N>::NFP, NCOLS = TcDims<N>::NCOLS, BSZ = TcDims<N>::BSZ;
  constexpr int BFSZ = TcDims<N>::BFSZ, NFACE = TcDims<N>::NFACE, NPP = MixedDims<N>::NPP;
  __shared__ __align__(128) float sB[2 * BSZ];
  __shared__ __align__(128) float sBF[2 * BFSZ];
  __shared__ float sdq[4][NP][33];
  __shared__ float sbase[4][32];
  __shared__ float sfh[4][NE3][32];
  __shared__ float scorr[4][3][32];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ double sdt;
  for (int i = threadIdx.x; i < 2 * BSZ; i += blockDim.x) sB[i] = a.Btc[i];
  for (int i = threadIdx.x; i < 2 * BFSZ; i += blockDim.x) sBF[i] = a.BtcF[i];
  tc::fence_proxy_async();  // sB and sBF are read by the tensor core
  const int n = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
  if (n == 0) {
    tc::alloc(&tmem_base, NCOLS);
    tc::fence_before();
  }
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
      const float* fh = a.fhat + (static_cast<size_t>(eslot[e] >> 1) * 4 + n) * NEP;
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(&sfh[n][e * NE + p][lane]));
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(fh + p));
      }
      if (eslot[e] & 1) {
        const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(&scorr[n][e][lane]));
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst),
                     "l"(a.corr + static_cast<size_t>(eslot[e] >> 1) * 4 + n));
      }
    }
    asm volatile("cp.async.commit_group;\n" ::);
  }
  stage_tail_prefetch<N>(a, blockIdx.x, n, lane, sK, s);
  float dq0[NP], ds[NP];
  if (active) {
#pragma unroll
    for (int i = 0; i < NP; ++i) dq0[i] = a.dQ0[off + i * sK];
    if (s >= 1) {
#pragma unroll
      for (int i = 0; i < NP; ++i) ds[i] = a.D[s][off + i * sK];
    } else {
#pragma unroll
      for (int i = 0; i < NP; ++i) ds[i] = 0.0f;
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) sdq[n][i][lane] = dq0[i] + (ds[i] - ds[0]);
    sbase[n][lane] = a.base[static_cast<size_t>(k) * 4 + n].x;
  }
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
  tc::fence_after();
  const uint32_t tbase = tmem_base;
  const uint32_t trow = tbase + (static_cast<uint32_t>(n * 32) << 16);  // this warp's 32 TMEM lanes
  // This thread's GEMM row in the permuted K order (Fr_0, Fs_0, Fr_1, Fs_1, ...,
  // then the 3 NpEdge edge DOFs, then zeros; the host permutes DivInt's columns
  // the same way), written to Tensor Memory 16 columns at a time as soon as a
  // chunk is complete, so only one chunk is live in registers.  Every thread
  // of the warp takes part in the stores (they are warp-collective); threads
  // past the last element compute on zeros and their rows are never read.
  float dof[NFP];
  auto flush = [&](int j) {  // j: index just written; stores its chunk when complete
    if ((j & 15) == 15) {
      const int c = j >> 4;
      uint32_t hi[16], lo[16];
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const float x = dof[16 * c + t];
        hi[t] = tc::to_tf32(x);
        lo[t] = tc::to_tf32(x - __uint_as_float(hi[t]));
      }
      tc::st16(trow + 16 * c, hi);
      tc::st16(trow + TcDims<N>::COL_LO + 16 * c, lo);
    }
  };
  const float Jd = active ? a.geo[k] : 0.0f, J0 = active ? a.geo[sK + k] : 0.0f;
  const float J1 = active ? a.geo[2 * sK + k] : 0.0f, J2 = active ? a.geo[3 * sK + k] : 0.0f;
  const float J3 = active ? a.geo[4 * sK + k] : 0.0f;
  const float ooJ = active ? a.geo[5 * sK + k] : 0.0f;
  {
    const float bq[4] = {active ? sbase[0][lane] : 1.0f, active ? sbase[1][lane] : 0.0f,
                         active ? sbase[2][lane] : 0.0f, active ? sbase[3][lane] : 1.0f};
    const float gm1 = a.gamma - 1.0f;
    const BasePrim b = base_prim(bq, gm1);
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      if (active) {
#pragma unroll
        for (int c = 0; c < 4; ++c) d[c] = sdq[c][i][lane];
      }
      const DeltaPrim q = delta_prim(b, d, gm1);
      float fx, fy;
      delta_flux_c(n, b, d, q, &fx, &fy);
      dof[2 * i] = Jd * (J0 * fx + J1 * fy);
      flush(2 * i);
      dof[2 * i + 1] = Jd * (J2 * fx + J3 * fy);
      flush(2 * i + 1);
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const bool right = eslot[e] & 1;
    const float ii = eII[e];
    const float cc = (active && right) ? scorr[n][e][lane] : 0.0f;
#pragma unroll
    for (int p = 0; p < NE; ++p) {
      const int j = 2 * NP + e * NE + p;
      const float f = active ? (right ? -(sfh[n][e * NE + NE - 1 - p][lane] - cc) : sfh[n][e * NE + p][lane]) : 0.0f;
      dof[j] = f * ii;
      flush(j);
    }
  }
#pragma unroll
  for (int j = 2 * NP + 3 * NE; j < NFP; ++j) {
    dof[j] = 0.0f;
    flush(j);
  }
  tc::wait_st();
  tc::fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::fence_after();
    constexpr uint32_t idesc = tc::idesc_tf32(128, TcDims<N>::NOUT);
    constexpr uint32_t lbo = 128, sbo = (NFP / 4) * 128;
    const uint32_t bhi = tc::smem_u32(sB), blo = tc::smem_u32(sB + BSZ);
    const uint32_t dcol = tbase + TcDims<N>::COL_D;
#pragma unroll
    for (int kk = 0; kk < NFP / 8; ++kk) {
      const uint64_t dh = tc::smem_desc(bhi + 256 * kk, lbo, sbo);
      const uint64_t dl = tc::smem_desc(blo + 256 * kk, lbo, sbo);
      const uint32_t ahi = tbase + 8 * kk, alo = tbase + TcDims<N>::COL_LO + 8 * kk;
      tc::mma_tf32_ts(dcol, ahi, dh, idesc, kk > 0 ? 1u : 0u);
      tc::mma_tf32_ts(dcol, ahi, dl, idesc, 1u);
      tc::mma_tf32_ts(dcol, alo, dh, idesc, 1u);
    }
    tc::commit(&mbar);
  }
  bool ok = tc::mbar_wait(&mbar, 0, 1 << 20);
  if (!ok) {
    if (lane == 0) atomicOr(a.err, 1u);
    ok = tc::mbar_wait(&mbar, 0, 1 << 20);  // let the MMAs drain before the TMEM is reused or freed
  }
  tc::fence_after();
  uint32_t dv[16];
  tc::ld16(trow + TcDims<N>::COL_D, dv);
  tc::wait_ld();
  float rmax = -3.4028235e38f, rabs = 0.0f;
  float2 rs2 = make_float2(0.0f, 0.0f);
  // the next stage's faces: on the tensor cores unless the divergence's wait gave up
  const bool faces = s >= 0 && !a.rhsOnly;
  const bool tcFaces = __syncthreads_and(ok) && faces;
  float dqn[NPP];
#pragma unroll
  for (int r = 0; r < NPP; ++r) dqn[r] = 0.0f;
  if (active) {
    float rhs[NP];
#pragma unroll
    for (int r = 0; r < NP; ++r) rhs[r] = -__uint_as_float(dv[r]) * ooJ;
    if (tcFaces)
      stage_tail<N, true>(a, eslot, n, k, off, sK, s, rhs, dq0, ds, dtk, rmax, rabs, rs2, dqn);
    else
      stage_tail<N>(a, eslot, n, k, off, sK, s, rhs, dq0, ds, dtk, rmax, rabs, rs2);
  }
  if (tcFaces) {
    uint32_t hi[16], lo[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const float x = (t < NPP) ? dqn[t < NPP ? t : 0] : 0.0f;
      hi[t] = tc::to_tf32(x);
      lo[t] = tc::to_tf32(x - __uint_as_float(hi[t]));
    }
    tc::st16(trow, hi);
    tc::st16(trow + 16, lo);
    tc::wait_st();
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::fence_after();
      constexpr uint32_t idescF = tc::idesc_tf32(128, NFACE);
      constexpr uint32_t lbo = 128, sbo = (TcDims<N>::KF / 4) * 128;
      const uint32_t bhi = tc::smem_u32(sBF), blo = tc::smem_u32(sBF + BFSZ);
      const uint32_t dcol = tbase + TcDims<N>::COL_D;
#pragma unroll
      for (int kk = 0; kk < TcDims<N>::KF / 8; ++kk) {
        const uint64_t dh = tc::smem_desc(bhi + 256 * kk, lbo, sbo);
        const uint64_t dl = tc::smem_desc(blo + 256 * kk, lbo, sbo);
        tc::mma_tf32_ts(dcol, tbase + 8 * kk, dh, idescF, kk > 0 ? 1u : 0u);
        tc::mma_tf32_ts(dcol, tbase + 8 * kk, dl, idescF, 1u);
        tc::mma_tf32_ts(dcol, tbase + 16 + 8 * kk, dh, idescF, 1u);
      }
      tc::commit(&mbar);
    }
    bool okF = tc::mbar_wait(&mbar, 1, 1 << 20);
    if (!okF) {
      if (lane == 0) atomicOr(a.err, 1u);
      tc::mbar_wait(&mbar, 1, 1 << 20);
    }
    tc::fence_after();
    uint32_t fv[NFACE];
    tc::ld16(trow + TcDims<N>::COL_D, fv);
    if constexpr (NFACE > 16) tc::ld16(trow + TcDims<N>::COL_D + 16, fv + 16);
    tc::wait_ld();
    if (active) {
      float f[MixedDims<N>::NE3];
#pragma unroll
      for (int q = 0; q < MixedDims<N>::NE3; ++q) f[q] = __uint_as_float(fv[q]);
      store_faces<N>(a, eslot, n, f);
    }
  }
  tc::fence_before();
  __syncthreads();
  // The columns are freed even when both bounded waits gave up: a CTA that kept
  // them would leave later CTAs on this SM in tcgen05.alloc, which waits without
  // bound, while an MMA still pending at the free can only disturb a step that
  // already reports the timeout.
  if (n == 0) {
    tc::fence_after();
    tc::dealloc(tbase, NCOLS);
  }
  if (s == 4 && !a.rhsOnly) {
    residual_commit(a.sc, n, lane, rmax, rabs, rs2);
  }
}

}  // namespace gcfd
