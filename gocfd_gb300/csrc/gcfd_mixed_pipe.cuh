// Persistent, TMA-pipelined stage kernel of the mixed path.
//
// Same arithmetic as k_mixed_stage (FMA divergence) and k_mixed_stage_tc
// (3xTF32 divergence on tcgen05), reorganised for latency: a grid of
// (SMs x resident CTAs) CTAs walks the 32-element blocks, and while a CTA
// computes block j, the Tensor Memory Accelerator already copies block j+1's
// inputs into the other half of a double-buffered shared-memory tile:
//   dQ0, D_s     [4][NP][32] FP32 tiles (3-D tensor maps over [n][i][k])
//   geo [6][32], eslot [3][32], IInII [3][32], base [32][8]
// so the element loads leave the critical path.  One elected thread issues the
// copies (cp.async.bulk.tensor, completion on an mbarrier) and L2 prefetches of
// what the stage update will read one block later (the compensated state, and
// at stage 4 the increments D2, D3 and the stage-3 RHS).  The edge fluxes are
// a gather by edge slot and stay per-thread cp.async copies, overlapped with
// the interior flux work as in the one-block kernels.
//
// Every wait is bounded: a copy that does not land sets bit 2 of the error
// word, the CTA waits (bounded) for its copy in flight, frees its Tensor Memory
// and stops.
#pragma once
#include <cuda.h>

#include "gcfd_mixed.cuh"
#include "gcfd_mixed_tc.cuh"
#include "gcfd_tc.cuh"

namespace gcfd {

// Tensor maps of the stage kernel's inputs (built once per context).
struct StageMaps {
  CUtensorMap dQ0;        // [4][NP][K] FP32, box (32, NP, 4)
  CUtensorMap D[5];       // D[1..4], same box (D[0] unused)
  CUtensorMap R3, Qhi, Qlo;
  CUtensorMap QhiRow, QloRow;  // box (32, 1, 4): solution point 0 only
  CUtensorMap geo;        // [6][K], box (32, 6)
  CUtensorMap eslot;      // [3][K] int32, box (32, 3)
  CUtensorMap II;         // [3][K], box (32, 3)
  CUtensorMap base;       // [K][8] FP32 (4 float2), box (8, 32)
};

namespace tma {

__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(tc::smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void load2d(uint32_t dst, const CUtensorMap* m, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];\n" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(m)), "r"(tc::smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void load3d(uint32_t dst, const CUtensorMap* m, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(m)), "r"(tc::smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}
__device__ __forceinline__ void prefetch3d(const CUtensorMap* m, int x, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global [%0, {%1, %2, %3}];\n" ::"l"(
                   reinterpret_cast<uint64_t>(m)),
               "r"(x), "r"(y), "r"(z)
               : "memory");
}

}  // namespace tma

// Shared-memory layout (bytes; every TMA destination 128-byte aligned).
template <int N, bool TC>
struct PipeLayout {
  static constexpr int NP = MixedDims<N>::NP, NE3 = MixedDims<N>::NE3, NPP = MixedDims<N>::NPP;
  static constexpr int NF = MixedDims<N>::NF;
  __host__ __device__ static constexpr int al(int b) { return (b + 127) & ~127; }
  static constexpr int TILE = 4 * NP * 32 * 4;  // one [4][NP][32] FP32 tile
  static constexpr int Q0 = 0;
  static constexpr int DS = Q0 + al(TILE);
  static constexpr int GEO = DS + al(TILE);
  static constexpr int ESL = GEO + al(6 * 32 * 4);
  static constexpr int II = ESL + al(3 * 32 * 4);
  static constexpr int BASE = II + al(3 * 32 * 4);
  static constexpr int BUF = BASE + al(32 * 8 * 4);  // one pipeline buffer
  static constexpr int FH = 2 * BUF;                 // [4][NE3][32] gathered edge fluxes
  static constexpr int CORR = FH + al(4 * NE3 * 32 * 4);
  static constexpr int OPS = CORR + al(4 * 3 * 32 * 4);
  static constexpr int OPS_BYTES = TC ? 2 * TcDims<N>::BSZ * 4 : 0;  // DivInt hi/lo for the tensor core
  static constexpr int BAR = OPS + al(OPS_BYTES);
  static constexpr int BYTES = BAR + 64;
  // Bytes one block's copies deliver (the full boxes, out-of-range elements included).
  __host__ __device__ static constexpr uint32_t tx_bytes(int stage) {
    return static_cast<uint32_t>((stage >= 1 ? 2 : 1) * TILE + (6 + 3 + 3 + 8) * 32 * 4);
  }
};

constexpr int kPipeWaitLimit = 1 << 20;

template <int N, bool TC>
__global__ void __launch_bounds__(128, 4) k_mixed_stage_pipe(const __grid_constant__ StageMaps maps, MixedArgs a) {
  using L = PipeLayout<N, TC>;
  constexpr int NP = MixedDims<N>::NP, NE = MixedDims<N>::NE, NE3 = MixedDims<N>::NE3;
  constexpr int NPP = MixedDims<N>::NPP, NEP = MixedDims<N>::NEP;
  constexpr int NFP = TcDims<N>::NFP, BSZ = TcDims<N>::BSZ, NCOLS = TcDims<N>::NCOLS;
  extern __shared__ __align__(128) unsigned char sm[];
  const int n = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = a.stage;
  const int nblk = (a.K + 31) >> 5;
  if (tc::smem_u32(sm) & 127) {  // TMA destinations must be 128-byte aligned
    if (threadIdx.x == 0) atomicOr(a.err, 2u);
    return;
  }
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L::BAR);  // [0], [1]: tile copies; [2]: MMA
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + L::BAR + 32);
  double* sdt = reinterpret_cast<double*>(sm + L::BAR + 40);
  float* sOps = reinterpret_cast<float*>(sm + L::OPS);
  float* sfh = reinterpret_cast<float*>(sm + L::FH);      // [4][NE3][32]
  float* scorr = reinterpret_cast<float*>(sm + L::CORR);  // [4][3][32]
  if (TC) {
    for (int i = threadIdx.x; i < 2 * BSZ; i += blockDim.x) sOps[i] = a.Btc[i];
    tc::fence_proxy_async();  // read by the tensor core
  }
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_init(&bar[2], 1);
  }
  if (TC && n == 0) {
    tc::alloc(tslot, NCOLS);
    tc::fence_before();
  }
  if (threadIdx.x == 0 && needs_global_dt(a, s)) *sdt = global_stage_dt(a, s);
  __syncthreads();
  const double dtGlobal = needs_global_dt(a, s) ? *sdt : 0.0;
  if (TC) tc::fence_after();
  const uint32_t tbase = TC ? *tslot : 0u;
  const uint32_t trow = tbase + (static_cast<uint32_t>(n * 32) << 16);  // this warp's TMEM lanes
  const size_t sK = static_cast<size_t>(a.K);
  const uint32_t txBytes = L::tx_bytes(s);

  auto issue = [&](int blk, int buf) {
    uint64_t* b = &bar[buf];
    const uint32_t dst = tc::smem_u32(sm + buf * L::BUF);
    const int x = blk * 32;
    tma::expect_tx(b, txBytes);
    tma::load3d(dst + L::Q0, &maps.dQ0, b, x, 0, 0);
    if (s >= 1) tma::load3d(dst + L::DS, &maps.D[s], b, x, 0, 0);
    tma::load2d(dst + L::GEO, &maps.geo, b, x, 0);
    tma::load2d(dst + L::ESL, &maps.eslot, b, x, 0);
    tma::load2d(dst + L::II, &maps.II, b, x, 0);
    tma::load2d(dst + L::BASE, &maps.base, b, 0, x);
  };
  // What stage_tail reads from global memory, into L2 ahead of use.
  auto prefetch_tail = [&](int blk) {
    if (s < 0 || a.rhsOnly) return;
    const int x = blk * 32;
    if (s == 4) {
      tma::prefetch3d(&maps.Qhi, x, 0, 0);
      tma::prefetch3d(&maps.Qlo, x, 0, 0);
      tma::prefetch3d(&maps.D[2], x, 0, 0);
      tma::prefetch3d(&maps.D[3], x, 0, 0);
      tma::prefetch3d(&maps.R3, x, 0, 0);
    } else {
      tma::prefetch3d(&maps.QhiRow, x, 0, 0);
      tma::prefetch3d(&maps.QloRow, x, 0, 0);
    }
  };

  int blk = blockIdx.x;
  if (threadIdx.x == 0 && blk < nblk) {
    issue(blk, 0);
    prefetch_tail(blk);
  }
  float rmax = -3.4028235e38f, rabs = 0.0f;
  float2 rs2 = make_float2(0.0f, 0.0f);
  for (int j = 0; blk < nblk; ++j, blk += gridDim.x) {
    const int buf = j & 1;
    const uint32_t par = (j >> 1) & 1;
    const bool tout = !tc::mbar_wait(&bar[buf], par, kPipeWaitLimit);
    // Uniform decision; also certifies that every thread is done with block
    // j-1, whose buffer the next copy overwrites.
    if (__syncthreads_or(tout)) {
      if (threadIdx.x == 0) {
        atomicOr(a.err, 4u);
        tc::mbar_wait(&bar[buf], par, kPipeWaitLimit);  // the copy in flight
      }
      __syncthreads();
      break;
    }
    const int nxt = blk + gridDim.x;
    if (threadIdx.x == 0 && nxt < nblk) {
      issue(nxt, buf ^ 1);
      prefetch_tail(nxt);
    }
    const unsigned char* B = sm + buf * L::BUF;
    const float* tQ0 = reinterpret_cast<const float*>(B + L::Q0);
    const float* tDs = reinterpret_cast<const float*>(B + L::DS);
    const float* tGeo = reinterpret_cast<const float*>(B + L::GEO);
    const int* tEsl = reinterpret_cast<const int*>(B + L::ESL);
    const float* tII = reinterpret_cast<const float*>(B + L::II);
    const float* tBase = reinterpret_cast<const float*>(B + L::BASE);
    const int k = blk * 32 + lane;
    const bool active = k < a.K;
    const size_t off = static_cast<size_t>(n) * NP * sK + k;

    // Edge fluxes of this block: per-thread gather, waited for after the interior work.
    int eslot[3];
    float eII[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      eslot[e] = tEsl[e * 32 + lane];
      eII[e] = tII[e * 32 + lane];
    }
    if (active) {
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        const float* fh = a.fhat + (static_cast<size_t>(eslot[e] >> 1) * 4 + n) * NEP;
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          const uint32_t dst = tc::smem_u32(&sfh[(n * NE3 + e * NE + p) * 32 + lane]);
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(fh + p));
        }
        if (eslot[e] & 1) {
          const uint32_t dst = tc::smem_u32(&scorr[(n * 3 + e) * 32 + lane]);
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst),
                       "l"(a.corr + static_cast<size_t>(eslot[e] >> 1) * 4 + n));
        }
      }
    }
    asm volatile("cp.async.commit_group;\n" ::);
    // Local time step (DT persists across stages; warp 0 rewrites it in the
    // update, after a CTA barrier).
    double dtLocal = dtGlobal;
    if (active && a.localDT && s >= 0 && !a.rhsOnly) {
      double v = (s == 0) ? -100.0 : a.DT[k];
#pragma unroll
      for (int e = 0; e < 3; ++e) v = fmax(v, a.edgeSpeed[eslot[e] >> 1]);
      dtLocal = a.cfl / v;
    }
    const float Jd = tGeo[lane], J0 = tGeo[32 + lane], J1 = tGeo[64 + lane];
    const float J2 = tGeo[96 + lane], J3 = tGeo[128 + lane], ooJ = tGeo[160 + lane];
    const float gm1 = a.gamma - 1.0f;
    float bq[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) bq[c] = active ? tBase[lane * 8 + 2 * c] : ((c == 0 || c == 3) ? 1.0f : 0.0f);
    const BasePrim b = base_prim(bq, gm1);
    float d0[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) d0[c] = (s >= 1) ? tDs[(c * NP) * 32 + lane] : 0.0f;
    float rhs[NP];
    if constexpr (TC) {
      // The GEMM row in the permuted K order (Fr_0, Fs_0, Fr_1, ..., edge
      // DOFs, zeros), split hi/lo and stored to Tensor Memory 16 columns at a time.
      float dof[NFP];
      auto flush = [&](int jj) {
        if ((jj & 15) == 15) {
          const int c = jj >> 4;
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
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        float d[4];
#pragma unroll
        for (int c = 0; c < 4; ++c)
          d[c] = tQ0[(c * NP + i) * 32 + lane] + ((s >= 1) ? tDs[(c * NP + i) * 32 + lane] - d0[c] : 0.0f);
        const DeltaPrim q = delta_prim(b, d, gm1);
        float fx, fy;
        delta_flux_c(n, b, d, q, &fx, &fy);
        dof[2 * i] = Jd * (J0 * fx + J1 * fy);
        flush(2 * i);
        dof[2 * i + 1] = Jd * (J2 * fx + J3 * fy);
        flush(2 * i + 1);
      }
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        const bool right = eslot[e] & 1;
        const float ii = eII[e];
        const float cc = (active && right) ? scorr[(n * 3 + e) * 32 + lane] : 0.0f;
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          const int jj = 2 * NP + e * NE + p;
          const float f = active ? (right ? -(sfh[(n * NE3 + e * NE + NE - 1 - p) * 32 + lane] - cc)
                                          : sfh[(n * NE3 + e * NE + p) * 32 + lane])
                                 : 0.0f;
          dof[jj] = f * ii;
          flush(jj);
        }
      }
#pragma unroll
      for (int jj = 2 * NP + 3 * NE; jj < NFP; ++jj) {
        dof[jj] = 0.0f;
        flush(jj);
      }
      tc::wait_st();
      tc::fence_before();
      __syncthreads();
      if (threadIdx.x == 0) {
        tc::fence_after();
        constexpr uint32_t idesc = tc::idesc_tf32(128, TcDims<N>::NOUT);
        constexpr uint32_t lbo = 128, sbo = (NFP / 4) * 128;
        const uint32_t bhi = tc::smem_u32(sOps), blo = tc::smem_u32(sOps + BSZ);
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
        tc::commit(&bar[2]);
      }
      if (!tc::mbar_wait(&bar[2], j & 1, kPipeWaitLimit)) {
        if (lane == 0) atomicOr(a.err, 1u);
        tc::mbar_wait(&bar[2], j & 1, kPipeWaitLimit);  // let the MMAs drain
      }
      tc::fence_after();
      uint32_t dv[16];
      tc::ld16(trow + TcDims<N>::COL_D, dv);
      tc::wait_ld();
#pragma unroll
      for (int r = 0; r < NP; ++r) rhs[r] = -__uint_as_float(dv[r]) * ooJ;
    } else {
      float acc[NP];
#pragma unroll
      for (int r = 0; r < NP; ++r) acc[r] = 0.0f;
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        float d[4];
#pragma unroll
        for (int c = 0; c < 4; ++c)
          d[c] = tQ0[(c * NP + i) * 32 + lane] + ((s >= 1) ? tDs[(c * NP + i) * 32 + lane] - d0[c] : 0.0f);
        const DeltaPrim q = delta_prim(b, d, gm1);
        float fx, fy;
        delta_flux_c(n, b, d, q, &fx, &fy);
        const float Fr = Jd * (J0 * fx + J1 * fy);
        const float Fs = Jd * (J2 * fx + J3 * fy);
#pragma unroll
        for (int r = 0; r < NP; ++r)
          acc[r] = fmaf(div_op<N>(i * NPP + r), Fr, fmaf(div_op<N>((NP + i) * NPP + r), Fs, acc[r]));
      }
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        const bool right = eslot[e] & 1;
        const float ii = eII[e];
        const float cc = (active && right) ? scorr[(n * 3 + e) * 32 + lane] : 0.0f;
#pragma unroll
        for (int p = 0; p < NE; ++p) {
          const float dof = active ? (right ? -(sfh[(n * NE3 + e * NE + NE - 1 - p) * 32 + lane] - cc) * ii
                                            : sfh[(n * NE3 + e * NE + p) * 32 + lane] * ii)
                                   : 0.0f;
#pragma unroll
          for (int r = 0; r < NP; ++r) acc[r] = fmaf(div_op<N>((2 * NP + e * NE + p) * NPP + r), dof, acc[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < NP; ++r) rhs[r] = -acc[r] * ooJ;
      // DT[k] was read above by every variable's thread; warp 0 rewrites it.
      if (a.localDT) __syncthreads();
    }
    if (active) {
      float dq0[NP], ds[NP];
#pragma unroll
      for (int r = 0; r < NP; ++r) {
        dq0[r] = tQ0[(n * NP + r) * 32 + lane];
        ds[r] = (s >= 1) ? tDs[(n * NP + r) * 32 + lane] : 0.0f;
      }
      stage_tail<N>(a, eslot, n, k, off, sK, s, rhs, dq0, ds, dtLocal, rmax, rabs, rs2);
    }
    if (TC) tc::fence_before();  // this block's TMEM reads before the next block's stores
  }
  if (TC) {
    __syncthreads();
    // freed even after a wait that gave up (see k_mixed_stage_tc): kept
    // columns would hold later CTAs in an unbounded tcgen05.alloc
    if (n == 0) {
      tc::fence_after();
      tc::dealloc(tbase, NCOLS);
    }
  }
  if (s == 4 && !a.rhsOnly) {
    residual_commit(a.sc, n, lane, rmax, rabs, rs2);
  }
}

}  // namespace gcfd
