// Device kernels of the DFR right-hand side and SSP(5,4) step.
//
// Data layout in HBM (one global element range; the reference's shards are
// contiguous K ranges and are stitched together on upload):
//   state      Q[n][i][k]    FP64, n = 0..3, i = 0..Np-1, k = 0..K-1
//   faces      QF[n][j][k]   T,    j = e*NpEdge + p (element-local edge e, CCW point p)
//   edge DOFs  FE[n][j][k]   T,    RT edge DOFs (normal flux * ||n||, owner sign/order)
// so a warp reads 32 consecutive elements of one row: every global access is
// coalesced.  One thread owns one element (kernels a, b, e) or one mesh edge
// (kernel c); each element-edge slot of FE is written by exactly one mesh
// edge, so no atomics are needed for the flux scatter.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "euler_physics.cuh"

namespace gcfd {

template <int N>
struct Dims {
  static constexpr int NP = (N + 1) * (N + 2) / 2;
  static constexpr int NE = N + 2;
  static constexpr int NE3 = 3 * (N + 2);
  static constexpr int NF = (N + 2) * (N + 4);
};

struct Scalars {
  unsigned long long gmax[5];   // per stage max edge wave speed (non-negative double bits)
  double time;                  // solver time, frozen for the BCs during a step
  double rhs_time;              // BC time of a standalone RHS evaluation
  double dt[5];                 // per stage dt (global time stepping)
  unsigned long long rmax[4];   // signed max of the final increment, order-preserving key
  unsigned long long rabs[4];   // max |R| (double bits)
  double rsum2[4];              // sum R^2
  unsigned long long gvisc[5];  // per stage max viscous wave speed (artificial dissipation)
  int steps;
  unsigned int errFlags;        // sticky device error bits (1: a tensor-core wait ran out, 2: misaligned
                                //   dynamic shared memory, 4: a TMA copy wait ran out)
  double* rpart;                // [unit][4] per-unit sums of R^2 of the final stage, and
  double* rpart2;               // [kResidBlocks][4] their block sums: both reduced in a fixed order
                                //   (k_resid_blocks, k_step_end), so the residual norms are deterministic
};

__device__ __forceinline__ unsigned long long order_key(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Copies an operator matrix into shared memory in the kernel's arithmetic type.
template <typename T>
__device__ __forceinline__ void stage_operator(T* dst, const double* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = static_cast<T>(src[i]);
}

// ---------------------------------------------------------------------------
// (a) solution points -> edge points: QF = FluxEdgeInterp * Q  per variable,
// InterpolateSolutionToEdges (edges.go:485-488).
template <int N, typename T>
__global__ void __launch_bounds__(128) k_interp(const double* __restrict__ Q, T* __restrict__ QF,
                                                const double* __restrict__ Iop, int K) {
  constexpr int NP = Dims<N>::NP, NE3 = Dims<N>::NE3;
  __shared__ T sI[NE3 * NP];
  stage_operator(sI, Iop, NE3 * NP);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const size_t sK = static_cast<size_t>(K);
#pragma unroll 1
  for (int n = 0; n < 4; ++n) {
    T q[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) q[i] = static_cast<T>(Q[(n * NP + i) * sK + k]);
#pragma unroll 2
    for (int j = 0; j < NE3; ++j) {
      T acc = T(0);
#pragma unroll
      for (int i = 0; i < NP; ++i) acc += sI[j * NP + i] * q[i];
      QF[(n * NE3 + j) * sK + k] = acc;
    }
  }
}

// ---------------------------------------------------------------------------
// (c) edge Riemann fluxes and boundary conditions, CalculateEdgeEulerFlux
// (edges.go:325-452) fused with SetRTFluxOnEdges (edges.go:454-483) and the
// per-edge wave-speed aggregate StoreEdgeAggregates (edges.go:246-289).
template <typename T>
struct EdgeArgs {
  const T* QF;
  T* FE;
  int K, nInt, nBC;
  // interior edges [0, nInt)
  const int* kL;
  const int* kR;
  const int* eLR;        // eL | eR << 2
  const double* nx;      // left outward unit normal
  const double* ny;
  const double* IIL;     // ||n|| scale of the left and right connection
  const double* IIR;
  const double* oohK;    // 1 / hK of the left element
  // boundary edges [nInt, nInt + nBC): kL, eLR (eL only), nx, ny, IIL, oohK share
  // the arrays above at offset nInt; flag and flux-point coordinates are extra.
  const int* bcFlag;
  const double* bx;      // nBC x NpEdge flux-point x of the left element's edge
  const double* by;
  double* edgeSpeed;     // per edge (same order) max wave speed
  unsigned long long* gmax;
  const double* time;
  int flux;
  Gas<T> gas;
  FreeStreamT<T> fsFar, fsIn, fsOut;
  T vbeta, vx0, vy0, vgamma;
};

template <int N, typename T>
__global__ void __launch_bounds__(128) k_edge_flux(EdgeArgs<T> a) {
  constexpr int NE = Dims<N>::NE, NE3 = Dims<N>::NE3;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int nTot = a.nInt + a.nBC;
  T smax = T(0);
  bool active = e < nTot;
  if (active) {
    const size_t sK = static_cast<size_t>(a.K);
    const int kL = a.kL[e];
    const int eL = a.eLR[e] & 3;
    const T nx = static_cast<T>(a.nx[e]), ny = static_cast<T>(a.ny[e]);
    const T IIL = static_cast<T>(a.IIL[e]);
    const T oohK = static_cast<T>(a.oohK[e]);
    smax = T(-1);
    if (e < a.nInt) {
      const int kR = a.kR[e];
      const int eR = a.eLR[e] >> 2;
      const T IIR = static_cast<T>(a.IIR[e]);
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const int jL = eL * NE + p, jR = eR * NE + (NE - 1 - p);
        T qL[4], qR[4], f[4];
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          qL[n] = a.QF[(n * NE3 + jL) * sK + kL];
          qR[n] = a.QF[(n * NE3 + jR) * sK + kR];
        }
        riemann_flux(a.flux, a.gas, qL, qR, nx, ny, f);
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          a.FE[(n * NE3 + jL) * sK + kL] = f[n] * IIL;
          a.FE[(n * NE3 + jR) * sK + kR] = -f[n] * IIR;
        }
        const T ws = oohK * (speed(qL[0], qL[1], qL[2]) + sound_speed(a.gas, qL[0], qL[1], qL[2], qL[3]));
        smax = dmax(smax, ws);
      }
    } else {
      const int b = e - a.nInt;
      const int flag = a.bcFlag[b];
      const T t = static_cast<T>(*a.time);
#pragma unroll
      for (int p = 0; p < NE; ++p) {
        const int jL = eL * NE + p;
        T qi[4], qb[4], f[4];
#pragma unroll
        for (int n = 0; n < 4; ++n) qi[n] = a.QF[(n * NE3 + jL) * sK + kL];
        bool wall = false;
        switch (flag) {
          case 4:  // BC_Far
            riemann_bc(a.fsFar, qi, a.fsFar.qinf, nx, ny, qb);
            break;
          case 1:  // BC_In
            riemann_bc(a.fsIn, qi, a.fsIn.qinf, nx, ny, qb);
            break;
          case 8:  // BC_Out
            riemann_bc(a.fsOut, qi, a.fsOut.qinf, nx, ny, qb);
            break;
          case 9: {  // BC_IVortex: exact state through the characteristic BC
            T ex[4];
            ivortex_state(a.vbeta, a.vx0, a.vy0, a.vgamma, t, static_cast<T>(a.bx[b * NE + p]),
                          static_cast<T>(a.by[b * NE + p]), ex);
            riemann_bc(a.fsFar, qi, ex, nx, ny, qb);
            break;
          }
          case 5:  // BC_Wall
          case 6:  // BC_Cyl
            wall = true;
#pragma unroll
            for (int n = 0; n < 4; ++n) qb[n] = qi[n];
            break;
          default:  // BC_None: physical flux of the interior state
#pragma unroll
            for (int n = 0; n < 4; ++n) qb[n] = qi[n];
            break;
        }
        if (wall) {
          const T pw = pressure(a.gas, qi[0], qi[1], qi[2], qi[3]);
          f[0] = T(0); f[1] = nx * pw; f[2] = ny * pw; f[3] = T(0);
        } else {
          T Fx[4], Fy[4];
          euler_flux(a.gas, qb, Fx, Fy);
#pragma unroll
          for (int n = 0; n < 4; ++n) f[n] = nx * Fx[n] + ny * Fy[n];
        }
#pragma unroll
        for (int n = 0; n < 4; ++n) a.FE[(n * NE3 + jL) * sK + kL] = f[n] * IIL;
        const T ws = oohK * (speed(qb[0], qb[1], qb[2]) + sound_speed(a.gas, qb[0], qb[1], qb[2], qb[3]));
        smax = dmax(smax, ws);
      }
    }
    a.edgeSpeed[e] = static_cast<double>(smax);
  }
  double m = active ? static_cast<double>(smax) : 0.0;
  m = warp_max(m);  // wave speeds are >= 0, so their bit patterns order like integers
  if ((threadIdx.x & 31) == 0)
    atomicMax(a.gmax, static_cast<unsigned long long>(__double_as_longlong(m)));
}

// ---------------------------------------------------------------------------
// (b) RT divergence with the interior transformed fluxes computed in place
// (SetRTFluxInternal euler.go:701-726 + RHSInternalPoints euler.go:665-699),
// fused with (e) the SSP(5,4) stage update (rkAdvance, euler.go:460-566) and
// the residual norms of the final stage.
template <typename T>
struct UpdateArgs {
  int K;
  int stage;                 // 0..4 RK stage; -1: write -Div(F)/J into rhsOut only
  const double* Qs;          // stage input state
  double* Q0;
  double* Q1;
  double* Q2;
  double* Q3;
  double* Q4;
  double* R;                 // Residual (stage 3 RHS, final increment)
  const T* FE;
  const double* Div;         // DivInt, Np x NpFlux
  const double* Jdet;
  const double* Jinv;        // 4 x K
  Scalars* sc;
  double cfl, finalTime;
  int localDT;
  const double* edgeSpeed;
  const int* elemEdge;       // 3 x K, into edgeSpeed
  double* DT;                // K, persistent across stages (local time stepping)
  double* rhsOut;            // stage == -1
  Gas<T> gas;
  // artificial dissipation (read by k_diss_update)
  const double* DissX;       // [4][Np + 3NpEdge][K]
  const double* DissY;
  const double* VF;          // [edge][4][NpEdge] viscous normal flux
  const double* viscSpeed;   // per edge
  const unsigned long long* sigV;  // per vertex sigma (double bits)
  const int* etov;           // [3][K]
  const double* V;           // Np x Np
  const double* Vinv;
  const double* mf;          // Np
  const double* IIE;         // [3][K]
  const int* ekL;
  const int* eLR;
  const unsigned long long* gvisc;  // per stage
  double* DTVisc;            // K, persistent (CalcElementMaxWaveSpeed never resets it)
  double cdiff;              // 1/(N+1)^2
  double* tapeRHS;           // when set, the stage's RHS is stored there (adjoint tape)
  double* tapeRHSpre;        // k_diss_update: the RHS before the modal filter (adjoint tape)
};

static __constant__ double kSSP[5][6] = {
    {0.391752226571890, 0, 0, 0, 0, 0},
    {0.444370493651235, 0.555629506348765, 0.368410593050371, 0, 0, 0},
    {0.620101851488403, 0.379898148511597, 0.251891774271694, 0, 0, 0},
    {0.178079954393132, 0.821920045606868, 0.544974750228521, 0, 0, 0},
    {0.517231671970585, 0.096059710526146, 0.386708617503269, 0.063692468666290,
     0.226007483236906, 0}};

// One point of the SSP(5,4) stage update (rkAdvance, euler.go:460-566); the
// final stage folds the increment into the residual partials.
template <typename T>
__device__ __forceinline__ void ssp_stage_update(const UpdateArgs<T>& a, size_t ind, double rhs, double dtk,
                                                 double& rmax, double& rabs, double& rs2) {
  const int s = a.stage;
  const double dtRHS = dtk * rhs;
  if (s == 0) {
    a.Q1[ind] = a.Q0[ind] + kSSP[0][0] * dtRHS;
  } else if (s == 1) {
    a.Q2[ind] = kSSP[1][0] * a.Q0[ind] + kSSP[1][1] * a.Q1[ind] + kSSP[1][2] * dtRHS;
  } else if (s == 2) {
    a.Q3[ind] = kSSP[2][0] * a.Q0[ind] + kSSP[2][1] * a.Q2[ind] + kSSP[2][2] * dtRHS;
  } else if (s == 3) {
    a.R[ind] = rhs;
    a.Q4[ind] = kSSP[3][0] * a.Q0[ind] + kSSP[3][1] * a.Q3[ind] + kSSP[3][2] * dtRHS;
  } else {
    const double dtR3 = dtk * a.R[ind];
    const double q0 = a.Q0[ind];
    const double inc = -q0 + kSSP[4][0] * a.Q2[ind] + kSSP[4][1] * a.Q3[ind] + kSSP[4][2] * a.Q4[ind] +
                       kSSP[4][3] * dtR3 + kSSP[4][4] * dtRHS;
    a.R[ind] = inc;
    a.Q0[ind] = q0 + inc;
    rmax = fmax(rmax, inc);
    rabs = fmax(rabs, fabs(inc));
    rs2 += inc * inc;
    if (inc != inc) rabs = inc;  // keep NaN visible
  }
}

// Block-wide residual partials of the final stage -> Scalars: the maxima by
// (order-independent) atomics, the FP64 sums of squares of each warp into its
// own slot of sc->rpart (unit = blockIdx.x * 4 + warp), summed by k_resid_blocks
// and k_step_end.
__device__ __forceinline__ void residual_reduce(Scalars* sc, const double rmax[4], const double rabs[4],
                                                const double rs2[4]) {
  const size_t unit = static_cast<size_t>(blockIdx.x) * 4 + (threadIdx.x >> 5);
#pragma unroll
  for (int n = 0; n < 4; ++n) {
    const unsigned long long km = warp_max_u64(order_key(rmax[n]));
    const double am = warp_max(rabs[n]);
    const double s2 = warp_sum(rs2[n]);
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&sc->rmax[n], km);
      atomicMax(&sc->rabs[n], static_cast<unsigned long long>(__double_as_longlong(am)));
      sc->rpart[unit * 4 + n] = s2;
    }
  }
}

// stage -1: write -Div(F)/J to rhsOut. Steps with artificial dissipation use
// that form too, into a scratch array; k_diss_update then adds the viscous
// terms, filters and applies the stage update.
template <int N, typename T>
__global__ void __launch_bounds__(128) k_div_update(UpdateArgs<T> a) {
  constexpr int NP = Dims<N>::NP, NE3 = Dims<N>::NE3, NF = Dims<N>::NF;
  __shared__ T sD[NP * NF];
  stage_operator(sD, a.Div, NP * NF);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = k < a.K;
  const size_t sK = static_cast<size_t>(a.K);
  double rloc_max[4], rloc_abs[4], rloc_s2[4];
#pragma unroll
  for (int n = 0; n < 4; ++n) { rloc_max[n] = -1.7976931348623157e308; rloc_abs[n] = 0.0; rloc_s2[n] = 0.0; }
  if (active) {
    const double jd = a.Jdet[k];
    const T Jd = static_cast<T>(jd);
    const T J0 = static_cast<T>(a.Jinv[k]), J1 = static_cast<T>(a.Jinv[sK + k]);
    const T J2 = static_cast<T>(a.Jinv[2 * sK + k]), J3 = static_cast<T>(a.Jinv[3 * sK + k]);
    T acc[4][NP];
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int r = 0; r < NP; ++r) acc[n][r] = T(0);
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      T q[4], Fx[4], Fy[4];
#pragma unroll
      for (int n = 0; n < 4; ++n) q[n] = static_cast<T>(a.Qs[(n * NP + i) * sK + k]);
      euler_flux(a.gas, q, Fx, Fy);
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const T Fr = Jd * (J0 * Fx[n] + J1 * Fy[n]);
        const T Fs = Jd * (J2 * Fx[n] + J3 * Fy[n]);
#pragma unroll
        for (int r = 0; r < NP; ++r) acc[n][r] += sD[r * NF + i] * Fr + sD[r * NF + NP + i] * Fs;
      }
    }
#pragma unroll
    for (int j = 0; j < NE3; ++j) {
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const T f = a.FE[(n * NE3 + j) * sK + k];
#pragma unroll
        for (int r = 0; r < NP; ++r) acc[n][r] += sD[r * NF + 2 * NP + j] * f;
      }
    }
    const T mooj = -(T(1) / Jd);
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int r = 0; r < NP; ++r) acc[n][r] = acc[n][r] * mooj;
    if (a.stage < 0) {
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int r = 0; r < NP; ++r)
          a.rhsOut[(n * NP + r) * sK + k] = static_cast<double>(acc[n][r]);
    } else {
      // Time step of this stage (CalcElementMaxWaveSpeed, calculateGlobalDT,
      // CalculateLocalDT: edges.go:291-323, euler.go:945-1002).
      double dtk;
      if (a.localDT) {
        double v = (a.stage == 0) ? -100.0 : a.DT[k];
#pragma unroll
        for (int ed = 0; ed < 3; ++ed) v = fmax(v, a.edgeSpeed[a.elemEdge[ed * sK + k]]);
        dtk = a.cfl / v;
        a.DT[k] = dtk;
      } else {
        const double gm = __longlong_as_double(static_cast<long long>(a.sc->gmax[a.stage]));
        dtk = a.cfl / gm;
        const double t = a.sc->time;
        if (t + dtk > a.finalTime) dtk = a.finalTime - t;
        if (k == 0) a.sc->dt[a.stage] = dtk;
      }
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int r = 0; r < NP; ++r) {
          if (a.tapeRHS) a.tapeRHS[(n * NP + r) * sK + k] = static_cast<double>(acc[n][r]);
          ssp_stage_update(a, (n * NP + r) * sK + k, static_cast<double>(acc[n][r]), dtk, rloc_max[n],
                           rloc_abs[n], rloc_s2[n]);
        }
    }
  }
  if (a.stage == 4) residual_reduce(a.sc, rloc_max, rloc_abs, rloc_s2);
}

// Step bookkeeping: reset the per-stage reductions before a step, advance the
// time by the last stage's dt after it (Solve, euler.go:176-181).
static __global__ void k_step_begin(Scalars* sc) {
  const int t = threadIdx.x;
  if (t < 5) {
    sc->gmax[t] = 0ULL;
    sc->gvisc[t] = 0ULL;
  }
  if (t < 4) {
    sc->rmax[t] = 0ULL;
    sc->rabs[t] = 0ULL;
  }
}
// The residual sums of squares of a step: the final stage wrote one FP64 sum
// per unit into sc->rpart; k_resid_blocks sums fixed contiguous runs of units
// (block b takes units [b*per, (b+1)*per), thread t every 256th of them, then a
// fixed tree) into sc->rpart2, and k_step_end sums those kResidBlocks values
// the same way.  The order never depends on scheduling, so the norms are the
// same bits run to run.
constexpr int kResidBlocks = 128;
constexpr int kResidBlockThreads = 256;

// Fixed-order block sum of 4 per-thread values; thread 0 returns the totals.
template <int T>
__device__ __forceinline__ void block_sum4(double s[4], double (*red)[T / 32]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int n = 0; n < 4; ++n) {
    s[n] = warp_sum(s[n]);
    if (lane == 0) red[n][w] = s[n];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      double v = 0.0;
      for (int i = 0; i < T / 32; ++i) v += red[n][i];
      s[n] = v;
    }
  }
}

static __global__ void __launch_bounds__(kResidBlockThreads) k_resid_blocks(Scalars* sc, int nunits) {
  __shared__ double red[4][kResidBlockThreads / 32];
  const int per = (nunits + kResidBlocks - 1) / kResidBlocks;
  const int u0 = blockIdx.x * per, u1 = min(u0 + per, nunits);
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  const double2* p = reinterpret_cast<const double2*>(sc->rpart);
  for (int u = u0 + threadIdx.x; u < u1; u += kResidBlockThreads) {
    const double2 a = p[2 * u], b = p[2 * u + 1];
    s[0] += a.x;
    s[1] += a.y;
    s[2] += b.x;
    s[3] += b.y;
  }
  block_sum4<kResidBlockThreads>(s, red);
  if (threadIdx.x == 0)
#pragma unroll
    for (int n = 0; n < 4; ++n) sc->rpart2[blockIdx.x * 4 + n] = s[n];
}

static __global__ void __launch_bounds__(kResidBlocks) k_step_end(Scalars* sc, int localDT) {
  __shared__ double red[4][kResidBlocks / 32];
  double s[4];
#pragma unroll
  for (int n = 0; n < 4; ++n) s[n] = sc->rpart2[threadIdx.x * 4 + n];
  block_sum4<kResidBlocks>(s, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int n = 0; n < 4; ++n) sc->rsum2[n] = s[n];
    if (!localDT) sc->time += sc->dt[4];
    sc->steps += 1;
  }
}

}  // namespace gcfd
