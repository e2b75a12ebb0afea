// The kernels of one polynomial order: this file is compiled once per order
// with -DGCFD_ORDER=N (0..4) and exports that order's launcher table
// (order_ops_N) and the set-up that must sit beside the kernels: the mixed
// path's constant-memory operators, the tensor-core operand and the launch
// shapes of the tensor-core and persistent stage kernels.
#include <cstring>

#include "gcfd_launch.cuh"

#ifndef GCFD_ORDER
#error "compile with -DGCFD_ORDER=<0..4>"
#endif
#define GCFD_CAT2(a, b) a##b
#define GCFD_CAT(a, b) GCFD_CAT2(a, b)

namespace gcfd_host {
namespace {

constexpr int kN = GCFD_ORDER;

// Tensor-core operand: DivInt (16 x NFP, zero padded, columns in the stage
// kernel's K order) split into TF32 hi and lo parts, each laid out as the
// kernel's shared-memory B operand, and
// the dynamic shared memory that keeps the stage kernel's CTAs per SM within
// the Tensor Memory they allocate (512 columns per SM).
float tf32_round(float x) {
  uint32_t u;
  std::memcpy(&u, &x, sizeof(u));
  u = (u + 0x1000u) & 0xFFFFE000u;  // nearest, ties away from zero, like cvt.rna.tf32.f32
  float r;
  std::memcpy(&r, &u, sizeof(r));
  return r;
}

template <int N>
int build_tc_n(gcfd_ctx* c) {
  constexpr int NFP = TcDims<N>::NFP, BSZ = TcDims<N>::BSZ, NCOLS = TcDims<N>::NCOLS;
  std::vector<float> b(2 * static_cast<size_t>(BSZ), 0.f);
  // K order of the kernel's rows: Fr_0, Fs_0, Fr_1, Fs_1, ..., then the edge DOFs.
  const int Np = c->Np;
  for (int r = 0; r < Np; ++r)
    for (int j = 0; j < c->NF; ++j) {
      const int col = j < 2 * Np ? ((j & 1) ? Np + j / 2 : j / 2) : j;
      const double v = c->el.DivInt(r, col);
      const float hi = tf32_round(static_cast<float>(v));
      const float lo = tf32_round(static_cast<float>(v - static_cast<double>(hi)));
      b[tc_b_index(r, j, NFP)] = hi;
      b[BSZ + tc_b_index(r, j, NFP)] = lo;
    }
  int rc = upload(c, &c->mBtc, b);
  if (rc) return rc;
  // FluxEdgeInterp (3 NpEdge x Np) as the face GEMM's B: N = face point q, K = solution point i.
  constexpr int KF = TcDims<N>::KF, BFSZ = TcDims<N>::BFSZ;
  std::vector<float> bf(2 * static_cast<size_t>(BFSZ), 0.f);
  for (int q = 0; q < 3 * c->NE; ++q)
    for (int i = 0; i < Np; ++i) {
      const double v = c->el.FluxEdgeInterp(q, i);
      const float hi = tf32_round(static_cast<float>(v));
      const float lo = tf32_round(static_cast<float>(v - static_cast<double>(hi)));
      bf[tc_b_index(q, i, KF)] = hi;
      bf[BFSZ + tc_b_index(q, i, KF)] = lo;
    }
  if ((rc = upload(c, &c->mBtcF, bf))) return rc;
  cudaFuncAttributes attr{};
  GCFD_CUDA(c, cudaFuncGetAttributes(&attr, k_mixed_stage_tc<N>));
  const int perSM = 512 / NCOLS;  // CTAs whose TMEM fits at once
  int smemPerSM = 0;
  GCFD_CUDA(c, cudaDeviceGetAttribute(&smemPerSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->prm.device));
  // Smallest per-CTA footprint (with the shared memory the runtime reserves per
  // CTA) at which perSM + 1 CTAs no longer fit on an SM.
  int reserved = 0;
  GCFD_CUDA(c, cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, c->prm.device));
  const int want = smemPerSM / (perSM + 1) + 1 - reserved;
  c->tcDynSmem = std::max(0, want - static_cast<int>(attr.sharedSizeBytes));
  if (c->tcDynSmem > 48 * 1024)
    GCFD_CUDA(c, cudaFuncSetAttribute(k_mixed_stage_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      c->tcDynSmem));
  return GCFD_OK;
}

// cuTensorMapEncodeTiled, resolved through the runtime so the library needs no libcuda link.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Tensor maps and launch shape of the persistent stage kernel.  K % 4 != 0
// (row strides not a multiple of 16 bytes) keeps the one-block kernels.
template <int N, bool TC>
int build_pipe_n(gcfd_ctx* c) {
  c->pipe = false;
  if (c->K % 4 != 0) return GCFD_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
      q != cudaDriverEntryPointSuccess || fn == nullptr) {
    cudaGetLastError();
    return fail(c, GCFD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  }
  const auto enc = reinterpret_cast<EncodeTiledFn>(fn);
  const cuuint64_t K = static_cast<cuuint64_t>(c->K), NP = static_cast<cuuint64_t>(c->Np);
  const cuuint32_t es[3] = {1, 1, 1};
  auto map3 = [&](CUtensorMap* m, float* p, cuuint32_t rows) {
    const cuuint64_t dims[3] = {K, NP, 4};
    const cuuint64_t strides[2] = {K * 4, NP * K * 4};
    const cuuint32_t box[3] = {32, rows, 4};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, p, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  auto map2 = [&](CUtensorMap* m, CUtensorMapDataType t, void* p, cuuint64_t d0, cuuint64_t d1, cuuint64_t stride,
                  cuuint32_t b0, cuuint32_t b1) {
    const cuuint64_t dims[2] = {d0, d1};
    const cuuint64_t strides[1] = {stride};
    const cuuint32_t box[2] = {b0, b1};
    return enc(m, t, 2, p, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  StageMaps& M = c->pipeMaps;
  const cuuint32_t np = static_cast<cuuint32_t>(c->Np);
  bool ok = map3(&M.dQ0, c->dQ0, np);
  for (int i = 1; i <= 4; ++i) ok = ok && map3(&M.D[i], c->Dk[i], np);
  M.D[0] = M.D[1];
  ok = ok && map3(&M.R3, c->R3, np) && map3(&M.Qhi, c->Qhi, np) && map3(&M.Qlo, c->Qlo, np) &&
       map3(&M.QhiRow, c->Qhi, 1) && map3(&M.QloRow, c->Qlo, 1);
  ok = ok && map2(&M.geo, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, c->mgeo, K, 6, K * 4, 32, 6) &&
       map2(&M.eslot, CU_TENSOR_MAP_DATA_TYPE_INT32, c->meslot, K, 3, K * 4, 32, 3) &&
       map2(&M.II, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, c->mII, K, 3, K * 4, 32, 3) &&
       map2(&M.base, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, c->mbase, 8, K, 32, 8, 32);
  if (!ok) return fail(c, GCFD_ERR_CUDA, "tensor map encoding failed for the stage kernel");
  int smem = PipeLayout<N, TC>::BYTES;
  if (TC) {
    // Pad the footprint so no more CTAs share an SM than its Tensor Memory holds.
    const int perSM = 512 / TcDims<N>::NCOLS;
    int smemPerSM = 0, reserved = 0;
    GCFD_CUDA(c, cudaDeviceGetAttribute(&smemPerSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->prm.device));
    GCFD_CUDA(c, cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, c->prm.device));
    smem = std::max(smem, smemPerSM / (perSM + 1) + 1 - reserved);
  }
  GCFD_CUDA(c, cudaFuncSetAttribute(k_mixed_stage_pipe<N, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int occ = 0, sms = 0;
  GCFD_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mixed_stage_pipe<N, TC>, 128, smem));
  if (TC) occ = std::min(occ, 512 / TcDims<N>::NCOLS);
  if (occ < 1) return fail(c, GCFD_ERR_CUDA, "stage kernel: no CTA fits on an SM");
  GCFD_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->prm.device));
  c->pipeGrid = sms * occ;
  c->pipeSmem = smem;
  c->pipe = true;
  return GCFD_OK;
}

// The mixed path's FP32 operators into this order's constant-memory copies
// (identical for every context of the same order, so concurrent contexts
// agree): DivInt^T, rows = flux DOF j, cols = output point r padded to NPP;
// FluxEdgeInterp^T, rows = solution point i, cols = face point padded to NE3P;
// and the modal filter's operators (PerssonC0 on the mixed path).
int mixed_consts(gcfd_ctx* c) {
  constexpr int NPP = MixedDims<kN>::NPP, NE3P = MixedDims<kN>::NE3P;
  const int Np = c->Np, NF = c->NF, NE = c->NE;
  std::vector<float> divT(static_cast<size_t>(NF) * NPP, 0.f), iop(static_cast<size_t>(NPP) * NE3P, 0.f);
  for (int j = 0; j < NF; ++j)
    for (int r = 0; r < Np; ++r) divT[static_cast<size_t>(j) * NPP + r] = static_cast<float>(c->el.DivInt(r, j));
  for (int j = 0; j < 3 * NE; ++j)
    for (int i = 0; i < Np; ++i) iop[static_cast<size_t>(i) * NE3P + j] = static_cast<float>(c->el.FluxEdgeInterp(j, i));
  const void* const d[5] = {&cDivT0, &cDivT1, &cDivT2, &cDivT3, &cDivT4};
  const void* const io[5] = {&cIopT0, &cIopT1, &cIopT2, &cIopT3, &cIopT4};
  const void* const sv[5] = {&cV0, &cV1, &cV2, &cV3, &cV4};
  const void* const svi[5] = {&cVi0, &cVi1, &cVi2, &cVi3, &cVi4};
  const void* const smf[5] = {&cMf0, &cMf1, &cMf2, &cMf3, &cMf4};
  GCFD_CUDA(c, cudaMemcpyToSymbol(d[kN], divT.data(), divT.size() * sizeof(float)));
  GCFD_CUDA(c, cudaMemcpyToSymbol(io[kN], iop.data(), iop.size() * sizeof(float)));
  std::vector<float> V(static_cast<size_t>(Np) * Np), Vi(V.size()), mf(Np);
  for (size_t q = 0; q < V.size(); ++q) {
    V[q] = static_cast<float>(c->el.V.v[q]);
    Vi[q] = static_cast<float>(c->el.Vinv.v[q]);
  }
  for (int q = 0; q < Np; ++q) mf[q] = static_cast<float>(c->el.ModeFilter[q]);
  GCFD_CUDA(c, cudaMemcpyToSymbol(sv[kN], V.data(), V.size() * sizeof(float)));
  GCFD_CUDA(c, cudaMemcpyToSymbol(svi[kN], Vi.data(), Vi.size() * sizeof(float)));
  GCFD_CUDA(c, cudaMemcpyToSymbol(smf[kN], mf.data(), mf.size() * sizeof(float)));
  return c->tc ? build_tc_n<kN>(c) : GCFD_OK;
}

int mixed_pipe(gcfd_ctx* c) { return c->tc ? build_pipe_n<kN, true>(c) : build_pipe_n<kN, false>(c); }

}  // namespace

const OrderOps* GCFD_CAT(order_ops_, GCFD_ORDER)() {
  static const OrderOps o{
      Ops{&Launch<kN, double>::step, &Launch<kN, double>::rhs, nullptr, nullptr},
      Ops{&MixedLaunch<kN>::step, &MixedLaunch<kN>::rhs, &MixedLaunch<kN>::prep_state,
          &MixedLaunch<kN>::prep_state_range},
      &mixed_consts, &mixed_pipe, &MixedLaunch<kN>::tape_step};
  return &o;
}

}  // namespace gcfd_host
