// libgcfd: residual norms without allocation (gcfd_residual_norms_static).
//
// The per-block partials live in one file-scope device array of fixed size;
// the first call on each device (more exactly: on each CUDA context current on
// it) looks up its address with cudaGetSymbolAddress (with that device
// current) and caches it together with the context handle, so a context that
// was destroyed and recreated (cudaDeviceReset) gets a fresh lookup.  Pass 1:
// block b reduces points [b*kResidChunk, (b+1)*kResidChunk) of each variable
// into 12 slots (order key of the signed max, bit pattern of max |R|, sum of
// squares).  Pass 2: one block reduces the nblk partials in a fixed order and
// writes 12 result slots, copied to the host.  The sums are therefore
// deterministic run to run.  No slot needs clearing: pass 2 reads only slots
// that pass 1 of the same call wrote.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "gcfd_ctx.hpp"

// 16384 blocks x 12 partial slots + 12 result slots (1.5 MiB); see
// GCFD_RESID_STATIC_MAX_POINTS.  Host code must not pass this name to a
// kernel: on the host it is a stand-in, and the device address comes from
// cudaGetSymbolAddress.
static __device__ __align__(256) unsigned long long g_resid_scratch[16384 * 12 + 12];

namespace gcfd_host {
namespace {

constexpr int kResidThreads = 256;
constexpr int kResidChunk = 2048;                // points per block and variable
constexpr int kResidMaxBlocks = 16384;           // => GCFD_RESID_STATIC_MAX_POINTS
constexpr int kResidResult = kResidMaxBlocks * 12;
static_assert(static_cast<long long>(kResidChunk) * kResidMaxBlocks == GCFD_RESID_STATIC_MAX_POINTS,
              "the header's limit must match the scratch layout");

constexpr int kMaxDevices = 64;
std::mutex g_resid_mutex;
unsigned long long* g_resid_ptr[kMaxDevices] = {};
void* g_resid_ctx[kMaxDevices] = {};  // CUcontext the cached address belongs to

__device__ __forceinline__ void resid_block_reduce(unsigned long long& key, unsigned long long& ab, double& s2,
                                                   unsigned long long* sk, unsigned long long* sa,
                                                   double* ss) {
  key = warp_max_u64(key);
  ab = warp_max_u64(ab);
  s2 = warp_sum(s2);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sk[w] = key;
    sa[w] = ab;
    ss[w] = s2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kResidThreads / 32; ++i) {
      key = key > sk[i] ? key : sk[i];
      ab = ab > sa[i] ? ab : sa[i];
      s2 += ss[i];
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kResidThreads) k_resid_partial(const double* __restrict__ R, long long npts,
                                                                  unsigned long long* scratch) {
  __shared__ unsigned long long sk[kResidThreads / 32], sa[kResidThreads / 32];
  __shared__ double ss[kResidThreads / 32];
  const long long lo = static_cast<long long>(blockIdx.x) * kResidChunk;
  const long long hi = lo + kResidChunk < npts ? lo + kResidChunk : npts;
  for (int n = 0; n < 4; ++n) {
    const double* r = R + n * npts;
    unsigned long long key = 0ULL, ab = 0ULL;
    double s2 = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += kResidThreads) {
      const double x = r[i];
      const unsigned long long k = order_key(x);
      const unsigned long long a = static_cast<unsigned long long>(__double_as_longlong(fabs(x)));
      key = key > k ? key : k;
      ab = ab > a ? ab : a;  // NaN bit patterns rank above +inf, so a NaN stays visible
      s2 += x * x;
    }
    resid_block_reduce(key, ab, s2, sk, sa, ss);
    if (threadIdx.x == 0) {
      unsigned long long* o = scratch + static_cast<size_t>(blockIdx.x) * 12 + n * 3;
      o[0] = key;
      o[1] = ab;
      o[2] = static_cast<unsigned long long>(__double_as_longlong(s2));
    }
  }
}

__global__ void __launch_bounds__(kResidThreads) k_resid_final(unsigned long long* scratch, int nblk) {
  __shared__ unsigned long long sk[kResidThreads / 32], sa[kResidThreads / 32];
  __shared__ double ss[kResidThreads / 32];
  for (int n = 0; n < 4; ++n) {
    unsigned long long key = 0ULL, ab = 0ULL;
    double s2 = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kResidThreads) {
      const unsigned long long* p = scratch + static_cast<size_t>(b) * 12 + n * 3;
      key = key > p[0] ? key : p[0];
      ab = ab > p[1] ? ab : p[1];
      s2 += __longlong_as_double(static_cast<long long>(p[2]));
    }
    resid_block_reduce(key, ab, s2, sk, sa, ss);
    if (threadIdx.x == 0) {
      unsigned long long* o = scratch + kResidResult + n * 3;
      o[0] = key;
      o[1] = ab;
      o[2] = static_cast<unsigned long long>(__double_as_longlong(s2));
    }
  }
}

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

// The driver's current context of the calling thread, or nullptr when the
// driver entry point is not available.
void* current_context() {
  static CtxGetCurrentFn fn = []() -> CtxGetCurrentFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  CUcontext ctx = nullptr;
  if (fn && fn(&ctx) == CUDA_SUCCESS) return static_cast<void*>(ctx);
  return nullptr;
}

// Device address of the scratch array for the current device, looked up once
// per device and context.
int resid_scratch(unsigned long long** out) {
  static_assert(sizeof(g_resid_scratch) == sizeof(unsigned long long) * (kResidResult + 12),
                "scratch size must match the slot layout");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(nullptr, GCFD_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(nullptr, GCFD_ERR_UNSUPPORTED, "device ordinal beyond the residual scratch table");
  std::lock_guard<std::mutex> lock(g_resid_mutex);
  void* ctx = current_context();
  if (!g_resid_ptr[dev] || (ctx && ctx != g_resid_ctx[dev])) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_resid_scratch);
    if (e != cudaSuccess || !p)
      return fail(nullptr, GCFD_ERR_CUDA,
                  std::string("cudaGetSymbolAddress(residual scratch): ") + cudaGetErrorString(e));
    g_resid_ptr[dev] = static_cast<unsigned long long*>(p);
    g_resid_ctx[dev] = current_context();
  }
  *out = g_resid_ptr[dev];
  return GCFD_OK;
}

}  // namespace
}  // namespace gcfd_host

using namespace gcfd_host;

extern "C" {

int gcfd_residual_norms_static(const double* dR, int32_t Np, int32_t K, void* stream, double* resid_max4,
                               double* resid_absmax4, double* resid_rms4) {
  if (!dR) return fail(nullptr, GCFD_ERR_ARG, "gcfd_residual_norms_static: dR is NULL");
  if (Np < 1 || K < 1) return fail(nullptr, GCFD_ERR_ARG, "gcfd_residual_norms_static: Np and K must be >= 1");
  const long long npts = static_cast<long long>(Np) * K;
  if (npts > GCFD_RESID_STATIC_MAX_POINTS)
    return fail(nullptr, GCFD_ERR_SHAPE,
                "gcfd_residual_norms_static: Np x K = " + std::to_string(npts) + " exceeds the fixed scratch limit " +
                    std::to_string(GCFD_RESID_STATIC_MAX_POINTS) + " (GCFD_RESID_STATIC_MAX_POINTS)");
  unsigned long long* scratch = nullptr;
  int rc = resid_scratch(&scratch);
  if (rc) return rc;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblk = static_cast<int>((npts + kResidChunk - 1) / kResidChunk);
  k_resid_partial<<<nblk, kResidThreads, 0, s>>>(dR, npts, scratch);
  k_resid_final<<<1, kResidThreads, 0, s>>>(scratch, nblk);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(nullptr, GCFD_ERR_CUDA, std::string("gcfd_residual_norms_static launch: ") + cudaGetErrorString(e));
  unsigned long long h[12];
  e = cudaMemcpyAsync(h, scratch + kResidResult, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return fail(nullptr, GCFD_ERR_CUDA, std::string("gcfd_residual_norms_static: ") + cudaGetErrorString(e));
  bool finite = true;
  for (int n = 0; n < 4; ++n) {
    double am, s2;
    std::memcpy(&am, &h[n * 3 + 1], sizeof(am));
    std::memcpy(&s2, &h[n * 3 + 2], sizeof(s2));
    const double rms = std::sqrt(s2 / static_cast<double>(npts));
    if (resid_max4) resid_max4[n] = decode_order_key(h[n * 3]);
    if (resid_absmax4) resid_absmax4[n] = am;
    if (resid_rms4) resid_rms4[n] = rms;
    if (!(std::isfinite(am) && std::isfinite(rms))) finite = false;
  }
  if (!finite) return fail(nullptr, GCFD_ERR_NAN, "gcfd_residual_norms_static: non-finite increment");
  return GCFD_OK;
}

}  // extern "C"

