// Host-side context of libgcfd shared by its translation units: the device
// buffers and settings of one solver (struct gcfd_ctx), the error and
// allocation helpers, and the per-order launcher tables.  The kernels of each
// polynomial order N are compiled in their own translation units
// (gcfd_order.cu and gcfd_order_adj.cu, built once per N with -DGCFD_ORDER=N);
// the rest of the library reaches them through order_ops() / adj_ops().
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gcfd.h"
#include "dfr_element.hpp"
#include "gcfd_mixed_pipe.cuh"
#include "mesh.hpp"

using namespace gcfd;

struct HostFreeStream {
  double qinf[4];
  double pinf, cinf, gamma, minf;
};

template <typename T>
FreeStreamT<T> to_device_fs(const HostFreeStream& h) {
  FreeStreamT<T> f;
  for (int n = 0; n < 4; ++n) f.qinf[n] = static_cast<T>(h.qinf[n]);
  f.pinf = static_cast<T>(h.pinf);
  f.cinf = static_cast<T>(h.cinf);
  f.gamma = static_cast<T>(h.gamma);
  f.minf = static_cast<T>(h.minf);
  return f;
}

struct gcfd_ctx {
  std::string err;
  gcfd_params prm{};
  int N = 0, K = 0, Np = 0, NE = 0, NF = 0, nEdges = 0, nInt = 0, nBC = 0;
  bool fp32 = false;
  DFRElement el;
  Topology topo;
  HostFreeStream fsFar{}, fsIn{}, fsOut{};
  double vbeta = 5.0, vx0 = 5.0, vy0 = 0.0, vgamma = 1.4;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  double* Q[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double* R = nullptr;
  double* Qtmp = nullptr;
  double* rhsOut = nullptr;
  double* rpart = nullptr;  // residual units of the final stage, Scalars::rpart
  void* QF = nullptr;
  void* FE = nullptr;
  double *Iop = nullptr, *Div = nullptr, *Jdet = nullptr, *Jinv = nullptr;
  int *ekL = nullptr, *ekR = nullptr, *eLR = nullptr, *bcFlag = nullptr, *elemEdge = nullptr;
  double *enx = nullptr, *eny = nullptr, *eIIL = nullptr, *eIIR = nullptr, *eoohK = nullptr;
  double *bx = nullptr, *by = nullptr, *edgeSpeed = nullptr, *DT = nullptr;
  Scalars* sc = nullptr;
  // mixed (delta form) path
  float* dQ0 = nullptr;
  float* Dk[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  float* R3 = nullptr;
  float* P23 = nullptr;  // A2 D2 + A3 D3, formed at stage 2 for the final stage
  float *mfaces = nullptr, *mfhat = nullptr, *mcorr = nullptr;
  float2* mbase = nullptr;
  double* mexBC = nullptr;
  float *Qhi = nullptr, *Qlo = nullptr;
  bool fp64Stale = false;  // mixed path: Q[0] lags the compensated state
  cudaStream_t stream2 = nullptr;
  cudaEvent_t evFork = nullptr, evJoin = nullptr;
  cudaEvent_t evChunk[8] = {};  // chunked state copies (mixed path)
  float *mgeo = nullptr, *mII = nullptr;
  int* meslot = nullptr;
  float *mnx = nullptr, *mny = nullptr, *moohK = nullptr;
  bool dirty = true;  // Q0 changed outside a step: the stage-0 data must be rebuilt
  bool tc = false;     // mixed path with the divergence GEMM on the tensor cores (3xTF32)
  float* mBtc = nullptr;
  float* mBtcF = nullptr;  // tensor-core path: FluxEdgeInterp split hi / lo (face GEMM operand)
  int tcDynSmem = 0;   // dynamic shared memory that caps the stage kernel's CTAs per SM to its TMEM share
  // persistent TMA-pipelined stage kernel (needs K % 4 == 0 for 16-byte row strides)
  bool pipe = false;   // built and usable
  bool pipeOn = false;  // selected (gcfd_set_option)
  int pipeGrid = 0, pipeSmem = 0;
  StageMaps pipeMaps{};
  // artificial dissipation (PerssonC0, FP64 path)
  bool diss = false;
  unsigned long long *sigV = nullptr, *epsV = nullptr;
  double *DissX = nullptr, *DissY = nullptr, *VF = nullptr, *viscSpeed = nullptr;
  double *DTVisc = nullptr, *dDiv = nullptr, *dBary = nullptr, *dV = nullptr, *dVinv = nullptr;
  double *dmf = nullptr, *dSensP = nullptr, *dMass = nullptr, *dSensD = nullptr, *dhK = nullptr;
  double *dnxE = nullptr, *dnyE = nullptr, *dIIE = nullptr;
  int* detov = nullptr;
  int nverts = 0;
  double dissKappa = 5.0;
  // adjoint (FP64 path): per-step tape, adjoint work arrays, recorded window
  bool adjReady = false;
  double* tapeRHS[5] = {};
  double* tapeES[5] = {};
  double* tapeDT[5] = {};
  double* tapeQF[5] = {};
  Scalars* tapeSc0 = nullptr;  // scalars before the taped step (BC time)
  Scalars* tapeSc = nullptr;   // after it (per-stage gmax and dt)
  double* Qb[5] = {};
  double *Qbf = nullptr, *Rb3 = nullptr, *QFb = nullptr, *FEb = nullptr;
  double *carry = nullptr, *dtOwnK = nullptr, *esBar = nullptr;
  double* adjS = nullptr;      // [0,5) dt adjoints, [5,9) Qinf adjoint, [9] t-bar current, [10] t-bar next, [11] J
  int* argEdge = nullptr;      // [5]
  // adjoint of the mixed path (FP32 arrays, same layouts; the stage states are
  // Q0 + D_s with the forward's own increments Dk)
  float* tapeRHS32[5] = {};
  float* Qb32[5] = {};
  float *Qbf32 = nullptr, *QF32 = nullptr, *QFb32 = nullptr, *FEb32 = nullptr;
  bool adjFacesPending = false;  // QFb32 holds stage-0 face adjoints not yet in Qbf32
  float* tapeQ0hi = nullptr;     // where the next taped step writes its starting Qhi
  double *dXs = nullptr, *dYs = nullptr, *edgeW = nullptr;
  // adjoint of the dissipation
  double* tapeQ2pre = nullptr;
  double* tapeDTV[5] = {};
  double* tapeVS[5] = {};
  double* tapeRHSpre[5] = {};
  double *sigE = nullptr, *epsE = nullptr, *SeE = nullptr, *alphaBar = nullptr, *carryV = nullptr;
  double *sigVbar = nullptr, *epsVbar = nullptr, *VFbar = nullptr, *DissXbar = nullptr, *DissYbar = nullptr;
  double *RbE = nullptr, *vsBar = nullptr;
  int *sigArg = nullptr, *epsArg = nullptr, *argVisc = nullptr;
  int winSteps = 0, winEvery = 1;
  bool winTaped = false;  // the recording kept every step's tape (slots 1..winSteps)
  // device blocks of the current adjoint window, and those of earlier windows
  // kept for reuse (pointer, bytes)
  std::vector<std::pair<void*, size_t>> winAllocs, winPool;
  // Segment tape: one slot per step of a checkpoint segment, so each step of
  // the segment is recomputed once with its tape kept (slot 0 is the
  // context's own stage arrays and tape); empty when it did not fit.
  struct TapeSlot {
    double* Q[5];  // Q[1..4]: stage states
    double *rhs[5], *es[5], *dt[5], *dtv[5], *vs[5], *rhspre[5];
    double* q2pre;
    Scalars *sc0, *sc;
    float* D[5];       // mixed path: D[1..4] stage increments
    float* rhs32[5];   // mixed path: stage RHS
    double* q0;        // window-taped slots, FP64 path: the step's starting state
    float* q0hi;       // window-taped slots, mixed path: the step's starting hi
  };
  std::vector<TapeSlot> slots;
  bool facesFromState = false;  // reverse stages rebuild their faces (the segment tape keeps none)
  // the mesh as given (post-processing: point location, edge-point coordinates)
  std::vector<double> meshVX, meshVY;
  std::vector<int32_t> meshEToV;
  std::shared_ptr<void> post;  // post-processing state (gcfd_post.cu), built on first use
  std::shared_ptr<void> graphOut;  // solution-output graph element and buffers (gcfd_graph.cu), on first use
  double *ckpt = nullptr, *ckptT = nullptr, *segQ = nullptr, *segT = nullptr, *endQ = nullptr;
  double *ckptV = nullptr, *segV = nullptr, *endV = nullptr;  // DTVisc (dissipation), K per entry
  Scalars* endSc = nullptr;
  std::vector<int> edgeOrder;             // device edge i -> topology edge
  // mesh and solution points on the device (gcfd_geometry.cu)
  double *dVX = nullptr, *dVY = nullptr, *dRS = nullptr;
  int32_t* dEToV = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graphExec = nullptr;
  cudaEvent_t ev[10] = {};
  bool evReady = false;

  ~gcfd_ctx() {
    if (graphExec) cudaGraphExecDestroy(graphExec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (void* p : allocs) cudaFree(p);
    for (auto& b : winAllocs) cudaFree(b.first);
    for (auto& b : winPool) cudaFree(b.first);
    for (auto& e : evChunk)
      if (e) cudaEventDestroy(e);
    if (evFork) cudaEventDestroy(evFork);
    if (evJoin) cudaEventDestroy(evJoin);
    if (stream2) cudaStreamDestroy(stream2);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace gcfd_host {

// Records msg as the context's error (or, with c == NULL, as the error of the
// calling thread's last context-free call) and returns code.
int fail(gcfd_ctx* c, int code, const std::string& msg);

#define GCFD_CUDA(ctx, call)                                                               \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? GCFD_ERR_OOM : GCFD_ERR_CUDA,     \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    }                                                                                      \
  } while (0)

template <typename P>
inline int dalloc(gcfd_ctx* c, P** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(P) > 0 ? count * sizeof(P) : 16);
  if (e != cudaSuccess)
    return fail(c, e == cudaErrorMemoryAllocation ? GCFD_ERR_OOM : GCFD_ERR_CUDA,
                std::string("cudaMalloc: ") + cudaGetErrorString(e));
  c->allocs.push_back(q);
  *p = static_cast<P*>(q);
  return GCFD_OK;
}

template <typename P>
inline int upload(gcfd_ctx* c, P** p, const std::vector<P>& h) {
  int rc = dalloc(c, p, h.size());
  if (rc) return rc;
  if (!h.empty()) GCFD_CUDA(c, cudaMemcpy(*p, h.data(), h.size() * sizeof(P), cudaMemcpyHostToDevice));
  return GCFD_OK;
}

// Launchers of one step / one RHS for the context's order and arithmetic.
struct Ops {
  void (*step)(gcfd_ctx*, cudaEvent_t*, double*, int*);
  void (*rhs)(gcfd_ctx*);
  void (*prep)(gcfd_ctx*);                  // rebuild stage-0 data from Q0 (mixed path), or nullptr
  void (*prep_range)(gcfd_ctx*, int, int);  // the same for elements [k0, k1)
};

// Everything of one order N that instantiates kernels (gcfd_order.cu).
struct OrderOps {
  Ops fp64, mixed;
  int (*mixed_consts)(gcfd_ctx*);  // FP32 operators into constant memory, tensor-core operand and launch shape
  int (*mixed_pipe)(gcfd_ctx*);    // tensor maps and grid of the persistent stage kernel
  void (*mixed_tape)(gcfd_ctx*);   // one mixed step with the adjoint tape (stage RHS, edge speeds, dt)
};

// Adjoint launchers of one order (gcfd_order_adj.cu).
struct AdjOps {
  void (*tape_step)(gcfd_ctx*);
  void (*reverse_step)(gcfd_ctx*, const double*);   // tape_step, then reverse_taped
  void (*reverse_taped)(gcfd_ctx*, const double*);
  void (*rhs_vjp)(gcfd_ctx*);
  void (*functional)(gcfd_ctx*, int);
  void (*mixed_reverse_taped)(gcfd_ctx*, const float*);  // FP32 adjoint of a step taped by mixed_tape,
                                                         // from the step's starting hi part
  void (*mixed_bar_convert)(gcfd_ctx*, bool);  // Qbf (FP64) -> Qbf32 (true) or back (false)
  int (*mixed_consts)(gcfd_ctx*);              // FP32 operators of the mixed reverse sweep
  void (*mixed_finish_faces)(gcfd_ctx*);       // the sweep's last deferred face transpose into Qbf32
};

const OrderOps* order_ops_0();
const OrderOps* order_ops_1();
const OrderOps* order_ops_2();
const OrderOps* order_ops_3();
const OrderOps* order_ops_4();
const AdjOps* adj_ops_0();
const AdjOps* adj_ops_1();
const AdjOps* adj_ops_2();
const AdjOps* adj_ops_3();
const AdjOps* adj_ops_4();

// The tables for order N (0..4), or nullptr.
const OrderOps* order_ops(int N);
const AdjOps* adj_ops(int N);
// The forward launchers of the context (its order and arithmetic).
inline Ops ctx_ops(const gcfd_ctx* c) {
  const OrderOps* o = order_ops(c->N);
  return c->fp32 ? o->mixed : o->fp64;
}

// The residual units (slots of Scalars::rpart) the final stage of a step writes:
// FP64 path, one per warp of k_div_update / k_diss_update; mixed path, one per
// CTA of the stage-4 kernel (the persistent kernel runs fewer CTAs).
inline int resid_units(const gcfd_ctx* c) {
  const int blocks32 = (c->K + 31) / 32;
  if (!c->fp32) return (c->K + 127) / 128 * 4;
  if (!c->diss && c->pipe && c->pipeOn) return std::min(c->pipeGrid, blocks32);
  return blocks32;
}

// Shared host helpers (gcfd.cu).
int sync_fp64_state(gcfd_ctx* c);
int prepare_if_dirty(gcfd_ctx* c);

// Device geometry (gcfd_geometry.cu): per-element geometry and per-edge tables
// from the mesh arrays and the device edge lists; the mixed path's FP32 copies;
// solution-point coordinates; the initial state into Q[0].
int device_geometry(gcfd_ctx* c, const gcfd_mesh* m, const std::vector<int>& kL, const std::vector<int>& kR,
                    const std::vector<int>& eLR);
int device_geometry_mixed(gcfd_ctx* c);
int device_solution_points(gcfd_ctx* c, double** X, double** Y);
int device_initial_state(gcfd_ctx* c);
int check_shards(gcfd_ctx* c, int nshards, const int32_t* Kmax);
int copy_shards(gcfd_ctx* c, double* dst, int nshards, const int32_t* Kmax, const double* const* Q,
                bool toDevice, double* const* Qout);
double decode_order_key(unsigned long long k);

}  // namespace gcfd_host
