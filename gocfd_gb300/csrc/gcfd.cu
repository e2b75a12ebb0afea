// libgcfd: device context, kernel launchers, per-step CUDA graph and the C ABI
// declared in include/gcfd.h.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <type_traits>
#include <string>
#include <vector>

#include "../../include/gcfd.h"
#include "dfr_element.hpp"
#include "gcfd_kernels.cuh"
#include "gcfd_mixed.cuh"
#include "gcfd_mixed_tc.cuh"
#include "gcfd_mixed_pipe.cuh"
#include "gcfd_mixed_diss.cuh"
#include "gcfd_diss.cuh"
#include "gcfd_adjoint.cuh"
#include "gcfd_adjoint_diss.cuh"
#include "mesh.hpp"

using namespace gcfd;

namespace {

thread_local std::string g_create_error;

struct HostFreeStream {
  double qinf[4];
  double pinf, cinf, gamma, minf;
};

// NewFreeStream (fluids.go:378-395).
HostFreeStream freestream_from_mach(double minf, double gamma, double alpha) {
  const double pi = 3.14159265358979323846;
  HostFreeStream f;
  const double ooggm1 = 1.0 / (gamma * (gamma - 1.0));
  f.qinf[0] = 1.0;
  f.qinf[1] = minf * std::cos(alpha * pi / 180.0);
  f.qinf[2] = minf * std::sin(alpha * pi / 180.0);
  f.qinf[3] = ooggm1 + 0.5 * minf * minf;
  f.gamma = gamma;
  f.minf = minf;
  const double oorho = 1.0 / f.qinf[0];
  const double u = f.qinf[1] * oorho, v = f.qinf[2] * oorho;
  const double p = (gamma - 1.0) * (f.qinf[3] - 0.5 * f.qinf[0] * (u * u + v * v));
  f.pinf = p;
  f.cinf = std::sqrt(std::fabs(gamma * p * oorho));
  return f;
}

// NewFreestreamFromQinf (fluids.go:397-406): Minf stays 0.
HostFreeStream freestream_from_q(double gamma, const double q[4]) {
  HostFreeStream f;
  for (int n = 0; n < 4; ++n) f.qinf[n] = q[n];
  f.gamma = gamma;
  f.minf = 0.0;
  const double oorho = 1.0 / q[0];
  const double u = q[1] * oorho, v = q[2] * oorho;
  const double p = (gamma - 1.0) * (q[3] - 0.5 * q[0] * (u * u + v * v));
  f.pinf = p;
  f.cinf = std::sqrt(std::fabs(gamma * p * oorho));
  return f;
}

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

}  // namespace

struct gcfd_ctx {
  std::string err;
  gcfd_params prm{};
  int N = 0, K = 0, Np = 0, NE = 0, NF = 0, nEdges = 0, nInt = 0, nBC = 0;
  bool fp32 = false;
  DFRElement el;
  Topology topo;
  Geometry geo;
  HostFreeStream fsFar{}, fsIn{}, fsOut{};
  double vbeta = 5.0, vx0 = 5.0, vy0 = 0.0, vgamma = 1.4;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  double* Q[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double* R = nullptr;
  double* Qtmp = nullptr;
  double* rhsOut = nullptr;
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
  std::vector<void*> winAllocs;
  double *ckpt = nullptr, *ckptT = nullptr, *segQ = nullptr, *segT = nullptr, *endQ = nullptr;
  double *ckptV = nullptr, *segV = nullptr, *endV = nullptr;  // DTVisc (dissipation), K per entry
  Scalars* endSc = nullptr;
  std::vector<int> edgeOrder;             // device edge i -> topology edge
  std::vector<double> hnx, hny, hoohK;    // per device edge
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
    for (void* p : winAllocs) cudaFree(p);
    for (auto& e : evChunk)
      if (e) cudaEventDestroy(e);
    if (evFork) cudaEventDestroy(evFork);
    if (evJoin) cudaEventDestroy(evJoin);
    if (stream2) cudaStreamDestroy(stream2);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int fail(gcfd_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_error = msg;
  return code;
}

#define GCFD_CUDA(ctx, call)                                                               \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? GCFD_ERR_OOM : GCFD_ERR_CUDA,     \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    }                                                                                      \
  } while (0)

template <typename P>
int dalloc(gcfd_ctx* c, P** p, size_t count) {
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
int upload(gcfd_ctx* c, P** p, const std::vector<P>& h) {
  int rc = dalloc(c, p, h.size());
  if (rc) return rc;
  if (!h.empty()) GCFD_CUDA(c, cudaMemcpy(*p, h.data(), h.size() * sizeof(P), cudaMemcpyHostToDevice));
  return GCFD_OK;
}

// ---------------------------------------------------------------------------
// Launchers, one instantiation per (order, arithmetic type).
template <int N, typename T>
struct Launch {
  static EdgeArgs<T> edge_args(gcfd_ctx* c, const double* time) {
    EdgeArgs<T> a;
    a.QF = static_cast<const T*>(c->QF);
    a.FE = static_cast<T*>(c->FE);
    a.K = c->K;
    a.nInt = c->nInt;
    a.nBC = c->nBC;
    a.kL = c->ekL;
    a.kR = c->ekR;
    a.eLR = c->eLR;
    a.nx = c->enx;
    a.ny = c->eny;
    a.IIL = c->eIIL;
    a.IIR = c->eIIR;
    a.oohK = c->eoohK;
    a.bcFlag = c->bcFlag;
    a.bx = c->bx;
    a.by = c->by;
    a.edgeSpeed = c->edgeSpeed;
    a.gmax = nullptr;
    a.time = time;
    a.flux = c->prm.flux_type;
    const double g = c->fsFar.gamma;
    a.gas = Gas<T>{static_cast<T>(g), static_cast<T>(g - 1.0), static_cast<T>(1.0 / (g - 1.0))};
    a.fsFar = to_device_fs<T>(c->fsFar);
    a.fsIn = to_device_fs<T>(c->fsIn);
    a.fsOut = to_device_fs<T>(c->fsOut);
    a.vbeta = static_cast<T>(c->vbeta);
    a.vx0 = static_cast<T>(c->vx0);
    a.vy0 = static_cast<T>(c->vy0);
    a.vgamma = static_cast<T>(c->vgamma);
    return a;
  }
  static UpdateArgs<T> update_args(gcfd_ctx* c, int stage, const double* Qs) {
    UpdateArgs<T> a;
    a.K = c->K;
    a.stage = stage;
    a.Qs = Qs;
    a.Q0 = c->Q[0];
    a.Q1 = c->Q[1];
    a.Q2 = c->Q[2];
    a.Q3 = c->Q[3];
    a.Q4 = c->Q[4];
    a.R = c->R;
    a.FE = static_cast<const T*>(c->FE);
    a.Div = c->Div;
    a.Jdet = c->Jdet;
    a.Jinv = c->Jinv;
    a.sc = c->sc;
    a.cfl = c->prm.cfl;
    a.finalTime = c->prm.final_time;
    a.localDT = c->prm.local_time_stepping;
    a.edgeSpeed = c->edgeSpeed;
    a.elemEdge = c->elemEdge;
    a.DT = c->DT;
    a.rhsOut = c->rhsOut;
    const double g = c->fsFar.gamma;
    a.gas = Gas<T>{static_cast<T>(g), static_cast<T>(g - 1.0), static_cast<T>(1.0 / (g - 1.0))};
    a.DissX = c->DissX;
    a.DissY = c->DissY;
    a.VF = c->VF;
    a.viscSpeed = c->viscSpeed;
    a.sigV = c->sigV;
    a.etov = c->detov;
    a.V = c->dV;
    a.Vinv = c->dVinv;
    a.mf = c->dmf;
    a.IIE = c->dIIE;
    a.ekL = c->ekL;
    a.eLR = c->eLR;
    a.gvisc = c->sc->gvisc;
    a.DTVisc = c->DTVisc;
    a.cdiff = 1.0 / (double(c->N + 1) * double(c->N + 1));
    a.tapeRHS = nullptr;
    a.tapeRHSpre = nullptr;
    return a;
  }
  static DissArgs diss_args(gcfd_ctx* c, int stage, double* Qs) {
    DissArgs a;
    a.K = c->K;
    a.nInt = c->nInt;
    a.nBC = c->nBC;
    a.stage = stage;
    a.Qs = Qs;
    a.Qlim = Qs;
    a.QF = static_cast<double*>(c->QF);
    a.Iop = c->Iop;
    a.etov = c->detov;
    a.hK = c->dhK;
    a.SensP = c->dSensP;
    a.Mass = c->dMass;
    a.SensD = c->dSensD;
    a.V = c->dV;
    a.Vinv = c->dVinv;
    a.mf = c->dmf;
    a.Div = c->dDiv;
    a.Bary = c->dBary;
    a.Jinv = c->Jinv;
    a.Jdet = c->Jdet;
    a.nxE = c->dnxE;
    a.nyE = c->dnyE;
    a.IIE = c->dIIE;
    a.elemEdge = c->elemEdge;
    a.ekL = c->ekL;
    a.ekR = c->ekR;
    a.eLR = c->eLR;
    a.enx = c->enx;
    a.eny = c->eny;
    a.eIIL = c->eIIL;
    a.eoohK = c->eoohK;
    a.sigV = c->sigV;
    a.epsV = c->epsV;
    a.DissX = c->DissX;
    a.DissY = c->DissY;
    a.VF = c->VF;
    a.viscSpeed = c->viscSpeed;
    a.gvisc = (stage >= 0) ? &c->sc->gvisc[stage] : &c->sc->gvisc[0];
    a.kappa = c->dissKappa;
    a.eps0 = 5.0 / 1.5;
    a.S0 = 4.0 / std::pow(double(c->N + 1), 4.0);
    a.omega = double(c->N * c->N);
    a.sigE = a.epsE = a.SeE = nullptr;
    a.faces32 = c->mfaces;
    a.base32 = c->mbase;
    a.eslot32 = c->meslot;
    a.DissX32 = reinterpret_cast<float*>(c->DissX);  // mixed path only; half of the FP64 arrays' memory
    a.DissY32 = reinterpret_cast<float*>(c->DissY);
    a.VF32 = reinterpret_cast<float*>(c->VF);
    return a;
  }
  static int grid(int n) { return (n + 127) / 128; }
  // Sensor, vertex smoothing, rkStep-2 limiter and faces (replaces interp).
  static void diss_front(gcfd_ctx* c, int stage, double* Qs) {
    cudaMemsetAsync(c->sigV, 0, sizeof(unsigned long long) * c->nverts, c->stream);
    cudaMemsetAsync(c->epsV, 0, sizeof(unsigned long long) * c->nverts, c->stream);
    const DissArgs d = diss_args(c, stage, Qs);
    k_diss_sensor<N><<<grid(c->K), 128, 0, c->stream>>>(d);
    if (stage == 2) k_diss_limit<N><<<grid(4 * c->K), 128, 0, c->stream>>>(d);
    interp(c, Qs);
  }
  static void diss_middle(gcfd_ctx* c, int stage, double* Qs) {
    const DissArgs d = diss_args(c, stage, Qs);
    constexpr int NF = Dims<N>::NF;
    k_diss_grad<N><<<grid(c->K), 128, sizeof(double) * (NF * NF + NF * 3), c->stream>>>(d);
    k_diss_edge<N><<<grid(c->nInt + c->nBC), 128, 0, c->stream>>>(d);
  }

  static void interp(gcfd_ctx* c, const double* Qs) {
    k_interp<N, T><<<grid(c->K), 128, 0, c->stream>>>(Qs, static_cast<T*>(c->QF), c->Iop, c->K);
  }
  static void edge(gcfd_ctx* c, const double* time, unsigned long long* gmax) {
    EdgeArgs<T> a = edge_args(c, time);
    a.gmax = gmax;
    k_edge_flux<N, T><<<grid(c->nInt + c->nBC), 128, 0, c->stream>>>(a);
  }
  static void update(gcfd_ctx* c, int stage, const double* Qs) {
    if (c->diss) {
      // Euler RHS into rhsOut, then dissipation + filter + stage update.
      if constexpr (std::is_same<T, double>::value) {
        k_div_update<N, T><<<grid(c->K), 128, 0, c->stream>>>(update_args(c, -1, Qs));
        k_diss_update<N><<<grid(c->K), 128, 0, c->stream>>>(update_args(c, stage, Qs));
      }
    } else {
      k_div_update<N, T><<<grid(c->K), 128, 0, c->stream>>>(update_args(c, stage, Qs));
    }
  }
  // One RK step: RungeKutta5SSP.Step (euler.go:408-418).
  static void step(gcfd_ctx* c, cudaEvent_t* ev, double* ms, int* launches) {
    auto mark = [&](int i) {
      if (ev) cudaEventRecord(ev[i], c->stream);
    };
    auto acc = [&](int fam, int a, int b) {
      if (!ev) return;
      cudaEventSynchronize(ev[b]);
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[a], ev[b]);
      ms[fam] += t;
      launches[fam] += 1;
    };
    mark(0);
    k_step_begin<<<1, 32, 0, c->stream>>>(c->sc);
    mark(1);
    acc(3, 0, 1);
    for (int s = 0; s < 5; ++s) {
      mark(2);
      if (c->diss) diss_front(c, s, c->Q[s]);
      else interp(c, c->Q[s]);
      mark(3);
      edge(c, &c->sc->time, &c->sc->gmax[s]);
      if (c->diss) diss_middle(c, s, c->Q[s]);
      mark(4);
      update(c, s, c->Q[s]);
      mark(5);
      acc(0, 2, 3);
      acc(1, 3, 4);
      acc(2, 4, 5);
    }
    mark(6);
    k_step_end<<<1, 32, 0, c->stream>>>(c->sc, c->prm.local_time_stepping);
    mark(7);
    acc(3, 6, 7);
  }
  static void rhs(gcfd_ctx* c) {
    if (c->diss) diss_front(c, -1, c->Qtmp);
    else interp(c, c->Qtmp);
    edge(c, &c->sc->rhs_time, &c->sc->gmax[0]);
    if (c->diss) diss_middle(c, -1, c->Qtmp);
    update(c, -1, c->Qtmp);
  }
};

// Mixed (delta form) path: edge + stage kernels per RK stage.
template <int N>
struct MixedLaunch {
  static MixedArgs args(gcfd_ctx* c, int stage, double* Q0, const double* time,
                        unsigned long long* gmax) {
    MixedArgs a;
    a.K = c->K;
    a.nInt = c->nInt;
    a.nBC = c->nBC;
    a.stage = stage;
    a.Q0 = Q0;
    a.Qhi = c->Qhi;
    a.Qlo = c->Qlo;
    a.dQ0 = c->dQ0;
    for (int i = 0; i < 5; ++i) a.D[i] = c->Dk[i];
    a.R3 = c->R3;
    a.faces = c->mfaces;
    a.fhat = c->mfhat;
    a.corr = c->mcorr;
    a.base = c->mbase;
    a.geo = c->mgeo;
    a.II = c->mII;
    a.eslot = c->meslot;
    a.ekL = c->ekL;
    a.ekR = c->ekR;
    a.enx = c->mnx;
    a.eny = c->mny;
    a.eoohK = c->moohK;
    a.bcFlag = c->bcFlag;
    a.bx = c->bx;
    a.by = c->by;
    a.exBC = c->mexBC;
    a.edgeSpeed = c->edgeSpeed;
    a.gmax = gmax;
    a.time = time;
    a.sc = c->sc;
    a.cfl = c->prm.cfl;
    a.finalTime = c->prm.final_time;
    a.localDT = c->prm.local_time_stepping;
    a.DT = c->DT;
    a.flux = c->prm.flux_type;
    a.gamma = static_cast<float>(c->fsFar.gamma);
    a.gammaD = c->fsFar.gamma;
    a.fsFar = to_device_fs<double>(c->fsFar);
    a.fsIn = to_device_fs<double>(c->fsIn);
    a.fsOut = to_device_fs<double>(c->fsOut);
    a.vbeta = c->vbeta;
    a.vx0 = c->vx0;
    a.vy0 = c->vy0;
    a.vgamma = c->vgamma;
    a.rhsOut = c->rhsOut;
    a.Btc = c->mBtc;
    a.DissX32 = reinterpret_cast<const float*>(c->DissX);
    a.DissY32 = reinterpret_cast<const float*>(c->DissY);
    a.VF32 = reinterpret_cast<const float*>(c->VF);
    a.err = reinterpret_cast<unsigned int*>(&c->sc->errFlags);
    a.rhsOnly = 0;
    a.gviscS = nullptr;
    a.cdiff = 0.0;
    return a;
  }
  static int gridE(gcfd_ctx* c) { return (c->K + 31) / 32; }
  static void stage_kernel(gcfd_ctx* c, const MixedArgs& a) {
    if (c->pipe && c->pipeOn) {
      const int g = std::min(c->pipeGrid, gridE(c));
      if (c->tc)
        k_mixed_stage_pipe<N, true><<<g, 128, c->pipeSmem, c->stream>>>(c->pipeMaps, a);
      else
        k_mixed_stage_pipe<N, false><<<g, 128, c->pipeSmem, c->stream>>>(c->pipeMaps, a);
      return;
    }
    if (c->tc)
      k_mixed_stage_tc<N><<<gridE(c), 128, c->tcDynSmem, c->stream>>>(a);
    else
      k_mixed_stage<N><<<gridE(c), 128, 0, c->stream>>>(a);
  }
  // Interior edges on the main stream; boundary edges (FP64, transcendental
  // work, few threads) concurrently on a forked stream, joined before the stage.
  static void edges(gcfd_ctx* c, int s, double* Q0, const double* time, unsigned long long* gmax,
                    bool fork) {
    const MixedArgs a = args(c, s, Q0, time, gmax);
    cudaStream_t sb = c->stream;
    if (fork && c->nBC > 0) {
      cudaEventRecord(c->evFork, c->stream);
      cudaStreamWaitEvent(c->stream2, c->evFork, 0);
      sb = c->stream2;
    }
    if (c->nBC > 0)
      k_mixed_edge_bc<N><<<(c->nBC + 7) / 8, dim3(8, MixedDims<N>::NE), 0, sb>>>(a);
    if (c->nInt > 0) {
      const int nb = (c->nInt + 127) / 128;
      switch (c->prm.flux_type) {
        case GCFD_FLUX_ROE_ER: k_mixed_edge<N, kFluxRoeER><<<nb, 128, 0, c->stream>>>(a); break;
        case GCFD_FLUX_ROE: k_mixed_edge<N, kFluxRoe><<<nb, 128, 0, c->stream>>>(a); break;
        case GCFD_FLUX_LAX: k_mixed_edge<N, kFluxLax><<<nb, 128, 0, c->stream>>>(a); break;
        default: k_mixed_edge<N, kFluxAverage><<<nb, 128, 0, c->stream>>>(a); break;
      }
    }
    if (fork && c->nBC > 0) {
      cudaEventRecord(c->evJoin, c->stream2);
      cudaStreamWaitEvent(c->stream, c->evJoin, 0);
    }
  }
  static void prepare(gcfd_ctx* c, double* Q0) { prepare_range(c, Q0, 0, c->K); }
  static void prepare_range(gcfd_ctx* c, double* Q0, int k0, int k1) {
    if (k1 <= k0) return;
    k_mixed_prepare<N><<<(k1 - k0 + 31) / 32, 128, 0, c->stream>>>(args(c, 0, Q0, nullptr, nullptr), k0, k1);
  }
  static void step(gcfd_ctx* c, cudaEvent_t* ev, double* ms, int* launches) {
    auto mark = [&](int i) {
      if (ev) cudaEventRecord(ev[i], c->stream);
    };
    auto acc = [&](int fam, int x, int y) {
      if (!ev) return;
      cudaEventSynchronize(ev[y]);
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[x], ev[y]);
      ms[fam] += t;
      launches[fam] += 1;
    };
    if (ev) {  // profiling also times the stage-0 preparation once
      mark(8);
      prepare(c, c->Q[0]);
      mark(9);
      acc(0, 8, 9);
    }
    mark(0);
    k_step_begin<<<1, 32, 0, c->stream>>>(c->sc);
    mark(1);
    acc(3, 0, 1);
    for (int s = 0; s < 5; ++s) {
      if (c->diss) {  // dissipation: no per-family split
        diss_stage(c, s);
        continue;
      }
      mark(2);
      edges(c, s, c->Q[0], &c->sc->time, &c->sc->gmax[s], ev == nullptr);
      mark(3);
      stage_kernel(c, args(c, s, c->Q[0], &c->sc->time, &c->sc->gmax[s]));
      mark(4);
      acc(1, 2, 3);
      acc(2, 3, 4);
    }
    mark(6);
    k_step_end<<<1, 32, 0, c->stream>>>(c->sc, c->prm.local_time_stepping);
    mark(7);
    acc(3, 6, 7);
  }
  static void rhs(gcfd_ctx* c) {
    prepare(c, c->Qtmp);
    if (c->diss) diss_front(c, -1, c->Qtmp);
    edges(c, -1, c->Qtmp, &c->sc->rhs_time, &c->sc->gmax[0], false);
    if (c->diss) diss_middle(c, -1, c->Qtmp);
    stage_kernel(c, args(c, -1, c->Qtmp, &c->sc->rhs_time, &c->sc->gmax[0]));
    if (c->diss)
      k_mixed_diss_update<N><<<gridE(c), 128, 0, c->stream>>>(args(c, -1, c->Qtmp, &c->sc->rhs_time,
                                                                    &c->sc->gmax[0]),
                                                               Launch<N, double>::update_args(c, -1, c->Qtmp));
  }
  // Sensor, vertex smoothing and the rkStep-2 limiter on the mixed state (the
  // limiter rewrites D2, the faces and the reference states it changes).
  static void diss_front(gcfd_ctx* c, int stage, double* Qs) {
    cudaMemsetAsync(c->sigV, 0, sizeof(unsigned long long) * c->nverts, c->stream);
    cudaMemsetAsync(c->epsV, 0, sizeof(unsigned long long) * c->nverts, c->stream);
    const DissArgs d = Launch<N, double>::diss_args(c, stage, Qs);
    const MixedArgs m = args(c, stage, c->Q[0], &c->sc->time, &c->sc->gmax[stage < 0 ? 0 : stage]);
    k_diss_sensor_mixed<N><<<(c->K + 127) / 128, 128, 0, c->stream>>>(d, m);
    if (stage == 2) k_mixed_limit<N><<<gridE(c), 128, 0, c->stream>>>(d, m);
  }
  // The RT gradient in FP32 (delta form), then the viscous edge fluxes.
  static void diss_middle(gcfd_ctx* c, int stage, double* Qs) {
    const DissArgs d = Launch<N, double>::diss_args(c, stage, Qs);
    const MixedArgs m = args(c, stage, c->Q[0], &c->sc->time, &c->sc->gmax[stage < 0 ? 0 : stage]);
    constexpr int NF = Dims<N>::NF;
    k_diss_grad_mixed<N><<<(c->K + 127) / 128, 128, sizeof(float) * (NF * NF + NF * 3), c->stream>>>(d, m);
    k_diss_edge_mixed<N><<<(c->nInt + c->nBC + 127) / 128, 128, 0, c->stream>>>(d);
  }
  // One stage with the PerssonC0 dissipation: FP64 stage state for the
  // dissipation kernels (Q[1] is free on the mixed path), the Euler RHS of the
  // stage from the delta-form kernel, then the dissipated update.
  static void diss_stage(gcfd_ctx* c, int s) {
    using L = Launch<N, double>;
    double* Qs64 = c->Q[1];  // not read: the dissipation kernels take the mixed state
    diss_front(c, s, Qs64);
    edges(c, s, c->Q[0], &c->sc->time, &c->sc->gmax[s], true);
    diss_middle(c, s, Qs64);
    MixedArgs m = args(c, s, c->Q[0], &c->sc->time, &c->sc->gmax[s]);
    m.rhsOnly = 1;
    stage_kernel(c, m);
    MixedArgs m2 = args(c, s, c->Q[0], &c->sc->time, &c->sc->gmax[s]);
    m2.gviscS = c->sc->gvisc;
    m2.cdiff = 1.0 / (double(c->N + 1) * double(c->N + 1));
    k_mixed_diss_update<N><<<gridE(c), 128, 0, c->stream>>>(m2, L::update_args(c, s, Qs64));
  }
  static void prep_state(gcfd_ctx* c) { prepare(c, c->Q[0]); }
  static void prep_state_range(gcfd_ctx* c, int k0, int k1) { prepare_range(c, c->Q[0], k0, k1); }
};

// Adjoint launchers (FP64 path).
template <int N>
struct AdjLaunch {
  using L = Launch<N, double>;
  static int grid(int n) { return (n + 127) / 128; }
  static EdgeArgs<double> edge_args(gcfd_ctx* c, const double* time) {
    EdgeArgs<double> e = L::edge_args(c, time);
    e.QF = static_cast<const double*>(c->QF);
    return e;
  }
  static AdjEdgeArgs adj_edge_args(gcfd_ctx* c) {
    AdjEdgeArgs x;
    x.FEb = c->FEb;
    x.QFb = c->QFb;
    x.qinfb = c->adjS + 5;
    x.tb = c->adjS + 9;
    x.esBar = c->esBar;
    x.useManualRoe = 1;
    return x;
  }
  static AdjArgs adj_args(gcfd_ctx* c, int s, const double* Qs, const double* Qbn, double* Qbs) {
    AdjArgs a;
    a.K = c->K;
    a.stage = s;
    a.localDT = c->prm.local_time_stepping;
    a.Qs = Qs;
    a.Qbn = Qbn;
    a.rhs = s >= 0 ? c->tapeRHS[s] : nullptr;
    a.rhs3 = c->tapeRHS[3];
    a.Qb0 = c->Qb[0];
    a.Qbs = Qbs;
    a.Qb2 = c->Qb[2];
    a.Qb3 = c->Qb[3];
    a.Rb3 = c->Rb3;
    a.dtS = c->tapeSc->dt;
    a.dtK = s >= 0 ? c->tapeDT[s] : nullptr;
    a.dtbarG = c->adjS;
    a.dtOwnK = c->dtOwnK;
    a.DivInt = c->Div;
    a.Jdet = c->Jdet;
    a.Jinv = c->Jinv;
    a.FEb = c->FEb;
    const double g = c->fsFar.gamma;
    a.gas = Gas<double>{g, g - 1.0, 1.0 / (g - 1.0)};
    return a;
  }
  // Forward step with the tape: the same launches as L::step (so the states
  // are bit-identical to the recorded trajectory), plus per-stage copies of
  // the edge speeds, local dt and faces, the stage RHS written by the update
  // kernel, and with the dissipation the rkStep-2 state before the limiter,
  // DTVisc before each stage, the viscous speeds and the pre-filter RHS.
  static void tape_step(gcfd_ctx* c) {
    cudaMemcpyAsync(c->tapeSc0, c->sc, sizeof(Scalars), cudaMemcpyDeviceToDevice, c->stream);
    k_step_begin<<<1, 32, 0, c->stream>>>(c->sc);
    void* faces = c->QF;
    const size_t SB = sizeof(double) * 4 * c->Np * static_cast<size_t>(c->K);
    for (int s = 0; s < 5; ++s) {
      c->QF = c->tapeQF[s];  // the stage's faces stay on the tape
      if (c->diss) {
        if (s == 2) cudaMemcpyAsync(c->tapeQ2pre, c->Q[2], SB, cudaMemcpyDeviceToDevice, c->stream);
        cudaMemcpyAsync(c->tapeDTV[s], c->DTVisc, sizeof(double) * c->K, cudaMemcpyDeviceToDevice, c->stream);
        L::diss_front(c, s, c->Q[s]);
      } else {
        L::interp(c, c->Q[s]);
      }
      L::edge(c, &c->sc->time, &c->sc->gmax[s]);
      if (c->diss) {
        L::diss_middle(c, s, c->Q[s]);
        cudaMemcpyAsync(c->tapeVS[s], c->viscSpeed, sizeof(double) * c->nEdges, cudaMemcpyDeviceToDevice,
                        c->stream);
      }
      c->QF = faces;
      cudaMemcpyAsync(c->tapeES[s], c->edgeSpeed, sizeof(double) * c->nEdges, cudaMemcpyDeviceToDevice,
                      c->stream);
      if (c->diss) {
        k_div_update<N, double><<<grid(c->K), 128, 0, c->stream>>>(L::update_args(c, -1, c->Q[s]));
        UpdateArgs<double> u = L::update_args(c, s, c->Q[s]);
        u.tapeRHS = c->tapeRHS[s];
        u.tapeRHSpre = c->tapeRHSpre[s];
        k_diss_update<N><<<grid(c->K), 128, 0, c->stream>>>(u);
      } else {
        UpdateArgs<double> u = L::update_args(c, s, c->Q[s]);
        u.tapeRHS = c->tapeRHS[s];
        k_div_update<N, double><<<grid(c->K), 128, 0, c->stream>>>(u);
      }
      if (c->prm.local_time_stepping)
        cudaMemcpyAsync(c->tapeDT[s], c->DT, sizeof(double) * c->K, cudaMemcpyDeviceToDevice, c->stream);
    }
    k_step_end<<<1, 32, 0, c->stream>>>(c->sc, c->prm.local_time_stepping);
    cudaMemcpyAsync(c->tapeSc, c->sc, sizeof(Scalars), cudaMemcpyDeviceToDevice, c->stream);
  }
  static void edges(gcfd_ctx* c, const EdgeArgs<double>& e, const AdjEdgeArgs& x) {
    if (c->nInt > 0) {
      if (e.flux == kFluxRoe && x.useManualRoe)
        k_adj_edge<N, true><<<grid(c->nInt), 128, 0, c->stream>>>(e, x);
      else
        k_adj_edge<N, false><<<grid(c->nInt), 128, 0, c->stream>>>(e, x);
    }
    if (c->nBC > 0) k_adj_edge_bc<N><<<grid(c->nBC * Dims<N>::NE), 128, 0, c->stream>>>(e, x);
  }
  static AdjDissArgs adj_diss_args(gcfd_ctx* c, const double* Qsens, int s) {
    AdjDissArgs x;
    x.nverts = c->nverts;
    x.Qsens = Qsens;
    x.rhsPre = c->tapeRHSpre[s < 0 ? 0 : s];
    x.RbE = c->RbE;
    x.alphaBar = c->alphaBar;
    x.sigVbar = c->sigVbar;
    x.epsVbar = c->epsVbar;
    x.VFbar = c->VFbar;
    x.DissXbar = c->DissXbar;
    x.DissYbar = c->DissYbar;
    x.QFb = c->QFb;
    x.vsBar = c->vsBar;
    x.sigArg = c->sigArg;
    x.epsArg = c->epsArg;
    x.sigE = c->sigE;
    x.SeE = c->SeE;
    x.Q2pre = c->tapeQ2pre;
    x.Qlim = c->Qb[2];
    return x;
  }
  // Dissipation, reverse, part 1 (before the Euler part): recompute the
  // stage's sensor and vertex maxima, then the update / filter / AddDissipation
  // adjoint; the Euler RHS adjoint is left in RbE.
  static void diss_reverse_update(gcfd_ctx* c, int s, const double* Qs, const double* Qsens, const double* Qbn,
                                  double* Qbs, const double* faces) {
    cudaMemsetAsync(c->sigV, 0, sizeof(unsigned long long) * c->nverts, c->stream);
    cudaMemsetAsync(c->epsV, 0, sizeof(unsigned long long) * c->nverts, c->stream);
    DissArgs d = L::diss_args(c, s, const_cast<double*>(Qsens));
    d.sigE = c->sigE;
    d.epsE = c->epsE;
    d.SeE = c->SeE;
    k_diss_sensor<N><<<grid(c->K), 128, 0, c->stream>>>(d);
    cudaMemsetAsync(c->sigArg, 0x7f, sizeof(int) * c->nverts, c->stream);
    cudaMemsetAsync(c->epsArg, 0x7f, sizeof(int) * c->nverts, c->stream);
    k_diss_argmax<<<grid(c->K), 128, 0, c->stream>>>(d, c->sigE, c->epsE, c->sigArg, c->epsArg);
    cudaMemsetAsync(c->sigVbar, 0, sizeof(double) * c->nverts, c->stream);
    cudaMemsetAsync(c->epsVbar, 0, sizeof(double) * c->nverts, c->stream);
    cudaMemsetAsync(c->VFbar, 0, sizeof(double) * (c->nInt + c->nBC) * 4 * c->NE, c->stream);
    d.Qs = Qs;
    d.QF = const_cast<double*>(faces);
    k_adj_diss_update<N><<<grid(c->K), 128, 0, c->stream>>>(d, adj_args(c, s, Qs, Qbn, Qbs),
                                                             adj_diss_args(c, Qsens, s));
  }
  // Dissipation, reverse, part 2 (after the Euler edge and speed adjoints):
  // viscous edges, gradient, face transpose, limiter (rkStep 2), sensor.
  static void diss_reverse_rest(gcfd_ctx* c, int s, const double* Qs, const double* Qsens, double* Qbs,
                                const double* faces) {
    DissArgs d = L::diss_args(c, s, const_cast<double*>(Qs));
    d.QF = const_cast<double*>(faces);
    const AdjDissArgs x = adj_diss_args(c, Qsens, s);
    k_adj_diss_edge<N><<<grid(c->nInt + c->nBC), 128, 0, c->stream>>>(d, x);
    constexpr int NF = Dims<N>::NF;
    k_adj_diss_grad<N><<<grid(c->K), 128, sizeof(double) * (NF * NF + NF * 3), c->stream>>>(d, x, Qbs);
    k_adj_interp<N><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb, c->Iop, Qbs, c->K);
    if (s == 2) k_adj_diss_limit<N><<<grid(4 * c->K), 128, 0, c->stream>>>(d, x);
    k_adj_diss_alpha<<<grid(c->K), 128, 0, c->stream>>>(d, x);
    k_adj_diss_sensor<N><<<grid(c->K), 128, 0, c->stream>>>(d, x, Qbs);
  }
  // The reverse of stage s.  Q0 is the step's initial state.
  static void reverse_stage(gcfd_ctx* c, int s, const double* Q0) {
    const double* Qs = (s == 0) ? Q0 : c->Q[s];
    const double* Qbn = (s == 4) ? c->Qbf : c->Qb[s + 1];
    const double* Qsens = (s == 2) ? c->tapeQ2pre : Qs;
    if (c->diss) {
      diss_reverse_update(c, s, Qs, Qsens, Qbn, c->Qb[s], c->tapeQF[s]);
      k_adj_div<N><<<grid(c->K), 128, 0, c->stream>>>(adj_args(c, -1, Qs, c->RbE, c->Qb[s]));
    } else {
      k_adj_div<N><<<grid(c->K), 128, 0, c->stream>>>(adj_args(c, s, Qs, Qbn, c->Qb[s]));
    }
    EdgeArgs<double> e = edge_args(c, &c->tapeSc0->time);
    e.QF = c->tapeQF[s];
    const AdjEdgeArgs x = adj_edge_args(c);
    const int nE = c->nInt + c->nBC;
    edges(c, e, x);
    cudaMemsetAsync(c->esBar, 0, sizeof(double) * nE, c->stream);
    if (c->diss) cudaMemsetAsync(c->vsBar, 0, sizeof(double) * nE, c->stream);
    AdjDtArgs d;
    d.K = c->K;
    d.stage = s;
    d.nEdges = nE;
    d.cfl = c->prm.cfl;
    d.finalTime = c->prm.final_time;
    d.gmaxS = reinterpret_cast<const double*>(c->tapeSc->gmax);
    d.tn = &c->tapeSc0->time;
    d.dtbarG = c->adjS;
    d.tbarNext = c->adjS + 10;
    d.tbarCur = c->adjS + 9;
    d.argEdge = c->argEdge + s;
    d.esBar = c->esBar;
    d.dtPrev = s > 0 ? c->tapeDT[s - 1] : nullptr;
    d.edgeSpeed = c->tapeES[s];
    d.elemEdge = c->elemEdge;
    d.dtOwnK = c->dtOwnK;
    d.carry = c->carry;
    d.diss = c->diss ? 1 : 0;
    d.cdiff = 1.0 / (double(c->N + 1) * double(c->N + 1));
    d.gviscS = reinterpret_cast<const double*>(c->tapeSc->gvisc);
    d.argVisc = c->argVisc + s;
    d.vsBar = c->vsBar;
    d.dtvPrev = c->diss ? c->tapeDTV[s] : nullptr;
    d.viscSpeed = c->diss ? c->tapeVS[s] : nullptr;
    d.carryV = c->carryV;
    if (c->prm.local_time_stepping) {
      k_adj_lts<<<grid(c->K), 128, 0, c->stream>>>(d);
    } else {
      cudaMemsetAsync(c->argEdge + s, 0x7f, sizeof(int), c->stream);
      k_adj_argmax<<<grid(nE), 128, 0, c->stream>>>(c->tapeES[s], d.gmaxS, s, nE, c->argEdge + s);
      if (c->diss) {
        cudaMemsetAsync(c->argVisc + s, 0x7f, sizeof(int), c->stream);
        k_adj_argmax<<<grid(nE), 128, 0, c->stream>>>(c->tapeVS[s], d.gviscS, s, nE, c->argVisc + s);
      }
      k_adj_gsel<<<1, 32, 0, c->stream>>>(d);
    }
    k_adj_speed<N><<<grid(nE), 128, 0, c->stream>>>(e, x);
    if (c->diss)
      diss_reverse_rest(c, s, Qs, Qsens, c->Qb[s], c->tapeQF[s]);
    else
      k_adj_interp<N><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb, c->Iop, c->Qb[s], c->K);
  }
  // Adjoint of one step whose initial state is Q0 (already in c->Q[0]) and
  // time is in c->sc.  In: Qbf, adjS[10] (t-bar of the step's end).  Out:
  // Qbf <- adjoint of Q0, adjS[10] <- t-bar of the step's start.  carryV (the
  // DTVisc adjoint) runs on across steps.
  static void reverse_step(gcfd_ctx* c, const double* Q0) {
    tape_step(c);
    // no zeroing of the stage adjoints: the first write to each is a store
    cudaMemsetAsync(c->adjS, 0, sizeof(double) * 5, c->stream);
    cudaMemcpyAsync(c->adjS + 9, c->adjS + 10, sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
    cudaMemsetAsync(c->carry, 0, sizeof(double) * c->K, c->stream);
    for (int s = 4; s >= 0; --s) reverse_stage(c, s, Q0);
    std::swap(c->Qbf, c->Qb[0]);
    cudaMemcpyAsync(c->adjS + 10, c->adjS + 9, sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  }
  // RHS adjoint at c->Qtmp and sc->rhs_time: Qb[0] <- J^T Qbf.
  static void rhs_vjp(gcfd_ctx* c) {
    const size_t S = sizeof(double) * 4 * c->Np * static_cast<size_t>(c->K);
    void* faces = c->QF;
    if (c->diss) {  // the forward RHS once more, keeping the pre-filter RHS
      c->QF = c->tapeQF[0];
      L::diss_front(c, -1, c->Qtmp);
      L::edge(c, &c->sc->rhs_time, &c->sc->gmax[0]);
      L::diss_middle(c, -1, c->Qtmp);
      k_div_update<N, double><<<grid(c->K), 128, 0, c->stream>>>(L::update_args(c, -1, c->Qtmp));
      UpdateArgs<double> u = L::update_args(c, -1, c->Qtmp);
      u.tapeRHSpre = c->tapeRHSpre[0];
      k_diss_update<N><<<grid(c->K), 128, 0, c->stream>>>(u);
    } else {
      L::interp(c, c->Qtmp);
    }
    cudaMemsetAsync(c->Qb[0], 0, S, c->stream);
    const EdgeArgs<double> e = edge_args(c, &c->sc->rhs_time);
    if (c->diss) {
      diss_reverse_update(c, -1, c->Qtmp, c->Qtmp, c->Qbf, c->Qb[0], static_cast<const double*>(c->QF));
      k_adj_div<N><<<grid(c->K), 128, 0, c->stream>>>(adj_args(c, -1, c->Qtmp, c->RbE, c->Qb[0]));
    } else {
      k_adj_div<N><<<grid(c->K), 128, 0, c->stream>>>(adj_args(c, -1, c->Qtmp, c->Qbf, c->Qb[0]));
    }
    edges(c, e, adj_edge_args(c));
    if (c->diss) {
      cudaMemsetAsync(c->vsBar, 0, sizeof(double) * (c->nInt + c->nBC), c->stream);
      diss_reverse_rest(c, -1, c->Qtmp, c->Qtmp, c->Qb[0], static_cast<const double*>(c->QF));
      c->QF = faces;
    } else {
      k_adj_interp<N><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb, c->Iop, c->Qb[0], c->K);
    }
  }
  // Functionals of the current state Q[0]: J into adjS[11], dJ/dQ into Qb[0],
  // dJ/dt into adjS[9].
  static void functional(gcfd_ctx* c, int kind) {
    const size_t S = sizeof(double) * 4 * c->Np * static_cast<size_t>(c->K);
    cudaMemsetAsync(c->Qb[0], 0, S, c->stream);
    if (kind == GCFD_FUNC_VORTEX_ERROR) {
      k_func_vortex<N><<<grid(c->K), 128, 0, c->stream>>>(c->Q[0], c->dXs, c->dYs, c->K, c->vbeta, c->vx0, c->vy0,
                                                          c->vgamma, &c->sc->time, c->Qb[0], c->adjS + 11,
                                                          c->adjS + 9);
      return;
    }
    L::interp(c, c->Q[0]);
    cudaMemsetAsync(c->QFb, 0, sizeof(double) * 4 * 3 * c->NE * static_cast<size_t>(c->K), c->stream);
    const EdgeArgs<double> e = edge_args(c, &c->sc->time);
    if (c->nBC > 0)
      k_func_wall<N><<<grid(c->nBC), 128, 0, c->stream>>>(e, c->edgeW, kind == GCFD_FUNC_WALL_FORCE_Y, c->QFb,
                                                          c->adjS + 11);
    k_adj_interp<N><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb, c->Iop, c->Qb[0], c->K);
  }
};

struct AdjOps {
  void (*tape_step)(gcfd_ctx*);
  void (*reverse_step)(gcfd_ctx*, const double*);
  void (*rhs_vjp)(gcfd_ctx*);
  void (*functional)(gcfd_ctx*, int);
};

template <int N>
AdjOps adj_ops_for() {
  return AdjOps{&AdjLaunch<N>::tape_step, &AdjLaunch<N>::reverse_step, &AdjLaunch<N>::rhs_vjp,
                &AdjLaunch<N>::functional};
}

bool select_adj_ops(int N, AdjOps* o) {
  switch (N) {
    case 0: *o = adj_ops_for<0>(); return true;
    case 1: *o = adj_ops_for<1>(); return true;
    case 2: *o = adj_ops_for<2>(); return true;
    case 3: *o = adj_ops_for<3>(); return true;
    case 4: *o = adj_ops_for<4>(); return true;
    default: return false;
  }
}

// Mixed path: rebuild the FP64 state Q[0] from the compensated pair.
void to_fp64_range(gcfd_ctx* c, int k0, int k1) {
  if (k1 <= k0) return;
  const size_t n = static_cast<size_t>(4) * c->Np * (k1 - k0);
  k_mixed_to_fp64<<<static_cast<int>(std::min<size_t>((n + 255) / 256, 152 * 16)), 256, 0, c->stream>>>(
      c->Qhi, c->Qlo, c->Q[0], c->K, 4 * c->Np, k0, k1);
}

int sync_fp64_state(gcfd_ctx* c) {
  if (!c->fp32 || !c->fp64Stale) return GCFD_OK;
  to_fp64_range(c, 0, c->K);
  GCFD_CUDA(c, cudaGetLastError());
  c->fp64Stale = false;
  return GCFD_OK;
}

// Host <-> device state copies of the element range [k0, k1) of the sharded
// host state (shard np covers [S_np, S_np + Kmax[np])) on the given stream.
int copy_shards_range(gcfd_ctx* c, int nshards, const int32_t* Kmax, const double* const* Qin,
                      double* const* Qout, bool toDevice, int k0, int k1, cudaStream_t st) {
  const size_t pitch = static_cast<size_t>(c->K) * sizeof(double);
  long long s0 = 0;
  for (int np = 0; np < nshards; ++np) {
    const long long a = std::max<long long>(s0, k0), b = std::min<long long>(s0 + Kmax[np], k1);
    if (b > a) {
      const size_t hp = static_cast<size_t>(Kmax[np]) * sizeof(double), w = static_cast<size_t>(b - a) * sizeof(double);
      for (int n = 0; n < 4; ++n) {
        double* d = c->Q[0] + static_cast<size_t>(n) * c->Np * c->K + a;
        if (toDevice) {
          if (!Qin[np * 4 + n]) return fail(c, GCFD_ERR_ARG, "null state pointer");
          GCFD_CUDA(c, cudaMemcpy2DAsync(d, pitch, Qin[np * 4 + n] + (a - s0), hp, w, c->Np, cudaMemcpyHostToDevice,
                                         st));
        } else {
          if (!Qout[np * 4 + n]) return fail(c, GCFD_ERR_ARG, "null state pointer");
          GCFD_CUDA(c, cudaMemcpy2DAsync(Qout[np * 4 + n] + (a - s0), hp, d, pitch, w, c->Np,
                                         cudaMemcpyDeviceToHost, st));
        }
      }
    }
    s0 += Kmax[np];
  }
  return GCFD_OK;
}



struct Ops {
  void (*step)(gcfd_ctx*, cudaEvent_t*, double*, int*);
  void (*rhs)(gcfd_ctx*);
  void (*prep)(gcfd_ctx*);  // rebuild stage-0 data from Q0 (mixed path), or nullptr
  void (*prep_range)(gcfd_ctx*, int, int);  // the same for elements [k0, k1)
};

template <int N>
Ops ops_for(bool fp32) {
  if (fp32)
    return Ops{&MixedLaunch<N>::step, &MixedLaunch<N>::rhs, &MixedLaunch<N>::prep_state,
               &MixedLaunch<N>::prep_state_range};
  return Ops{&Launch<N, double>::step, &Launch<N, double>::rhs, nullptr, nullptr};
}

bool select_ops(int N, bool fp32, Ops* o) {
  switch (N) {
    case 0: *o = ops_for<0>(fp32); return true;
    case 1: *o = ops_for<1>(fp32); return true;
    case 2: *o = ops_for<2>(fp32); return true;
    case 3: *o = ops_for<3>(fp32); return true;
    case 4: *o = ops_for<4>(fp32); return true;
    default: return false;
  }
}

// Mixed path: the state moves in kStateChunks element ranges, and each range's
// conversion (hi/lo split, dQ0, faces, reference states on the way in; hi + lo
// to FP64 on the way out) runs on the compute stream while the next range's copy
// is in flight on the second stream.
constexpr int kStateChunks = 8;

int set_state_overlapped(gcfd_ctx* c, int nshards, const int32_t* Kmax, const double* const* Q) {
  Ops o;
  select_ops(c->N, c->fp32, &o);
  const int step = ((c->K + kStateChunks - 1) / kStateChunks + 31) & ~31;
  GCFD_CUDA(c, cudaEventRecord(c->evFork, c->stream));  // earlier work on Q0 first
  GCFD_CUDA(c, cudaStreamWaitEvent(c->stream2, c->evFork, 0));
  for (int j = 0, k0 = 0; k0 < c->K; ++j, k0 += step) {
    const int k1 = std::min(c->K, k0 + step);
    int rc = copy_shards_range(c, nshards, Kmax, Q, nullptr, true, k0, k1, c->stream2);
    if (rc) return rc;
    GCFD_CUDA(c, cudaEventRecord(c->evChunk[j], c->stream2));
    GCFD_CUDA(c, cudaStreamWaitEvent(c->stream, c->evChunk[j], 0));
    o.prep_range(c, k0, k1);
  }
  GCFD_CUDA(c, cudaGetLastError());
  c->dirty = false;
  c->fp64Stale = false;
  return GCFD_OK;
}

int get_state_overlapped(gcfd_ctx* c, int nshards, const int32_t* Kmax, double* const* Q) {
  const int step = ((c->K + kStateChunks - 1) / kStateChunks + 31) & ~31;
  for (int j = 0, k0 = 0; k0 < c->K; ++j, k0 += step) {
    const int k1 = std::min(c->K, k0 + step);
    to_fp64_range(c, k0, k1);
    GCFD_CUDA(c, cudaEventRecord(c->evChunk[j], c->stream));
    GCFD_CUDA(c, cudaStreamWaitEvent(c->stream2, c->evChunk[j], 0));
    int rc = copy_shards_range(c, nshards, Kmax, nullptr, Q, false, k0, k1, c->stream2);
    if (rc) return rc;
  }
  GCFD_CUDA(c, cudaGetLastError());
  GCFD_CUDA(c, cudaEventRecord(c->evJoin, c->stream2));
  GCFD_CUDA(c, cudaStreamWaitEvent(c->stream, c->evJoin, 0));
  c->fp64Stale = false;
  return GCFD_OK;
}

int capture_graph(gcfd_ctx* c) {
  Ops o;
  select_ops(c->N, c->fp32, &o);
  GCFD_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  o.step(c, nullptr, nullptr, nullptr);
  cudaGraph_t g = nullptr;
  GCFD_CUDA(c, cudaStreamEndCapture(c->stream, &g));
  c->graph = g;
  GCFD_CUDA(c, cudaGraphInstantiate(&c->graphExec, g, 0));
  return GCFD_OK;
}

int prepare_if_dirty(gcfd_ctx* c) {
  if (!c->dirty) return GCFD_OK;
  Ops o;
  select_ops(c->N, c->fp32, &o);
  if (o.prep) o.prep(c);
  GCFD_CUDA(c, cudaGetLastError());
  c->dirty = false;
  return GCFD_OK;
}

int check_shards(gcfd_ctx* c, int nshards, const int32_t* Kmax) {
  if (nshards <= 0 || !Kmax) return fail(c, GCFD_ERR_ARG, "nshards must be > 0 with Kmax given");
  long long tot = 0;
  for (int i = 0; i < nshards; ++i) {
    if (Kmax[i] < 0) return fail(c, GCFD_ERR_SHAPE, "negative shard size");
    tot += Kmax[i];
  }
  if (tot != c->K)
    return fail(c, GCFD_ERR_SHAPE, "shard sizes sum to " + std::to_string(tot) + ", mesh has K=" +
                                       std::to_string(c->K));
  return GCFD_OK;
}

int copy_shards(gcfd_ctx* c, double* dst, int nshards, const int32_t* Kmax, const double* const* Q,
                bool toDevice, double* const* Qout) {
  const size_t pitch = static_cast<size_t>(c->K) * sizeof(double);
  long long k0 = 0;
  for (int np = 0; np < nshards; ++np) {
    const size_t w = static_cast<size_t>(Kmax[np]) * sizeof(double);
    if (w == 0) continue;
    for (int n = 0; n < 4; ++n) {
      double* d = dst + static_cast<size_t>(n) * c->Np * c->K + k0;
      if (toDevice) {
        if (!Q[np * 4 + n]) return fail(c, GCFD_ERR_ARG, "null state pointer");
        GCFD_CUDA(c, cudaMemcpy2DAsync(d, pitch, Q[np * 4 + n], w, w, c->Np, cudaMemcpyHostToDevice,
                                       c->stream));
      } else {
        if (!Qout[np * 4 + n]) return fail(c, GCFD_ERR_ARG, "null state pointer");
        GCFD_CUDA(c, cudaMemcpy2DAsync(Qout[np * 4 + n], w, d, pitch, w, c->Np,
                                       cudaMemcpyDeviceToHost, c->stream));
      }
    }
    k0 += Kmax[np];
  }
  return GCFD_OK;
}

// Initial condition, InitializeSolution (euler.go:728-794).
std::vector<double> initial_state(gcfd_ctx* c) {
  const int K = c->K, Np = c->Np;
  std::vector<double> q(static_cast<size_t>(4) * Np * K);
  for (int i = 0; i < Np; ++i)
    for (int k = 0; k < K; ++k) {
      double s[4];
      const size_t pt = static_cast<size_t>(i) * K + k;
      if (c->prm.init_type == GCFD_INIT_IVORTEX) {
        const double x = c->geo.xSol[pt], y = c->geo.ySol[pt];
        const double pi = 3.14159265358979323846, g = c->vgamma, GM1 = g - 1.0;
        double u = 1.0, v = 0.0;
        const double r2 = (x - c->vx0) * (x - c->vx0) + (y - c->vy0) * (y - c->vy0);
        const double ex1r = std::exp(1.0 - r2);
        const double tv1 = 1.0 - (GM1 * c->vbeta * c->vbeta * std::exp(2.0 * (1.0 - r2)) / (16.0 * g * pi * pi));
        u -= c->vbeta * ex1r * (y - c->vy0) * (0.5 / pi);
        v += c->vbeta * ex1r * (x - c->vx0) * (0.5 / pi);
        const double rho = std::pow(tv1, 1.0 / GM1), p = std::pow(rho, g);
        s[0] = rho; s[1] = rho * u; s[2] = rho * v;
        s[3] = p * (1.0 / GM1) + 0.5 * rho * (u * u + v * v);
      } else if (c->prm.init_type == GCFD_INIT_SHOCKTUBE) {
        const double* src = (c->geo.xSol[pt] < 0.5) ? c->fsIn.qinf : c->fsOut.qinf;
        for (int n = 0; n < 4; ++n) s[n] = src[n];
      } else {
        for (int n = 0; n < 4; ++n) s[n] = c->fsFar.qinf[n];
      }
      for (int n = 0; n < 4; ++n) q[(static_cast<size_t>(n) * Np + i) * K + k] = s[n];
    }
  return q;
}

// Buffers and operators of the artificial dissipation (FP64 path).
int build_diss(gcfd_ctx* c, const gcfd_mesh* m) {
  const int K = c->K, Np = c->Np, NE = c->NE;
  const int NR = Np + 3 * NE;
  int rc;
  c->nverts = m->nverts;
  if ((rc = dalloc(c, &c->sigV, static_cast<size_t>(c->nverts)))) return rc;
  if ((rc = dalloc(c, &c->epsV, static_cast<size_t>(c->nverts)))) return rc;
  if ((rc = dalloc(c, &c->DissX, static_cast<size_t>(4) * NR * K))) return rc;
  if ((rc = dalloc(c, &c->DissY, static_cast<size_t>(4) * NR * K))) return rc;
  if ((rc = dalloc(c, &c->VF, static_cast<size_t>(c->nEdges) * 4 * NE))) return rc;
  if ((rc = dalloc(c, &c->viscSpeed, static_cast<size_t>(c->nEdges)))) return rc;
  if ((rc = dalloc(c, &c->DTVisc, static_cast<size_t>(K)))) return rc;
  GCFD_CUDA(c, cudaMemset(c->DTVisc, 0, sizeof(double) * K));
  if ((rc = upload(c, &c->dDiv, c->el.Div.v))) return rc;
  if ((rc = upload(c, &c->dBary, c->el.Bary.v))) return rc;
  if ((rc = upload(c, &c->dV, c->el.V.v))) return rc;
  if ((rc = upload(c, &c->dVinv, c->el.Vinv.v))) return rc;
  if ((rc = upload(c, &c->dmf, c->el.ModeFilter))) return rc;
  if ((rc = upload(c, &c->dSensP, c->el.SensP.v))) return rc;
  if ((rc = upload(c, &c->dMass, c->el.MassMatrix.v))) return rc;
  if ((rc = upload(c, &c->dSensD, c->el.SensD.v))) return rc;
  if ((rc = upload(c, &c->dhK, c->geo.hK))) return rc;
  if ((rc = upload(c, &c->dnxE, c->geo.nx))) return rc;
  if ((rc = upload(c, &c->dnyE, c->geo.ny))) return rc;
  if ((rc = upload(c, &c->dIIE, c->geo.IInII))) return rc;
  std::vector<int> ev(static_cast<size_t>(3) * K);
  for (int k = 0; k < K; ++k)
    for (int v = 0; v < 3; ++v) ev[static_cast<size_t>(v) * K + k] = m->etov[3 * k + v];
  if ((rc = upload(c, &c->detov, ev))) return rc;
  return GCFD_OK;
}

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

int build_tc(gcfd_ctx* c) {
  switch (c->N) {
    case 0: return build_tc_n<0>(c);
    case 1: return build_tc_n<1>(c);
    case 2: return build_tc_n<2>(c);
    case 3: return build_tc_n<3>(c);
    case 4: return build_tc_n<4>(c);
    default: return fail(c, GCFD_ERR_UNSUPPORTED, "tensor-core path: N <= 4");
  }
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

int build_pipe(gcfd_ctx* c) {
  switch (c->N) {
    case 0: return c->tc ? build_pipe_n<0, true>(c) : build_pipe_n<0, false>(c);
    case 1: return c->tc ? build_pipe_n<1, true>(c) : build_pipe_n<1, false>(c);
    case 2: return c->tc ? build_pipe_n<2, true>(c) : build_pipe_n<2, false>(c);
    case 3: return c->tc ? build_pipe_n<3, true>(c) : build_pipe_n<3, false>(c);
    case 4: return c->tc ? build_pipe_n<4, true>(c) : build_pipe_n<4, false>(c);
    default: return GCFD_OK;
  }
}

// The mixed path's FP32 operators into the per-order constant-memory copies
// (identical for every context of the same order, so concurrent contexts agree).
int upload_const_ops(gcfd_ctx* c, const std::vector<float>& divT, const std::vector<float>& iopT) {
  const void* d = nullptr;
  const void* i = nullptr;
  switch (c->N) {
    case 0: d = &cDivT0; i = &cIopT0; break;
    case 1: d = &cDivT1; i = &cIopT1; break;
    case 2: d = &cDivT2; i = &cIopT2; break;
    case 3: d = &cDivT3; i = &cIopT3; break;
    case 4: d = &cDivT4; i = &cIopT4; break;
    default: return fail(c, GCFD_ERR_UNSUPPORTED, "mixed path: N <= 4");
  }
  GCFD_CUDA(c, cudaMemcpyToSymbol(d, divT.data(), divT.size() * sizeof(float)));
  GCFD_CUDA(c, cudaMemcpyToSymbol(i, iopT.data(), iopT.size() * sizeof(float)));
  // The modal filter's operators (PerssonC0 on the mixed path).
  const void* sv[5] = {&cV0, &cV1, &cV2, &cV3, &cV4};
  const void* svi[5] = {&cVi0, &cVi1, &cVi2, &cVi3, &cVi4};
  const void* smf[5] = {&cMf0, &cMf1, &cMf2, &cMf3, &cMf4};
  const int np = c->Np;
  std::vector<float> V(static_cast<size_t>(np) * np), Vi(V.size()), mf(np);
  for (size_t q = 0; q < V.size(); ++q) {
    V[q] = static_cast<float>(c->el.V.v[q]);
    Vi[q] = static_cast<float>(c->el.Vinv.v[q]);
  }
  for (int q = 0; q < np; ++q) mf[q] = static_cast<float>(c->el.ModeFilter[q]);
  GCFD_CUDA(c, cudaMemcpyToSymbol(sv[c->N], V.data(), V.size() * sizeof(float)));
  GCFD_CUDA(c, cudaMemcpyToSymbol(svi[c->N], Vi.data(), Vi.size() * sizeof(float)));
  GCFD_CUDA(c, cudaMemcpyToSymbol(smf[c->N], mf.data(), mf.size() * sizeof(float)));
  return GCFD_OK;
}

// Buffers and FP32 operator / geometry copies of the mixed path.
int build_mixed(gcfd_ctx* c) {
  const int K = c->K, Np = c->Np, NE = c->NE, NF = c->NF;
  const int NPP = (Np + 3) & ~3;
  const size_t nS = static_cast<size_t>(4) * Np * K;
  int rc;
  if ((rc = dalloc(c, &c->dQ0, nS))) return rc;
  for (int i = 1; i <= 4; ++i)
    if ((rc = dalloc(c, &c->Dk[i], nS))) return rc;
  if ((rc = dalloc(c, &c->R3, nS))) return rc;
  const int NEP = (NE + 1) & ~1;  // edge-major stride, see MixedDims::NEP
  if ((rc = dalloc(c, &c->mfaces, static_cast<size_t>(c->nEdges) * 2 * 4 * NEP))) return rc;
  if ((rc = dalloc(c, &c->mfhat, static_cast<size_t>(c->nEdges) * 4 * NEP))) return rc;
  if ((rc = dalloc(c, &c->mcorr, static_cast<size_t>(c->nEdges) * 4))) return rc;
  if ((rc = dalloc(c, &c->mbase, static_cast<size_t>(K) * 4))) return rc;
  if ((rc = dalloc(c, &c->Qhi, nS))) return rc;
  if ((rc = dalloc(c, &c->Qlo, nS))) return rc;
  GCFD_CUDA(c, cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
  GCFD_CUDA(c, cudaEventCreateWithFlags(&c->evFork, cudaEventDisableTiming));
  GCFD_CUDA(c, cudaEventCreateWithFlags(&c->evJoin, cudaEventDisableTiming));
  for (auto& e : c->evChunk) GCFD_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  if ((rc = dalloc(c, &c->mexBC, static_cast<size_t>(std::max(c->nBC, 1)) * NE * 4))) return rc;
  GCFD_CUDA(c, cudaMemset(c->mfaces, 0, sizeof(float) * c->nEdges * 2 * 4 * NEP));
  GCFD_CUDA(c, cudaMemset(c->mfhat, 0, sizeof(float) * c->nEdges * 4 * NEP));
  GCFD_CUDA(c, cudaMemset(c->mcorr, 0, sizeof(float) * c->nEdges * 4));
  // DivInt^T, rows = flux DOF j, cols = output point r padded to NPP.
  // FluxEdgeInterp^T, rows = solution point i, cols = face point padded to NE3P.
  const int NE3P = (3 * NE + 3) & ~3;
  std::vector<float> divT(static_cast<size_t>(NF) * NPP, 0.f), iop(static_cast<size_t>(NPP) * NE3P, 0.f);
  for (int j = 0; j < NF; ++j)
    for (int r = 0; r < Np; ++r) divT[static_cast<size_t>(j) * NPP + r] = static_cast<float>(c->el.DivInt(r, j));
  for (int j = 0; j < 3 * NE; ++j)
    for (int i = 0; i < Np; ++i) iop[static_cast<size_t>(i) * NE3P + j] = static_cast<float>(c->el.FluxEdgeInterp(j, i));
  if ((rc = upload_const_ops(c, divT, iop))) return rc;
  if (c->tc && (rc = build_tc(c))) return rc;
  const Geometry& g = c->geo;
  std::vector<float> geo(static_cast<size_t>(6) * K), ii(static_cast<size_t>(3) * K);
  for (int k = 0; k < K; ++k) {
    geo[k] = static_cast<float>(g.Jdet[k]);
    for (int q = 0; q < 4; ++q) geo[static_cast<size_t>(q + 1) * K + k] = static_cast<float>(g.Jinv[4 * k + q]);
    geo[static_cast<size_t>(5) * K + k] = static_cast<float>(1.0 / g.Jdet[k]);
    for (int e = 0; e < 3; ++e) ii[static_cast<size_t>(e) * K + k] = static_cast<float>(g.IInII[static_cast<size_t>(e) * K + k]);
  }
  if ((rc = upload(c, &c->mgeo, geo))) return rc;
  if ((rc = upload(c, &c->mII, ii))) return rc;
  std::vector<int> slot(static_cast<size_t>(3) * K);
  std::vector<int> pos(c->topo.nEdges);
  for (int i = 0; i < c->nEdges; ++i) pos[c->edgeOrder[i]] = i;
  for (int k = 0; k < K; ++k)
    for (int e = 0; e < 3; ++e) {
      const int en = c->topo.elemEdge[3 * k + e];
      const int side = (c->topo.kL[en] == k && c->topo.eL[en] == e) ? 0 : 1;
      slot[static_cast<size_t>(e) * K + k] = pos[en] * 2 + side;
    }
  if ((rc = upload(c, &c->meslot, slot))) return rc;
  std::vector<float> nx(c->nEdges), ny(c->nEdges), oh(c->nEdges);
  for (int i = 0; i < c->nEdges; ++i) {
    nx[i] = static_cast<float>(c->hnx[i]);
    ny[i] = static_cast<float>(c->hny[i]);
    oh[i] = static_cast<float>(c->hoohK[i]);
  }
  if ((rc = upload(c, &c->mnx, nx))) return rc;
  if ((rc = upload(c, &c->mny, ny))) return rc;
  if ((rc = upload(c, &c->moohK, oh))) return rc;
  return build_pipe(c);
}

int build_context(gcfd_ctx* c, const gcfd_mesh* m) {
  const gcfd_params& p = c->prm;
  c->N = p.N;
  c->fp32 = (p.precision == GCFD_PREC_FP32 || p.precision == GCFD_PREC_TF32X3);
  c->tc = (p.precision == GCFD_PREC_TF32X3);
  // NewEuler creates the dissipation only for PerssonC0 with N > 0 (euler.go:107-112);
  // the sensor ramp takes Kappa when given, else 5 (dissipation.go:140-147).
  c->diss = (p.limiter == GCFD_LIMITER_PERSSON_C0) && p.N > 0;
  c->dissKappa = (p.kappa != 0.0) ? p.kappa : 5.0;
  try {
    c->el = build_dfr_element(p.N);
  } catch (const std::exception& e) {
    return fail(c, GCFD_ERR_UNSUPPORTED, e.what());
  }
  c->Np = c->el.Np;
  c->NE = c->el.NpEdge;
  c->NF = c->el.NpFlux;
  c->K = m->K;
  std::string msg = build_topology(m->nverts, m->K, m->etov, m->nbc, m->bc_v1, m->bc_v2, m->bc_flag,
                                   &c->topo);
  if (!msg.empty()) return fail(c, GCFD_ERR_ARG, msg);
  build_geometry(c->el, c->topo, m->vx, m->vy, m->etov, &c->geo);
  for (int k = 0; k < c->K; ++k)
    if (!(c->geo.Jdet[k] > 0.0))
      return fail(c, GCFD_ERR_ARG, "element " + std::to_string(k) +
                                       " is not counter-clockwise (|J| <= 0)");

  // Free streams and BC relabelling of InitializeSolution (euler.go:728-794).
  c->fsFar = freestream_from_mach(p.minf, p.gamma, p.alpha);
  c->fsIn = c->fsFar;
  c->fsOut = c->fsFar;
  c->vx0 = p.vortex_x0;
  c->vy0 = p.vortex_y0;
  if (p.init_type == GCFD_INIT_IVORTEX) {
    const double q[4] = {1, 1, 0, 3};
    c->fsFar = freestream_from_q(1.4, q);
    for (int& b : c->topo.bc)
      if (b == BC_Wall) b = BC_IVortex;
  } else if (p.init_type == GCFD_INIT_SHOCKTUBE) {
    const double g = 1.4;
    const double qi[4] = {1, 0, 0, 1 / (g - 1)}, qo[4] = {0.125, 0, 0, 0.1 / (g - 1)};
    c->fsIn = freestream_from_q(g, qi);
    c->fsOut = freestream_from_q(g, qo);
  }

  // Edge tables: interior edges first, then boundary edges, each in mesh order.
  const Topology& t = c->topo;
  const Geometry& g = c->geo;
  std::vector<int> order;
  for (int en = 0; en < t.nEdges; ++en)
    if (t.kR[en] >= 0) order.push_back(en);
  c->nInt = static_cast<int>(order.size());
  for (int en = 0; en < t.nEdges; ++en)
    if (t.kR[en] < 0) order.push_back(en);
  c->nEdges = t.nEdges;
  c->nBC = c->nEdges - c->nInt;
  const int K = c->K, NE = c->NE, Np = c->Np;
  std::vector<int> kL(c->nEdges), kR(c->nEdges), eLR(c->nEdges), flag(std::max(c->nBC, 1));
  std::vector<double> nx(c->nEdges), ny(c->nEdges), IIL(c->nEdges), IIR(c->nEdges), oohK(c->nEdges);
  std::vector<double> bx(static_cast<size_t>(std::max(c->nBC, 1)) * NE), by(bx.size());
  std::vector<int> elemEdge(static_cast<size_t>(3) * K);
  std::vector<int> pos(t.nEdges);
  for (int i = 0; i < c->nEdges; ++i) {
    const int en = order[i];
    pos[en] = i;
    kL[i] = t.kL[en];
    kR[i] = t.kR[en] >= 0 ? t.kR[en] : 0;
    eLR[i] = t.eL[en] | ((t.eR[en] >= 0 ? t.eR[en] : 0) << 2);
    const size_t fl = static_cast<size_t>(t.eL[en]) * K + t.kL[en];
    nx[i] = g.nx[fl];
    ny[i] = g.ny[fl];
    IIL[i] = g.IInII[fl];
    IIR[i] = t.kR[en] >= 0 ? g.IInII[static_cast<size_t>(t.eR[en]) * K + t.kR[en]] : 0.0;
    oohK[i] = 1.0 / g.hK[t.kL[en]];
    if (i >= c->nInt) {
      const int b = i - c->nInt;
      flag[b] = t.bc[en];
      for (int q = 0; q < NE; ++q) {
        const size_t row = static_cast<size_t>(2 * Np + t.eL[en] * NE + q);
        element_point(m->etov, m->vx, m->vy, t.kL[en], c->el.rFlux[row], c->el.sFlux[row],
                      &bx[static_cast<size_t>(b) * NE + q], &by[static_cast<size_t>(b) * NE + q]);
      }
    }
  }
  for (int k = 0; k < K; ++k)
    for (int ed = 0; ed < 3; ++ed)
      elemEdge[static_cast<size_t>(ed) * K + k] = pos[t.elemEdge[3 * k + ed]];
  c->edgeOrder = order;
  c->hnx = nx;
  c->hny = ny;
  c->hoohK = oohK;

  GCFD_CUDA(c, cudaSetDevice(p.device));
  GCFD_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  const size_t nState = static_cast<size_t>(4) * Np * K;
  const size_t nFace = static_cast<size_t>(4) * 3 * NE * K;
  const size_t tsz = c->fp32 ? sizeof(float) : sizeof(double);
  int rc;
  for (int s = 0; s < 5; ++s)
    if ((rc = dalloc(c, &c->Q[s], nState))) return rc;
  if ((rc = dalloc(c, &c->R, nState))) return rc;
  if ((rc = dalloc(c, &c->Qtmp, nState))) return rc;
  if ((rc = dalloc(c, &c->rhsOut, nState))) return rc;
  if (!c->fp32) {
    char* qf = nullptr;
    if ((rc = dalloc(c, &qf, nFace * tsz))) return rc;
    c->QF = qf;
    char* fe = nullptr;
    if ((rc = dalloc(c, &fe, nFace * tsz))) return rc;
    c->FE = fe;
  } else {
    if ((rc = build_mixed(c))) return rc;
  }
  if (c->diss && (rc = build_diss(c, m))) return rc;
  if ((rc = upload(c, &c->Iop, c->el.FluxEdgeInterp.v))) return rc;
  if ((rc = upload(c, &c->Div, c->el.DivInt.v))) return rc;
  if ((rc = upload(c, &c->Jdet, g.Jdet))) return rc;
  std::vector<double> jinvT(static_cast<size_t>(4) * K);
  for (int k = 0; k < K; ++k)
    for (int q = 0; q < 4; ++q) jinvT[static_cast<size_t>(q) * K + k] = g.Jinv[4 * k + q];
  if ((rc = upload(c, &c->Jinv, jinvT))) return rc;
  if ((rc = upload(c, &c->ekL, kL))) return rc;
  if ((rc = upload(c, &c->ekR, kR))) return rc;
  if ((rc = upload(c, &c->eLR, eLR))) return rc;
  if ((rc = upload(c, &c->bcFlag, flag))) return rc;
  if ((rc = upload(c, &c->elemEdge, elemEdge))) return rc;
  if ((rc = upload(c, &c->enx, nx))) return rc;
  if ((rc = upload(c, &c->eny, ny))) return rc;
  if ((rc = upload(c, &c->eIIL, IIL))) return rc;
  if ((rc = upload(c, &c->eIIR, IIR))) return rc;
  if ((rc = upload(c, &c->eoohK, oohK))) return rc;
  if ((rc = upload(c, &c->bx, bx))) return rc;
  if ((rc = upload(c, &c->by, by))) return rc;
  if ((rc = dalloc(c, &c->edgeSpeed, static_cast<size_t>(c->nEdges)))) return rc;
  if ((rc = dalloc(c, &c->DT, static_cast<size_t>(K)))) return rc;
  if ((rc = dalloc(c, &c->sc, 1))) return rc;
  GCFD_CUDA(c, cudaMemset(c->sc, 0, sizeof(Scalars)));
  GCFD_CUDA(c, cudaMemset(c->DT, 0, sizeof(double) * K));
  GCFD_CUDA(c, cudaMemset(c->R, 0, sizeof(double) * nState));
  std::vector<double> q0 = initial_state(c);
  GCFD_CUDA(c, cudaMemcpy(c->Q[0], q0.data(), nState * sizeof(double), cudaMemcpyHostToDevice));
  for (auto& e : c->ev) GCFD_CUDA(c, cudaEventCreate(&e));
  if ((rc = capture_graph(c))) return rc;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  return GCFD_OK;
}

}  // namespace

extern "C" {

int gcfd_create(const gcfd_mesh* mesh, const gcfd_params* params, gcfd_ctx** out) {
  g_create_error.clear();
  if (!mesh || !params || !out) return fail(nullptr, GCFD_ERR_ARG, "null argument");
  *out = nullptr;
  if (mesh->K <= 0 || mesh->nverts < 3 || !mesh->vx || !mesh->vy || !mesh->etov)
    return fail(nullptr, GCFD_ERR_ARG, "mesh needs K > 0, nverts >= 3 and vertex/element arrays");
  if (mesh->nbc < 0 || (mesh->nbc > 0 && (!mesh->bc_v1 || !mesh->bc_v2 || !mesh->bc_flag)))
    return fail(nullptr, GCFD_ERR_ARG, "boundary edge arrays missing");
  if (params->N < 0 || params->N > 4)
    return fail(nullptr, GCFD_ERR_UNSUPPORTED, "PolynomialOrder must be 0..4");
  if (params->precision != GCFD_PREC_FP64 && params->precision != GCFD_PREC_FP32 &&
      params->precision != GCFD_PREC_TF32X3)
    return fail(nullptr, GCFD_ERR_UNSUPPORTED, "unknown precision mode");
  if (params->flux_type < 0 || params->flux_type > 3)
    return fail(nullptr, GCFD_ERR_ARG, "unknown flux type");
  if (params->init_type < 0 || params->init_type > 2)
    return fail(nullptr, GCFD_ERR_ARG, "unknown init type");
  if (params->limiter != GCFD_LIMITER_NONE && params->limiter != GCFD_LIMITER_PERSSON_C0)
    return fail(nullptr, GCFD_ERR_ARG, "unknown limiter");
  if (!(params->cfl > 0.0)) return fail(nullptr, GCFD_ERR_ARG, "CFL must be > 0");
  std::unique_ptr<gcfd_ctx> c(new gcfd_ctx());
  c->prm = *params;
  int rc = build_context(c.get(), mesh);
  if (rc != GCFD_OK) {
    g_create_error = c->err;
    return rc;
  }
  *out = c.release();
  return GCFD_OK;
}

int gcfd_destroy(gcfd_ctx* ctx) {
  if (!ctx) return GCFD_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  delete ctx;
  return GCFD_OK;
}

int gcfd_read_mesh(const char* path, gcfd_mesh* out) {
  if (!path || !out) return fail(nullptr, GCFD_ERR_ARG, "null argument");
  MeshFile m;
  const std::string msg = read_mesh_file(path, &m);
  if (!msg.empty()) return fail(nullptr, GCFD_ERR_ARG, msg);
  auto copy = [](const auto& v) {
    using T = typename std::decay_t<decltype(v)>::value_type;
    T* p = new T[std::max<size_t>(v.size(), 1)];
    std::copy(v.begin(), v.end(), p);
    return p;
  };
  out->nverts = static_cast<int32_t>(m.vx.size());
  out->vx = copy(m.vx);
  out->vy = copy(m.vy);
  out->K = static_cast<int32_t>(m.etov.size() / 3);
  out->etov = copy(m.etov);
  out->nbc = static_cast<int32_t>(m.bc_flag.size());
  out->bc_v1 = copy(m.bc_v1);
  out->bc_v2 = copy(m.bc_v2);
  out->bc_flag = copy(m.bc_flag);
  return GCFD_OK;
}

void gcfd_free_mesh(gcfd_mesh* m) {
  if (!m) return;
  delete[] m->vx;
  delete[] m->vy;
  delete[] m->etov;
  delete[] m->bc_v1;
  delete[] m->bc_v2;
  delete[] m->bc_flag;
  *m = gcfd_mesh{};
}

const char* gcfd_last_error(const gcfd_ctx* ctx) {
  return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

int gcfd_dims(const gcfd_ctx* c, int32_t* K, int32_t* Np, int32_t* NpEdge, int32_t* NpFlux,
              int32_t* nEdges) {
  if (!c) return GCFD_ERR_ARG;
  if (K) *K = c->K;
  if (Np) *Np = c->Np;
  if (NpEdge) *NpEdge = c->NE;
  if (NpFlux) *NpFlux = c->NF;
  if (nEdges) *nEdges = c->nEdges;
  return GCFD_OK;
}

int gcfd_set_state(gcfd_ctx* c, int32_t nshards, const int32_t* Kmax, const double* const* Q) {
  if (!c || !Q) return c ? fail(c, GCFD_ERR_ARG, "null state") : GCFD_ERR_ARG;
  int rc = check_shards(c, nshards, Kmax);
  if (rc) return rc;
  if (c->fp32) {
    if ((rc = set_state_overlapped(c, nshards, Kmax, Q))) return rc;
  } else {
    if ((rc = copy_shards(c, c->Q[0], nshards, Kmax, Q, true, nullptr))) return rc;
    c->dirty = true;
    c->fp64Stale = false;
  }
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  return GCFD_OK;
}

int gcfd_get_state(gcfd_ctx* c, int32_t nshards, const int32_t* Kmax, double* const* Q) {
  if (!c || !Q) return c ? fail(c, GCFD_ERR_ARG, "null state") : GCFD_ERR_ARG;
  int rc = check_shards(c, nshards, Kmax);
  if (rc) return rc;
  if (c->fp32 && c->fp64Stale) {
    if ((rc = get_state_overlapped(c, nshards, Kmax, Q))) return rc;
  } else {
    if ((rc = sync_fp64_state(c))) return rc;
    if ((rc = copy_shards(c, c->Q[0], nshards, Kmax, nullptr, false, Q))) return rc;
  }
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  return GCFD_OK;
}

int gcfd_set_state_device(gcfd_ctx* c, const double* dQ) {
  if (!c || !dQ) return c ? fail(c, GCFD_ERR_ARG, "null state") : GCFD_ERR_ARG;
  GCFD_CUDA(c, cudaMemcpyAsync(c->Q[0], dQ, sizeof(double) * 4 * c->Np * static_cast<size_t>(c->K),
                               cudaMemcpyDeviceToDevice, c->stream));
  c->dirty = true;
  c->fp64Stale = false;
  return GCFD_OK;
}

int gcfd_get_state_device(gcfd_ctx* c, double* dQ) {
  if (!c || !dQ) return c ? fail(c, GCFD_ERR_ARG, "null state") : GCFD_ERR_ARG;
  int rc = sync_fp64_state(c);
  if (rc) return rc;
  GCFD_CUDA(c, cudaMemcpyAsync(dQ, c->Q[0], sizeof(double) * 4 * c->Np * static_cast<size_t>(c->K),
                               cudaMemcpyDeviceToDevice, c->stream));
  return GCFD_OK;
}

int gcfd_set_time(gcfd_ctx* c, double time) {
  if (!c) return GCFD_ERR_ARG;
  GCFD_CUDA(c, cudaMemcpyAsync(&c->sc->time, &time, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  return GCFD_OK;
}

int gcfd_get_time(gcfd_ctx* c, double* time, int32_t* steps) {
  if (!c) return GCFD_ERR_ARG;
  Scalars h;
  GCFD_CUDA(c, cudaMemcpyAsync(&h, c->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, c->stream));
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  if (time) *time = h.time;
  if (steps) *steps = h.steps;
  return GCFD_OK;
}

int gcfd_rhs(gcfd_ctx* c, double time, int32_t nshards, const int32_t* Kmax, const double* const* Q,
             double* const* RHS) {
  if (!c || !Q || !RHS) return c ? fail(c, GCFD_ERR_ARG, "null state") : GCFD_ERR_ARG;
  int rc = check_shards(c, nshards, Kmax);
  if (rc) return rc;
  if ((rc = sync_fp64_state(c))) return rc;  // the RHS reuses the stage-0 buffers
  if ((rc = copy_shards(c, c->Qtmp, nshards, Kmax, Q, true, nullptr))) return rc;
  GCFD_CUDA(c, cudaMemcpyAsync(&c->sc->rhs_time, &time, sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
  Ops o;
  select_ops(c->N, c->fp32, &o);
  o.rhs(c);
  c->dirty = true;  // the mixed path's stage-0 buffers now hold the RHS input
  GCFD_CUDA(c, cudaGetLastError());
  if ((rc = copy_shards(c, c->rhsOut, nshards, Kmax, nullptr, false, RHS))) return rc;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  return GCFD_OK;
}

static double decode_order_key(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  double d;
  std::memcpy(&d, &b, sizeof(d));
  return d;
}

int gcfd_step(gcfd_ctx* c, int32_t nsteps, double* time, double* dt_last, double* resid_max4,
              double* resid_absmax4, double* resid_rms4) {
  if (!c) return GCFD_ERR_ARG;
  if (nsteps < 0) return fail(c, GCFD_ERR_ARG, "nsteps must be >= 0");
  int rc = prepare_if_dirty(c);
  if (rc) return rc;
  for (int i = 0; i < nsteps; ++i) GCFD_CUDA(c, cudaGraphLaunch(c->graphExec, c->stream));
  if (nsteps > 0 && c->fp32) c->fp64Stale = true;
  Scalars h;
  GCFD_CUDA(c, cudaMemcpyAsync(&h, c->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, c->stream));
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  if (time) *time = h.time;
  if (dt_last) *dt_last = h.dt[4];
  bool finite = true;
  const double cnt = static_cast<double>(c->Np) * c->K;
  for (int n = 0; n < 4; ++n) {
    double am;
    std::memcpy(&am, &h.rabs[n], sizeof(am));
    const double mx = decode_order_key(h.rmax[n]);
    const double rms = std::sqrt(h.rsum2[n] / cnt);
    if (resid_max4) resid_max4[n] = mx;
    if (resid_absmax4) resid_absmax4[n] = am;
    if (resid_rms4) resid_rms4[n] = rms;
    if (nsteps > 0 && !(std::isfinite(am) && std::isfinite(rms))) finite = false;
  }
  if (h.errFlags & 2u)
    return fail(c, GCFD_ERR_CUDA, "stage kernel: dynamic shared memory is not 128-byte aligned");
  if (h.errFlags)
    return fail(c, GCFD_ERR_TIMEOUT,
                (h.errFlags & 4u) ? "a TMA copy of the stage kernel did not complete within its wait bound"
                                  : "a tensor-core completion wait ran out of its iteration bound");
  if (!finite) return fail(c, GCFD_ERR_NAN, "non-finite RK increment (solution diverged)");
  return GCFD_OK;
}

int gcfd_enqueue_steps(gcfd_ctx* c, int32_t nsteps) {
  if (!c) return GCFD_ERR_ARG;
  if (nsteps < 0) return fail(c, GCFD_ERR_ARG, "nsteps must be >= 0");
  int rc = prepare_if_dirty(c);
  if (rc) return rc;
  for (int i = 0; i < nsteps; ++i) GCFD_CUDA(c, cudaGraphLaunch(c->graphExec, c->stream));
  if (nsteps > 0 && c->fp32) c->fp64Stale = true;
  return GCFD_OK;
}

int gcfd_get_stream(gcfd_ctx* c, void** stream) {
  if (!c || !stream) return GCFD_ERR_ARG;
  *stream = static_cast<void*>(c->stream);
  return GCFD_OK;
}

int gcfd_set_option(gcfd_ctx* c, int32_t option, int32_t value) {
  if (!c) return GCFD_ERR_ARG;
  if (option != GCFD_OPT_STAGE_PIPELINE) return fail(c, GCFD_ERR_ARG, "unknown option");
  if (value != 0 && value != 1) return fail(c, GCFD_ERR_ARG, "GCFD_OPT_STAGE_PIPELINE takes 0 or 1");
  if (c->pipeOn == (value == 1)) return GCFD_OK;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  c->pipeOn = (value == 1);
  if (c->graphExec) GCFD_CUDA(c, cudaGraphExecDestroy(c->graphExec));
  if (c->graph) GCFD_CUDA(c, cudaGraphDestroy(c->graph));
  c->graphExec = nullptr;
  c->graph = nullptr;
  return capture_graph(c);
}

int gcfd_get_option(const gcfd_ctx* c, int32_t option, int32_t* value) {
  if (!c || !value) return GCFD_ERR_ARG;
  if (option != GCFD_OPT_STAGE_PIPELINE) return GCFD_ERR_ARG;
  *value = (c->fp32 && c->pipe && c->pipeOn) ? 1 : 0;
  return GCFD_OK;
}

int gcfd_profile_step(gcfd_ctx* c, double* kernel_ms4, int32_t* launches4) {
  if (!c || !kernel_ms4 || !launches4) return GCFD_ERR_ARG;
  double ms[4] = {0, 0, 0, 0};
  int l[4] = {0, 0, 0, 0};
  int rc = sync_fp64_state(c);
  if (rc) return rc;
  Ops o;
  select_ops(c->N, c->fp32, &o);
  o.step(c, c->ev, ms, l);
  c->dirty = false;
  if (c->fp32) c->fp64Stale = true;
  GCFD_CUDA(c, cudaGetLastError());
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int i = 0; i < 4; ++i) {
    kernel_ms4[i] = ms[i];
    launches4[i] = l[i];
  }
  return GCFD_OK;
}

int gcfd_host_operator(int32_t N, int32_t which, double* out, int32_t* rows, int32_t* cols) {
  DFRElement e;
  try {
    e = build_dfr_element(N);
  } catch (const std::exception& ex) {
    g_create_error = ex.what();
    return GCFD_ERR_UNSUPPORTED;
  }
  const DMat* m = nullptr;
  DMat tmp;
  switch (which) {
    case 0: m = &e.FluxEdgeInterp; break;
    case 1: m = &e.DivInt; break;
    case 2: m = &e.Div; break;
    case 3: m = &e.V; break;
    case 4:
      tmp = DMat(e.Np, 2);
      for (int i = 0; i < e.Np; ++i) { tmp(i, 0) = e.r[i]; tmp(i, 1) = e.s[i]; }
      m = &tmp;
      break;
    case 5:
      tmp = DMat(e.NpFlux, 2);
      for (int i = 0; i < e.NpFlux; ++i) { tmp(i, 0) = e.rFlux[i]; tmp(i, 1) = e.sFlux[i]; }
      m = &tmp;
      break;
    default: return GCFD_ERR_ARG;
  }
  if (rows) *rows = m->rows;
  if (cols) *cols = m->cols;
  if (out) std::memcpy(out, m->v.data(), m->v.size() * sizeof(double));
  return GCFD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Adjoint entry points.
namespace {

int adj_check(gcfd_ctx* c) {
  if (c->fp32) return fail(c, GCFD_ERR_UNSUPPORTED, "the adjoint runs on the FP64 path only");
  return GCFD_OK;
}

// Interpolatory weights of the NpEdge edge flux points on [-1, 1], normalised
// to sum to one (exact for polynomials of degree NpEdge - 1 along the edge).
std::vector<double> edge_weights(const gcfd_ctx* c) {
  const int NE = c->NE, off = 2 * c->Np;
  std::vector<double> t(NE), A(static_cast<size_t>(NE) * NE), w(NE);
  for (int p = 0; p < NE; ++p) t[p] = c->el.rFlux[off + p];
  for (int m = 0; m < NE; ++m) {
    for (int p = 0; p < NE; ++p) A[m * NE + p] = std::pow(t[p], m);
    w[m] = (m % 2 == 0) ? 1.0 / (m + 1) : 0.0;
  }
  // Gaussian elimination with partial pivoting
  for (int col = 0; col < NE; ++col) {
    int piv = col;
    for (int r = col + 1; r < NE; ++r)
      if (std::fabs(A[r * NE + col]) > std::fabs(A[piv * NE + col])) piv = r;
    if (piv != col) {
      for (int j = 0; j < NE; ++j) std::swap(A[col * NE + j], A[piv * NE + j]);
      std::swap(w[col], w[piv]);
    }
    for (int r = col + 1; r < NE; ++r) {
      const double f = A[r * NE + col] / A[col * NE + col];
      for (int j = col; j < NE; ++j) A[r * NE + j] -= f * A[col * NE + j];
      w[r] -= f * w[col];
    }
  }
  for (int r = NE - 1; r >= 0; --r) {
    double s = w[r];
    for (int j = r + 1; j < NE; ++j) s -= A[r * NE + j] * w[j];
    w[r] = s / A[r * NE + r];
  }
  return w;
}

// Buffers of gcfd_functional (any path): the state adjoint, face adjoints,
// scalars, solution-point coordinates, edge weights and FP64 faces.
int func_init(gcfd_ctx* c) {
  if (c->adjS) return GCFD_OK;
  const size_t S = static_cast<size_t>(4) * c->Np * c->K;
  const size_t F = static_cast<size_t>(4) * 3 * c->NE * c->K;
  int rc;
  if (!c->QF) {  // the mixed path keeps its faces elsewhere
    double* qf = nullptr;
    if ((rc = dalloc(c, &qf, F))) return rc;
    c->QF = qf;
  }
  if ((rc = dalloc(c, &c->Qb[0], S))) return rc;
  if ((rc = dalloc(c, &c->QFb, F))) return rc;
  if ((rc = upload(c, &c->dXs, c->geo.xSol))) return rc;
  if ((rc = upload(c, &c->dYs, c->geo.ySol))) return rc;
  if ((rc = upload(c, &c->edgeW, edge_weights(c)))) return rc;
  if ((rc = dalloc(c, &c->adjS, 16))) return rc;
  GCFD_CUDA(c, cudaMemsetAsync(c->adjS, 0, sizeof(double) * 16, c->stream));
  return GCFD_OK;
}

int adj_init(gcfd_ctx* c) {
  if (c->adjReady) return GCFD_OK;
  int rc = adj_check(c);
  if (rc) return rc;
  if ((rc = func_init(c))) return rc;
  const size_t S = static_cast<size_t>(4) * c->Np * c->K;
  const size_t F = static_cast<size_t>(4) * 3 * c->NE * c->K;
  const int nE = c->nInt + c->nBC;
  for (int s = 0; s < 5; ++s) {
    if ((rc = dalloc(c, &c->tapeRHS[s], S))) return rc;
    if ((rc = dalloc(c, &c->tapeES[s], static_cast<size_t>(nE)))) return rc;
    if ((rc = dalloc(c, &c->tapeDT[s], static_cast<size_t>(c->K)))) return rc;
    if ((rc = dalloc(c, &c->tapeQF[s], F))) return rc;
    if (s > 0 && (rc = dalloc(c, &c->Qb[s], S))) return rc;
  }
  if ((rc = dalloc(c, &c->tapeSc0, 1))) return rc;
  if ((rc = dalloc(c, &c->tapeSc, 1))) return rc;
  if ((rc = dalloc(c, &c->Qbf, S))) return rc;
  if ((rc = dalloc(c, &c->Rb3, S))) return rc;
  if ((rc = dalloc(c, &c->FEb, F))) return rc;
  if ((rc = dalloc(c, &c->carry, static_cast<size_t>(c->K)))) return rc;
  if ((rc = dalloc(c, &c->dtOwnK, static_cast<size_t>(c->K)))) return rc;
  if ((rc = dalloc(c, &c->esBar, static_cast<size_t>(nE)))) return rc;
  if ((rc = dalloc(c, &c->argEdge, 8))) return rc;
  if (c->diss) {
    const size_t NR = static_cast<size_t>(c->Np) + 3 * c->NE;
    if ((rc = dalloc(c, &c->tapeQ2pre, S))) return rc;
    for (int s = 0; s < 5; ++s) {
      if ((rc = dalloc(c, &c->tapeDTV[s], static_cast<size_t>(c->K)))) return rc;
      if ((rc = dalloc(c, &c->tapeVS[s], static_cast<size_t>(nE)))) return rc;
      if ((rc = dalloc(c, &c->tapeRHSpre[s], S))) return rc;
    }
    for (double** p : {&c->sigE, &c->epsE, &c->SeE, &c->alphaBar, &c->carryV})
      if ((rc = dalloc(c, p, static_cast<size_t>(c->K)))) return rc;
    if ((rc = dalloc(c, &c->sigVbar, static_cast<size_t>(c->nverts)))) return rc;
    if ((rc = dalloc(c, &c->epsVbar, static_cast<size_t>(c->nverts)))) return rc;
    if ((rc = dalloc(c, &c->VFbar, static_cast<size_t>(nE) * 4 * c->NE))) return rc;
    if ((rc = dalloc(c, &c->DissXbar, 4 * NR * c->K))) return rc;
    if ((rc = dalloc(c, &c->DissYbar, 4 * NR * c->K))) return rc;
    if ((rc = dalloc(c, &c->RbE, S))) return rc;
    if ((rc = dalloc(c, &c->vsBar, static_cast<size_t>(nE)))) return rc;
    if ((rc = dalloc(c, &c->sigArg, static_cast<size_t>(c->nverts)))) return rc;
    if ((rc = dalloc(c, &c->epsArg, static_cast<size_t>(c->nverts)))) return rc;
    if ((rc = dalloc(c, &c->argVisc, 8))) return rc;
  }
  c->adjReady = true;
  return GCFD_OK;
}

int win_alloc(gcfd_ctx* c, double** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(double) > 0 ? count * sizeof(double) : 16);
  if (e != cudaSuccess)
    return fail(c, e == cudaErrorMemoryAllocation ? GCFD_ERR_OOM : GCFD_ERR_CUDA,
                std::string("cudaMalloc (adjoint window): ") + cudaGetErrorString(e));
  c->winAllocs.push_back(q);
  *p = static_cast<double*>(q);
  return GCFD_OK;
}

}  // namespace

extern "C" {

int gcfd_functional(gcfd_ctx* c, int32_t kind, double* J, int32_t nshards, const int32_t* Kmax,
                    double* const* Qbar, double* tbar) {
  if (!c || !J) return c ? fail(c, GCFD_ERR_ARG, "null J") : GCFD_ERR_ARG;
  if (kind < GCFD_FUNC_WALL_FORCE_X || kind > GCFD_FUNC_VORTEX_ERROR)
    return fail(c, GCFD_ERR_ARG, "unknown functional kind");
  int rc = func_init(c);
  if (rc) return rc;
  if (Qbar && (rc = check_shards(c, nshards, Kmax))) return rc;
  if ((rc = sync_fp64_state(c))) return rc;
  AdjOps o;
  select_adj_ops(c->N, &o);
  GCFD_CUDA(c, cudaMemsetAsync(c->adjS + 9, 0, sizeof(double) * 3, c->stream));
  o.functional(c, kind);
  GCFD_CUDA(c, cudaGetLastError());
  double h[3];
  GCFD_CUDA(c, cudaMemcpyAsync(h, c->adjS + 9, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if (Qbar && (rc = copy_shards(c, c->Qb[0], nshards, Kmax, nullptr, false, Qbar))) return rc;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  *J = h[2];
  if (tbar) *tbar = h[0];
  return GCFD_OK;
}

int gcfd_rhs_vjp(gcfd_ctx* c, double time, int32_t nshards, const int32_t* Kmax, const double* const* Q,
                 const double* const* RHSbar, double* const* Qbar, double* qinf_bar4, double* time_bar) {
  if (!c || !Q || !RHSbar || !Qbar) return c ? fail(c, GCFD_ERR_ARG, "null state") : GCFD_ERR_ARG;
  int rc = adj_init(c);
  if (rc) return rc;
  if ((rc = check_shards(c, nshards, Kmax))) return rc;
  if ((rc = copy_shards(c, c->Qtmp, nshards, Kmax, Q, true, nullptr))) return rc;
  if ((rc = copy_shards(c, c->Qbf, nshards, Kmax, RHSbar, true, nullptr))) return rc;
  GCFD_CUDA(c, cudaMemcpyAsync(&c->sc->rhs_time, &time, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  GCFD_CUDA(c, cudaMemsetAsync(c->adjS + 5, 0, sizeof(double) * 5, c->stream));
  AdjOps o;
  select_adj_ops(c->N, &o);
  o.rhs_vjp(c);
  GCFD_CUDA(c, cudaGetLastError());
  double h[5];
  GCFD_CUDA(c, cudaMemcpyAsync(h, c->adjS + 5, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = copy_shards(c, c->Qb[0], nshards, Kmax, nullptr, false, Qbar))) return rc;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  if (qinf_bar4)
    for (int i = 0; i < 4; ++i) qinf_bar4[i] = h[i];
  if (time_bar) *time_bar = h[4];
  return GCFD_OK;
}

int gcfd_record_steps(gcfd_ctx* c, int32_t nsteps, int32_t every, double* time, double* dt_last) {
  if (!c) return GCFD_ERR_ARG;
  if (nsteps < 1 || every < 1) return fail(c, GCFD_ERR_ARG, "nsteps and checkpoint_every must be >= 1");
  int rc = adj_init(c);
  if (rc) return rc;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  for (void* p : c->winAllocs) cudaFree(p);
  c->winAllocs.clear();
  c->winSteps = 0;
  const size_t S = static_cast<size_t>(4) * c->Np * c->K;
  const int nck = (nsteps + every - 1) / every;
  if ((rc = win_alloc(c, &c->ckpt, S * nck))) return rc;
  if ((rc = win_alloc(c, &c->ckptT, static_cast<size_t>(nck)))) return rc;
  if ((rc = win_alloc(c, &c->segQ, S * std::min(every, nsteps)))) return rc;
  if ((rc = win_alloc(c, &c->segT, static_cast<size_t>(std::min(every, nsteps))))) return rc;
  if ((rc = win_alloc(c, &c->endQ, S))) return rc;
  const size_t KV = c->diss ? static_cast<size_t>(c->K) : 0;  // DTVisc persists across steps
  if (c->diss) {
    if ((rc = win_alloc(c, &c->ckptV, KV * nck))) return rc;
    if ((rc = win_alloc(c, &c->segV, KV * std::min(every, nsteps)))) return rc;
    if ((rc = win_alloc(c, &c->endV, KV))) return rc;
  }
  double* sc = nullptr;
  if ((rc = win_alloc(c, &sc, (sizeof(Scalars) + 7) / 8))) return rc;
  c->endSc = reinterpret_cast<Scalars*>(sc);
  for (int n = 0; n < nsteps; ++n) {
    if (n % every == 0) {
      const int j = n / every;
      GCFD_CUDA(c, cudaMemcpyAsync(c->ckpt + S * j, c->Q[0], S * sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      GCFD_CUDA(c, cudaMemcpyAsync(c->ckptT + j, &c->sc->time, sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      if (c->diss)
        GCFD_CUDA(c, cudaMemcpyAsync(c->ckptV + KV * j, c->DTVisc, KV * sizeof(double), cudaMemcpyDeviceToDevice,
                                     c->stream));
    }
    GCFD_CUDA(c, cudaGraphLaunch(c->graphExec, c->stream));
  }
  GCFD_CUDA(c, cudaMemcpyAsync(c->endQ, c->Q[0], S * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  if (c->diss)
    GCFD_CUDA(c, cudaMemcpyAsync(c->endV, c->DTVisc, KV * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  GCFD_CUDA(c, cudaMemcpyAsync(c->endSc, c->sc, sizeof(Scalars), cudaMemcpyDeviceToDevice, c->stream));
  Scalars h;
  GCFD_CUDA(c, cudaMemcpyAsync(&h, c->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, c->stream));
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  c->winSteps = nsteps;
  c->winEvery = every;
  if (time) *time = h.time;
  if (dt_last) *dt_last = h.dt[4];
  return GCFD_OK;
}

int gcfd_step_vjp(gcfd_ctx* c, int32_t nshards, const int32_t* Kmax, const double* const* Qfinal_bar,
                  double tfinal_bar, double* const* Q0_bar, double* qinf_bar4, double* t0_bar) {
  if (!c || !Qfinal_bar || !Q0_bar) return c ? fail(c, GCFD_ERR_ARG, "null adjoint") : GCFD_ERR_ARG;
  int rc = adj_check(c);
  if (rc) return rc;
  if (c->winSteps < 1) return fail(c, GCFD_ERR_ARG, "no recorded window: call gcfd_record_steps first");
  if ((rc = check_shards(c, nshards, Kmax))) return rc;
  AdjOps o;
  select_adj_ops(c->N, &o);
  const size_t S = static_cast<size_t>(4) * c->Np * c->K;
  const size_t SB = S * sizeof(double);
  if ((rc = copy_shards(c, c->Qbf, nshards, Kmax, Qfinal_bar, true, nullptr))) return rc;
  GCFD_CUDA(c, cudaMemsetAsync(c->adjS, 0, sizeof(double) * 12, c->stream));
  GCFD_CUDA(c, cudaMemcpyAsync(c->adjS + 10, &tfinal_bar, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  const size_t KV = c->diss ? static_cast<size_t>(c->K) : 0;
  if (c->diss) GCFD_CUDA(c, cudaMemsetAsync(c->carryV, 0, KV * sizeof(double), c->stream));
  const int every = c->winEvery, nsteps = c->winSteps;
  const int nseg = (nsteps + every - 1) / every;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int n0 = seg * every, m = std::min(every, nsteps - n0);
    GCFD_CUDA(c, cudaMemcpyAsync(c->Q[0], c->ckpt + S * seg, SB, cudaMemcpyDeviceToDevice, c->stream));
    GCFD_CUDA(c, cudaMemcpyAsync(&c->sc->time, c->ckptT + seg, sizeof(double), cudaMemcpyDeviceToDevice,
                                 c->stream));
    if (c->diss)
      GCFD_CUDA(c, cudaMemcpyAsync(c->DTVisc, c->ckptV + KV * seg, KV * sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
    for (int i = 0; i < m; ++i) {
      GCFD_CUDA(c, cudaMemcpyAsync(c->segQ + S * i, c->Q[0], SB, cudaMemcpyDeviceToDevice, c->stream));
      GCFD_CUDA(c, cudaMemcpyAsync(c->segT + i, &c->sc->time, sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      if (c->diss)
        GCFD_CUDA(c, cudaMemcpyAsync(c->segV + KV * i, c->DTVisc, KV * sizeof(double), cudaMemcpyDeviceToDevice,
                                     c->stream));
      if (i + 1 < m) GCFD_CUDA(c, cudaGraphLaunch(c->graphExec, c->stream));
    }
    for (int i = m - 1; i >= 0; --i) {
      GCFD_CUDA(c, cudaMemcpyAsync(c->Q[0], c->segQ + S * i, SB, cudaMemcpyDeviceToDevice, c->stream));
      GCFD_CUDA(c, cudaMemcpyAsync(&c->sc->time, c->segT + i, sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      if (c->diss)
        GCFD_CUDA(c, cudaMemcpyAsync(c->DTVisc, c->segV + KV * i, KV * sizeof(double), cudaMemcpyDeviceToDevice,
                                     c->stream));
      o.reverse_step(c, c->segQ + S * i);
      GCFD_CUDA(c, cudaGetLastError());
    }
  }
  double h[6];
  GCFD_CUDA(c, cudaMemcpyAsync(h, c->adjS + 5, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = copy_shards(c, c->Qbf, nshards, Kmax, nullptr, false, Q0_bar))) return rc;
  // back to the window's end
  GCFD_CUDA(c, cudaMemcpyAsync(c->Q[0], c->endQ, SB, cudaMemcpyDeviceToDevice, c->stream));
  GCFD_CUDA(c, cudaMemcpyAsync(c->sc, c->endSc, sizeof(Scalars), cudaMemcpyDeviceToDevice, c->stream));
  if (c->diss)
    GCFD_CUDA(c, cudaMemcpyAsync(c->DTVisc, c->endV, KV * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  if (qinf_bar4)
    for (int i = 0; i < 4; ++i) qinf_bar4[i] = h[i];
  if (t0_bar) *t0_bar = h[5];
  return GCFD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Residual norms without allocation (gcfd_residual_norms_static).
//
// The per-block partials live in one file-scope device array of fixed size;
// the first call on each device looks up its address with
// cudaGetSymbolAddress (with that device current) and caches it.  Pass 1:
// block b reduces points [b*kResidChunk, (b+1)*kResidChunk) of each variable
// into 12 slots (order key of the signed max, bit pattern of max |R|, sum of
// squares).  Pass 2: one block reduces the nblk partials in a fixed order and
// writes 12 result slots, copied to the host.  The sums are therefore
// deterministic run to run.  No slot needs clearing: pass 2 reads only slots
// that pass 1 of the same call wrote.
namespace {

constexpr int kResidThreads = 256;
constexpr int kResidChunk = 2048;                // points per block and variable
constexpr int kResidMaxBlocks = 16384;           // => GCFD_RESID_STATIC_MAX_POINTS
constexpr int kResidResult = kResidMaxBlocks * 12;
static_assert(static_cast<long long>(kResidChunk) * kResidMaxBlocks == GCFD_RESID_STATIC_MAX_POINTS,
              "the header's limit must match the scratch layout");

__device__ __align__(256) unsigned long long g_resid_scratch[kResidResult + 12];

constexpr int kMaxDevices = 64;
std::mutex g_resid_mutex;
unsigned long long* g_resid_ptr[kMaxDevices] = {};

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

// Device address of the scratch array for the current device, looked up once.
int resid_scratch(unsigned long long** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(nullptr, GCFD_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(nullptr, GCFD_ERR_UNSUPPORTED, "device ordinal beyond the residual scratch table");
  std::lock_guard<std::mutex> lock(g_resid_mutex);
  if (!g_resid_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_resid_scratch);
    if (e != cudaSuccess || !p)
      return fail(nullptr, GCFD_ERR_CUDA,
                  std::string("cudaGetSymbolAddress(residual scratch): ") + cudaGetErrorString(e));
    g_resid_ptr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_resid_ptr[dev];
  return GCFD_OK;
}

}  // namespace

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
