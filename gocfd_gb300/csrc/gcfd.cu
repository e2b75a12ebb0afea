// libgcfd: context creation and state transfer, the per-step CUDA graph and
// the forward entry points of the C ABI declared in include/gcfd.h.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "gcfd_ctx.hpp"

namespace gcfd_host {

namespace {
thread_local std::string g_create_error;
}  // namespace

int fail(gcfd_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_error = msg;
  return code;
}

const OrderOps* order_ops(int N) {
  switch (N) {
    case 0: return order_ops_0();
    case 1: return order_ops_1();
    case 2: return order_ops_2();
    case 3: return order_ops_3();
    case 4: return order_ops_4();
    default: return nullptr;
  }
}

const AdjOps* adj_ops(int N) {
  switch (N) {
    case 0: return adj_ops_0();
    case 1: return adj_ops_1();
    case 2: return adj_ops_2();
    case 3: return adj_ops_3();
    case 4: return adj_ops_4();
    default: return nullptr;
  }
}

namespace {

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

// Mixed path: rebuild the FP64 state Q[0] from the compensated pair.
void to_fp64_range(gcfd_ctx* c, int k0, int k1) {
  if (k1 <= k0) return;
  const size_t n = static_cast<size_t>(4) * c->Np * (k1 - k0);
  k_mixed_to_fp64<<<static_cast<int>(std::min<size_t>((n + 255) / 256, 152 * 16)), 256, 0, c->stream>>>(
      c->Qhi, c->Qlo, c->Q[0], c->K, 4 * c->Np, k0, k1);
}

}  // namespace

int sync_fp64_state(gcfd_ctx* c) {
  if (!c->fp32 || !c->fp64Stale) return GCFD_OK;
  to_fp64_range(c, 0, c->K);
  GCFD_CUDA(c, cudaGetLastError());
  c->fp64Stale = false;
  return GCFD_OK;
}

namespace {

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



// Mixed path: the state moves in kStateChunks element ranges, and each range's
// conversion (hi/lo split, dQ0, faces, reference states on the way in; hi + lo
// to FP64 on the way out) runs on the compute stream while the next range's copy
// is in flight on the second stream.
constexpr int kStateChunks = 8;

int set_state_overlapped(gcfd_ctx* c, int nshards, const int32_t* Kmax, const double* const* Q) {
  const Ops o = ctx_ops(c);
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
  const Ops o = ctx_ops(c);
  GCFD_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  o.step(c, nullptr, nullptr, nullptr);
  cudaGraph_t g = nullptr;
  GCFD_CUDA(c, cudaStreamEndCapture(c->stream, &g));
  c->graph = g;
  GCFD_CUDA(c, cudaGraphInstantiate(&c->graphExec, g, 0));
  return GCFD_OK;
}

}  // namespace

int prepare_if_dirty(gcfd_ctx* c) {
  if (!c->dirty) return GCFD_OK;
  const Ops o = ctx_ops(c);
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

namespace {

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
  std::vector<int> ev(static_cast<size_t>(3) * K);
  for (int k = 0; k < K; ++k)
    for (int v = 0; v < 3; ++v) ev[static_cast<size_t>(v) * K + k] = m->etov[3 * k + v];
  if ((rc = upload(c, &c->detov, ev))) return rc;
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
  if ((rc = dalloc(c, &c->P23, nS))) return rc;
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
  if ((rc = order_ops(c->N)->mixed_consts(c))) return rc;
  if ((rc = device_geometry_mixed(c))) return rc;
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
  return order_ops(c->N)->mixed_pipe(c);
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
  c->meshVX.assign(m->vx, m->vx + m->nverts);
  c->meshVY.assign(m->vy, m->vy + m->nverts);
  c->meshEToV.assign(m->etov, m->etov + 3 * static_cast<size_t>(m->K));

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
  std::vector<double> bx(static_cast<size_t>(std::max(c->nBC, 1)) * NE), by(bx.size());
  std::vector<int> elemEdge(static_cast<size_t>(3) * K);
  std::vector<int> pos(t.nEdges);
  for (int i = 0; i < c->nEdges; ++i) {
    const int en = order[i];
    pos[en] = i;
    kL[i] = t.kL[en];
    kR[i] = t.kR[en] >= 0 ? t.kR[en] : 0;
    eLR[i] = t.eL[en] | ((t.eR[en] >= 0 ? t.eR[en] : 0) << 2);
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

  GCFD_CUDA(c, cudaSetDevice(p.device));
  GCFD_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  const size_t nState = static_cast<size_t>(4) * Np * K;
  const size_t nFace = static_cast<size_t>(4) * 3 * NE * K;
  const size_t tsz = c->fp32 ? sizeof(float) : sizeof(double);
  int rc;
  // geometry and per-edge tables on the device (gcfd_geometry.cu)
  if ((rc = device_geometry(c, m, kL, kR, eLR))) return rc;
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
  if ((rc = upload(c, &c->bcFlag, flag))) return rc;
  if ((rc = upload(c, &c->elemEdge, elemEdge))) return rc;
  if ((rc = upload(c, &c->bx, bx))) return rc;
  if ((rc = upload(c, &c->by, by))) return rc;
  if ((rc = dalloc(c, &c->edgeSpeed, static_cast<size_t>(c->nEdges)))) return rc;
  if ((rc = dalloc(c, &c->DT, static_cast<size_t>(K)))) return rc;
  if ((rc = dalloc(c, &c->sc, 1))) return rc;
  GCFD_CUDA(c, cudaMemset(c->sc, 0, sizeof(Scalars)));
  const size_t nunit = static_cast<size_t>((K + 31) / 32 + 8);
  if ((rc = dalloc(c, &c->rpart, 4 * (nunit + kResidBlocks)))) return rc;
  GCFD_CUDA(c, cudaMemset(c->rpart, 0, sizeof(double) * 4 * (nunit + kResidBlocks)));
  double* rp[2] = {c->rpart, c->rpart + 4 * nunit};
  GCFD_CUDA(c, cudaMemcpy(&c->sc->rpart, rp, sizeof(rp), cudaMemcpyHostToDevice));
  GCFD_CUDA(c, cudaMemset(c->DT, 0, sizeof(double) * K));
  GCFD_CUDA(c, cudaMemset(c->R, 0, sizeof(double) * nState));
  if ((rc = device_initial_state(c))) return rc;
  for (auto& e : c->ev) GCFD_CUDA(c, cudaEventCreate(&e));
  if ((rc = capture_graph(c))) return rc;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  return GCFD_OK;
}

}  // namespace
}  // namespace gcfd_host

using namespace gcfd_host;

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
  const Ops o = ctx_ops(c);
  o.rhs(c);
  c->dirty = true;  // the mixed path's stage-0 buffers now hold the RHS input
  GCFD_CUDA(c, cudaGetLastError());
  if ((rc = copy_shards(c, c->rhsOut, nshards, Kmax, nullptr, false, RHS))) return rc;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  return GCFD_OK;
}

}  // extern "C"

double gcfd_host::decode_order_key(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  double d;
  std::memcpy(&d, &b, sizeof(d));
  return d;
}

extern "C" {

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
  if (option == GCFD_OPT_WINDOW_TAPED) {
    *value = (c->winSteps > 0 && c->winTaped) ? 1 : 0;
    return GCFD_OK;
  }
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
  const Ops o = ctx_ops(c);
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
