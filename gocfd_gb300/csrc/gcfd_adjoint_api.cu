// libgcfd: the adjoint entry points of the C ABI (functionals, RHS and
// checkpointed-window vector-Jacobian products) declared in include/gcfd.h.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "gcfd_ctx.hpp"

namespace gcfd_host {
namespace {

// The mixed path's adjoint (FP32 reverse of the mixed forward) covers the
// Euler RHS and step without the artificial dissipation, with the FMA or
// tensor-core stage kernel.
int adj_check(gcfd_ctx* c) {
  if (c->fp32 && c->diss)
    return fail(c, GCFD_ERR_UNSUPPORTED, "the adjoint of the mixed path runs without the PerssonC0 dissipation");
  if (c->fp32 && c->pipe && c->pipeOn)
    return fail(c, GCFD_ERR_UNSUPPORTED, "the adjoint of the mixed path does not run with the pipelined stage kernel");
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
  if ((rc = device_solution_points(c, &c->dXs, &c->dYs))) return rc;
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
  if (c->fp32) {  // FP32 adjoint arrays; the stage increments are the forward's own
    for (int s = 0; s < 5; ++s) {
      if ((rc = dalloc(c, &c->tapeRHS32[s], S))) return rc;
      if ((rc = dalloc(c, &c->tapeES[s], static_cast<size_t>(nE)))) return rc;
      if ((rc = dalloc(c, &c->tapeDT[s], static_cast<size_t>(c->K)))) return rc;
      if ((rc = dalloc(c, &c->Qb32[s], S))) return rc;
    }
    if ((rc = dalloc(c, &c->Qbf32, S))) return rc;
    for (float** p : {&c->QF32, &c->QFb32, &c->FEb32})
      if ((rc = dalloc(c, p, F))) return rc;
    if ((rc = dalloc(c, &c->tapeSc0, 1))) return rc;
    if ((rc = dalloc(c, &c->tapeSc, 1))) return rc;
    if ((rc = dalloc(c, &c->Qbf, S))) return rc;  // FP64 staging of the caller's adjoints
    if ((rc = dalloc(c, &c->carry, static_cast<size_t>(c->K)))) return rc;
    if ((rc = dalloc(c, &c->dtOwnK, static_cast<size_t>(c->K)))) return rc;
    if ((rc = dalloc(c, &c->esBar, static_cast<size_t>(nE)))) return rc;
    if ((rc = dalloc(c, &c->argEdge, 8))) return rc;
    if ((rc = adj_ops(c->N)->mixed_consts(c))) return rc;
    c->adjReady = true;
    return GCFD_OK;
  }
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

// Device blocks of adjoint windows.  gcfd_record_steps hands the previous
// window's blocks to c->winPool, and each request of the new window takes a
// pooled block of the same size first: repeated windows of one shape (an
// optimisation loop) allocate nothing after the first.  A cudaMalloc that
// fails frees the pool and is tried once more; gcfd_destroy frees everything.
void release_pool(gcfd_ctx* c) {
  for (auto& b : c->winPool) cudaFree(b.first);
  c->winPool.clear();
}

void* win_block(gcfd_ctx* c, size_t bytes) {
  for (size_t i = 0; i < c->winPool.size(); ++i)
    if (c->winPool[i].second == bytes) {
      void* p = c->winPool[i].first;
      c->winPool.erase(c->winPool.begin() + static_cast<std::ptrdiff_t>(i));
      c->winAllocs.emplace_back(p, bytes);
      return p;
    }
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    release_pool(c);
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
  }
  c->winAllocs.emplace_back(p, bytes);
  return p;
}

// Frees blocks of the current window taken since its first `keep` blocks.
void drop_blocks(gcfd_ctx* c, size_t keep) {
  while (c->winAllocs.size() > keep) {
    cudaFree(c->winAllocs.back().first);
    c->winAllocs.pop_back();
  }
}

int win_alloc(gcfd_ctx* c, double** p, size_t count) {
  void* q = win_block(c, count * sizeof(double) > 0 ? count * sizeof(double) : 16);
  if (!q) return fail(c, GCFD_ERR_OOM, "cudaMalloc (adjoint window): out of memory");
  *p = static_cast<double*>(q);
  return GCFD_OK;
}

// Point the context's stage arrays and tape at segment-tape slot i.
void bind_slot(gcfd_ctx* c, int i) {
  const gcfd_ctx::TapeSlot& t = c->slots[i];
  if (c->fp32) {
    for (int s = 0; s < 5; ++s) {
      if (s > 0) c->Dk[s] = t.D[s];
      c->tapeRHS32[s] = t.rhs32[s];
      c->tapeES[s] = t.es[s];
      c->tapeDT[s] = t.dt[s];
    }
    c->tapeSc0 = t.sc0;
    c->tapeSc = t.sc;
    return;
  }
  for (int s = 0; s < 5; ++s) {
    if (s > 0) c->Q[s] = t.Q[s];
    c->tapeRHS[s] = t.rhs[s];
    c->tapeES[s] = t.es[s];
    c->tapeDT[s] = t.dt[s];
    c->tapeDTV[s] = t.dtv[s];
    c->tapeVS[s] = t.vs[s];
    c->tapeRHSpre[s] = t.rhspre[s];
  }
  c->tapeQ2pre = t.q2pre;
  c->tapeSc0 = t.sc0;
  c->tapeSc = t.sc;
}

// Slot 0 is the context's own stage arrays and tape; slots 1.. are allocated
// per window (they go with the window's allocations; withQ0: each also keeps
// its step's starting state, for a window taped while recording).  Returns
// false, with nothing kept, when they do not fit in device memory.
bool alloc_slots_mixed(gcfd_ctx* c, int nslots, bool withQ0);

bool alloc_slots(gcfd_ctx* c, int nslots, bool withQ0) {
  if (c->fp32) return alloc_slots_mixed(c, nslots, withQ0);
  c->slots.clear();
  gcfd_ctx::TapeSlot base{};
  for (int s = 0; s < 5; ++s) {
    base.Q[s] = c->Q[s];
    base.rhs[s] = c->tapeRHS[s];
    base.es[s] = c->tapeES[s];
    base.dt[s] = c->tapeDT[s];
    base.dtv[s] = c->tapeDTV[s];
    base.vs[s] = c->tapeVS[s];
    base.rhspre[s] = c->tapeRHSpre[s];
  }
  base.q2pre = c->tapeQ2pre;
  base.sc0 = c->tapeSc0;
  base.sc = c->tapeSc;
  c->slots.push_back(base);
  const size_t S = static_cast<size_t>(4) * c->Np * c->K, K = c->K, nE = c->nInt + c->nBC;
  const size_t per = 9 * S + 5 * (nE + K) + 2 * ((sizeof(Scalars) + 7) / 8) +
                     (c->diss ? S + 5 * (K + nE + S) : 0) + (withQ0 ? S : 0);
  const size_t keep = c->winAllocs.size();
  for (int i = 1; i < nslots; ++i) {
    void* p = win_block(c, per * sizeof(double));
    if (!p) {
      drop_blocks(c, keep);
      c->slots.resize(1);
      return false;
    }
    double* d = static_cast<double*>(p);
    gcfd_ctx::TapeSlot t{};
    auto take = [&](size_t n) {
      double* r = d;
      d += n;
      return r;
    };
    for (int s = 1; s < 5; ++s) t.Q[s] = take(S);
    for (int s = 0; s < 5; ++s) {
      t.rhs[s] = take(S);
      t.es[s] = take(nE);
      t.dt[s] = take(K);
    }
    t.sc0 = reinterpret_cast<Scalars*>(take((sizeof(Scalars) + 7) / 8));
    t.sc = reinterpret_cast<Scalars*>(take((sizeof(Scalars) + 7) / 8));
    if (withQ0) t.q0 = take(S);
    if (c->diss) {
      t.q2pre = take(S);
      for (int s = 0; s < 5; ++s) {
        t.dtv[s] = take(K);
        t.vs[s] = take(nE);
        t.rhspre[s] = take(S);
      }
    }
    c->slots.push_back(t);
  }
  return true;
}

// The mixed path's slots: the stage increments D1..D4 and stage RHS in FP32,
// edge speeds, local dt and scalars as on the FP64 path.
bool alloc_slots_mixed(gcfd_ctx* c, int nslots, bool withQ0) {
  c->slots.clear();
  gcfd_ctx::TapeSlot base{};
  for (int s = 0; s < 5; ++s) {
    base.D[s] = c->Dk[s];
    base.rhs32[s] = c->tapeRHS32[s];
    base.es[s] = c->tapeES[s];
    base.dt[s] = c->tapeDT[s];
  }
  base.sc0 = c->tapeSc0;
  base.sc = c->tapeSc;
  c->slots.push_back(base);
  const size_t S = static_cast<size_t>(4) * c->Np * c->K, K = c->K, nE = c->nInt + c->nBC;
  auto rup = [](size_t b) { return (b + 255) & ~static_cast<size_t>(255); };
  const size_t bS = rup(S * sizeof(float)), bE = rup(nE * sizeof(double)), bK = rup(K * sizeof(double));
  const size_t bSc = rup(sizeof(Scalars));
  const size_t per = 9 * bS + 5 * (bE + bK) + 2 * bSc + (withQ0 ? bS : 0);
  const size_t keep = c->winAllocs.size();
  for (int i = 1; i < nslots; ++i) {
    void* p = win_block(c, per);
    if (!p) {
      drop_blocks(c, keep);
      c->slots.resize(1);
      return false;
    }
    char* d = static_cast<char*>(p);
    auto take = [&](size_t n) {
      char* r = d;
      d += n;
      return r;
    };
    gcfd_ctx::TapeSlot t{};
    for (int s = 1; s < 5; ++s) t.D[s] = reinterpret_cast<float*>(take(bS));
    for (int s = 0; s < 5; ++s) {
      t.rhs32[s] = reinterpret_cast<float*>(take(bS));
      t.es[s] = reinterpret_cast<double*>(take(bE));
      t.dt[s] = reinterpret_cast<double*>(take(bK));
    }
    t.sc0 = reinterpret_cast<Scalars*>(take(bSc));
    t.sc = reinterpret_cast<Scalars*>(take(bSc));
    if (withQ0) t.q0hi = reinterpret_cast<float*>(take(bS));
    c->slots.push_back(t);
  }
  return true;
}

// gcfd_step_vjp on the mixed path: the recorded window's segments are
// recomputed by the mixed forward from their FP64 checkpoints (hi + lo of the
// compensated state), each step taped (stage RHS, edge speeds, dt; the stage
// increments stay in the slot's D arrays), and reversed in FP32.
int step_vjp_mixed(gcfd_ctx* c, int32_t nshards, const int32_t* Kmax, const double* const* Qfinal_bar,
                   double tfinal_bar, double* const* Q0_bar, double* qinf_bar4, double* t0_bar) {
  const AdjOps& o = *adj_ops(c->N);
  const OrderOps& fo = *order_ops(c->N);
  const Ops fwd = fo.mixed;
  const size_t S = static_cast<size_t>(4) * c->Np * c->K;
  const size_t SB = S * sizeof(double);
  int rc;
  if ((rc = copy_shards(c, c->Qbf, nshards, Kmax, Qfinal_bar, true, nullptr))) return rc;
  o.mixed_bar_convert(c, true);
  c->adjFacesPending = false;
  GCFD_CUDA(c, cudaMemsetAsync(c->adjS, 0, sizeof(double) * 12, c->stream));
  GCFD_CUDA(c, cudaMemcpyAsync(c->adjS + 10, &tfinal_bar, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  const int every = c->winEvery, nsteps = c->winSteps;
  const int nseg = c->winTaped ? 0 : (nsteps + every - 1) / every;
  if (c->winTaped) {  // the recording kept every step's tape: reverse only
    for (int i = nsteps - 1; i >= 0; --i) {
      bind_slot(c, i + 1);
      o.mixed_reverse_taped(c, c->slots[i + 1].q0hi);
      GCFD_CUDA(c, cudaGetLastError());
    }
    bind_slot(c, 0);
  }
  // The hi part of the compensated state at the start of each taped step (the
  // reverse sweep evaluates the stage states as hi + D_s in FP32) is written by
  // the step's stage-4 kernel into c->tapeQ0hi.
  float* hiTmp = reinterpret_cast<float*>(c->Qtmp);  // S doubles of room
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int n0 = seg * every, m = std::min(every, nsteps - n0);
    GCFD_CUDA(c, cudaMemcpyAsync(c->Q[0], c->ckpt + S * seg, SB, cudaMemcpyDeviceToDevice, c->stream));
    GCFD_CUDA(c, cudaMemcpyAsync(&c->sc->time, c->ckptT + seg, sizeof(double), cudaMemcpyDeviceToDevice,
                                 c->stream));
    c->fp64Stale = false;
    fwd.prep(c);
    if (m > 1 && static_cast<int>(c->slots.size()) >= m) {
      // segment tape: each step recomputed once with its tape in its own slot,
      // segQ entry i receiving the step's starting hi from its stage-4 kernel
      for (int i = 0; i < m; ++i) {
        c->tapeQ0hi = reinterpret_cast<float*>(c->segQ + S * i);
        bind_slot(c, i);
        fo.mixed_tape(c);
        GCFD_CUDA(c, cudaGetLastError());
      }
      c->tapeQ0hi = nullptr;
      for (int i = m - 1; i >= 0; --i) {
        bind_slot(c, i);
        o.mixed_reverse_taped(c, reinterpret_cast<const float*>(c->segQ + S * i));
        GCFD_CUDA(c, cudaGetLastError());
      }
      bind_slot(c, 0);
      c->fp64Stale = true;
      continue;
    }
    // without it: the segment's steps once through the graph, keeping each
    // step's starting state in FP64 (segQ), then per step in reverse order the
    // state restored and prepared (the last step's is current already), one
    // taped step (its starting hi into hiTmp) and its reverse
    for (int i = 0; i < m; ++i) {
      if ((rc = sync_fp64_state(c))) return rc;
      GCFD_CUDA(c, cudaMemcpyAsync(c->segQ + S * i, c->Q[0], SB, cudaMemcpyDeviceToDevice, c->stream));
      GCFD_CUDA(c, cudaMemcpyAsync(c->segT + i, &c->sc->time, sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      if (i + 1 < m) {
        GCFD_CUDA(c, cudaGraphLaunch(c->graphExec, c->stream));
        c->fp64Stale = true;
      }
    }
    for (int i = m - 1; i >= 0; --i) {
      if (i < m - 1) {
        GCFD_CUDA(c, cudaMemcpyAsync(c->Q[0], c->segQ + S * i, SB, cudaMemcpyDeviceToDevice, c->stream));
        GCFD_CUDA(c, cudaMemcpyAsync(&c->sc->time, c->segT + i, sizeof(double), cudaMemcpyDeviceToDevice,
                                     c->stream));
        c->fp64Stale = false;
        fwd.prep(c);
      }
      c->tapeQ0hi = hiTmp;
      fo.mixed_tape(c);
      c->tapeQ0hi = nullptr;
      c->fp64Stale = true;
      o.mixed_reverse_taped(c, hiTmp);
      GCFD_CUDA(c, cudaGetLastError());
    }
  }
  o.mixed_finish_faces(c);
  o.mixed_bar_convert(c, false);
  double h[6];
  GCFD_CUDA(c, cudaMemcpyAsync(h, c->adjS + 5, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = copy_shards(c, c->Qbf, nshards, Kmax, nullptr, false, Q0_bar))) return rc;
  // back to the window's end: the FP64 state, rebuilt into the mixed state by
  // the next step
  GCFD_CUDA(c, cudaMemcpyAsync(c->Q[0], c->endQ, SB, cudaMemcpyDeviceToDevice, c->stream));
  GCFD_CUDA(c, cudaMemcpyAsync(c->sc, c->endSc, sizeof(Scalars), cudaMemcpyDeviceToDevice, c->stream));
  c->dirty = true;
  c->fp64Stale = false;
  GCFD_CUDA(c, cudaStreamSynchronize(c->stream));
  if (qinf_bar4)
    for (int i = 0; i < 4; ++i) qinf_bar4[i] = h[i];
  if (t0_bar) *t0_bar = h[5];
  return GCFD_OK;
}

}  // namespace
}  // namespace gcfd_host

using namespace gcfd_host;

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
  const AdjOps& o = *adj_ops(c->N);
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
  // One RHS adjoint costs about one RHS: it runs the FP64 kernels on every
  // context (the mixed path's FP32 transpose of a single RHS loses up to ~5e-5
  // relative at N = 1 and 4 to DivInt's cancellation; over a step dt scales
  // that away, which is where the FP32 reverse sweep runs).
  if (c->fp32 && !c->FEb) {
    double* fe = nullptr;
    if ((rc = dalloc(c, &fe, static_cast<size_t>(4) * 3 * c->NE * c->K))) return rc;
    c->FEb = fe;
  }
  const AdjOps& o = *adj_ops(c->N);
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
  if (!c->slots.empty()) bind_slot(c, 0);
  c->slots.clear();
  c->winPool.insert(c->winPool.end(), c->winAllocs.begin(), c->winAllocs.end());
  c->winAllocs.clear();
  c->segQ = c->segT = nullptr;
  c->winSteps = 0;
  const size_t S = static_cast<size_t>(4) * c->Np * c->K;
  const int nck = (nsteps + every - 1) / every;
  if ((rc = win_alloc(c, &c->ckpt, S * nck))) return rc;
  if ((rc = win_alloc(c, &c->ckptT, static_cast<size_t>(nck)))) return rc;
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
  // One segment for the whole window (every >= nsteps): when a tape slot per
  // step fits in device memory the recording itself keeps every step's tape
  // (slots 1..nsteps; slot 0, the context's own arrays, stays free for
  // gcfd_step) and the reverse sweep recomputes nothing.
  c->winTaped = every >= nsteps && alloc_slots(c, nsteps + 1, true);
  if (!c->winTaped) {  // the segment's starting states, for the reverse sweep
    if ((rc = win_alloc(c, &c->segQ, S * std::min(every, nsteps)))) return rc;
    if ((rc = win_alloc(c, &c->segT, static_cast<size_t>(std::min(every, nsteps))))) return rc;
  }
  // Otherwise the segment tape (one slot per step of a segment) when it fits;
  // without it every step of a segment is recomputed twice in the reverse sweep.
  if (!c->winTaped && every > 1) alloc_slots(c, std::min(every, nsteps), false);
  if ((rc = prepare_if_dirty(c))) return rc;
  if (c->winTaped && !c->fp32) {  // FP64: the step's starting state and time, then the taped step
    GCFD_CUDA(c, cudaMemcpyAsync(c->ckpt, c->Q[0], S * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    GCFD_CUDA(c, cudaMemcpyAsync(c->ckptT, &c->sc->time, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (c->diss)
      GCFD_CUDA(c, cudaMemcpyAsync(c->ckptV, c->DTVisc, KV * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    const AdjOps& ao = *adj_ops(c->N);
    for (int n = 0; n < nsteps; ++n) {
      GCFD_CUDA(c, cudaMemcpyAsync(c->slots[n + 1].q0, c->Q[0], S * sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      bind_slot(c, n + 1);
      ao.tape_step(c);
      GCFD_CUDA(c, cudaGetLastError());
    }
    bind_slot(c, 0);
  } else if (c->winTaped) {
    if ((rc = sync_fp64_state(c))) return rc;
    GCFD_CUDA(c, cudaMemcpyAsync(c->ckpt, c->Q[0], S * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    GCFD_CUDA(c, cudaMemcpyAsync(c->ckptT, &c->sc->time, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    const OrderOps& fo = *order_ops(c->N);
    for (int n = 0; n < nsteps; ++n) {
      c->tapeQ0hi = c->slots[n + 1].q0hi;  // the step's starting hi, from its stage-4 kernel
      bind_slot(c, n + 1);
      fo.mixed_tape(c);
      GCFD_CUDA(c, cudaGetLastError());
    }
    c->tapeQ0hi = nullptr;
    bind_slot(c, 0);
    c->fp64Stale = true;
  }
  for (int n = 0; n < (c->winTaped ? 0 : nsteps); ++n) {
    if (n % every == 0) {
      const int j = n / every;
      if ((rc = sync_fp64_state(c))) return rc;  // mixed path: the checkpoint is hi + lo in FP64
      GCFD_CUDA(c, cudaMemcpyAsync(c->ckpt + S * j, c->Q[0], S * sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      GCFD_CUDA(c, cudaMemcpyAsync(c->ckptT + j, &c->sc->time, sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      if (c->diss)
        GCFD_CUDA(c, cudaMemcpyAsync(c->ckptV + KV * j, c->DTVisc, KV * sizeof(double), cudaMemcpyDeviceToDevice,
                                     c->stream));
    }
    GCFD_CUDA(c, cudaGraphLaunch(c->graphExec, c->stream));
    if (c->fp32) c->fp64Stale = true;
  }
  if ((rc = sync_fp64_state(c))) return rc;
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
  if (c->fp32) return step_vjp_mixed(c, nshards, Kmax, Qfinal_bar, tfinal_bar, Q0_bar, qinf_bar4, t0_bar);
  const AdjOps& o = *adj_ops(c->N);
  const size_t S = static_cast<size_t>(4) * c->Np * c->K;
  const size_t SB = S * sizeof(double);
  if ((rc = copy_shards(c, c->Qbf, nshards, Kmax, Qfinal_bar, true, nullptr))) return rc;
  GCFD_CUDA(c, cudaMemsetAsync(c->adjS, 0, sizeof(double) * 12, c->stream));
  GCFD_CUDA(c, cudaMemcpyAsync(c->adjS + 10, &tfinal_bar, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  const size_t KV = c->diss ? static_cast<size_t>(c->K) : 0;
  if (c->diss) GCFD_CUDA(c, cudaMemsetAsync(c->carryV, 0, KV * sizeof(double), c->stream));
  const int every = c->winEvery, nsteps = c->winSteps;
  const int nseg = c->winTaped ? 0 : (nsteps + every - 1) / every;
  if (c->winTaped) {  // the recording kept every step's tape: reverse only, faces rebuilt from the stage states
    c->facesFromState = true;
    for (int i = nsteps - 1; i >= 0; --i) {
      bind_slot(c, i + 1);
      o.reverse_taped(c, c->slots[i + 1].q0);
      GCFD_CUDA(c, cudaGetLastError());
    }
    c->facesFromState = false;
    bind_slot(c, 0);
  }
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int n0 = seg * every, m = std::min(every, nsteps - n0);
    GCFD_CUDA(c, cudaMemcpyAsync(c->Q[0], c->ckpt + S * seg, SB, cudaMemcpyDeviceToDevice, c->stream));
    GCFD_CUDA(c, cudaMemcpyAsync(&c->sc->time, c->ckptT + seg, sizeof(double), cudaMemcpyDeviceToDevice,
                                 c->stream));
    if (c->diss)
      GCFD_CUDA(c, cudaMemcpyAsync(c->DTVisc, c->ckptV + KV * seg, KV * sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
    const bool taped = m > 1 && static_cast<int>(c->slots.size()) >= m;
    for (int i = 0; i < m; ++i) {
      GCFD_CUDA(c, cudaMemcpyAsync(c->segQ + S * i, c->Q[0], SB, cudaMemcpyDeviceToDevice, c->stream));
      GCFD_CUDA(c, cudaMemcpyAsync(c->segT + i, &c->sc->time, sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
      if (c->diss)
        GCFD_CUDA(c, cudaMemcpyAsync(c->segV + KV * i, c->DTVisc, KV * sizeof(double), cudaMemcpyDeviceToDevice,
                                     c->stream));
      if (taped) {  // the recompute keeps each step's tape in its own slot
        bind_slot(c, i);
        o.tape_step(c);
        GCFD_CUDA(c, cudaGetLastError());
      } else if (i + 1 < m) {
        GCFD_CUDA(c, cudaGraphLaunch(c->graphExec, c->stream));
      }
    }
    if (taped) {
      c->facesFromState = true;
      for (int i = m - 1; i >= 0; --i) {
        bind_slot(c, i);
        o.reverse_taped(c, c->segQ + S * i);
        GCFD_CUDA(c, cudaGetLastError());
      }
      c->facesFromState = false;
      bind_slot(c, 0);
      continue;
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
