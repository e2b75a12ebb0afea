// Adjoint launchers of one polynomial order: compiled once per order with
// -DGCFD_ORDER=N (0..4), exporting adj_ops_N.
#include "gcfd_adjoint.cuh"
#include "gcfd_adjoint_diss.cuh"
#include "gcfd_adjoint_mixed.cuh"
#include "gcfd_launch.cuh"

#ifndef GCFD_ORDER
#error "compile with -DGCFD_ORDER=<0..4>"
#endif
#define GCFD_CAT2(a, b) a##b
#define GCFD_CAT(a, b) GCFD_CAT2(a, b)

namespace gcfd_host {
namespace {

constexpr int kN = GCFD_ORDER;

// Adjoint launchers (FP64 path, and the FP32 reverse of the mixed path).
template <int N>
struct AdjLaunch {
  using L = Launch<N, double>;
  static int grid(int n) { return (n + 127) / 128; }
  static EdgeArgs<double> edge_args(gcfd_ctx* c, const double* time) {
    EdgeArgs<double> e = L::edge_args(c, time);
    e.QF = static_cast<const double*>(c->QF);
    return e;
  }
  static AdjEdgeArgs<double> adj_edge_args(gcfd_ctx* c, const double* faces) {
    AdjEdgeArgs<double> x;
    x.QF = faces;
    x.FEb = c->FEb;
    x.QFb = c->QFb;
    x.qinfb = c->adjS + 5;
    x.tb = c->adjS + 9;
    x.esBar = c->esBar;
    x.useManualRoe = 1;
    return x;
  }
  static AdjArgs<double> adj_args(gcfd_ctx* c, int s, const double* Qs, const double* Qbn, double* Qbs) {
    AdjArgs<double> a;
    a.K = c->K;
    a.stage = s;
    a.localDT = c->prm.local_time_stepping;
    a.Qs = Qs;
    a.Qs32 = nullptr;
    a.Ds = nullptr;
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
    k_resid_blocks<<<kResidBlocks, kResidBlockThreads, 0, c->stream>>>(c->sc, resid_units(c));
    k_step_end<<<1, kResidBlocks, 0, c->stream>>>(c->sc, c->prm.local_time_stepping);
    cudaMemcpyAsync(c->tapeSc, c->sc, sizeof(Scalars), cudaMemcpyDeviceToDevice, c->stream);
  }
  template <typename T>
  static void edges(gcfd_ctx* c, const EdgeArgs<double>& e, const AdjEdgeArgs<T>& x) {
    if (c->nInt > 0) {
      if (e.flux == kFluxRoe && x.useManualRoe)
        k_adj_edge<N, true, T><<<grid(c->nInt), 128, 0, c->stream>>>(e, x);
      else
        k_adj_edge<N, false, T><<<grid(c->nInt), 128, 0, c->stream>>>(e, x);
    }
    // boundary points: dual numbers, a long dependent chain per thread (on the
    // narrow FP64 pipe for the FP64 path), so one warp per block spreads them
    // over every SM
    constexpr int G = std::is_same<T, float>::value ? 3 : 1;  // threads per point (k_adj_edge_bc)
    if (c->nBC > 0) k_adj_edge_bc<N, T><<<(c->nBC * Dims<N>::NE * G + 31) / 32, 32, 0, c->stream>>>(e, x);
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
    k_adj_interp<N, double><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb, c->Iop, Qbs, c->K);
    if (s == 2) k_adj_diss_limit<N><<<grid(4 * c->K), 128, 0, c->stream>>>(d, x);
    k_adj_diss_alpha<<<grid(c->K), 128, 0, c->stream>>>(d, x);
    k_adj_diss_sensor<N><<<grid(c->K), 128, 0, c->stream>>>(d, x, Qbs);
  }
  // The time-step adjoints of stage s (after the edge adjoints): the dt
  // adjoint onto the wave speed that set it (global: the argmax edge; local:
  // per element), with the viscous limit of the dissipation.  esBar is left
  // for k_adj_speed.
  static void dt_reverse(gcfd_ctx* c, int s) {
    const int nE = c->nInt + c->nBC;
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
  }
  // esBar onto the face states: with global dt one warp on the stage's argmax
  // edge (every other edge has esBar = 0), with local dt a thread per edge.
  template <typename T>
  static void speed_reverse(gcfd_ctx* c, int s, const EdgeArgs<double>& e, const AdjEdgeArgs<T>& x) {
    if (c->prm.local_time_stepping)
      k_adj_speed<N, T><<<grid(c->nInt + c->nBC), 128, 0, c->stream>>>(e, x);
    else
      k_adj_speed_one<N, T><<<1, 32, 0, c->stream>>>(e, x, c->argEdge + s);
  }
  // The reverse of stage s.  Q0 is the step's initial state.  With a segment
  // tape the stage faces are not taped (they are FluxEdgeInterp of the stage
  // state, after the rkStep-2 limiter where it applies) and are rebuilt here.
  static void reverse_stage(gcfd_ctx* c, int s, const double* Q0) {
    const double* Qs = (s == 0) ? Q0 : c->Q[s];
    if (c->facesFromState) {
      void* f = c->QF;
      c->QF = c->tapeQF[s];
      L::interp(c, Qs);
      c->QF = f;
    }
    const double* Qbn = (s == 4) ? c->Qbf : c->Qb[s + 1];
    const double* Qsens = (s == 2) ? c->tapeQ2pre : Qs;
    if (c->diss) {
      diss_reverse_update(c, s, Qs, Qsens, Qbn, c->Qb[s], c->tapeQF[s]);
      k_adj_div<N, double><<<grid(c->K), 128, 0, c->stream>>>(adj_args(c, -1, Qs, c->RbE, c->Qb[s]));
    } else {
      k_adj_div<N, double><<<grid(c->K), 128, 0, c->stream>>>(adj_args(c, s, Qs, Qbn, c->Qb[s]));
    }
    EdgeArgs<double> e = edge_args(c, &c->tapeSc0->time);
    e.QF = c->tapeQF[s];
    const AdjEdgeArgs<double> x = adj_edge_args(c, c->tapeQF[s]);
    edges(c, e, x);
    dt_reverse(c, s);
    speed_reverse(c, s, e, x);
    if (c->diss)
      diss_reverse_rest(c, s, Qs, Qsens, c->Qb[s], c->tapeQF[s]);
    else
      k_adj_interp<N, double><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb, c->Iop, c->Qb[s], c->K);
  }
  // Adjoint of one step whose initial state is Q0 (already in c->Q[0]) and
  // time is in c->sc.  In: Qbf, adjS[10] (t-bar of the step's end).  Out:
  // Qbf <- adjoint of Q0, adjS[10] <- t-bar of the step's start.  carryV (the
  // DTVisc adjoint) runs on across steps.
  static void reverse_step(gcfd_ctx* c, const double* Q0) {
    tape_step(c);
    reverse_taped(c, Q0);
  }
  // The adjoint of a step whose tape is already bound (tape_step ran earlier
  // into the context's current tape slot).
  static void reverse_taped(gcfd_ctx* c, const double* Q0) {
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
      k_adj_div<N, double><<<grid(c->K), 128, 0, c->stream>>>(adj_args(c, -1, c->Qtmp, c->RbE, c->Qb[0]));
    } else {
      k_adj_div<N, double><<<grid(c->K), 128, 0, c->stream>>>(adj_args(c, -1, c->Qtmp, c->Qbf, c->Qb[0]));
    }
    edges(c, e, adj_edge_args(c, static_cast<const double*>(c->QF)));
    if (c->diss) {
      cudaMemsetAsync(c->vsBar, 0, sizeof(double) * (c->nInt + c->nBC), c->stream);
      diss_reverse_rest(c, -1, c->Qtmp, c->Qtmp, c->Qb[0], static_cast<const double*>(c->QF));
      c->QF = faces;
    } else {
      k_adj_interp<N, double><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb, c->Iop, c->Qb[0], c->K);
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
    k_adj_interp<N, double><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb, c->Iop, c->Qb[0], c->K);
  }

  // ---- mixed path: the FP32 adjoint of a step taped by the mixed forward ----
  static AdjArgs<float> adj_args32(gcfd_ctx* c, int s, const float* Q0hi, const float* Qbn, float* Qbs) {
    AdjArgs<float> a;
    a.K = c->K;
    a.stage = s;
    a.localDT = c->prm.local_time_stepping;
    a.Qs = nullptr;
    a.Qs32 = Q0hi;
    a.Ds = s > 0 ? c->Dk[s] : nullptr;
    a.Qbn = Qbn;
    a.rhs = s >= 0 ? c->tapeRHS32[s] : nullptr;
    a.rhs3 = c->tapeRHS32[3];
    a.Qb0 = c->Qb32[0];
    a.Qbs = Qbs;
    a.Qb2 = nullptr;  // k_adj_div32 takes the final state's shares from Qbf32
    a.Qb3 = nullptr;
    a.Rb3 = nullptr;
    a.dtS = c->tapeSc->dt;
    a.dtK = s >= 0 ? c->tapeDT[s] : nullptr;
    a.dtbarG = c->adjS;
    a.dtOwnK = c->dtOwnK;
    a.DivInt = c->Div;
    a.Jdet = c->Jdet;
    a.Jinv = c->Jinv;
    a.FEb = c->FEb32;
    const float g = static_cast<float>(c->fsFar.gamma);
    a.gas = Gas<float>{g, g - 1.0f, 1.0f / (g - 1.0f)};
    return a;
  }
  static AdjEdgeArgs<float> adj_edge_args32(gcfd_ctx* c) {
    AdjEdgeArgs<float> x;
    x.QF = c->QF32;
    x.FEb = c->FEb32;
    x.QFb = c->QFb32;
    x.qinfb = c->adjS + 5;
    x.tb = c->adjS + 9;
    x.esBar = c->esBar;
    x.useManualRoe = 1;
    return x;
  }
  // Stage s in reverse: the stage state is Q0 + D_s (the taped increments), its
  // faces are interpolated once more in FP32, then the kernels of the FP64
  // sweep in FP32 (the boundary points and wave-speed maxima in FP64).
  //
  // The face transpose of stage s + 1 rides in stage s's divergence kernel
  // (k_adj_div32), and stage 0's in the stage-4 kernel of the step reversed
  // next (c->adjFacesPending until then; mixed_finish_faces ends a sweep).
  static void mixed_reverse_stage(gcfd_ctx* c, int s, const float* Q0) {
    const float* Qbn = (s == 4) ? c->Qbf32 : c->Qb32[s + 1];
    const bool pending = (s < 4) || c->adjFacesPending;
    k_adj_div32<N><<<(c->K + 31) / 32, 128, 0, c->stream>>>(adj_args32(c, s, Q0, Qbn, c->Qb32[s]), c->mgeo,
                                                           pending ? c->QFb32 : nullptr, c->QF32, c->Qbf32,
                                                           c->tapeDT[4]);
    c->adjFacesPending = false;
    const EdgeArgs<double> e = edge_args(c, &c->tapeSc0->time);
    const AdjEdgeArgs<float> x = adj_edge_args32(c);
    edges(c, e, x);
    dt_reverse(c, s);
    speed_reverse(c, s, e, x);
    if (s == 0) c->adjFacesPending = true;
  }
  // The last stage-0 face transpose of a reverse sweep into its result Qbf32.
  static void mixed_finish_faces(gcfd_ctx* c) {
    if (!c->adjFacesPending) return;
    k_adj_interp<N, float><<<grid(4 * c->K), 128, 0, c->stream>>>(c->QFb32, c->Iop, c->Qbf32, c->K);
    c->adjFacesPending = false;
  }
  // The adjoint of a mixed step whose tape is bound; Q0 is the hi part of the
  // step's initial state.  In: Qbf32, adjS[10]; out: Qbf32 <- adjoint of Q0,
  // adjS[10] <- t-bar of the step's start.
  static void mixed_reverse_taped(gcfd_ctx* c, const float* Q0) {
    cudaMemsetAsync(c->adjS, 0, sizeof(double) * 5, c->stream);
    cudaMemcpyAsync(c->adjS + 9, c->adjS + 10, sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
    cudaMemsetAsync(c->carry, 0, sizeof(double) * c->K, c->stream);
    for (int s = 4; s >= 0; --s) mixed_reverse_stage(c, s, Q0);
    std::swap(c->Qbf32, c->Qb32[0]);
    cudaMemcpyAsync(c->adjS + 10, c->adjS + 9, sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  }
  // FP32 DivInt and FluxEdgeInterp into this unit's constant memory as the
  // packed pairs of k_adj_div32 (AdjDims), with DivInt's column sums in FP64.
  static int mixed_consts(gcfd_ctx* c) {
    constexpr int NP = AdjDims<N>::NP, NE3 = AdjDims<N>::NE3, NEH = AdjDims<N>::NEH, NPH = AdjDims<N>::NPH;
    const DMat& D = c->el.DivInt;
    const DMat& I = c->el.FluxEdgeInterp;
    std::vector<double> cs(c->NF, 0.0);
    for (int j = 0; j < c->NF; ++j)
      for (int r = 0; r < NP; ++r) cs[j] += D(r, j);
    auto f2 = [](double x, double y) { return make_float2(static_cast<float>(x), static_cast<float>(y)); };
    std::vector<float2> fs(NP * NP), de(NP * NEH), csfs(NP), cse(NEH), iopT(NE3 * NPH), iop(NP * NEH);
    for (int r = 0; r < NP; ++r) {
      for (int i = 0; i < NP; ++i) fs[r * NP + i] = f2(D(r, i), D(r, NP + i));
      for (int q = 0; q < NEH; ++q)
        de[r * NEH + q] = f2(D(r, 2 * NP + 2 * q), 2 * q + 1 < NE3 ? D(r, 2 * NP + 2 * q + 1) : 0.0);
    }
    for (int i = 0; i < NP; ++i) csfs[i] = f2(cs[i], cs[NP + i]);
    for (int q = 0; q < NEH; ++q) cse[q] = f2(cs[2 * NP + 2 * q], 2 * q + 1 < NE3 ? cs[2 * NP + 2 * q + 1] : 0.0);
    for (int j = 0; j < NE3; ++j)
      for (int h = 0; h < NPH; ++h) iopT[j * NPH + h] = f2(I(j, 2 * h), 2 * h + 1 < NP ? I(j, 2 * h + 1) : 0.0);
    for (int i = 0; i < NP; ++i)
      for (int q = 0; q < NEH; ++q) iop[i * NEH + q] = f2(I(2 * q, i), 2 * q + 1 < NE3 ? I(2 * q + 1, i) : 0.0);
    GCFD_CUDA(c, cudaMemcpyToSymbol(cAdjDivFS, fs.data(), fs.size() * sizeof(float2)));
    GCFD_CUDA(c, cudaMemcpyToSymbol(cAdjDivE, de.data(), de.size() * sizeof(float2)));
    GCFD_CUDA(c, cudaMemcpyToSymbol(cAdjCSFS, csfs.data(), csfs.size() * sizeof(float2)));
    GCFD_CUDA(c, cudaMemcpyToSymbol(cAdjCSE, cse.data(), cse.size() * sizeof(float2)));
    GCFD_CUDA(c, cudaMemcpyToSymbol(cAdjIopT, iopT.data(), iopT.size() * sizeof(float2)));
    GCFD_CUDA(c, cudaMemcpyToSymbol(cAdjIop, iop.data(), iop.size() * sizeof(float2)));
    return GCFD_OK;
  }
  static void mixed_bar_convert(gcfd_ctx* c, bool toFP32) {
    const size_t S = static_cast<size_t>(4) * c->Np * c->K;
    if (toFP32)
      k_convert<double, float><<<1024, 256, 0, c->stream>>>(c->Qbf, c->Qbf32, S);
    else
      k_convert<float, double><<<1024, 256, 0, c->stream>>>(c->Qbf32, c->Qbf, S);
  }
};

}  // namespace

const AdjOps* GCFD_CAT(adj_ops_, GCFD_ORDER)() {
  static const AdjOps o{&AdjLaunch<kN>::tape_step,       &AdjLaunch<kN>::reverse_step,
                        &AdjLaunch<kN>::reverse_taped,   &AdjLaunch<kN>::rhs_vjp,
                        &AdjLaunch<kN>::functional,      &AdjLaunch<kN>::mixed_reverse_taped,
                        &AdjLaunch<kN>::mixed_bar_convert, &AdjLaunch<kN>::mixed_consts,
                        &AdjLaunch<kN>::mixed_finish_faces};
  return &o;
}

}  // namespace gcfd_host
