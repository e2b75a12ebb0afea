// Kernel launchers of the forward step and RHS, one instantiation per order N
// and arithmetic: Launch<N, double> (FP64 path) and MixedLaunch<N> (mixed
// path).  Included by the per-order translation units only.
#pragma once
#include "gcfd_ctx.hpp"
#include "gcfd_diss.cuh"
#include "gcfd_kernels.cuh"
#include "gcfd_mixed.cuh"
#include "gcfd_mixed_diss.cuh"
#include "gcfd_mixed_pipe.cuh"
#include "gcfd_mixed_tc.cuh"

namespace gcfd_host {

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
    k_resid_blocks<<<kResidBlocks, kResidBlockThreads, 0, c->stream>>>(c->sc, resid_units(c));
    k_step_end<<<1, kResidBlocks, 0, c->stream>>>(c->sc, c->prm.local_time_stepping);
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
    a.P23 = c->P23;
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
    a.BtcF = c->mBtcF;
    a.DissX32 = reinterpret_cast<const float*>(c->DissX);
    a.DissY32 = reinterpret_cast<const float*>(c->DissY);
    a.VF32 = reinterpret_cast<const float*>(c->VF);
    a.err = reinterpret_cast<unsigned int*>(&c->sc->errFlags);
    a.rhsOnly = 0;
    a.tapeRHS = nullptr;
    a.tapeQ0 = nullptr;
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
    k_resid_blocks<<<kResidBlocks, kResidBlockThreads, 0, c->stream>>>(c->sc, resid_units(c));
    k_step_end<<<1, kResidBlocks, 0, c->stream>>>(c->sc, c->prm.local_time_stepping);
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
  // One step with the adjoint tape: the launches of step() (so the stage
  // increments Dk are those of the recorded trajectory), plus the stage RHS and
  // the step's starting Qhi (c->tapeQ0hi) written by the stage kernel, the edge
  // speeds written by the edge kernels straight into the tape (every edge's
  // speed is written at every stage and read only within it), per-stage copies
  // of the local dt, and the scalars before (BC time) and after (per-stage gmax
  // and dt).
  static void tape_step(gcfd_ctx* c) {
    double* const edgeSpeed = c->edgeSpeed;
    cudaMemcpyAsync(c->tapeSc0, c->sc, sizeof(Scalars), cudaMemcpyDeviceToDevice, c->stream);
    k_step_begin<<<1, 32, 0, c->stream>>>(c->sc);
    for (int s = 0; s < 5; ++s) {
      c->edgeSpeed = c->tapeES[s];
      edges(c, s, c->Q[0], &c->sc->time, &c->sc->gmax[s], true);
      MixedArgs a = args(c, s, c->Q[0], &c->sc->time, &c->sc->gmax[s]);
      a.tapeRHS = c->tapeRHS32[s];
      if (s == 4) a.tapeQ0 = c->tapeQ0hi;  // the step's starting hi, read by stage 4 anyway
      stage_kernel(c, a);
      if (c->prm.local_time_stepping)
        cudaMemcpyAsync(c->tapeDT[s], c->DT, sizeof(double) * c->K, cudaMemcpyDeviceToDevice, c->stream);
    }
    c->edgeSpeed = edgeSpeed;
    k_resid_blocks<<<kResidBlocks, kResidBlockThreads, 0, c->stream>>>(c->sc, resid_units(c));
    k_step_end<<<1, kResidBlocks, 0, c->stream>>>(c->sc, c->prm.local_time_stepping);
    cudaMemcpyAsync(c->tapeSc, c->sc, sizeof(Scalars), cudaMemcpyDeviceToDevice, c->stream);
  }
  static void prep_state(gcfd_ctx* c) { prepare(c, c->Q[0]); }
  static void prep_state_range(gcfd_ctx* c, int k0, int k1) { prepare_range(c, c->Q[0], k0, k1); }
};

}  // namespace gcfd_host
