// ORACLE (test infrastructure only): C++ FP64 restatement of gocfd's 2D Euler
// DFR right-hand side and SSP(5,4) Runge-Kutta step.  Only tests,
// __graft_entry__.smoke() and the CPU-baseline leg of bench.py may load it, as
// the checker and the timed CPU baseline; the product never links it.
//
// The loops follow the reference's own structure (one shard, ProcLimit = 1),
// with OpenMP over elements and edges for the CPU baseline:
//   RungeKutta5SSP.StepWorker / rkAdvance   model_problems/Euler2D/euler.go:420-653
//   SetRTFluxInternal                       euler.go:701-726, fluxes.go:53-87
//   RHSInternalPoints                       euler.go:665-699
//   InterpolateSolutionToEdges              edges.go:485-488
//   CalculateEdgeEulerFlux + BCs            edges.go:325-452, bcs.go:11-133
//   AvgFlux / LaxFlux / RoeFlux / RoeERFlux fluxes.go:135-190,284-503
//   SetRTFluxOnEdges                        edges.go:454-483
//   StoreEdgeAggregates / CalcElementMaxWaveSpeed  edges.go:246-323
//   calculateGlobalDT / CalculateLocalDT / InitializeDT  euler.go:655-663,945-1002
//   GetFlowFunctionBase                     fluids.go:422-469
//   IVortex.GetStateC                       isentropic_vortex/analytic_vortex.go:31-82
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

struct oracle_fs {
  double qinf[4];
  double pinf, cinf, gamma, minf;
};

struct oracle_problem {
  int32_t N, K, Np, NpEdge, NpFlux, nEdges;
  const double* FluxEdgeInterp;  // 3NpEdge x Np
  const double* DivInt;          // Np x NpFlux
  const double* Jdet;            // K
  const double* Jinv;            // K x 4
  const double* nx;              // 3 x K
  const double* ny;
  const double* IInII;
  const double* hK;              // K
  const double* FluxX;           // NpFlux x K
  const double* FluxY;
  const int64_t* kL;
  const int64_t* eL;
  const int64_t* kR;
  const int64_t* eR;
  const int64_t* bc;
  const int64_t* EtoEdge;        // K x 3
  int32_t flux_type;             // 0 average, 1 lax, 2 roe, 3 roe-er
  int32_t flux_mock;             // 0 Euler flux, 1 FluxCalcMomentumOnly (euler_test.go:896-901)
  int32_t local_dt;
  int32_t pad;
  double cfl, final_time;
  double gamma;                  // FSFar.Gamma, used by every flow function
  oracle_fs far, in, out;
  double vbeta, vx0, vy0, vgamma;
  // Artificial dissipation (PerssonC0, dissipation.go / dfr_shock_capturing.go); diss == 0 disables it.
  int32_t diss;
  int32_t nverts;
  const int64_t* EtoV;          // K x 3
  const double* V;              // Np x Np modal Vandermonde
  const double* Vinv;
  const double* SensD;          // Np x Np, I - Clipper
  const double* SensP;          // Np x Np, MassMatrix * SensD
  const double* Mass;           // Np x Np
  const double* ModeFilter;     // Np
  const double* Div;            // NpFlux x NpFlux
  const double* Bary;           // NpFlux x 3
  double kappa;                 // shock-finder Kappa (sigma ramp half width)
  double eps0;                  // viscosity scale (5 / 1.5)
};

}  // extern "C"

namespace {

struct Ctx {
  const oracle_problem* p;
  double GM1;
};

inline double pressure(double g, double rho, double rhoU, double rhoV, double E) {
  const double oorho = 1. / rho;
  const double u = rhoU * oorho, v = rhoV * oorho;
  const double U2 = u * u + v * v;
  const double q = 0.5 * rho * U2;
  return (g - 1.) * (E - q);
}
inline double sound_speed(double g, double rho, double rhoU, double rhoV, double E) {
  const double p = pressure(g, rho, rhoU, rhoV, E);
  return std::sqrt(std::fabs(g * p * (1. / rho)));
}
inline double velocity(double rho, double rhoU, double rhoV) {
  const double oorho = 1. / rho;
  const double u = rhoU * oorho, v = rhoV * oorho;
  return std::sqrt(u * u + v * v);
}

// CalculateFlux -> FluxCalcMock (FluxCalcBase or the momentum-only test mock).
inline void calc_flux(const oracle_problem* p, const double q[4], double Fx[4], double Fy[4]) {
  if (p->flux_mock == 1) {
    for (int n = 0; n < 4; ++n) { Fx[n] = q[1]; Fy[n] = q[2]; }
    return;
  }
  const double oorho = 1. / q[0];
  const double u = q[1] * oorho, v = q[2] * oorho;
  const double pr = pressure(p->gamma, q[0], q[1], q[2], q[3]);
  Fx[0] = q[1]; Fx[1] = q[1] * u + pr; Fx[2] = q[1] * v; Fx[3] = u * (q[3] + pr);
  Fy[0] = q[2]; Fy[1] = q[2] * u; Fy[2] = q[2] * v + pr; Fy[3] = v * (q[3] + pr);
}

void avg_flux(const oracle_problem* p, const double qL[4], const double qR[4], double nx, double ny,
              double f[4]) {
  double FxL[4], FyL[4], FxR[4], FyR[4];
  calc_flux(p, qL, FxL, FyL);
  calc_flux(p, qR, FxR, FyR);
  for (int n = 0; n < 4; ++n) {
    const double fx = 0.5 * (FxL[n] + FxR[n]), fy = 0.5 * (FyL[n] + FyR[n]);
    f[n] = nx * fx + ny * fy;
  }
}

void lax_flux(const oracle_problem* p, const double qL[4], const double qR[4], double nx, double ny,
              double f[4]) {
  const double g = p->gamma;
  const double rhoL = qL[0], rhoR = qR[0];
  const double rhoUL = qL[1], rhoVL = qL[2], rhoUR = qR[1], rhoVR = qR[2];
  const double EL = qL[3], ER = qR[3];
  const double uL = rhoUL / rhoL, vL = rhoVL / rhoL, uR = rhoUR / rhoR, vR = rhoVR / rhoR;
  const double pL = pressure(g, rhoL, rhoUL, rhoVL, EL), pR = pressure(g, rhoR, rhoUR, rhoVR, ER);
  const double CL = sound_speed(g, rhoL, rhoUL, rhoVL, EL), CR = sound_speed(g, rhoR, rhoUR, rhoVR, ER);
  const double maxV = std::max(std::sqrt(uL * uL + vL * vL) + CL, std::sqrt(uR * uR + vR * vR) + CR);
  f[0] = 0.5 * (nx * (rhoUL + rhoUR) + ny * (rhoVL + rhoVR));
  f[1] = 0.5 * (nx * (rhoUL * uL + rhoUR * uR + pL + pR) + ny * (rhoUL * vL + rhoUR * vR));
  f[2] = 0.5 * (nx * (rhoVL * uL + rhoVR * uR) + ny * (rhoVL * vL + rhoVR * vR + pL + pR));
  f[3] = 0.5 * (nx * ((pL + EL) * uL + (pR + ER) * uR) + ny * ((pL + EL) * vL + (pR + ER) * vR));
  for (int n = 0; n < 4; ++n) f[n] += 0.5 * maxV * (qL[n] - qR[n]);
}

void roe_flux(const oracle_problem* p, const double QL[4], const double QR[4], double nx, double ny,
              double f[4]) {
  const double g = p->gamma, GM1 = g - 1.;
  auto rotate = [&](double rhoU, double rhoV, double* ru, double* rv) {
    *ru = rhoU * nx + rhoV * ny;
    *rv = rhoU * (-ny) + rhoV * nx;
  };
  double rhoULr, rhoVLr, rhoURr, rhoVRr;
  rotate(QL[1], QL[2], &rhoULr, &rhoVLr);
  rotate(QR[1], QR[2], &rhoURr, &rhoVRr);
  const double rhoL = QL[0], uL = rhoULr / QL[0], vL = rhoVLr / QL[0];
  const double rhoR = QR[0], uR = rhoURr / QR[0], vR = rhoVRr / QR[0];
  const double pL = pressure(g, QL[0], QL[1], QL[2], QL[3]);
  const double pR = pressure(g, QR[0], QR[1], QR[2], QR[3]);
  const double hL = (QL[3] + pL) / rhoL, hR = (QR[3] + pR) / rhoR;
  const double rhoLs = std::sqrt(rhoL), rhoRs = std::sqrt(rhoR);
  const double rhoLsRs = rhoLs + rhoRs;
  const double rho = rhoLs * rhoRs;
  const double u = (rhoLs * uL + rhoRs * uR) / rhoLsRs;
  const double v = (rhoLs * vL + rhoRs * vR) / rhoLsRs;
  const double h = (rhoLs * hL + rhoRs * hR) / rhoLsRs;
  const double c2 = GM1 * (h - 0.5 * (u * u + v * v));
  const double C = std::sqrt(c2);
  double dW1 = -0.5 * (rho * (uR - uL)) / C + 0.5 * (pR - pL) / c2;
  double dW2 = (rhoR - rhoL) - (pR - pL) / c2;
  double dW3 = rho * (vR - vL);
  double dW4 = 0.5 * (rho * (uR - uL)) / C + 0.5 * (pR - pL) / c2;
  dW1 = std::fabs(u - C) * dW1;
  dW2 = std::fabs(u) * dW2;
  dW3 = std::fabs(u) * dW3;
  dW4 = std::fabs(u + C) * dW4;
  double n0 = 0.5 * (rhoULr + rhoURr);
  double n1 = 0.5 * (rhoULr * uL + rhoURr * uR + pL + pR);
  double n2 = 0.5 * (rhoVLr * uL + rhoVRr * uR);
  double n3 = 0.5 * ((pL + QL[3]) * uL + (pR + QR[3]) * uR);
  n0 -= 0.5 * (dW1 + dW2 + dW4);
  n1 -= 0.5 * (dW1 * (u - C) + dW2 * u + dW4 * (u + C));
  n2 -= 0.5 * (dW1 * v + dW2 * v + dW3 + dW4 * v);
  n3 -= 0.5 * (dW1 * (h - u * C) + 0.5 * dW2 * (u * u + v * v) + dW3 * v + dW4 * (h + u * C));
  f[0] = n0;
  f[1] = nx * n1 - ny * n2;
  f[2] = ny * n1 + nx * n2;
  f[3] = n3;
}

void roe_er_flux(const oracle_problem* p, const double qL[4], const double qR[4], double nx, double ny,
                 double f[4]) {
  const double g = p->gamma, GM1 = g - 1.;
  const double rhoL = qL[0], rhoR = qR[0];
  const double ooRhoL = 1. / rhoL, ooRhoR = 1. / rhoR;
  const double rhoLs = std::sqrt(rhoL), rhoRs = std::sqrt(rhoR);
  const double uL = qL[1] * ooRhoL, vL = qL[2] * ooRhoL, uR = qR[1] * ooRhoR, vR = qR[2] * ooRhoR;
  const double EL = qL[3], ER = qR[3];
  const double UL = nx * uL + ny * vL, UR = nx * uR + ny * vR;
  const double pL = pressure(g, qL[0], qL[1], qL[2], qL[3]), pR = pressure(g, qR[0], qR[1], qR[2], qR[3]);
  const double HL = EL + pL, HR = ER + pR;
  const double ooRs = 1. / (rhoLs + rhoRs);
  const double u = (rhoLs * uL + rhoRs * uR) * ooRs, v = (rhoLs * vL + rhoRs * vR) * ooRs;
  const double h = (HL + HR) * ooRs;
  const double rho = rhoLs * rhoRs;
  const double H = h * rho;
  const double U = nx * u + ny * v;
  const double C2 = GM1 * (h - 0.5 * (u * u + v * v));
  const double C = std::sqrt(C2);
  const double ooC = 1. / C;
  const double Uabs = std::fabs(U);
  f[0] = 0.5 * (UL * rhoL + UR * rhoR);
  f[1] = 0.5 * (UL * rhoL * uL + pL * nx + UR * rhoR * uR + pR * nx);
  f[2] = 0.5 * (UL * rhoL * vL + pL * ny + UR * rhoR * vR + pR * ny);
  f[3] = 0.5 * (UL * HL + UR * HR);
  const double Uef = 0.05 * C;
  const double du = uR - uL, dv = vR - vL;
  const double deltaV2 = du * du + dv * dv;
  const double ooVmag = 1. / std::sqrt(u * u + v * v);
  double n1x, n1y;
  if (deltaV2 < 0.01 * C2) { n1x = nx; n1y = ny; }
  else { n1x = ooVmag * du; n1y = ooVmag * dv; }
  const double n2x = n1y * (nx * n1y - n1x * ny), n2y = -n1x * (nx * n1y - n1x * ny);
  const double alp1 = nx * n1x + ny * n1y, alp2 = nx * n2x + ny * n2y;
  const double U1x = n1x * u, U1y = n1y * v, U2x = n2x * u, U2y = n2y * v;
  const double Urot = std::sqrt(alp1 * alp1 * (U1x * U1x + U1y * U1y)) + std::sqrt(alp2 * alp2 * (U2x * U2x + U2y * U2y));
  const double sigma = std::max(Uabs, std::min(Uef, Urot));
  // math.Copysign(x, 1) == |x|
  const double UabsPrime = Uabs - 0.25 * std::max(0., UR - UL) * (std::fabs(U + C) - std::fabs(U - C));
  const double dU = UR - UL, dP = pR - pL, dRho = rhoR - rhoL, dRhoU = rhoR * uR - rhoL * uL;
  const double dRhoV = rhoR * vR - rhoL * vL, dE = ER - EL;
  const double dPu = rho * dU * std::max(0., C - UabsPrime);
  const double swt = std::fabs(U) * std::min(UabsPrime, C);
  const double dPp = swt * dP * ooC;
  const double dUu = swt * dU * ooC;
  f[0] -= 0.5 * (sigma * dRho + (dPu + dPp) * 0 + dUu * rho);
  f[1] -= 0.5 * (sigma * dRhoU + (dPu + dPp) * nx + dUu * rho * u);
  f[2] -= 0.5 * (sigma * dRhoV + (dPu + dPp) * ny + dUu * rho * v);
  f[3] -= 0.5 * (sigma * dE + (dPu + dPp) * ny + dUu * H);
}

// RiemannBC (bcs.go:70-133).
void riemann_bc(const oracle_fs& FS, const double qq[4], const double QInf[4], double nx, double ny,
                double Q[4]) {
  const double rhoInt = qq[0], uInt = qq[1] / qq[0], vInt = qq[2] / qq[0];
  const double Gamma = FS.gamma, GM1 = Gamma - 1., OOGM1 = 1. / GM1;
  const double pInt = pressure(Gamma, qq[0], qq[1], qq[2], qq[3]);
  const double CInt = sound_speed(Gamma, qq[0], qq[1], qq[2], qq[3]);
  const double pInf = FS.pinf, CInf = FS.cinf;
  const double rhoInf = QInf[0], uInf = QInf[1] / QInf[0], vInf = QInf[2] / QInf[0];
  const double tx = -ny, ty = nx;
  const double VnormInt = nx * uInt + ny * vInt;
  if (FS.minf <= 1.) {
    const double VnormInf = nx * uInf + ny * vInf;
    const double Rinf = VnormInf - 2. * CInf * OOGM1;
    const double Rint = VnormInt + 2. * CInt * OOGM1;
    const double Vnorm = 0.5 * (Rint + Rinf);
    const double C = 0.25 * GM1 * (Rint - Rinf);
    double Vtang, Beta;
    if (VnormInt < 0) {
      Vtang = tx * uInf + ty * vInf;
      Beta = pInf / std::pow(rhoInf, Gamma);
    } else {
      Vtang = tx * uInt + ty * vInt;
      Beta = pInt / std::pow(rhoInt, Gamma);
    }
    const double u = Vnorm * nx + Vtang * tx;
    const double v = Vnorm * ny + Vtang * ty;
    const double rho = std::pow(C * C / (Gamma * Beta), OOGM1);
    const double pr = Beta * std::pow(rho, Gamma);
    Q[0] = rho; Q[1] = rho * u; Q[2] = rho * v; Q[3] = pr * OOGM1 + 0.5 * rho * (u * u + v * v);
  } else if (VnormInt < 0) {
    for (int n = 0; n < 4; ++n) Q[n] = QInf[n];
  } else {
    for (int n = 0; n < 4; ++n) Q[n] = qq[n];
  }
}

void ivortex_state(const oracle_problem* p, double t, double x, double y, double out[4]) {
  const double pi = M_PI;
  const double oo2pi = 0.5 * (1. / pi);
  const double Gamma = p->vgamma, GM1 = Gamma - 1, OOGM1 = 1. / GM1;
  const double pi2 = pi * pi, beta = p->vbeta, beta2 = beta * beta;
  const double fac = 16 * Gamma * pi2;
  double u = 1.0, v = 0.;
  const double xmut = x - u * t, ymvt = y - v * t;
  const double r2 = (xmut - p->vx0) * (xmut - p->vx0) + (ymvt - p->vy0) * (ymvt - p->vy0);
  const double ex1r = std::exp(1 - r2);
  const double tv1 = 1.0 - (GM1 * beta2 * std::exp(2.0 * (1.0 - r2)) / fac);
  u -= beta * ex1r * (ymvt - p->vy0) * oo2pi;
  v += beta * ex1r * (xmut - p->vx0) * oo2pi;
  const double rho = std::pow(tv1, OOGM1);
  const double pr = std::pow(rho, Gamma);
  const double q = 0.5 * rho * (u * u + v * v);
  out[0] = rho; out[1] = rho * u; out[2] = rho * v; out[3] = pr * (1. / (Gamma - 1.)) + q;
}

struct Work {
  std::vector<double> QFace, FRT, EdgeFlux, EdgeSpeed;
  Work(const oracle_problem* p) {
    const size_t K = p->K;
    QFace.assign(4 * 3 * p->NpEdge * K, 0.);
    FRT.assign(4 * p->NpFlux * K, 0.);
    EdgeFlux.assign(4 * static_cast<size_t>(p->nEdges) * p->NpEdge, 0.);
    EdgeSpeed.assign(p->nEdges, 0.);
  }
};

// Q_Face[n] = FluxEdgeInterp * Q[n]  (edges.go:485-488)
void interpolate_to_edges(const oracle_problem* p, const double* Q, double* QF) {
  const int K = p->K, Np = p->Np, NE3 = 3 * p->NpEdge;
#pragma omp parallel for schedule(static)
  for (int kb = 0; kb < K; kb += 256) {
    const int ke = std::min(K, kb + 256);
    for (int n = 0; n < 4; ++n)
      for (int j = 0; j < NE3; ++j) {
        double* dst = QF + (static_cast<size_t>(n) * NE3 + j) * K;
        for (int k = kb; k < ke; ++k) dst[k] = 0.;
        for (int i = 0; i < Np; ++i) {
          const double a = p->FluxEdgeInterp[j * Np + i];
          const double* src = Q + (static_cast<size_t>(n) * Np + i) * K;
          for (int k = kb; k < ke; ++k) dst[k] += a * src[k];
        }
      }
  }
}

// CalculateEdgeEulerFlux (edges.go:325-452): BCs overwrite the left face state
// in place; the normal flux of every edge lands in EdgeFlux in left order.
void edge_fluxes(const oracle_problem* p, double time, double* QF, double* EF, double* EQ = nullptr) {
  const int K = p->K, NE = p->NpEdge, NE3 = 3 * NE, Nint = p->Np;
#pragma omp parallel for schedule(static)
  for (int en = 0; en < p->nEdges; ++en) {
    const int kL = static_cast<int>(p->kL[en]), eL = static_cast<int>(p->eL[en]);
    const size_t fi = static_cast<size_t>(eL) * K + kL;
    const double nx = p->nx[fi], ny = p->ny[fi];
    const int shiftL = eL * NE;
    auto qf = [&](int n, int row, int k) -> double& { return QF[(static_cast<size_t>(n) * NE3 + row) * K + k]; };
    double* out = EF + static_cast<size_t>(en) * NE * 4;
    if (EQ)  // EdgeQValues: the left face state before any BC (edges.go:343-350)
      for (int i = 0; i < NE; ++i)
        for (int n = 0; n < 4; ++n) EQ[(static_cast<size_t>(en) * NE + i) * 4 + n] = qf(n, i + shiftL, kL);
    if (p->kR[en] >= 0) {
      const int kR = static_cast<int>(p->kR[en]), eR = static_cast<int>(p->eR[en]);
      const int shiftR = eR * NE;
      for (int i = 0; i < NE; ++i) {
        const int iL = i + shiftL, iR = NE - 1 - i + shiftR;
        double qL[4], qR[4], f[4];
        for (int n = 0; n < 4; ++n) { qL[n] = qf(n, iL, kL); qR[n] = qf(n, iR, kR); }
        switch (p->flux_type) {
          case 0: avg_flux(p, qL, qR, nx, ny, f); break;
          case 1: lax_flux(p, qL, qR, nx, ny, f); break;
          case 3: roe_er_flux(p, qL, qR, nx, ny, f); break;
          default: roe_flux(p, qL, qR, nx, ny, f); break;
        }
        for (int n = 0; n < 4; ++n) out[i * 4 + n] = f[n];
      }
    } else {
      const int bc = static_cast<int>(p->bc[en]);
      for (int i = 0; i < NE; ++i) {
        const int iL = i + shiftL;
        double qi[4], qb[4], f[4];
        for (int n = 0; n < 4; ++n) qi[n] = qf(n, iL, kL);
        bool calcNormal = true;
        switch (bc) {
          case 4: riemann_bc(p->far, qi, p->far.qinf, nx, ny, qb); break;
          case 1: riemann_bc(p->in, qi, p->in.qinf, nx, ny, qb); break;
          case 8: riemann_bc(p->out, qi, p->out.qinf, nx, ny, qb); break;
          case 9: {
            const size_t indFlux = static_cast<size_t>(2 * Nint + iL) * K + kL;
            double ex[4];
            ivortex_state(p, time, p->FluxX[indFlux], p->FluxY[indFlux], ex);
            riemann_bc(p->far, qi, ex, nx, ny, qb);
            break;
          }
          case 5: case 6: {  // WallBC (bcs.go:11-23)
            calcNormal = false;
            const double pr = pressure(p->gamma, qi[0], qi[1], qi[2], qi[3]);
            f[0] = 0; f[1] = nx * pr; f[2] = ny * pr; f[3] = 0;
            for (int n = 0; n < 4; ++n) qb[n] = qi[n];
            break;
          }
          default: for (int n = 0; n < 4; ++n) qb[n] = qi[n]; break;
        }
        for (int n = 0; n < 4; ++n) qf(n, iL, kL) = qb[n];
        if (calcNormal) {
          double Fx[4], Fy[4];
          calc_flux(p, qb, Fx, Fy);
          for (int n = 0; n < 4; ++n) f[n] = nx * Fx[n] + ny * Fy[n];
        }
        for (int n = 0; n < 4; ++n) out[i * 4 + n] = f[n];
      }
    }
  }
}

// StoreEdgeAggregates (edges.go:246-289) on the BC-overwritten face states.
void edge_aggregates(const oracle_problem* p, const double* QF, double* speed) {
  const int K = p->K, NE = p->NpEdge, NE3 = 3 * NE;
#pragma omp parallel for schedule(static)
  for (int en = 0; en < p->nEdges; ++en) {
    const int kL = static_cast<int>(p->kL[en]), shift = static_cast<int>(p->eL[en]) * NE;
    const double oohK = 1. / p->hK[kL];
    double m = -DBL_MAX;
    for (int i = shift; i < shift + NE; ++i) {
      double q[4];
      for (int n = 0; n < 4; ++n) q[n] = QF[(static_cast<size_t>(n) * NE3 + i) * K + kL];
      const double C = sound_speed(p->gamma, q[0], q[1], q[2], q[3]);
      const double U = velocity(q[0], q[1], q[2]);
      m = std::max(m, oohK * (U + C));
    }
    speed[en] = m;
  }
}

// SetRTFluxInternal + SetRTFluxOnEdges + RHSInternalPoints.
void assemble_rhs(const oracle_problem* p, const double* Q, const double* EF, double* FRT, double* RHS) {
  const int K = p->K, Np = p->Np, NE = p->NpEdge, NF = p->NpFlux, Nint = Np;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < K; ++k) {
    for (int n = 0; n < 4; ++n)
      for (int i = 0; i < NF; ++i) FRT[(static_cast<size_t>(n) * NF + i) * K + k] = 0.;
    const double JdetD = p->Jdet[k];
    const double* JinvD = p->Jinv + 4 * static_cast<size_t>(k);
    for (int i = 0; i < Nint; ++i) {
      double q[4], Fx[4], Fy[4];
      for (int n = 0; n < 4; ++n) q[n] = Q[(static_cast<size_t>(n) * Np + i) * K + k];
      calc_flux(p, q, Fx, Fy);
      for (int n = 0; n < 4; ++n) {
        FRT[(static_cast<size_t>(n) * NF + i) * K + k] = JdetD * (JinvD[0] * Fx[n] + JinvD[1] * Fy[n]);
        FRT[(static_cast<size_t>(n) * NF + i + Nint) * K + k] = JdetD * (JinvD[2] * Fx[n] + JinvD[3] * Fy[n]);
      }
    }
    for (int edgeNum = 0; edgeNum < 3; ++edgeNum) {
      const int shift = edgeNum * NE;
      const double IInII = p->IInII[static_cast<size_t>(edgeNum) * K + k];
      const int64_t en = p->EtoEdge[3 * static_cast<size_t>(k) + edgeNum];
      const bool owner = p->kL[en] == k;
      const double* nf = EF + static_cast<size_t>(en) * NE * 4;
      for (int n = 0; n < 4; ++n)
        for (int i = 0; i < NE; ++i) {
          const size_t ind = (static_cast<size_t>(n) * NF + 2 * Nint + i + shift) * K + k;
          FRT[ind] = owner ? nf[i * 4 + n] * IInII : -nf[(NE - i - 1) * 4 + n] * IInII;
        }
    }
  }
  // DivInt * F_RT_DOF, then * -1/|J|
#pragma omp parallel for schedule(static)
  for (int kb = 0; kb < K; kb += 256) {
    const int ke = std::min(K, kb + 256);
    for (int n = 0; n < 4; ++n)
      for (int r = 0; r < Np; ++r) {
        double* dst = RHS + (static_cast<size_t>(n) * Np + r) * K;
        for (int k = kb; k < ke; ++k) dst[k] = 0.;
        for (int j = 0; j < NF; ++j) {
          const double a = p->DivInt[r * NF + j];
          const double* src = FRT + (static_cast<size_t>(n) * NF + j) * K;
          for (int k = kb; k < ke; ++k) dst[k] += a * src[k];
        }
        for (int k = kb; k < ke; ++k) dst[k] *= -(1. / p->Jdet[k]);
      }
  }
}


// ---------------------------------------------------------------------------
// Artificial dissipation (PerssonC0): model_problems/Euler2D/dissipation.go and
// DG2D/dfr_shock_capturing.go.

struct DissWork {
  std::vector<double> Se, sigma, eps, sigV, epsV, Eps;  // Eps: NpFlux x K (C0 epsilon)
  std::vector<double> DissX, DissY;                      // 4 x NpFlux x K
  std::vector<double> EQ;                                // nEdges x NpEdge x 4 left face states
  std::vector<double> VF;                                // nEdges x NpEdge x 4 viscous normal flux
  std::vector<double> viscSpeed;                         // nEdges
  DissWork(const oracle_problem* p) {
    const size_t K = p->K;
    Se.assign(K, 0.); sigma.assign(K, 0.); eps.assign(K, 0.);
    sigV.assign(p->nverts, 0.); epsV.assign(p->nverts, 0.);
    Eps.assign(static_cast<size_t>(p->NpFlux) * K, 0.);
    DissX.assign(4 * static_cast<size_t>(p->NpFlux) * K, 0.);
    DissY.assign(DissX.size(), 0.);
    EQ.assign(static_cast<size_t>(p->nEdges) * p->NpEdge * 4, 0.);
    VF.assign(EQ.size(), 0.);
    viscSpeed.assign(p->nEdges, 0.);
  }
};

// UpdateSeMoment (dfr_shock_capturing.go:142-166), UpdateShockFinderSigma
// (dissipation.go:491-518, S0 = 4/(N+1)^4), CalculateElementViscosity
// (dissipation.go:397-412).  A NaN moment keeps sigma = 0.
void shock_sensor(const oracle_problem* p, const double* Q, DissWork& w) {
  const int K = p->K, Np = p->Np;
  const double S0 = 4. / std::pow(double(p->N + 1), 4.);
  const double left = S0 - p->kappa, right = S0 + p->kappa, ookappa = 0.5 / p->kappa;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < K; ++k) {
    double num = 0., den = 0.;
    for (int i = 0; i < Np; ++i) {
      double x = 0., y = 0., dq = 0.;
      for (int j = 0; j < Np; ++j) {
        const double rj = Q[static_cast<size_t>(j) * K + k];
        x += p->SensP[i * Np + j] * rj;
        y += p->Mass[i * Np + j] * rj;
        dq += p->SensD[i * Np + j] * rj;
      }
      num += dq * x;
      den += Q[static_cast<size_t>(i) * K + k] * y;
    }
    const double se = std::log10(num / den);
    double sigma = 0.;
    if (se < left) sigma = 0.;
    else if (se >= left && se <= right) sigma = 0.5 * (1. + std::sin(M_PI * ookappa * (se - S0)));
    else if (se > right) sigma = 1.;
    w.Se[k] = se;
    w.sigma[k] = sigma;
    w.eps[k] = p->eps0 * p->hK[k] * sigma;
  }
}

// MergeElementScalarToVertices (euler.go:1048-1065) with max, then
// MergeVertexScalarToElement (euler.go:1067-1086) with sum / 3 for sigma and
// InterpolateEpsilonSigma (dissipation.go:219-242) for epsilon.
void vertex_smoothing(const oracle_problem* p, DissWork& w) {
  const int K = p->K, NF = p->NpFlux;
  std::fill(w.sigV.begin(), w.sigV.end(), -1.);
  std::fill(w.epsV.begin(), w.epsV.end(), -1.);
  for (int k = 0; k < K; ++k)
    for (int v = 0; v < 3; ++v) {
      const int64_t vert = p->EtoV[3 * static_cast<size_t>(k) + v];
      w.sigV[vert] = std::max(w.sigV[vert], w.sigma[k]);
      w.epsV[vert] = std::max(w.epsV[vert], w.eps[k]);
    }
#pragma omp parallel for schedule(static)
  for (int k = 0; k < K; ++k) {
    double acc = 0.;
    for (int v = 0; v < 3; ++v) acc = acc + w.sigV[p->EtoV[3 * static_cast<size_t>(k) + v]];
    w.sigma[k] = acc / 3.;
    for (int i = 0; i < NF; ++i) {
      double e = 0.;
      for (int v = 0; v < 3; ++v) e += p->Bary[i * 3 + v] * w.epsV[p->EtoV[3 * static_cast<size_t>(k) + v]];
      w.Eps[static_cast<size_t>(i) * K + k] = e;
    }
  }
}

// limitAndFilterSolution (dissipation.go:606-622) for the 4 variables.
void limit_filter(const oracle_problem* p, double* U, const std::vector<double>& sigma) {
  const int K = p->K, Np = p->Np;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < K; ++k) {
    const double alpha = std::sin(0.5 * M_PI * sigma[k]);
    for (int n = 0; n < 4; ++n) {
      double* u = U + static_cast<size_t>(n) * Np * K + k;
      std::vector<double> m(Np, 0.);
      for (int i = 0; i < Np; ++i)
        for (int j = 0; j < Np; ++j) m[i] += p->Vinv[i * Np + j] * u[static_cast<size_t>(j) * K];
      for (int i = 1; i < Np; ++i) m[i] *= p->ModeFilter[i] * (1. - alpha);
      for (int i = 0; i < Np; ++i) {
        double acc = 0.;
        for (int j = 0; j < Np; ++j) acc += p->V[i * Np + j] * m[j];
        u[static_cast<size_t>(i) * K] = acc;
      }
    }
  }
}

// CalculateEpsilonGradient (dissipation.go:244-272) via
// GetSolutionGradientUsingRTElement (euler.go:864-918) and the RT metrics of
// CalculateRTBasedDerivativeMetrics (dfr_startup.go:213-254).
void epsilon_gradient(const oracle_problem* p, const double* Q, DissWork& w) {
  const int K = p->K, Np = p->Np, NE = p->NpEdge, NF = p->NpFlux;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < K; ++k) {
    const double* Ji = p->Jinv + 4 * static_cast<size_t>(k);
    const double ooJd = 1. / p->Jdet[k];
    std::vector<double> DX(NF), DY(NF);
    for (int n = 0; n < 4; ++n) {
      for (int i = 0; i < Np; ++i) {
        const double Un = Q[(static_cast<size_t>(n) * Np + i) * K + k];
        DX[i] = Ji[0] * Un;
        DY[i] = Ji[1] * Un;
        DX[i + Np] = Ji[2] * Un;
        DY[i + Np] = Ji[3] * Un;
      }
      for (int e = 0; e < 3; ++e) {
        const int64_t en = p->EtoEdge[3 * static_cast<size_t>(k) + e];
        const bool own = p->kL[en] == k;
        const size_t fi = static_cast<size_t>(e) * K + k;
        const double mx = ooJd * p->nx[fi] * p->IInII[fi], my = ooJd * p->ny[fi] * p->IInII[fi];
        for (int i = 0; i < NE; ++i) {
          const int ii = own ? i : NE - 1 - i;
          const double Un = w.EQ[(static_cast<size_t>(en) * NE + ii) * 4 + n];
          DX[2 * Np + e * NE + i] = mx * Un;
          DY[2 * Np + e * NE + i] = my * Un;
        }
      }
      for (int r = 0; r < NF; ++r) {
        double gx = 0., gy = 0.;
        for (int j = 0; j < NF; ++j) {
          gx += p->Div[r * NF + j] * DX[j];
          gy += p->Div[r * NF + j] * DY[j];
        }
        const double e = w.Eps[static_cast<size_t>(r) * K + k];
        w.DissX[(static_cast<size_t>(n) * NF + r) * K + k] = gx * e;
        w.DissY[(static_cast<size_t>(n) * NF + r) * K + k] = gy * e;
      }
    }
  }
}

// StoreEdgeAggregates' viscous part (edges.go:274-286) and StoreEdgeViscousFlux
// (edges.go:151-244), including its use of the left normal on both sides and
// of the stored left face states for both "sides" of the penalty jump.
void viscous_edges(const oracle_problem* p, DissWork& w) {
  const int K = p->K, NE = p->NpEdge, NF = p->NpFlux, Nint = p->Np;
  const double Omega = double(p->N * p->N);
#pragma omp parallel for schedule(static)
  for (int en = 0; en < p->nEdges; ++en) {
    const int kL = static_cast<int>(p->kL[en]), eL = static_cast<int>(p->eL[en]);
    const size_t fiL = static_cast<size_t>(eL) * K + kL;
    const double nxL = p->nx[fiL], nyL = p->ny[fiL];
    const double oohK = 1. / p->hK[kL];
    double vmax = -DBL_MAX;
    for (int i = 0; i < NE; ++i)
      vmax = std::max(oohK * oohK * w.Eps[static_cast<size_t>(2 * Nint + eL * NE + i) * K + kL], vmax);
    w.viscSpeed[en] = vmax;
    double* vf = w.VF.data() + static_cast<size_t>(en) * NE * 4;
    const int shiftL = eL * NE;
    if (p->kR[en] < 0) {
      for (int n = 0; n < 4; ++n)
        for (int i = 0; i < NE; ++i) {
          const size_t indL = static_cast<size_t>(n) * NF * K + static_cast<size_t>(2 * Nint + shiftL + i) * K + kL;
          vf[i * 4 + n] = nxL * w.DissX[indL] + nyL * w.DissY[indL];
        }
      continue;
    }
    const int kR = static_cast<int>(p->kR[en]), shiftR = static_cast<int>(p->eR[en]) * NE;
    const double len = (eL == 1) ? 2. * std::sqrt(2.) * p->IInII[fiL] : 2. * p->IInII[fiL];
    const double ooLen = 1. / len;
    for (int n = 0; n < 4; ++n)
      for (int i = 0; i < NE; ++i) {
        const size_t indL = static_cast<size_t>(n) * NF * K + static_cast<size_t>(2 * Nint + shiftL + i) * K + kL;
        const size_t indR = static_cast<size_t>(n) * NF * K + static_cast<size_t>(2 * Nint + shiftR + NE - 1 - i) * K + kR;
        const double vFL = nxL * w.DissX[indL] + nyL * w.DissY[indL];
        const double vFR = nxL * w.DissX[indR] + nyL * w.DissY[indR];
        vf[i * 4 + n] = 0.5 * (vFL + vFR);
      }
    for (int n = 0; n < 4; ++n)
      for (int i = 0; i < NE; ++i) {
        const double epsL = w.Eps[static_cast<size_t>(2 * Nint + shiftL + i) * K + kL];
        const double epsR = w.Eps[static_cast<size_t>(2 * Nint + shiftR + NE - 1 - i) * K + kR];
        const double lam = 0.5 * (epsL + epsR);
        const int ii = NE - 1 - i;
        const double* eq = w.EQ.data() + static_cast<size_t>(en) * NE * 4;
        vf[i * 4 + n] -= (Omega * lam * ooLen) * (eq[i * 4 + n] - eq[ii * 4 + n]);
      }
  }
}

// AddDissipation (dissipation.go:274-346): RHS += DivInt * DOF(eps grad Q) / |J|.
void add_dissipation(const oracle_problem* p, DissWork& w, double* RHS) {
  const int K = p->K, Np = p->Np, NE = p->NpEdge, NF = p->NpFlux;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < K; ++k) {
    const double Jd = p->Jdet[k];
    const double* Ji = p->Jinv + 4 * static_cast<size_t>(k);
    std::vector<double> DOF(NF);
    for (int n = 0; n < 4; ++n) {
      for (int i = 0; i < Np; ++i) {
        const size_t ind = (static_cast<size_t>(n) * NF + i) * K + k;
        DOF[i] = Jd * (Ji[0] * w.DissX[ind] + Ji[1] * w.DissY[ind]);
        DOF[i + Np] = Jd * (Ji[2] * w.DissX[ind] + Ji[3] * w.DissY[ind]);
      }
      for (int e = 0; e < 3; ++e) {
        const int64_t en = p->EtoEdge[3 * static_cast<size_t>(k) + e];
        const int sign = (p->kL[en] == k) ? 1 : -1;
        const double II = p->IInII[static_cast<size_t>(e) * K + k];
        for (int i = 0; i < NE; ++i) {
          const int ii = (sign == -1) ? NE - 1 - i : i;
          DOF[2 * Np + e * NE + i] = w.VF[(static_cast<size_t>(en) * NE + ii) * 4 + n] * II * double(sign);
        }
      }
      const double oojd = 1. / Jd;
      for (int r = 0; r < Np; ++r) {
        double d = 0.;
        for (int j = 0; j < NF; ++j) d += p->DivInt[r * NF + j] * DOF[j];
        RHS[(static_cast<size_t>(n) * Np + r) * K + k] += oojd * d;
      }
    }
  }
}

}  // namespace

extern "C" {

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// One RHS evaluation, as the reference tests compose it (euler_test.go:202-222).
// Q, RHS: 4 x Np x K.  QFaceOut (optional): BC-overwritten faces 4 x 3NpEdge x K.
// With dissipation enabled the RHS is the one a step uses at a stage other
// than rkStep 2: Euler RHS + AddDissipation, then the modal filter.
int oracle_rhs(const oracle_problem* p, double time, const double* Q, double* RHS, double* QFaceOut) {
  Work w(p);
  const bool diss = p->diss != 0;
  DissWork dw(p);
  if (diss) {
    shock_sensor(p, Q, dw);
    vertex_smoothing(p, dw);
  }
  interpolate_to_edges(p, Q, w.QFace.data());
  edge_fluxes(p, time, w.QFace.data(), w.EdgeFlux.data(), diss ? dw.EQ.data() : nullptr);
  assemble_rhs(p, Q, w.EdgeFlux.data(), w.FRT.data(), RHS);
  if (diss) {
    epsilon_gradient(p, Q, dw);
    viscous_edges(p, dw);
    add_dissipation(p, dw, RHS);
    limit_filter(p, RHS, dw.sigma);
  }
  if (QFaceOut) std::memcpy(QFaceOut, w.QFace.data(), w.QFace.size() * sizeof(double));
  return 0;
}

// Variant that takes face values directly (no interpolation), used by the
// polynomial-divergence known-answer test (CheckFlux0, euler_test.go:903-982).
int oracle_rhs_faces(const oracle_problem* p, double time, const double* Q, const double* QFaceIn,
                     double* RHS) {
  Work w(p);
  std::memcpy(w.QFace.data(), QFaceIn, w.QFace.size() * sizeof(double));
  edge_fluxes(p, time, w.QFace.data(), w.EdgeFlux.data());
  assemble_rhs(p, Q, w.EdgeFlux.data(), w.FRT.data(), RHS);
  return 0;
}

// nsteps SSP(5,4) steps (StepWorker x 5 + Time += GlobalDT).  Q (4 x Np x K) is
// updated in place; R (optional, 4 x Np x K) receives the final increment.
// DT (K) carries the per-element time step across stages and steps.
int oracle_step(const oracle_problem* p, int nsteps, double* Q, double* time, double* dt_last,
                double* R, double* DT, double* DTVisc) {
  const int K = p->K, Np = p->Np;
  const size_t S = static_cast<size_t>(4) * Np * K;
  std::vector<double> Q1(S), Q2(S), Q3(S), Q4(S), RHS(S), Res(S, 0.);
  std::vector<double> DTloc(K, 0.), DTVloc(K, 0.);
  double* dt = DT ? DT : DTloc.data();
  double* dtv = DTVisc ? DTVisc : DTVloc.data();
  Work w(p);
  const bool diss = p->diss != 0;
  DissWork dw(p);
  const double C_diff = 1. / (double(p->N + 1) * double(p->N + 1));
  double GlobalDT = 0.;
  for (int st = 0; st < nsteps; ++st) {
    for (int rkStep = 0; rkStep < 5; ++rkStep) {
      double* QQQ = rkStep == 0 ? Q : rkStep == 1 ? Q1.data() : rkStep == 2 ? Q2.data()
                  : rkStep == 3 ? Q3.data() : Q4.data();
      if (diss) {
        shock_sensor(p, QQQ, dw);
        vertex_smoothing(p, dw);
        if (rkStep == 2) limit_filter(p, QQQ, dw.sigma);
      }
      interpolate_to_edges(p, QQQ, w.QFace.data());
      edge_fluxes(p, *time, w.QFace.data(), w.EdgeFlux.data(), diss ? dw.EQ.data() : nullptr);
      if (diss) epsilon_gradient(p, QQQ, dw);
      edge_aggregates(p, w.QFace.data(), w.EdgeSpeed.data());
      if (diss) viscous_edges(p, dw);
      if (rkStep == 0)
        for (int k = 0; k < K; ++k) dt[k] = -100;
      double gmax = -DBL_MAX, gvisc = -DBL_MAX;
      for (int k = 0; k < K; ++k)
        for (int e = 0; e < 3; ++e) {
          const int64_t en = p->EtoEdge[3 * static_cast<size_t>(k) + e];
          const double s = w.EdgeSpeed[en];
          gmax = std::max(gmax, s);
          dt[k] = std::max(dt[k], s);
          if (diss) {
            const double v = dw.viscSpeed[en];
            gvisc = std::max(gvisc, v);
            dtv[k] = std::max(dtv[k], v);
          }
        }
      if (!p->local_dt) {
        GlobalDT = p->cfl / gmax;
        if (diss) GlobalDT = std::min(GlobalDT, C_diff / gvisc);
        if (*time + GlobalDT > p->final_time) GlobalDT = p->final_time - *time;
        for (int k = 0; k < K; ++k) dt[k] = GlobalDT;
      } else {
        for (int k = 0; k < K; ++k) dt[k] = p->cfl / dt[k];
        if (diss)
          for (int k = 0; k < K; ++k)
            if (dtv[k] > 1.e-9) {
              dtv[k] = C_diff / dtv[k];
              dt[k] = std::min(dt[k], dtv[k]);
            }
      }
      assemble_rhs(p, QQQ, w.EdgeFlux.data(), w.FRT.data(), RHS.data());
      if (diss) {
        add_dissipation(p, dw, RHS.data());
        limit_filter(p, RHS.data(), dw.sigma);
      }
#pragma omp parallel for schedule(static)
      for (int k = 0; k < K; ++k) {
        for (int n = 0; n < 4; ++n)
          for (int i = 0; i < Np; ++i) {
            const size_t ind = (static_cast<size_t>(n) * Np + i) * K + k;
            const double dtRHS = dt[k] * RHS[ind];
            switch (rkStep) {
              case 0: Q1[ind] = Q[ind] + 0.391752226571890 * dtRHS; break;
              case 1: Q2[ind] = 0.444370493651235 * Q[ind] + 0.555629506348765 * Q1[ind] + 0.368410593050371 * dtRHS; break;
              case 2: Q3[ind] = 0.620101851488403 * Q[ind] + 0.379898148511597 * Q2[ind] + 0.251891774271694 * dtRHS; break;
              case 3:
                Res[ind] = RHS[ind];
                Q4[ind] = 0.178079954393132 * Q[ind] + 0.821920045606868 * Q3[ind] + 0.544974750228521 * dtRHS;
                break;
              default: {
                const double dtR3 = dt[k] * Res[ind];
                Res[ind] = -Q[ind] + 0.517231671970585 * Q2[ind] + 0.096059710526146 * Q3[ind] +
                           0.386708617503269 * Q4[ind] + 0.063692468666290 * dtR3 + 0.226007483236906 * dtRHS;
                Q[ind] += Res[ind];
              }
            }
          }
      }
    }
    if (!p->local_dt) *time += GlobalDT;
  }
  if (dt_last) *dt_last = GlobalDT;
  if (R) std::memcpy(R, Res.data(), S * sizeof(double));
  return 0;
}

// The standalone indicator of ModeAliasShockFinder.ShockIndicator
// (dfr_shock_capturing.go:189-235): moment with the mass-matrix diagonal,
// S0 = 4/N^4; used by the reference's TestShockFinder.
double oracle_shock_indicator(const oracle_problem* p, const double* q, const double* Clipper, double kappa) {
  const int Np = p->Np;
  double mNum = 0., mDen = 0.;
  for (int i = 0; i < Np; ++i) {
    double c = 0.;
    for (int j = 0; j < Np; ++j) c += Clipper[i * Np + j] * q[j];
    const double mass = p->Mass[i + i * Np];
    const double t1 = q[i] - c;
    mNum += mass * (t1 * t1);
    mDen += mass * (q[i] * q[i]);
  }
  const double Se = std::log10(mNum / mDen);
  const double S0 = 4. / std::pow(double(p->N), 4.);
  const double left = S0 - kappa, right = S0 + kappa, ookappa = 0.5 / kappa;
  if (Se < left) return 0.;
  if (Se >= left && Se <= right) return 0.5 * (1. + std::sin(M_PI * ookappa * (Se - S0)));
  return 1.;
}

// EpsilonSigmaMaxToVertices (dissipation.go:163-217) on a given element
// scalar: the maximum over the elements sharing each vertex (TestDissipation).
int oracle_vertex_max(const oracle_problem* p, const double* elem, double* vert) {
  for (int v = 0; v < p->nverts; ++v) vert[v] = -DBL_MAX;
  for (int k = 0; k < p->K; ++k)
    for (int v = 0; v < 3; ++v) {
      const int64_t i = p->EtoV[3 * static_cast<size_t>(k) + v];
      vert[i] = std::max(vert[i], elem[k]);
    }
  return 0;
}

// Physical gradient at all NpFlux flux points from the RT element, with the
// edge values taken from each edge's left element (GetSolutionGradient,
// euler.go:864-918), for the polynomial exactness test of TestDissipation2.
// GX, GY: 4 x NpFlux x K.
int oracle_gradient(const oracle_problem* p, const double* Q, double* GX, double* GY) {
  Work w(p);
  DissWork dw(p);
  interpolate_to_edges(p, Q, w.QFace.data());
  edge_fluxes(p, 0., w.QFace.data(), w.EdgeFlux.data(), dw.EQ.data());
  std::fill(dw.Eps.begin(), dw.Eps.end(), 1.);
  epsilon_gradient(p, Q, dw);
  std::memcpy(GX, dw.DissX.data(), dw.DissX.size() * sizeof(double));
  std::memcpy(GY, dw.DissY.data(), dw.DissY.size() * sizeof(double));
  return 0;
}

// Element scalars of the last sensor evaluation, for tests: Se, sigma, eps per
// element after one sensor + vertex pass on Q.
int oracle_sensor(const oracle_problem* p, const double* Q, double* Se, double* sigmaElem, double* epsElem,
                  double* sigmaAvg, double* epsVertex) {
  DissWork dw(p);
  shock_sensor(p, Q, dw);
  std::memcpy(Se, dw.Se.data(), p->K * sizeof(double));
  std::memcpy(sigmaElem, dw.sigma.data(), p->K * sizeof(double));
  std::memcpy(epsElem, dw.eps.data(), p->K * sizeof(double));
  vertex_smoothing(p, dw);
  std::memcpy(sigmaAvg, dw.sigma.data(), p->K * sizeof(double));
  std::memcpy(epsVertex, dw.epsV.data(), p->nverts * sizeof(double));
  return 0;
}

}  // extern "C"
