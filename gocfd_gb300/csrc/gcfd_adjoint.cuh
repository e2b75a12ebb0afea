// Adjoint (vector-Jacobian products) of the FP64 right-hand side and of the
// SSP(5,4) step.  The forward restates RHSInternalPoints / CalculateEdgeEulerFlux
// / SetRTFluxOnEdges / rkAdvance (euler.go:460-726, edges.go:325-488); the
// adjoint is the exact transpose of that discrete map, including the
// dependence of the time step on the state (global: dt = CFL / max wave speed,
// clipped to FinalTime; local: the running max of CalculateLocalDT) and of the
// IVortex boundary state on the solver time.
//
// Per RK stage s, in reverse:
//   k_adj_div     R-bar from the stage output's adjoint, the SSP combination
//                 terms, the dt adjoint partials, DivInt^T, the interior flux
//                 Jacobian^T (reverse mode written out), edge-DOF adjoints
//   k_adj_edge    Riemann flux Jacobian^T per edge point (Roe in reverse mode,
//                 the other fluxes and every boundary condition by dual numbers)
//   k_adj_gsel /  the dt adjoint onto the wave speed that set it (global:
//   k_adj_lts     the argmax edge; local: per element, carried to the previous
//                 stage when the previous DT was the max)
//   k_adj_speed   wave speed Jacobian^T at each edge's max point
//   k_adj_interp  FluxEdgeInterp^T of the face adjoints
#pragma once
#include <type_traits>

#include "gcfd_dual.cuh"
#include "gcfd_kernels.cuh"

namespace gcfd {

// Euler flux (FluxCalcBase, fluxes.go:76-87) in reverse: qb += (dFx/dq)^T Fxb + (dFy/dq)^T Fyb.
template <typename T>
__device__ __forceinline__ void euler_flux_vjp(const Gas<T>& g, const T q[4], const T Fxb[4], const T Fyb[4],
                                               T qb[4]) {
  const T rho = q[0], m = q[1], n = q[2], E = q[3];
  const T oorho = T(1) / rho;
  const T u = m * oorho, v = n * oorho;
  const T p = g.gm1 * (E - T(0.5) * rho * (u * u + v * v));
  T mb = Fxb[0] + u * Fxb[1] + v * Fxb[2];
  T nb = Fyb[0] + u * Fyb[1] + v * Fyb[2];
  T ub = m * Fxb[1] + (E + p) * Fxb[3] + n * Fyb[1];
  T vb = m * Fxb[2] + n * Fyb[2] + (E + p) * Fyb[3];
  T Eb = u * Fxb[3] + v * Fyb[3];
  const T pb = Fxb[1] + u * Fxb[3] + Fyb[2] + v * Fyb[3];
  // p = gm1 (E - (m^2 + n^2) / (2 rho))
  T rhob = g.gm1 * T(0.5) * (u * u + v * v) * pb;
  mb -= g.gm1 * u * pb;
  nb -= g.gm1 * v * pb;
  Eb += g.gm1 * pb;
  // u = m / rho, v = n / rho
  mb += ub * oorho;
  nb += vb * oorho;
  rhob -= (u * ub + v * vb) * oorho;
  qb[0] += rhob;
  qb[1] += mb;
  qb[2] += nb;
  qb[3] += Eb;
}

// Static pressure (fluids.go:422-453) in reverse.
__device__ __forceinline__ void pressure_vjp(const Gas<double>& g, const double q[4], double pb, double qb[4]) {
  const double oorho = 1.0 / q[0];
  const double u = q[1] * oorho, v = q[2] * oorho;
  qb[0] += g.gm1 * 0.5 * (u * u + v * v) * pb;
  qb[1] -= g.gm1 * u * pb;
  qb[2] -= g.gm1 * v * pb;
  qb[3] += g.gm1 * pb;
}

template <typename T>
__device__ __forceinline__ T sgn(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }

// RoeFlux (fluxes.go:284-413) in reverse: QLb, QRb += (df/dQL)^T fb, (df/dQR)^T fb.
// Divisions are taken once as reciprocals (division is a multi-instruction
// sequence); the forward intermediates are recomputed from QL, QR.  T = double
// on the FP64 path, float on the mixed one.
template <typename T>
__device__ __forceinline__ void roe_vjp(const Gas<T>& g, const T QL[4], const T QR[4], T nx, T ny, const T fbo[4],
                                        T QLb[4], T QRb[4]) {
  // forward
  const T iL = T(1.0) / QL[0], iR = T(1.0) / QR[0];
  const T rhoULr = QL[1] * nx + QL[2] * ny, rhoVLr = -QL[1] * ny + QL[2] * nx;
  const T rhoURr = QR[1] * nx + QR[2] * ny, rhoVRr = -QR[1] * ny + QR[2] * nx;
  const T rhoL = QL[0], uL = rhoULr * iL, vL = rhoVLr * iL;
  const T rhoR = QR[0], uR = rhoURr * iR, vR = rhoVRr * iR;
  const T uxL = QL[1] * iL, uyL = QL[2] * iL, uxR = QR[1] * iR, uyR = QR[2] * iR;
  const T pL = g.gm1 * (QL[3] - T(0.5) * rhoL * (uxL * uxL + uyL * uyL));
  const T pR = g.gm1 * (QR[3] - T(0.5) * rhoR * (uxR * uxR + uyR * uyR));
  const T hL = (QL[3] + pL) * iL, hR = (QR[3] + pR) * iR;
  const T rhoLs = sqrt(rhoL), rhoRs = sqrt(rhoR);
  const T S = rhoLs + rhoRs, oS = T(1.0) / S;
  const T rho = rhoLs * rhoRs;
  const T u = (rhoLs * uL + rhoRs * uR) * oS;
  const T v = (rhoLs * vL + rhoRs * vR) * oS;
  const T h = (rhoLs * hL + rhoRs * hR) * oS;
  const T c2 = g.gm1 * (h - T(0.5) * (u * u + v * v));
  const T C = sqrt(c2), oC = T(1.0) / C, oc2 = oC * oC;
  const T du = uR - uL, dp = pR - pL;
  const T a1 = -T(0.5) * (rho * du) * oC + T(0.5) * dp * oc2;
  const T a2 = (rhoR - rhoL) - dp * oc2;
  const T a3 = rho * (vR - vL);
  const T a4 = T(0.5) * (rho * du) * oC + T(0.5) * dp * oc2;
  const T l1 = fabs(u - C), l2 = fabs(u), l4 = fabs(u + C);
  const T W1 = l1 * a1, W2 = l2 * a2, W3 = l2 * a3, W4 = l4 * a4;
  // output rotation: out0 = f0, out1 = nx f1 - ny f2, out2 = ny f1 + nx f2, out3 = f3
  const T f0b = fbo[0], f1b = nx * fbo[1] + ny * fbo[2], f2b = -ny * fbo[1] + nx * fbo[2], f3b = fbo[3];
  T rhoULrb = T(0.5) * f0b + T(0.5) * uL * f1b;
  T rhoURrb = T(0.5) * f0b + T(0.5) * uR * f1b;
  T rhoVLrb = T(0.5) * uL * f2b;
  T rhoVRrb = T(0.5) * uR * f2b;
  T uLb = T(0.5) * rhoULr * f1b + T(0.5) * rhoVLr * f2b + T(0.5) * (pL + QL[3]) * f3b;
  T uRb = T(0.5) * rhoURr * f1b + T(0.5) * rhoVRr * f2b + T(0.5) * (pR + QR[3]) * f3b;
  T vLb = T(0.0), vRb = T(0.0);
  T pLb = T(0.5) * f1b + T(0.5) * uL * f3b;
  T pRb = T(0.5) * f1b + T(0.5) * uR * f3b;
  T QL3b = T(0.5) * uL * f3b, QR3b = T(0.5) * uR * f3b;
  // dissipation terms: f0 -= T0/2, f1 -= T1/2, f2 -= T2/2, f3 -= T3/2
  const T T0b = -T(0.5) * f0b, T1b = -T(0.5) * f1b, T2b = -T(0.5) * f2b, T3b = -T(0.5) * f3b;
  const T W1b = T0b + (u - C) * T1b + v * T2b + (h - u * C) * T3b;
  const T W2b = T0b + u * T1b + v * T2b + T(0.5) * (u * u + v * v) * T3b;
  const T W3b = T2b + v * T3b;
  const T W4b = T0b + (u + C) * T1b + v * T2b + (h + u * C) * T3b;
  T ub = (W1 + W2 + W4) * T1b + (-W1 * C + W2 * u + W4 * C) * T3b;
  T vb = (W1 + W2 + W4) * T2b + (W2 * v + W3) * T3b;
  T hb = (W1 + W4) * T3b;
  T Cb = (-W1 + W4) * T1b + (-W1 * u + W4 * u) * T3b;
  // W = l * a
  const T a1b = l1 * W1b, a2b = l2 * W2b, a3b = l2 * W3b, a4b = l4 * W4b;
  const T l1b = a1 * W1b, l2b = a2 * W2b + a3 * W3b, l4b = a4 * W4b;
  const T s1 = sgn(u - C), s2 = sgn(u), s4 = sgn(u + C);
  ub += s1 * l1b + s2 * l2b + s4 * l4b;
  Cb += -s1 * l1b + s4 * l4b;
  // a1..a4
  const T a14 = a4b - a1b;
  T rhob = T(0.5) * du * oC * a14 + (vR - vL) * a3b;
  const T dub = T(0.5) * rho * oC * a14;
  Cb -= T(0.5) * rho * du * oc2 * a14;
  const T dpb = oc2 * (T(0.5) * (a1b + a4b) - a2b);
  T c2b = dp * oc2 * oc2 * (a2b - T(0.5) * (a1b + a4b));
  T rhoRb = a2b, rhoLb = -a2b;
  vRb += rho * a3b;
  vLb -= rho * a3b;
  uRb += dub;
  uLb -= dub;
  pRb += dpb;
  pLb -= dpb;
  // C = sqrt(c2); c2 = gm1 (h - (u^2 + v^2) / 2)
  c2b += T(0.5) * Cb * oC;
  hb += g.gm1 * c2b;
  ub -= g.gm1 * u * c2b;
  vb -= g.gm1 * v * c2b;
  // Roe averages
  uLb += rhoLs * oS * ub;
  uRb += rhoRs * oS * ub;
  vLb += rhoLs * oS * vb;
  vRb += rhoRs * oS * vb;
  const T hLb = rhoLs * oS * hb, hRb = rhoRs * oS * hb;
  const T rhoLsb = ((uL - u) * ub + (vL - v) * vb + (hL - h) * hb) * oS + rhoRs * rhob;
  const T rhoRsb = ((uR - u) * ub + (vR - v) * vb + (hR - h) * hb) * oS + rhoLs * rhob;
  rhoLb += T(0.5) * rhoLsb / rhoLs;
  rhoRb += T(0.5) * rhoRsb / rhoRs;
  // h = (E + p) / rho
  QL3b += hLb * iL;
  pLb += hLb * iL;
  rhoLb -= hL * iL * hLb;
  QR3b += hRb * iR;
  pRb += hRb * iR;
  rhoRb -= hR * iR * hRb;
  // rotated velocities
  rhoULrb += uLb * iL;
  rhoVLrb += vLb * iL;
  rhoLb -= (uL * uLb + vL * vLb) * iL;
  rhoURrb += uRb * iR;
  rhoVRrb += vRb * iR;
  rhoRb -= (uR * uRb + vR * vRb) * iR;
  // p = gm1 (E - (m^2 + n^2) / (2 rho))
  rhoLb += g.gm1 * T(0.5) * (uxL * uxL + uyL * uyL) * pLb;
  rhoRb += g.gm1 * T(0.5) * (uxR * uxR + uyR * uyR) * pRb;
  QLb[0] += rhoLb;
  QRb[0] += rhoRb;
  QLb[3] += QL3b + g.gm1 * pLb;
  QRb[3] += QR3b + g.gm1 * pRb;
  QLb[1] += nx * rhoULrb - ny * rhoVLrb - g.gm1 * uxL * pLb;
  QLb[2] += ny * rhoULrb + nx * rhoVLrb - g.gm1 * uyL * pLb;
  QRb[1] += nx * rhoURrb - ny * rhoVRrb - g.gm1 * uxR * pRb;
  QRb[2] += ny * rhoURrb + nx * rhoVRrb - g.gm1 * uyR * pRb;
}

// Any interior flux by forward-mode duals (8 tangents: QL then QR).
static __device__ __noinline__ void riemann_vjp_dual(int kind, const Gas<double>& g, const double QL[4], const double QR[4],
                                              double nx, double ny, const double fb[4], double QLb[4],
                                              double QRb[4]) {
  using D = Dual<8>;
  D qL[4], qR[4], f[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    qL[i] = seed<8>(QL[i], i);
    qR[i] = seed<8>(QR[i], 4 + i);
  }
  riemann_flux<D>(kind, dual_gas<8>(g), qL, qR, D(nx), D(ny), f);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    double sl = 0.0, sr = 0.0;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      sl += fb[n] * f[n].d[j];
      sr += fb[n] * f[n].d[4 + j];
    }
    QLb[j] += sl;
    QRb[j] += sr;
  }
}

// Edge-point wave speed oohK (|u| + c) (StoreEdgeAggregates, edges.go:274-286)
// in reverse, tangents in S.
template <typename S>
__device__ __forceinline__ void wave_speed_vjp(const Gas<double>& g, double oohK, const double q[4], double wb,
                                               double qb[4]) {
  using D = Dual<4, S>;
  D d[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] = seed<4, S>(q[i], i);
  const Gas<D> gd = dual_gas<4, S>(g);
  const D ws = D(oohK) * (speed(d[0], d[1], d[2]) + sound_speed(gd, d[0], d[1], d[2], d[3]));
#pragma unroll
  for (int i = 0; i < 4; ++i) qb[i] += wb * static_cast<double>(ws.d[i]);
}

// One boundary edge point by duals (tangents: interior face state 0..3, the
// far-field Qinf 4..7 with its derived pinf / cinf, solver time 8): the
// boundary flux n.F(qb) (or the wall pressure flux) and the wave speed of qb.
// bp indexes the boundary flux-point coordinates (boundary edge * NpEdge + point).
template <typename T>
__device__ __forceinline__ void bc_point(const EdgeArgs<double>& a, int flag, int bp, const T qi[4], T nx, T ny,
                                         const FreeStreamT<T>& far, const FreeStreamT<T>& in,
                                         const FreeStreamT<T>& out, T t, T oohK, T f[4], T& ws) {
  const Gas<T> g{T(a.gas.gamma), T(a.gas.gm1), T(a.gas.oogm1)};
  T qb[4];
  bool wall = false;
  switch (flag) {
    case 4: riemann_bc(far, qi, far.qinf, nx, ny, qb); break;
    case 1: riemann_bc(in, qi, in.qinf, nx, ny, qb); break;
    case 8: riemann_bc(out, qi, out.qinf, nx, ny, qb); break;
    case 9: {
      T ex[4];
      ivortex_state(T(a.vbeta), T(a.vx0), T(a.vy0), T(a.vgamma), t, T(a.bx[bp]), T(a.by[bp]), ex);
      riemann_bc(far, qi, ex, nx, ny, qb);
      break;
    }
    case 5:
    case 6:
      wall = true;
#pragma unroll
      for (int n = 0; n < 4; ++n) qb[n] = qi[n];
      break;
    default:
#pragma unroll
      for (int n = 0; n < 4; ++n) qb[n] = qi[n];
  }
  if (wall) {
    const T pw = pressure(g, qi[0], qi[1], qi[2], qi[3]);
    f[0] = T(0.0); f[1] = nx * pw; f[2] = ny * pw; f[3] = T(0.0);
  } else {
    T Fx[4], Fy[4];
    euler_flux(g, qb, Fx, Fy);
#pragma unroll
    for (int n = 0; n < 4; ++n) f[n] = nx * Fx[n] + ny * Fy[n];
  }
  ws = oohK * (speed(qb[0], qb[1], qb[2]) + sound_speed(g, qb[0], qb[1], qb[2], qb[3]));
}

// Reverse of bc_point: qib += J^T (fb, wsb); qinfb (4) and tb get the far-field and time parts.
// The inputs are numbered j = 0..8 (interior face state 0..3, Qinf 4..7, time
// 8); this evaluates the M of them from j0 on as dual tangents (all nine: one
// thread per point; three groups of three: three threads per point).  The
// tangents run in S: double on the FP64 path, float for the mixed path's
// reverse sweep (whose boundary Jacobians then cost FP32 rather than FP64 work).
template <typename S, int M = 9>
static __device__ __noinline__ void bc_point_vjp(const EdgeArgs<double>& a, int flag, int bp, const double qi[4],
                                          double nx, double ny, double t, double oohK, const double fb[4], double wsb,
                                          double qib[4], double qinfb[4], double* tb, int j0 = 0) {
  using D = Dual<M, S>;
  auto arg = [&](double v, int j) { return (j >= j0 && j < j0 + M) ? seed<M, S>(v, j - j0) : D(v); };
  D q[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i] = arg(qi[i], i);
  FreeStreamT<D> far, in, out;
  const Gas<D> gd = dual_gas<M, S>(a.gas);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    far.qinf[i] = arg(a.fsFar.qinf[i], 4 + i);
    in.qinf[i] = D(a.fsIn.qinf[i]);
    out.qinf[i] = D(a.fsOut.qinf[i]);
  }
  // pinf, cinf follow Qinf (FreeStream, fluids.go:370-406); values kept bit-equal to the forward's
  far.pinf = pressure(gd, far.qinf[0], far.qinf[1], far.qinf[2], far.qinf[3]);
  far.cinf = sound_speed(gd, far.qinf[0], far.qinf[1], far.qinf[2], far.qinf[3]);
  far.pinf.v = static_cast<S>(a.fsFar.pinf);
  far.cinf.v = static_cast<S>(a.fsFar.cinf);
  far.gamma = D(a.fsFar.gamma);
  far.minf = D(a.fsFar.minf);
  in.pinf = D(a.fsIn.pinf); in.cinf = D(a.fsIn.cinf); in.gamma = D(a.fsIn.gamma); in.minf = D(a.fsIn.minf);
  out.pinf = D(a.fsOut.pinf); out.cinf = D(a.fsOut.cinf); out.gamma = D(a.fsOut.gamma); out.minf = D(a.fsOut.minf);
  D f[4], ws;
  bc_point<D>(a, flag, bp, q, D(nx), D(ny), far, in, out, arg(t, 8), D(oohK), f, ws);
#pragma unroll
  for (int jj = 0; jj < M; ++jj) {
    const int j = j0 + jj;
    double s = wsb * static_cast<double>(ws.d[jj]);
#pragma unroll
    for (int n = 0; n < 4; ++n) s += fb[n] * static_cast<double>(f[n].d[jj]);
    if (j < 4) qib[j] += s;
    else if (j < 8) qinfb[j - 4] += s;
    else *tb += s;
  }
}

// T: the arithmetic and array type of the adjoint (double: FP64 path; float:
// mixed path, whose stage states are Q0 + D_s with the FP32 increments D_s).
template <typename T>
struct AdjArgs {
  int K, stage, localDT;
  const double* Qs;     // stage state (FP64 path)
  const float* Qs32;    // mixed path: the hi part of the step's initial state Q0
  const float* Ds;      // mixed path, stage > 0: the stage increment (state = Q0 + Ds)
  const T* Qbn;         // adjoint of the stage output (stage -1: the RHS adjoint)
  const T* rhs;         // taped RHS of this stage
  const T* rhs3;        // taped RHS of stage 3 (stage 4)
  T* Qb0;               // adjoint of the step's initial state (accumulated)
  T* Qbs;               // adjoint of this stage's state (accumulated)
  T* Qb2;               // stage 4 feeds the stage-2 and stage-3 states directly
  T* Qb3;
  T* Rb3;               // W3 dt4 Qbar_final, stage 4 -> stage 3
  const double* dtS;    // taped global dt per stage [5]
  const double* dtK;    // taped local dt of this stage [K]
  double* dtbarG;       // [5] global dt adjoints
  double* dtOwnK;       // [K] local dt adjoint of this stage
  const double* DivInt;
  const double* Jdet;
  const double* Jinv;
  T* FEb;               // [n][3NE][K]
  Gas<T> gas;
};

// Forward stage coefficients (rkAdvance, euler.go:460-566): stage s < 4 forms
// Q_{s+1} = alpha Q0 + beta Q_s + gamma dt RHS_s; stage 4 forms
// Q_final = A2 Q2 + A3 Q3 + A4 Q4 + W3 dt4 RHS_3 + C4 dt4 RHS_4.
__device__ __forceinline__ void stage_coeffs(int s, double& alpha, double& beta, double& gamma) {
  switch (s) {
    case 0: alpha = 1.0; beta = 0.0; gamma = kSSP[0][0]; break;
    case 1: alpha = kSSP[1][0]; beta = kSSP[1][1]; gamma = kSSP[1][2]; break;
    case 2: alpha = kSSP[2][0]; beta = kSSP[2][1]; gamma = kSSP[2][2]; break;
    default: alpha = kSSP[3][0]; beta = kSSP[3][1]; gamma = kSSP[3][2]; break;
  }
}

// Stage state value at flat index ind.
template <typename T>
__device__ __forceinline__ T stage_value(const AdjArgs<T>& a, size_t ind) {
  if (a.Qs32) return static_cast<T>(a.Qs32[ind]) + (a.Ds ? static_cast<T>(a.Ds[ind]) : T(0));
  return static_cast<T>(a.Qs[ind]);
}

template <int N, typename T>
__global__ void __launch_bounds__(128) k_adj_div(AdjArgs<T> a) {
  constexpr int NP = Dims<N>::NP, NE3 = Dims<N>::NE3, NF = Dims<N>::NF;
  __shared__ T sD[NP * NF];
  stage_operator(sD, a.DivInt, NP * NF);
  __syncthreads();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = k < a.K;
  const size_t sK = static_cast<size_t>(a.K);
  const int s = a.stage;
  T dtb = T(0);
  if (active) {
    T Rb[4][NP];
    if (s < 0) {
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int r = 0; r < NP; ++r) Rb[n][r] = a.Qbn[(n * NP + r) * sK + k];
    } else if (s == 4) {
      const T dt4 = static_cast<T>(a.localDT ? a.dtK[k] : a.dtS[4]);
      const T A2 = kSSP[4][0], A3 = kSSP[4][1], A4 = kSSP[4][2], W3 = kSSP[4][3], C4 = kSSP[4][4];
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int r = 0; r < NP; ++r) {
          const size_t ind = (n * NP + r) * sK + k;
          const T qb = a.Qbn[ind];
          Rb[n][r] = C4 * dt4 * qb;
          a.Rb3[ind] = W3 * dt4 * qb;
          dtb += qb * (W3 * a.rhs3[ind] + C4 * a.rhs[ind]);
          a.Qb2[ind] = A2 * qb;  // stage 4 is the first writer of the stage-2..4 adjoints
          a.Qb3[ind] = A3 * qb;
          a.Qbs[ind] = A4 * qb;
        }
    } else {
      double ald, bed, gad;
      stage_coeffs(s, ald, bed, gad);
      const T al = static_cast<T>(ald), be = static_cast<T>(bed), ga = static_cast<T>(gad);
      const T dt = static_cast<T>(a.localDT ? a.dtK[k] : a.dtS[s]);
#pragma unroll
      for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int r = 0; r < NP; ++r) {
          const size_t ind = (n * NP + r) * sK + k;
          const T qb = a.Qbn[ind];
          Rb[n][r] = ga * dt * qb + (s == 3 ? a.Rb3[ind] : T(0));
          dtb += ga * qb * a.rhs[ind];
          // first writers: stage 3 of the step's Q0 adjoint, stage 1 of its own
          if (s == 3) a.Qb0[ind] = al * qb;
          else a.Qb0[ind] += al * qb;
          if (s == 1) a.Qbs[ind] = be * qb;
          else if (be != T(0)) a.Qbs[ind] += be * qb;
        }
    }
    // RHS = -(1/J) DivInt . DOF  =>  DOFb = -(1/J) DivInt^T Rb
    const T Jd = static_cast<T>(a.Jdet[k]), mooj = -(T(1) / Jd);
    const T J0 = static_cast<T>(a.Jinv[k]), J1 = static_cast<T>(a.Jinv[sK + k]);
    const T J2 = static_cast<T>(a.Jinv[2 * sK + k]), J3 = static_cast<T>(a.Jinv[3 * sK + k]);
#pragma unroll 1
    for (int i = 0; i < NP; ++i) {
      T Fxb[4], Fyb[4], q[4], qb[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        T fr = T(0), fs = T(0);
#pragma unroll
        for (int r = 0; r < NP; ++r) {
          fr += sD[r * NF + i] * Rb[n][r];
          fs += sD[r * NF + NP + i] * Rb[n][r];
        }
        fr *= mooj;
        fs *= mooj;
        Fxb[n] = Jd * (J0 * fr + J2 * fs);
        Fyb[n] = Jd * (J1 * fr + J3 * fs);
        q[n] = stage_value(a, (n * NP + i) * sK + k);
      }
      euler_flux_vjp(a.gas, q, Fxb, Fyb, qb);
#pragma unroll
      for (int n = 0; n < 4; ++n) a.Qbs[(n * NP + i) * sK + k] += qb[n];
    }
#pragma unroll 1
    for (int j = 0; j < NE3; ++j) {
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        T d = T(0);
#pragma unroll
        for (int r = 0; r < NP; ++r) d += sD[r * NF + 2 * NP + j] * Rb[n][r];
        a.FEb[(n * NE3 + j) * sK + k] = mooj * d;
      }
    }
    if (s >= 0 && a.localDT) a.dtOwnK[k] = static_cast<double>(dtb);
  }
  if (s >= 0 && !a.localDT) {
    const double t = warp_sum(active ? static_cast<double>(dtb) : 0.0);
    if ((threadIdx.x & 31) == 0) atomicAdd(&a.dtbarG[s], t);
  }
}

template <typename T>
struct AdjEdgeArgs {
  const T* QF;     // [n][3NE][K] face states of the stage
  T* FEb;          // [n][3NE][K] edge DOF adjoints (from k_adj_div)
  T* QFb;          // [n][3NE][K] face adjoints (written here)
  double* qinfb;   // [4] far-field Qinf adjoint
  double* tb;      // solver-time adjoint
  double* esBar;   // per edge: adjoint of the edge's max wave speed
  int useManualRoe;
};

template <typename T>
__device__ __forceinline__ Gas<T> gas_as(const Gas<double>& g) {
  return Gas<T>{static_cast<T>(g.gamma), static_cast<T>(g.gm1), static_cast<T>(g.oogm1)};
}

// Interior edges [0, nInt): Riemann flux Jacobian^T at each edge point
// (ROE: the reverse-mode Roe adjoint in T; otherwise the dual-number one in FP64).
template <int N, bool ROE, typename T>
__global__ void __launch_bounds__(128) k_adj_edge(EdgeArgs<double> a, AdjEdgeArgs<T> x) {
  constexpr int NE = Dims<N>::NE, NE3 = Dims<N>::NE3;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.nInt) return;
  const size_t sK = static_cast<size_t>(a.K);
  const int kL = a.kL[e], kR = a.kR[e];
  const int eL = a.eLR[e] & 3, eR = a.eLR[e] >> 2;
  const T nx = static_cast<T>(a.nx[e]), ny = static_cast<T>(a.ny[e]);
  const T IIL = static_cast<T>(a.IIL[e]), IIR = static_cast<T>(a.IIR[e]);
  const Gas<T> g = gas_as<T>(a.gas);
#pragma unroll 1
  for (int p = 0; p < NE; ++p) {
    const int jL = eL * NE + p, jR = eR * NE + (NE - 1 - p);
    T qL[4], qR[4], fb[4], qLb[4] = {T(0), T(0), T(0), T(0)}, qRb[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      qL[n] = x.QF[(n * NE3 + jL) * sK + kL];
      qR[n] = x.QF[(n * NE3 + jR) * sK + kR];
      fb[n] = IIL * x.FEb[(n * NE3 + jL) * sK + kL] - IIR * x.FEb[(n * NE3 + jR) * sK + kR];
    }
    if (ROE) {
      roe_vjp<T>(g, qL, qR, nx, ny, fb, qLb, qRb);
    } else {
      double dL[4], dR[4], dfb[4], dLb[4] = {0.0, 0.0, 0.0, 0.0}, dRb[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        dL[n] = qL[n];
        dR[n] = qR[n];
        dfb[n] = fb[n];
      }
      riemann_vjp_dual(a.flux, a.gas, dL, dR, a.nx[e], a.ny[e], dfb, dLb, dRb);
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        qLb[n] = static_cast<T>(dLb[n]);
        qRb[n] = static_cast<T>(dRb[n]);
      }
    }
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      x.QFb[(n * NE3 + jL) * sK + kL] = qLb[n];
      x.QFb[(n * NE3 + jR) * sK + kR] = qRb[n];
    }
  }
}

// Boundary edges [nInt, nInt + nBC): boundary state and flux by dual numbers
// (the point values in FP64).  FP64 path: one thread per (boundary edge, edge
// point) with all nine tangents in FP64; mixed path (T = float): three threads
// per point, three FP32 tangents each.
template <int N, typename T>
__global__ void __launch_bounds__(128) k_adj_edge_bc(EdgeArgs<double> a, AdjEdgeArgs<T> x) {
  constexpr int NE = Dims<N>::NE, NE3 = Dims<N>::NE3;
  constexpr int G = std::is_same<T, float>::value ? 3 : 1;  // threads per point
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double qinfb[4] = {0.0, 0.0, 0.0, 0.0}, tb = 0.0;
  if (tid < a.nBC * NE * G) {
    const int pt = tid / G, g = tid - pt * G;
    const int b = pt / NE, p = pt - b * NE;
    const int e = a.nInt + b;
    const size_t sK = static_cast<size_t>(a.K);
    const int kL = a.kL[e];
    const int jL = (a.eLR[e] & 3) * NE + p;
    const double IIL = a.IIL[e];
    double qi[4], fb[4], qib[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      qi[n] = static_cast<double>(x.QF[(n * NE3 + jL) * sK + kL]);
      fb[n] = IIL * static_cast<double>(x.FEb[(n * NE3 + jL) * sK + kL]);
    }
    if (G == 1) {
      bc_point_vjp<T>(a, a.bcFlag[b], pt, qi, a.nx[e], a.ny[e], *a.time, a.oohK[e], fb, 0.0, qib, qinfb, &tb);
#pragma unroll
      for (int n = 0; n < 4; ++n) x.QFb[(n * NE3 + jL) * sK + kL] = static_cast<T>(qib[n]);
    } else {
      bc_point_vjp<T, 3>(a, a.bcFlag[b], pt, qi, a.nx[e], a.ny[e], *a.time, a.oohK[e], fb, 0.0, qib, qinfb, &tb,
                         3 * g);
      // group 0 owns face components 0..2, group 1 component 3
#pragma unroll
      for (int n = 0; n < 4; ++n)
        if (n / 3 == g) x.QFb[(n * NE3 + jL) * sK + kL] = static_cast<T>(qib[n]);
    }
  }
#pragma unroll
  for (int n = 0; n < 4; ++n) qinfb[n] = warp_sum(qinfb[n]);
  tb = warp_sum(tb);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int n = 0; n < 4; ++n)
      if (qinfb[n] != 0.0) atomicAdd(&x.qinfb[n], qinfb[n]);
    if (tb != 0.0) atomicAdd(x.tb, tb);
  }
}

// Global dt: the edge that set this stage's max wave speed.
static __global__ void k_adj_argmax(const double* edgeSpeed, const double* gmaxS, int stage, int nEdges, int* argEdge) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nEdges && edgeSpeed[g] == gmaxS[stage]) atomicMin(argEdge, g);
}

struct AdjDtArgs {
  int K, stage, nEdges;
  double cfl, finalTime;
  const double* gmaxS;     // taped per-stage max wave speed [5]
  const double* tn;        // taped step start time
  const double* dtbarG;    // [5]
  const double* tbarNext;  // adjoint of the step's end time (stage 4 only)
  double* tbarCur;         // adjoint of the step's start time
  const int* argEdge;
  double* esBar;           // per edge
  // local dt
  const double* dtPrev;    // taped local dt of stage s-1 [K] (stage > 0)
  const double* edgeSpeed; // taped edge speeds of this stage
  const int* elemEdge;     // [3][K]
  const double* dtOwnK;
  double* carry;           // [K]: adjoint carried to the previous stage's dt
  // viscous limit of the PerssonC0 dissipation (diss != 0)
  int diss;
  double cdiff;            // 1 / (N + 1)^2
  const double* gviscS;    // taped per-stage max viscous speed [5]
  const int* argVisc;      // global: the edge that set it
  double* vsBar;           // per edge: adjoint of the viscous speed
  const double* dtvPrev;   // local: taped DTVisc before this stage [K]
  const double* viscSpeed; // local: taped viscous speeds of this stage
  double* carryV;          // [K]: adjoint of DTVisc carried to the previous stage (and step)
};

// Global: dt = min-clip(CFL / gmax) (calculateGlobalDT, euler.go:945-971).
static __global__ void k_adj_gsel(AdjDtArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int s = a.stage;
  double dtb = a.dtbarG[s];
  if (s == 4) dtb += *a.tbarNext;  // Time += GlobalDT of the last stage
  const double gm = a.gmaxS[s];
  const double dtC = a.cfl / gm;
  const double gv = a.diss ? a.gviscS[s] : 0.0;
  const double dtV = a.diss ? a.cdiff / gv : 0.0;
  const bool visc = a.diss && fmin(dtC, dtV) == dtV && dtV < dtC;
  const double dtU = a.diss ? fmin(dtC, dtV) : dtC;
  if (*a.tn + dtU > a.finalTime) {
    *a.tbarCur -= dtb;  // dt = FinalTime - t
  } else if (visc) {
    const int g = *a.argVisc;
    if (g >= 0 && g < a.nEdges) a.vsBar[g] += -a.cdiff / (gv * gv) * dtb;
  } else {
    const int g = *a.argEdge;
    if (g >= 0 && g < a.nEdges) a.esBar[g] += -a.cfl / (gm * gm) * dtb;
  }
}

// Local: DT_k = CFL / max(DT_k(prev stage) or -100 at stage 0, edge speeds)
// (CalculateLocalDT, euler.go:973-1002).
static __global__ void k_adj_lts(AdjDtArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const size_t sK = static_cast<size_t>(a.K);
  const int s = a.stage;
  double v = (s == 0) ? -100.0 : a.dtPrev[k];
  int arg = -1;
  int eg[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    eg[e] = a.elemEdge[e * sK + k];
    const double w = a.edgeSpeed[eg[e]];
    if (w > v) { v = w; arg = e; }
  }
  double dtb = a.dtOwnK[k] + a.carry[k];
  if (a.diss) {
    // dv = max(DTVisc, viscous speeds); DTVisc <- Cdiff / dv when dv > 1e-9, and
    // dt = min(CFL / v, DTVisc) (CalculateLocalDT with the dissipation).
    double dv = a.dtvPrev[k];
    int argv = -1;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const double w = a.viscSpeed[eg[e]];
      if (w > dv) { dv = w; argv = e; }
    }
    double dvnb = a.carryV[k];
    if (dv > 1.e-9) {
      const double dvn = a.cdiff / dv;
      if (dvn < a.cfl / v) {  // the viscous limit set dt
        dvnb += dtb;
        dtb = 0.0;
      }
      dvnb = -a.cdiff / (dv * dv) * dvnb;
    }
    if (argv < 0) {
      a.carryV[k] = dvnb;
    } else {
      a.carryV[k] = 0.0;
      if (dvnb != 0.0) atomicAdd(&a.vsBar[eg[argv]], dvnb);
    }
  }
  const double vb = -a.cfl / (v * v) * dtb;
  if (arg < 0) {
    a.carry[k] = (s == 0) ? 0.0 : vb;
  } else {
    a.carry[k] = 0.0;
    atomicAdd(&a.esBar[eg[arg]], vb);
  }
}

// esBar[g] onto the face state at the edge's max wave-speed point (the point
// chosen in FP64, the tangents in T).
template <int N, typename T>
__global__ void __launch_bounds__(128) k_adj_speed(EdgeArgs<double> a, AdjEdgeArgs<T> x) {
  constexpr int NE = Dims<N>::NE, NE3 = Dims<N>::NE3;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.nInt + a.nBC) return;
  const double wbar = x.esBar[e];
  if (wbar == 0.0) return;
  const size_t sK = static_cast<size_t>(a.K);
  const int kL = a.kL[e];
  const int eL = a.eLR[e] & 3;
  const double nx = a.nx[e], ny = a.ny[e];
  const double oohK = a.oohK[e];
  const bool bc = e >= a.nInt;
  const int b = e - a.nInt;
  const int flag = bc ? a.bcFlag[b] : 0;
  const double t = *a.time;
  // the point the forward max picked: first strict increase (dmax(smax, ws) from -1)
  double best = -1.0;
  int pb = 0;
  for (int p = 0; p < NE; ++p) {
    const int jL = eL * NE + p;
    double qi[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) qi[n] = static_cast<double>(x.QF[(n * NE3 + jL) * sK + kL]);
    double ws;
    if (bc) {
      double f[4];
      bc_point<double>(a, flag, b * NE + p, qi, nx, ny, a.fsFar, a.fsIn, a.fsOut, t, oohK, f, ws);
    } else {
      ws = oohK * (speed(qi[0], qi[1], qi[2]) + sound_speed(a.gas, qi[0], qi[1], qi[2], qi[3]));
    }
    if (ws > best) { best = ws; pb = p; }
  }
  const int jL = eL * NE + pb;
  double qi[4], qib[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int n = 0; n < 4; ++n) qi[n] = static_cast<double>(x.QF[(n * NE3 + jL) * sK + kL]);
  if (bc) {
    double qinfb[4] = {0.0, 0.0, 0.0, 0.0}, tb = 0.0;
    const double fb[4] = {0.0, 0.0, 0.0, 0.0};
    bc_point_vjp<T>(a, flag, b * NE + pb, qi, nx, ny, t, oohK, fb, wbar, qib, qinfb, &tb);
#pragma unroll
    for (int n = 0; n < 4; ++n)
      if (qinfb[n] != 0.0) atomicAdd(&x.qinfb[n], qinfb[n]);
    if (tb != 0.0) atomicAdd(x.tb, tb);
  } else {
    wave_speed_vjp<T>(a.gas, oohK, qi, wbar, qib);
  }
#pragma unroll
  for (int n = 0; n < 4; ++n) x.QFb[(n * NE3 + jL) * sK + kL] += static_cast<T>(qib[n]);
}

// Global dt: the one edge that set the stage's dt (argEdge), one warp, lane p
// evaluating edge point p (k_adj_speed's work for that edge without a thread
// per edge of the mesh).
template <int N, typename T>
__global__ void __launch_bounds__(32) k_adj_speed_one(EdgeArgs<double> a, AdjEdgeArgs<T> x, const int* argEdge) {
  constexpr int NE = Dims<N>::NE, NE3 = Dims<N>::NE3;
  const int e = *argEdge;
  if (e < 0 || e >= a.nInt + a.nBC) return;
  const double wbar = x.esBar[e];
  if (wbar == 0.0) return;
  const int p = threadIdx.x;
  const size_t sK = static_cast<size_t>(a.K);
  const int kL = a.kL[e];
  const int eL = a.eLR[e] & 3;
  const double nx = a.nx[e], ny = a.ny[e];
  const double oohK = a.oohK[e];
  const bool bc = e >= a.nInt;
  const int b = e - a.nInt;
  const int flag = bc ? a.bcFlag[b] : 0;
  const double t = *a.time;
  double ws = -1.0;
  double qi[4];
  if (p < NE) {
    const int jL = eL * NE + p;
#pragma unroll
    for (int n = 0; n < 4; ++n) qi[n] = static_cast<double>(x.QF[(n * NE3 + jL) * sK + kL]);
    if (bc) {
      double f[4];
      bc_point<double>(a, flag, b * NE + p, qi, nx, ny, a.fsFar, a.fsIn, a.fsOut, t, oohK, f, ws);
    } else {
      ws = oohK * (speed(qi[0], qi[1], qi[2]) + sound_speed(a.gas, qi[0], qi[1], qi[2], qi[3]));
    }
  }
  // the forward's max is the first strict increase: the lowest point holding the max
  double m = ws;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  const unsigned hit = __ballot_sync(0xffffffffu, p < NE && ws == m && ws > -1.0);
  const int pb = hit ? __ffs(hit) - 1 : 0;
  if (p != pb) return;
  const int jL = eL * NE + pb;
  double qib[4] = {0.0, 0.0, 0.0, 0.0};
  if (bc) {
    double qinfb[4] = {0.0, 0.0, 0.0, 0.0}, tb = 0.0;
    const double fb[4] = {0.0, 0.0, 0.0, 0.0};
    bc_point_vjp<T>(a, flag, b * NE + pb, qi, nx, ny, t, oohK, fb, wbar, qib, qinfb, &tb);
#pragma unroll
    for (int n = 0; n < 4; ++n)
      if (qinfb[n] != 0.0) atomicAdd(&x.qinfb[n], qinfb[n]);
    if (tb != 0.0) atomicAdd(x.tb, tb);
  } else {
    wave_speed_vjp<T>(a.gas, oohK, qi, wbar, qib);
  }
#pragma unroll
  for (int n = 0; n < 4; ++n) x.QFb[(n * NE3 + jL) * sK + kL] += static_cast<T>(qib[n]);
}

// Qbs += FluxEdgeInterp^T QFb, one thread per (variable, element).
template <int N, typename T>
__global__ void __launch_bounds__(128) k_adj_interp(const T* QFb, const double* Iop, T* Qbs, int K) {
  constexpr int NP = Dims<N>::NP, NE3 = Dims<N>::NE3;
  __shared__ T sI[NE3 * NP];
  stage_operator(sI, Iop, NE3 * NP);
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * K) return;
  const int n = t / K, k = t - n * K;
  const size_t sK = static_cast<size_t>(K);
  T f[NE3];
#pragma unroll
  for (int j = 0; j < NE3; ++j) f[j] = QFb[(n * NE3 + j) * sK + k];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    T acc = T(0);
#pragma unroll
    for (int j = 0; j < NE3; ++j) acc += sI[j * NP + i] * f[j];
    Qbs[(n * NP + i) * sK + k] += acc;
  }
}

// Element-wise conversion between the FP64 interface arrays and the FP32 adjoint.
template <typename A, typename B>
__global__ void k_convert(const A* __restrict__ src, B* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    dst[i] = static_cast<B>(src[i]);
}


// ---------------------------------------------------------------------------
// Functionals of the state, with their gradients.

// Pressure force on Wall / Cyl boundary edges, sum over edges of
// |edge| sum_p w_p p(q_p) n_x (or n_y): the integrated wall pressure force of
// the wall dump in OutputFinal (euler.go:251-316), with the face states at the
// edge's flux points and the interpolatory weights of those points.
template <int N>
__global__ void __launch_bounds__(128) k_func_wall(EdgeArgs<double> a, const double* w, int ycomp, double* QFb,
                                                   double* J) {
  constexpr int NE = Dims<N>::NE, NE3 = Dims<N>::NE3;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  double jl = 0.0;
  if (b < a.nBC) {
    const int flag = a.bcFlag[b];
    if (flag == 5 || flag == 6) {
      const int e = a.nInt + b;
      const size_t sK = static_cast<size_t>(a.K);
      const int kL = a.kL[e];
      const int eL = a.eLR[e] & 3;
      const double nc = ycomp ? a.ny[e] : a.nx[e];
      const double len = a.IIL[e] * (eL == 1 ? 2.0 * sqrt(2.0) : 2.0);
      for (int p = 0; p < NE; ++p) {
        const int jL = eL * NE + p;
        double q[4], qb[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int n = 0; n < 4; ++n) q[n] = a.QF[(n * NE3 + jL) * sK + kL];
        const double c = len * w[p] * nc;
        jl += c * pressure(a.gas, q[0], q[1], q[2], q[3]);
        pressure_vjp(a.gas, q, c, qb);
#pragma unroll
        for (int n = 0; n < 4; ++n) QFb[(n * NE3 + jL) * sK + kL] += qb[n];
      }
    }
  }
  jl = warp_sum(jl);
  if ((threadIdx.x & 31) == 0 && jl != 0.0) atomicAdd(J, jl);
}

// Squared error against the exact isentropic vortex at the solver time,
// sum over solution points and variables of (Q - Q_exact(t))^2
// (IVortex.GetStateC, isentropic_vortex/analytic_vortex.go:31-82).
template <int N>
__global__ void __launch_bounds__(128) k_func_vortex(const double* Q, const double* X, const double* Y, int K,
                                                     double beta, double x0, double y0, double gamma,
                                                     const double* time, double* Qb, double* J, double* tb) {
  constexpr int NP = Dims<N>::NP;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double jl = 0.0, tl = 0.0;
  if (k < K) {
    const size_t sK = static_cast<size_t>(K);
    const Dual<1> t = seed<1>(*time, 0);
    for (int i = 0; i < NP; ++i) {
      const size_t pt = static_cast<size_t>(i) * sK + k;
      Dual<1> ex[4];
      ivortex_state(Dual<1>(beta), Dual<1>(x0), Dual<1>(y0), Dual<1>(gamma), t, Dual<1>(X[pt]), Dual<1>(Y[pt]), ex);
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const size_t ind = (n * NP + i) * sK + k;
        const double d = Q[ind] - ex[n].v;
        jl += d * d;
        Qb[ind] = 2.0 * d;
        tl -= 2.0 * d * ex[n].d[0];
      }
    }
  }
  jl = warp_sum(jl);
  tl = warp_sum(tl);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(J, jl);
    atomicAdd(tb, tl);
  }
}

}  // namespace gcfd
