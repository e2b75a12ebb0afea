// Pointwise 2D Euler physics shared by the device kernels, templated on the
// arithmetic type T (double for the FP64 drop-in path, float for the FP32 path).
// Every function restates one reference routine and keeps its order of
// operations so the FP64 path tracks the reference arithmetic closely.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gcfd {

enum FluxKind : int { kFluxAverage = 0, kFluxLax = 1, kFluxRoe = 2, kFluxRoeER = 3 };

template <typename T>
struct Gas {
  T gamma, gm1, oogm1;
};

template <typename T> __device__ __forceinline__ T dsqrt(T x);
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <typename T> __device__ __forceinline__ T dabs(T x);
template <> __device__ __forceinline__ double dabs<double>(double x) { return fabs(x); }
template <> __device__ __forceinline__ float dabs<float>(float x) { return fabsf(x); }
template <typename T> __device__ __forceinline__ T dpow(T x, T y);
template <> __device__ __forceinline__ double dpow<double>(double x, double y) { return pow(x, y); }
template <> __device__ __forceinline__ float dpow<float>(float x, float y) { return powf(x, y); }
template <typename T> __device__ __forceinline__ T dexp(T x);
template <> __device__ __forceinline__ double dexp<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float dexp<float>(float x) { return expf(x); }
template <typename T> __device__ __forceinline__ T dmax(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T dmin(T a, T b) { return a < b ? a : b; }

// Static pressure, model_problems/Euler2D/fluids.go:422-453.
template <typename T>
__device__ __forceinline__ T pressure(const Gas<T>& g, T rho, T rhoU, T rhoV, T E) {
  const T oorho = T(1) / rho;
  const T u = rhoU * oorho, v = rhoV * oorho;
  const T q = T(0.5) * rho * (u * u + v * v);
  return g.gm1 * (E - q);
}

// Sound speed sqrt(|gamma p / rho|), fluids.go:456-457.
template <typename T>
__device__ __forceinline__ T sound_speed(const Gas<T>& g, T rho, T rhoU, T rhoV, T E) {
  const T p = pressure(g, rho, rhoU, rhoV, E);
  return dsqrt(dabs(g.gamma * p * (T(1) / rho)));
}

// Velocity magnitude, fluids.go:448-449.
template <typename T>
__device__ __forceinline__ T speed(T rho, T rhoU, T rhoV) {
  const T oorho = T(1) / rho;
  const T u = rhoU * oorho, v = rhoV * oorho;
  return dsqrt(u * u + v * v);
}

// Physical flux vectors, FluxCalcBase (fluxes.go:76-87).
template <typename T>
__device__ __forceinline__ void euler_flux(const Gas<T>& g, const T q[4], T Fx[4], T Fy[4]) {
  const T oorho = T(1) / q[0];
  const T u = q[1] * oorho, v = q[2] * oorho;
  const T p = pressure(g, q[0], q[1], q[2], q[3]);
  Fx[0] = q[1]; Fx[1] = q[1] * u + p; Fx[2] = q[1] * v; Fx[3] = u * (q[3] + p);
  Fy[0] = q[2]; Fy[1] = q[2] * u; Fy[2] = q[2] * v + p; Fy[3] = v * (q[3] + p);
}

// Average of the two sides' fluxes dotted with the normal, AvgFlux (fluxes.go:135-159).
template <typename T>
__device__ __forceinline__ void flux_average(const Gas<T>& g, const T qL[4], const T qR[4], T nx,
                                             T ny, T f[4]) {
  T FxL[4], FyL[4], FxR[4], FyR[4];
  euler_flux(g, qL, FxL, FyL);
  euler_flux(g, qR, FxR, FyR);
#pragma unroll
  for (int n = 0; n < 4; ++n)
    f[n] = nx * (T(0.5) * (FxL[n] + FxR[n])) + ny * (T(0.5) * (FyL[n] + FyR[n]));
}

// Local Lax-Friedrichs, LaxFlux (fluxes.go:161-190).
template <typename T>
__device__ __forceinline__ void flux_lax(const Gas<T>& g, const T qL[4], const T qR[4], T nx, T ny,
                                         T f[4]) {
  const T rhoL = qL[0], rhoR = qR[0];
  const T rhoUL = qL[1], rhoVL = qL[2], rhoUR = qR[1], rhoVR = qR[2];
  const T EL = qL[3], ER = qR[3];
  const T uL = rhoUL / rhoL, vL = rhoVL / rhoL, uR = rhoUR / rhoR, vR = rhoVR / rhoR;
  const T pL = pressure(g, rhoL, rhoUL, rhoVL, EL), pR = pressure(g, rhoR, rhoUR, rhoVR, ER);
  const T CL = sound_speed(g, rhoL, rhoUL, rhoVL, EL), CR = sound_speed(g, rhoR, rhoUR, rhoVR, ER);
  const T maxV = dmax(dsqrt(uL * uL + vL * vL) + CL, dsqrt(uR * uR + vR * vR) + CR);
  f[0] = T(0.5) * (nx * (rhoUL + rhoUR) + ny * (rhoVL + rhoVR));
  f[1] = T(0.5) * (nx * (rhoUL * uL + rhoUR * uR + pL + pR) + ny * (rhoUL * vL + rhoUR * vR));
  f[2] = T(0.5) * (nx * (rhoVL * uL + rhoVR * uR) + ny * (rhoVL * vL + rhoVR * vR + pL + pR));
  f[3] = T(0.5) * (nx * ((pL + EL) * uL + (pR + ER) * uR) + ny * ((pL + EL) * vL + (pR + ER) * vR));
#pragma unroll
  for (int n = 0; n < 4; ++n) f[n] += T(0.5) * maxV * (qL[n] - qR[n]);
}

// Roe flux with rotation to the face frame, RoeFlux (fluxes.go:284-413).
template <typename T>
__device__ __forceinline__ void flux_roe(const Gas<T>& g, const T QL[4], const T QR[4], T nx, T ny,
                                         T f[4]) {
  const T rhoULr = QL[1] * nx + QL[2] * ny, rhoVLr = QL[1] * (-ny) + QL[2] * nx;
  const T rhoURr = QR[1] * nx + QR[2] * ny, rhoVRr = QR[1] * (-ny) + QR[2] * nx;
  const T rhoL = QL[0], uL = rhoULr / QL[0], vL = rhoVLr / QL[0];
  const T rhoR = QR[0], uR = rhoURr / QR[0], vR = rhoVRr / QR[0];
  const T pL = pressure(g, QL[0], QL[1], QL[2], QL[3]);
  const T pR = pressure(g, QR[0], QR[1], QR[2], QR[3]);
  const T hL = (QL[3] + pL) / rhoL, hR = (QR[3] + pR) / rhoR;
  const T rhoLs = dsqrt(rhoL), rhoRs = dsqrt(rhoR);
  const T rhoLsRs = rhoLs + rhoRs;
  const T rho = rhoLs * rhoRs;
  const T u = (rhoLs * uL + rhoRs * uR) / rhoLsRs;
  const T v = (rhoLs * vL + rhoRs * vR) / rhoLsRs;
  const T h = (rhoLs * hL + rhoRs * hR) / rhoLsRs;
  const T c2 = g.gm1 * (h - T(0.5) * (u * u + v * v));
  const T C = dsqrt(c2);
  T dW1 = -T(0.5) * (rho * (uR - uL)) / C + T(0.5) * (pR - pL) / c2;
  T dW2 = (rhoR - rhoL) - (pR - pL) / c2;
  T dW3 = rho * (vR - vL);
  T dW4 = T(0.5) * (rho * (uR - uL)) / C + T(0.5) * (pR - pL) / c2;
  dW1 = dabs(u - C) * dW1;
  dW2 = dabs(u) * dW2;
  dW3 = dabs(u) * dW3;
  dW4 = dabs(u + C) * dW4;
  T f0 = T(0.5) * (rhoULr + rhoURr);
  T f1 = T(0.5) * (rhoULr * uL + rhoURr * uR + pL + pR);
  T f2 = T(0.5) * (rhoVLr * uL + rhoVRr * uR);
  T f3 = T(0.5) * ((pL + QL[3]) * uL + (pR + QR[3]) * uR);
  f0 -= T(0.5) * (dW1 + dW2 + dW4);
  f1 -= T(0.5) * (dW1 * (u - C) + dW2 * u + dW4 * (u + C));
  f2 -= T(0.5) * (dW1 * v + dW2 * v + dW3 + dW4 * v);
  f3 -= T(0.5) * (dW1 * (h - u * C) + T(0.5) * dW2 * (u * u + v * v) + dW3 * v + dW4 * (h + u * C));
  f[0] = f0;
  f[1] = nx * f1 - ny * f2;
  f[2] = ny * f1 + nx * f2;
  f[3] = f3;
}

// Go's math.Copysign(x, 1) is |x|; RoeERFlux uses it as "sign".
template <typename T>
__device__ __forceinline__ T copysign_pos(T x) { return dabs(x); }

// Roe-ER flux, RoeERFlux (fluxes.go:415-503), energy dissipation term kept as written.
template <typename T>
__device__ __forceinline__ void flux_roe_er(const Gas<T>& g, const T qL[4], const T qR[4], T nx,
                                            T ny, T f[4]) {
  const T rhoL = qL[0], rhoR = qR[0];
  const T ooRhoL = T(1) / rhoL, ooRhoR = T(1) / rhoR;
  const T rhoLs = dsqrt(rhoL), rhoRs = dsqrt(rhoR);
  const T uL = qL[1] * ooRhoL, vL = qL[2] * ooRhoL, uR = qR[1] * ooRhoR, vR = qR[2] * ooRhoR;
  const T EL = qL[3], ER = qR[3];
  const T UL = nx * uL + ny * vL, UR = nx * uR + ny * vR;
  const T pL = pressure(g, qL[0], qL[1], qL[2], qL[3]), pR = pressure(g, qR[0], qR[1], qR[2], qR[3]);
  const T HL = EL + pL, HR = ER + pR;
  const T ooRs = T(1) / (rhoLs + rhoRs);
  const T u = (rhoLs * uL + rhoRs * uR) * ooRs, v = (rhoLs * vL + rhoRs * vR) * ooRs;
  const T h = (HL + HR) * ooRs;
  const T rho = rhoLs * rhoRs;
  const T H = h * rho;
  const T U = nx * u + ny * v;
  const T C2 = g.gm1 * (h - T(0.5) * (u * u + v * v));
  const T C = dsqrt(C2);
  const T ooC = T(1) / C;
  const T Uabs = dabs(U);
  f[0] = T(0.5) * (UL * rhoL + UR * rhoR);
  f[1] = T(0.5) * (UL * rhoL * uL + pL * nx + UR * rhoR * uR + pR * nx);
  f[2] = T(0.5) * (UL * rhoL * vL + pL * ny + UR * rhoR * vR + pR * ny);
  f[3] = T(0.5) * (UL * HL + UR * HR);
  const T Uef = T(0.05) * C;
  const T du = uR - uL, dv = vR - vL;
  const T deltaV2 = du * du + dv * dv;
  const T ooVmag = T(1) / dsqrt(u * u + v * v);
  T n1x, n1y;
  if (deltaV2 < T(0.01) * C2) { n1x = nx; n1y = ny; }
  else { n1x = ooVmag * du; n1y = ooVmag * dv; }
  const T n2x = n1y * (nx * n1y - n1x * ny), n2y = -n1x * (nx * n1y - n1x * ny);
  const T alp1 = nx * n1x + ny * n1y, alp2 = nx * n2x + ny * n2y;
  const T U1x = n1x * u, U1y = n1y * v, U2x = n2x * u, U2y = n2y * v;
  const T Urot = dsqrt(alp1 * alp1 * (U1x * U1x + U1y * U1y)) +
                 dsqrt(alp2 * alp2 * (U2x * U2x + U2y * U2y));
  const T sigma = dmax(Uabs, dmin(Uef, Urot));
  const T UabsPrime = Uabs - T(0.25) * dmax(T(0), UR - UL) * (copysign_pos(U + C) - copysign_pos(U - C));
  const T dU = UR - UL, dP = pR - pL, dRho = rhoR - rhoL;
  const T dRhoU = rhoR * uR - rhoL * uL, dRhoV = rhoR * vR - rhoL * vL, dE = ER - EL;
  const T dPu = rho * dU * dmax(T(0), C - UabsPrime);
  const T swt = copysign_pos(U) * dmin(UabsPrime, C);
  const T dPp = swt * dP * ooC;
  const T dUu = swt * dU * ooC;
  f[0] -= T(0.5) * (sigma * dRho + (dPu + dPp) * T(0) + dUu * rho);
  f[1] -= T(0.5) * (sigma * dRhoU + (dPu + dPp) * nx + dUu * rho * u);
  f[2] -= T(0.5) * (sigma * dRhoV + (dPu + dPp) * ny + dUu * rho * v);
  f[3] -= T(0.5) * (sigma * dE + (dPu + dPp) * ny + dUu * H);
}

template <typename T>
__device__ __forceinline__ void riemann_flux(int kind, const Gas<T>& g, const T qL[4],
                                             const T qR[4], T nx, T ny, T f[4]) {
  switch (kind) {
    case kFluxAverage: flux_average(g, qL, qR, nx, ny, f); break;
    case kFluxLax: flux_lax(g, qL, qR, nx, ny, f); break;
    case kFluxRoeER: flux_roe_er(g, qL, qR, nx, ny, f); break;
    default: flux_roe(g, qL, qR, nx, ny, f); break;
  }
}

// Free-stream state used by a far-field style boundary (FreeStream, fluids.go:370-406).
template <typename T>
struct FreeStreamT {
  T qinf[4];
  T pinf, cinf, gamma, minf;
};

// Characteristic boundary state, RiemannBC (bcs.go:70-133).  QInf may differ
// from fs.qinf (IVortex passes the exact state) while pinf/cinf stay fs's.
// FewerPow uses p = rho C^2 / gamma, equal to Beta rho^gamma by construction
// (rho^(gamma-1) = C^2 / (gamma Beta)), which saves one pow per point.
template <typename T, bool FewerPow = false>
__device__ __forceinline__ void riemann_bc(const FreeStreamT<T>& fs, const T qi[4],
                                           const T QInf[4], T nx, T ny, T out[4]) {
  const T Gamma = fs.gamma, GM1 = Gamma - T(1), OOGM1 = T(1) / GM1;
  const Gas<T> g{Gamma, GM1, OOGM1};
  const T rhoInt = qi[0], uInt = qi[1] / qi[0], vInt = qi[2] / qi[0];
  const T pInt = pressure(g, qi[0], qi[1], qi[2], qi[3]);
  const T CInt = sound_speed(g, qi[0], qi[1], qi[2], qi[3]);
  const T rhoInf = QInf[0], uInf = QInf[1] / QInf[0], vInf = QInf[2] / QInf[0];
  const T tx = -ny, ty = nx;
  const T VnormInt = nx * uInt + ny * vInt;
  if (fs.minf <= T(1)) {
    const T VnormInf = nx * uInf + ny * vInf;
    const T Rinf = VnormInf - T(2) * fs.cinf * OOGM1;
    const T Rint = VnormInt + T(2) * CInt * OOGM1;
    const T Vnorm = T(0.5) * (Rint + Rinf);
    const T C = T(0.25) * GM1 * (Rint - Rinf);
    T Vtang, Beta;
    if (VnormInt < T(0)) {
      Vtang = tx * uInf + ty * vInf;
      Beta = fs.pinf / dpow(rhoInf, Gamma);
    } else {
      Vtang = tx * uInt + ty * vInt;
      Beta = pInt / dpow(rhoInt, Gamma);
    }
    const T u = Vnorm * nx + Vtang * tx;
    const T v = Vnorm * ny + Vtang * ty;
    const T rho = dpow(C * C / (Gamma * Beta), OOGM1);
    const T p = FewerPow ? rho * C * C / Gamma : Beta * dpow(rho, Gamma);
    out[0] = rho;
    out[1] = rho * u;
    out[2] = rho * v;
    out[3] = p * OOGM1 + T(0.5) * rho * (u * u + v * v);
  } else if (VnormInt < T(0)) {
#pragma unroll
    for (int n = 0; n < 4; ++n) out[n] = QInf[n];
  } else {
#pragma unroll
    for (int n = 0; n < 4; ++n) out[n] = qi[n];
  }
}

// Isentropic vortex exact state, IVortex.GetState/GetStateC
// (isentropic_vortex/analytic_vortex.go:31-82).
template <typename T>
__device__ __forceinline__ void ivortex_state(T beta, T x0, T y0, T gamma, T t, T x, T y,
                                              T out[4]) {
  const T pi = T(3.14159265358979323846);
  const T oo2pi = T(0.5) * (T(1) / pi);
  const T GM1 = gamma - T(1), OOGM1 = T(1) / GM1;
  const T fac = T(16) * gamma * (pi * pi);
  T u = T(1), v = T(0);
  const T xmut = x - u * t, ymvt = y - v * t;
  const T r2 = (xmut - x0) * (xmut - x0) + (ymvt - y0) * (ymvt - y0);
  const T ex1r = dexp(T(1) - r2);
  const T tv1 = T(1) - (GM1 * beta * beta * dexp(T(2) * (T(1) - r2)) / fac);
  u -= beta * ex1r * (ymvt - y0) * oo2pi;
  v += beta * ex1r * (xmut - x0) * oo2pi;
  const T rho = dpow(tv1, OOGM1);
  const T p = dpow(rho, gamma);
  const T q = T(0.5) * rho * (u * u + v * v);
  out[0] = rho;
  out[1] = rho * u;
  out[2] = rho * v;
  out[3] = p * (T(1) / (gamma - T(1))) + q;
}

}  // namespace gcfd
