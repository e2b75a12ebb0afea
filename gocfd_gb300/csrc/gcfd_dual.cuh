// Forward-mode dual numbers for the pointwise physics of euler_physics.cuh.
// Dual<M, S> carries a value and M tangents in S (double unless stated); instantiating the physics templates
// with T = Dual<M> gives their Jacobian columns exactly (to rounding), which
// the adjoint kernels use for the rarely executed pieces (boundary states,
// wave speeds, the Lax / average / Roe-ER fluxes).  The hot Roe and interior
// flux adjoints are written out in reverse mode in gcfd_adjoint.cuh.
#pragma once
#include "euler_physics.cuh"

namespace gcfd {

template <int M, typename S = double>
struct Dual {
  S v;
  S d[M];
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(double x) : v(static_cast<S>(x)) {
#pragma unroll
    for (int i = 0; i < M; ++i) d[i] = S(0);
  }
  __device__ __forceinline__ Dual& operator+=(const Dual& b) {
    v += b.v;
#pragma unroll
    for (int i = 0; i < M; ++i) d[i] += b.d[i];
    return *this;
  }
  __device__ __forceinline__ Dual& operator-=(const Dual& b) {
    v -= b.v;
#pragma unroll
    for (int i = 0; i < M; ++i) d[i] -= b.d[i];
    return *this;
  }
};

template <int M, typename S = double>
__device__ __forceinline__ Dual<M, S> seed(double v, int i) {
  Dual<M, S> r(v);
  r.d[i] = S(1);
  return r;
}

template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator-(const Dual<M, S>& a) {
  Dual<M, S> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator+(const Dual<M, S>& a, const Dual<M, S>& b) {
  Dual<M, S> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator-(const Dual<M, S>& a, const Dual<M, S>& b) {
  Dual<M, S> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator*(const Dual<M, S>& a, const Dual<M, S>& b) {
  Dual<M, S> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator/(const Dual<M, S>& a, const Dual<M, S>& b) {
  Dual<M, S> r;
  const S ib = S(1) / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator+(const Dual<M, S>& a, double b) { return a + Dual<M, S>(b); }
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator+(double a, const Dual<M, S>& b) { return Dual<M, S>(a) + b; }
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator-(const Dual<M, S>& a, double b) { return a - Dual<M, S>(b); }
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator-(double a, const Dual<M, S>& b) { return Dual<M, S>(a) - b; }
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator*(const Dual<M, S>& a, double b) {
  const S c = static_cast<S>(b);
  Dual<M, S> r;
  r.v = a.v * c;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = a.d[i] * c;
  return r;
}
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator*(double a, const Dual<M, S>& b) { return b * a; }
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator/(const Dual<M, S>& a, double b) { return a / Dual<M, S>(b); }
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> operator/(double a, const Dual<M, S>& b) { return Dual<M, S>(a) / b; }

template <int M, typename S>
__device__ __forceinline__ bool operator<(const Dual<M, S>& a, const Dual<M, S>& b) { return a.v < b.v; }
template <int M, typename S>
__device__ __forceinline__ bool operator>(const Dual<M, S>& a, const Dual<M, S>& b) { return a.v > b.v; }
template <int M, typename S>
__device__ __forceinline__ bool operator<=(const Dual<M, S>& a, const Dual<M, S>& b) { return a.v <= b.v; }
template <int M, typename S>
__device__ __forceinline__ bool operator>=(const Dual<M, S>& a, const Dual<M, S>& b) { return a.v >= b.v; }

// Elementary functions.  At the kinks (|x| at 0, sqrt at 0) the derivative is
// taken as 0, the value a central difference gives for |x|.
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> dsqrt(Dual<M, S> x) {
  Dual<M, S> r;
  r.v = sqrt(x.v);
  const S s = r.v > S(0) ? S(0.5) / r.v : S(0);
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = s * x.d[i];
  return r;
}
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> dabs(Dual<M, S> x) {
  const S s = x.v > S(0) ? S(1) : (x.v < S(0) ? S(-1) : S(0));
  Dual<M, S> r;
  r.v = fabs(x.v);
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = s * x.d[i];
  return r;
}
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> dexp(Dual<M, S> x) {
  Dual<M, S> r;
  r.v = exp(x.v);
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = r.v * x.d[i];
  return r;
}
// x^y; the log term only when y carries a tangent (y is gamma or 1/(gamma-1)
// in every call here, so log(x) of a negative base is never formed).
template <int M, typename S>
__device__ __forceinline__ Dual<M, S> dpow(Dual<M, S> x, Dual<M, S> y) {
  Dual<M, S> r;
  r.v = pow(x.v, y.v);
  const S dx = y.v * pow(x.v, y.v - S(1));
  bool ytan = false;
#pragma unroll
  for (int i = 0; i < M; ++i) ytan |= (y.d[i] != S(0));
  const S dy = ytan ? r.v * log(x.v) : S(0);
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = dx * x.d[i] + (ytan ? dy * y.d[i] : S(0));
  return r;
}

template <int M, typename S = double>
__device__ __forceinline__ Gas<Dual<M, S>> dual_gas(const Gas<double>& g) {
  return Gas<Dual<M, S>>{Dual<M, S>(g.gamma), Dual<M, S>(g.gm1), Dual<M, S>(g.oogm1)};
}

}  // namespace gcfd
