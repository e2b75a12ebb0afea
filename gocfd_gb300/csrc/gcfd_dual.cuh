// Forward-mode dual numbers for the pointwise physics of euler_physics.cuh.
// Dual<M> carries a value and M tangents; instantiating the physics templates
// with T = Dual<M> gives their Jacobian columns exactly (to rounding), which
// the adjoint kernels use for the rarely executed pieces (boundary states,
// wave speeds, the Lax / average / Roe-ER fluxes).  The hot Roe and interior
// flux adjoints are written out in reverse mode in gcfd_adjoint.cuh.
#pragma once
#include "euler_physics.cuh"

namespace gcfd {

template <int M>
struct Dual {
  double v;
  double d[M];
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(double x) : v(x) {
#pragma unroll
    for (int i = 0; i < M; ++i) d[i] = 0.0;
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

template <int M>
__device__ __forceinline__ Dual<M> seed(double v, int i) {
  Dual<M> r(v);
  r.d[i] = 1.0;
  return r;
}

template <int M>
__device__ __forceinline__ Dual<M> operator-(const Dual<M>& a) {
  Dual<M> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int M>
__device__ __forceinline__ Dual<M> operator+(const Dual<M>& a, const Dual<M>& b) {
  Dual<M> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int M>
__device__ __forceinline__ Dual<M> operator-(const Dual<M>& a, const Dual<M>& b) {
  Dual<M> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int M>
__device__ __forceinline__ Dual<M> operator*(const Dual<M>& a, const Dual<M>& b) {
  Dual<M> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int M>
__device__ __forceinline__ Dual<M> operator/(const Dual<M>& a, const Dual<M>& b) {
  Dual<M> r;
  const double ib = 1.0 / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int M> __device__ __forceinline__ Dual<M> operator+(const Dual<M>& a, double b) { return a + Dual<M>(b); }
template <int M> __device__ __forceinline__ Dual<M> operator+(double a, const Dual<M>& b) { return Dual<M>(a) + b; }
template <int M> __device__ __forceinline__ Dual<M> operator-(const Dual<M>& a, double b) { return a - Dual<M>(b); }
template <int M> __device__ __forceinline__ Dual<M> operator-(double a, const Dual<M>& b) { return Dual<M>(a) - b; }
template <int M> __device__ __forceinline__ Dual<M> operator*(const Dual<M>& a, double b) {
  Dual<M> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int M> __device__ __forceinline__ Dual<M> operator*(double a, const Dual<M>& b) { return b * a; }
template <int M> __device__ __forceinline__ Dual<M> operator/(const Dual<M>& a, double b) { return a / Dual<M>(b); }
template <int M> __device__ __forceinline__ Dual<M> operator/(double a, const Dual<M>& b) { return Dual<M>(a) / b; }

template <int M> __device__ __forceinline__ bool operator<(const Dual<M>& a, const Dual<M>& b) { return a.v < b.v; }
template <int M> __device__ __forceinline__ bool operator>(const Dual<M>& a, const Dual<M>& b) { return a.v > b.v; }
template <int M> __device__ __forceinline__ bool operator<=(const Dual<M>& a, const Dual<M>& b) { return a.v <= b.v; }
template <int M> __device__ __forceinline__ bool operator>=(const Dual<M>& a, const Dual<M>& b) { return a.v >= b.v; }

// Elementary functions.  At the kinks (|x| at 0, sqrt at 0) the derivative is
// taken as 0, the value a central difference gives for |x|.
template <int M>
__device__ __forceinline__ Dual<M> dsqrt(Dual<M> x) {
  Dual<M> r;
  r.v = sqrt(x.v);
  const double s = r.v > 0.0 ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = s * x.d[i];
  return r;
}
template <int M>
__device__ __forceinline__ Dual<M> dabs(Dual<M> x) {
  const double s = x.v > 0.0 ? 1.0 : (x.v < 0.0 ? -1.0 : 0.0);
  Dual<M> r;
  r.v = fabs(x.v);
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = s * x.d[i];
  return r;
}
template <int M>
__device__ __forceinline__ Dual<M> dexp(Dual<M> x) {
  Dual<M> r;
  r.v = exp(x.v);
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = r.v * x.d[i];
  return r;
}
// x^y; the log term only when y carries a tangent (y is gamma or 1/(gamma-1)
// in every call here, so log(x) of a negative base is never formed).
template <int M>
__device__ __forceinline__ Dual<M> dpow(Dual<M> x, Dual<M> y) {
  Dual<M> r;
  r.v = pow(x.v, y.v);
  const double dx = y.v * pow(x.v, y.v - 1.0);
  bool ytan = false;
#pragma unroll
  for (int i = 0; i < M; ++i) ytan |= (y.d[i] != 0.0);
  const double dy = ytan ? r.v * log(x.v) : 0.0;
#pragma unroll
  for (int i = 0; i < M; ++i) r.d[i] = dx * x.d[i] + (ytan ? dy * y.d[i] : 0.0);
  return r;
}

template <int M>
__device__ __forceinline__ Gas<Dual<M>> dual_gas(const Gas<double>& g) {
  return Gas<Dual<M>>{Dual<M>(g.gamma), Dual<M>(g.gm1), Dual<M>(g.oogm1)};
}

}  // namespace gcfd
