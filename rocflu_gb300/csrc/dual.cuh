// Forward-mode dual numbers: a value and N directional derivatives.  The
// point-wise physics of physics.cuh is generic in its scalar type, so the same
// flux, reconstruction and limiter code evaluated on Dual<N> gives exact
// local Jacobians (tangent kernels) and, for N inputs of a face, the rows of
// the transposed flux Jacobian (adjoint kernels).  Comparisons and branch
// decisions use the value only: derivatives follow the active branch.
#pragma once
#include <cmath>

namespace rflu {

// T is the arithmetic type of value and derivatives: double in the FP64
// modes, float for the mixed mode's flux and limiter Jacobians.
template <int N, typename T = double>
struct Dual {
  T v;
  T d[N];
  __host__ __device__ Dual() : v(T(0)) {
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = T(0);
  }
  __host__ __device__ Dual(double x) : v(T(x)) {  // NOLINT: constants promote implicitly
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = T(0);
  }
  __host__ __device__ static Dual seed(double x, int k) {
    Dual r(x);
    r.d[k] = T(1);
    return r;
  }
  // rounding between arithmetic types (the mixed mode's FP64 first-order
  // paths feeding FP32 fluxes)
  template <typename U>
  __host__ __device__ explicit Dual(const Dual<N, U> &o) : v(T(o.v)) {
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = T(o.d[k]);
  }
};

#define RFLU_DUAL_BINOP(op, expr_d)                                                                \
  template <int N, typename T>                                                                     \
  __host__ __device__ inline Dual<N, T> operator op(const Dual<N, T> &a, const Dual<N, T> &b) {    \
    Dual<N, T> r;                                                                                  \
    r.v = a.v op b.v;                                                                    \
    _Pragma("unroll") for (int k = 0; k < N; ++k) r.d[k] = expr_d;                       \
    return r;                                                                            \
  }
RFLU_DUAL_BINOP(+, a.d[k] + b.d[k])
RFLU_DUAL_BINOP(-, a.d[k] - b.d[k])
RFLU_DUAL_BINOP(*, a.d[k] * b.v + a.v * b.d[k])
#undef RFLU_DUAL_BINOP

template <int N, typename T>
__host__ __device__ inline Dual<N, T> operator/(const Dual<N, T> &a, const Dual<N, T> &b) {
  Dual<N, T> r;
  const T ib = T(1) / b.v;
  r.v = a.v / b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <int N, typename T>
__host__ __device__ inline Dual<N, T> operator-(const Dual<N, T> &a) {
  Dual<N, T> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int N, typename T> __host__ __device__ inline bool operator<(const Dual<N, T> &a, const Dual<N, T> &b) { return a.v < b.v; }
template <int N, typename T> __host__ __device__ inline bool operator>(const Dual<N, T> &a, const Dual<N, T> &b) { return a.v > b.v; }
template <int N, typename T> __host__ __device__ inline bool operator<=(const Dual<N, T> &a, const Dual<N, T> &b) { return a.v <= b.v; }
template <int N, typename T> __host__ __device__ inline bool operator>=(const Dual<N, T> &a, const Dual<N, T> &b) { return a.v >= b.v; }
template <int N, typename T> __host__ __device__ inline bool operator==(const Dual<N, T> &a, const Dual<N, T> &b) { return a.v == b.v; }
template <int N, typename T> __host__ __device__ inline bool operator!=(const Dual<N, T> &a, const Dual<N, T> &b) { return a.v != b.v; }

template <int N, typename T>
__host__ __device__ inline Dual<N, T> sqrt_(const Dual<N, T> &a) {
  Dual<N, T> r;
  r.v = sqrt(a.v);
  const T h = (r.v > T(0)) ? T(0.5) / r.v : T(0);
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * h;
  return r;
}
// x ** y with y a constant of the gas model: d(x^y) = y x^(y-1) dx
template <int N, typename T>
__host__ __device__ inline Dual<N, T> powConstExp(const Dual<N, T> &a, const Dual<N, T> &y) {
  Dual<N, T> r;
  r.v = pow(a.v, y.v);
  const T s = y.v * pow(a.v, y.v - T(1));
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * s;
  return r;
}
template <int N, typename T>
__host__ __device__ inline Dual<N, T> fabs_(const Dual<N, T> &a) {
  return (a.v < T(0)) ? -a : a;
}
template <int N, typename T>
__host__ __device__ inline Dual<N, T> copysign_(const Dual<N, T> &a, const Dual<N, T> &b) {
  // d/db copysign(a, b) = 0 away from b = 0
  const bool flip = (signbit(a.v) != signbit(b.v));
  return flip ? -a : a;
}

template <typename S> struct ValueOf { __host__ __device__ static double get(const S &x) { return (double)x; } };
template <int N, typename T> struct ValueOf<Dual<N, T>> {
  __host__ __device__ static double get(const Dual<N, T> &x) { return (double)x.v; }
};

}  // namespace rflu
