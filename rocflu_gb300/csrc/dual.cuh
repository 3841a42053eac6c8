// Forward-mode dual numbers: a value and N directional derivatives.  The
// point-wise physics of physics.cuh is generic in its scalar type, so the same
// flux, reconstruction and limiter code evaluated on Dual<N> gives exact
// local Jacobians (tangent kernels) and, for N inputs of a face, the rows of
// the transposed flux Jacobian (adjoint kernels).  Comparisons and branch
// decisions use the value only: derivatives follow the active branch.
#pragma once
#include <cmath>

namespace rflu {

template <int N>
struct Dual {
  double v;
  double d[N];
  __host__ __device__ Dual() : v(0.0) {
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = 0.0;
  }
  __host__ __device__ Dual(double x) : v(x) {  // NOLINT: constants promote implicitly
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = 0.0;
  }
  __host__ __device__ static Dual seed(double x, int k) {
    Dual r(x);
    r.d[k] = 1.0;
    return r;
  }
};

#define RFLU_DUAL_BINOP(op, expr_d)                                                      \
  template <int N>                                                                       \
  __host__ __device__ inline Dual<N> operator op(const Dual<N> &a, const Dual<N> &b) {   \
    Dual<N> r;                                                                           \
    r.v = a.v op b.v;                                                                    \
    _Pragma("unroll") for (int k = 0; k < N; ++k) r.d[k] = expr_d;                       \
    return r;                                                                            \
  }
RFLU_DUAL_BINOP(+, a.d[k] + b.d[k])
RFLU_DUAL_BINOP(-, a.d[k] - b.d[k])
RFLU_DUAL_BINOP(*, a.d[k] * b.v + a.v * b.d[k])
#undef RFLU_DUAL_BINOP

template <int N>
__host__ __device__ inline Dual<N> operator/(const Dual<N> &a, const Dual<N> &b) {
  Dual<N> r;
  const double ib = 1.0 / b.v;
  r.v = a.v / b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N> &a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int N> __host__ __device__ inline bool operator<(const Dual<N> &a, const Dual<N> &b) { return a.v < b.v; }
template <int N> __host__ __device__ inline bool operator>(const Dual<N> &a, const Dual<N> &b) { return a.v > b.v; }
template <int N> __host__ __device__ inline bool operator<=(const Dual<N> &a, const Dual<N> &b) { return a.v <= b.v; }
template <int N> __host__ __device__ inline bool operator>=(const Dual<N> &a, const Dual<N> &b) { return a.v >= b.v; }
template <int N> __host__ __device__ inline bool operator==(const Dual<N> &a, const Dual<N> &b) { return a.v == b.v; }
template <int N> __host__ __device__ inline bool operator!=(const Dual<N> &a, const Dual<N> &b) { return a.v != b.v; }

template <int N>
__host__ __device__ inline Dual<N> sqrt_(const Dual<N> &a) {
  Dual<N> r;
  r.v = sqrt(a.v);
  const double h = (r.v > 0.0) ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * h;
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> fabs_(const Dual<N> &a) {
  return (a.v < 0.0) ? -a : a;
}
template <int N>
__host__ __device__ inline Dual<N> copysign_(const Dual<N> &a, const Dual<N> &b) {
  // d/db copysign(a, b) = 0 away from b = 0
  const bool flip = (signbit(a.v) != signbit(b.v));
  return flip ? -a : a;
}

template <typename S> struct ValueOf { __host__ __device__ static double get(const S &x) { return (double)x; } };
template <int N> struct ValueOf<Dual<N>> { __host__ __device__ static double get(const Dual<N> &x) { return x.v; } };

}  // namespace rflu
