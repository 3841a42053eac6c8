// Tangent and adjoint of the residual (filled in by the adjoint kernels).
#pragma once
namespace rflu {
namespace RFLU_NS {
template <typename R>
struct AdjointOps {
  static constexpr void (*jvp)(const View<R> &, const double *, double *, double *, cudaStream_t) = nullptr;
  static constexpr void (*vjp)(const View<R> &, const double *, double *, double *, cudaStream_t) = nullptr;
  static constexpr void (*patchPressure)(const View<R> &, int, double *, double *, double *, cudaStream_t) = nullptr;
};
}  // namespace RFLU_NS
}  // namespace rflu
