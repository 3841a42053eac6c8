// Launcher table of one precision mode.  Each kernel translation unit
// (kernels_fp64.cu, kernels_fp64x.cu, kernels_mixed.cu) fills one table; the
// C ABI picks the table from rflu_num_desc::precision.
#pragma once
#include <cuda_runtime.h>

#include "ctx.h"

namespace rflu {

template <typename R>
struct Ops {
  void (*initState)(const View<R> &, cudaStream_t);
  // permute-in + initState of the reference cells o0 .. o1-1
  void (*initFromRef)(const View<R> &, const double *cvRef, int o0, int o1, cudaStream_t);
  void (*gradLimit)(const View<R> &, cudaStream_t);
  void (*faceFlux)(const View<R> &, cudaStream_t);
  void (*gatherRhs)(const View<R> &, cudaStream_t);
  void (*gatherUpdate)(const View<R> &, int, const double *, cudaStream_t);
  void (*timestep)(const View<R> &, cudaStream_t);
  void (*stepEnd)(const View<R> &, cudaStream_t);
  void (*stepStart)(const View<R> &, cudaStream_t);  // dt reduction + first-stage gradients
  void (*configure)(const View<R> &);                  // mesh-dependent kernel attributes
  int (*tileGrid)(const View<R> &, int withDt);        // CTAs of the persistent tiled kernels
  // tangent / adjoint of the residual (FP64 modes only; null elsewhere)
  void (*jvp)(const View<R> &, const double *cvDot, double *rhsDot, double *work, cudaStream_t);
  void (*vjp)(const View<R> &, const double *rhsBar, double *cvBar, double *work, cudaStream_t);
  void (*patchPressure)(const View<R> &, int iPatch, double *J, double *cvBar, double *work, cudaStream_t);
  // fills the adjoint's mesh-dependent arrays (View::tsW) once they exist
  void (*adjointSetup)(const View<R> &, cudaStream_t);
  // RKUpdateMP + RFLU_SetVarsContWrapper + AfterUpdateMP from View::rhs
  void (*updateFromRhs)(const View<R> &, int, const double *, cudaStream_t);
  // View::rhs += a (5,nCells) array in the reference's cell order
  void (*addRhs)(const View<R> &, const double *, cudaStream_t);
  // the limiter's active branches of every cell (second order; adjoint.cuh)
  void (*limiterBranches)(const View<R> &, int *, double *work, cudaStream_t);
};

// The mixed mode's Newton-refined FP64 reciprocal and square root against
// IEEE FP64 division and sqrt on n generated values: the largest relative
// errors (kernels_mixed.cu).
cudaError_t mixedRefineCheck(long long n, unsigned long long seed, double *maxRel);

const Ops<double> *opsFp64();
const Ops<double> *opsFp64Exact();
const Ops<float> *opsMixed();

}  // namespace rflu
