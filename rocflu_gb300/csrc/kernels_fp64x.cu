// Kernel instantiation of the fp64x mode: FP64 in the reference's evaluation order without FMA contraction (-fmad=false): bit-exact with the CPU restatement.
#define RFLU_NS fp64x
#include "kernels.cuh"
#include "adjoint.cuh"
#include "ops.h"

namespace rflu {
const Ops<double> *opsFp64Exact() {
  using L = fp64x::Launch<double>;
  static const Ops<double> ops = {L::initState, L::initFromRef, L::gradLimit, L::faceFlux,  L::gatherRhs, L::gatherUpdate,
                                 L::timestep,  L::stepEnd,   L::stepStart, L::configure, L::tileGrid, fp64x::AdjointOps<double>::jvp, fp64x::AdjointOps<double>::vjp,
                                 fp64x::AdjointOps<double>::patchPressure, L::adjointSetup,
                                 L::updateFromRhs, L::addRhs, fp64x::AdjointOps<double>::limiterBranches};
  return &ops;
}
}  // namespace rflu
