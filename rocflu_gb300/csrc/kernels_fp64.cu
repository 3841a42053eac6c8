// Kernel instantiation of the fp64 mode: FP64, fused multiply-add allowed (-fmad=true).
#define RFLU_NS fp64
#include "kernels.cuh"
#include "adjoint.cuh"
#include "ops.h"

namespace rflu {
const Ops<double> *opsFp64() {
  using L = fp64::Launch<double>;
  static const Ops<double> ops = {L::initState, L::initFromRef, L::gradLimit, L::faceFlux,  L::gatherRhs, L::gatherUpdate,
                                 L::timestep,  L::stepEnd,   L::stepStart, L::configure, L::tileGrid, fp64::AdjointOps<double>::jvp, fp64::AdjointOps<double>::vjp,
                                 fp64::AdjointOps<double>::patchPressure, L::adjointSetup,
                                 L::updateFromRhs, L::addRhs, fp64::AdjointOps<double>::limiterBranches};
  return &ops;
}
}  // namespace rflu
