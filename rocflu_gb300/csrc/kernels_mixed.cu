// Kernel instantiation of the mixed mode: FP32 state, gradients and fluxes; FP64 master cv, pressure/sound-speed recovery, checks and RK combination.
#define RFLU_NS mixed
#include "kernels.cuh"
#include "adjoint.cuh"
#include "ops.h"

namespace rflu {
const Ops<float> *opsMixed() {
  using L = mixed::Launch<float>;
  static const Ops<float> ops = {L::initState, L::initFromRef, L::gradLimit, L::faceFlux,  L::gatherRhs, L::gatherUpdate,
                                 L::timestep,  L::stepEnd,   L::stepStart, L::configure, L::tileGrid, mixed::AdjointOps<float>::jvp, mixed::AdjointOps<float>::vjp,
                                 mixed::AdjointOps<float>::patchPressure, L::adjointSetup};
  return &ops;
}
}  // namespace rflu
