// Kernel instantiation of the mixed mode: FP32 state, gradients and fluxes; FP64 master cv, pressure/sound-speed recovery, checks and RK combination.
#define RFLU_NS mixed
#include "kernels.cuh"
#include "adjoint.cuh"
#include "ops.h"

#include <cstring>

namespace rflu {
// rflu_gpu_check_refinements: kRefineCheck compiled with this unit's flags.
cudaError_t mixedRefineCheck(long long n, unsigned long long seed, double *maxRel) {
  unsigned long long *d = nullptr, h[2] = {0, 0};
  cudaError_t e = cudaMalloc(&d, sizeof h);
  if (e != cudaSuccess) return e;
  e = cudaMemset(d, 0, sizeof h);
  if (e == cudaSuccess) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    mixed::kRefineCheck<<<sms * 8, 256>>>(n, seed, 100, d);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  }
  cudaFree(d);
  for (int k = 0; k < 2; ++k) std::memcpy(&maxRel[k], &h[k], sizeof(double));
  return e;
}

const Ops<float> *opsMixed() {
  using L = mixed::Launch<float>;
  static const Ops<float> ops = {L::initState, L::initFromRef, L::gradLimit, L::faceFlux,  L::gatherRhs, L::gatherUpdate,
                                 L::timestep,  L::stepEnd,   L::stepStart, L::configure, L::tileGrid, mixed::AdjointOps<float>::jvp, mixed::AdjointOps<float>::vjp,
                                 mixed::AdjointOps<float>::patchPressure, L::adjointSetup,
                                 L::updateFromRhs, L::addRhs, mixed::AdjointOps<float>::limiterBranches};
  return &ops;
}
}  // namespace rflu
