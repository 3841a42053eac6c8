// C ABI of the device path (include/rflu_gpu.h): context creation (cell
// renumbering, CSR structures, least-squares weights), state transfer and the
// stage / step / residual drivers.  Kernels live in kernels_*.cu.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rflu_gpu.h"
#include "args.h"
#include "convert.cuh"
#include "constr.h"
#include "ctx.h"
#include "errors.h"
#include "ops.h"
#include "tiles.h"

namespace rflu {

std::string &lastError() {
  static thread_local std::string msg;
  return msg;
}

namespace {

#define RFLU_CUDA(call)                                                                       \
  do {                                                                                        \
    cudaError_t err_ = (call);                                                                \
    if (err_ != cudaSuccess)                                                                  \
      return fail(RFLU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_));       \
  } while (0)

// --- small device helpers of the ABI --------------------------------------
__global__ void kSetScalars(Scalars *sc, double time, double endTime, int resetCounters) {
  sc->time = time;
  sc->endTime = endTime;
  sc->finished = 0;
  sc->stepsDone = 0;
  if (resetCounters) {
    sc->nanCells = sc->posFixCells = sc->negPCells = 0;
    sc->firstBadCell = INT_MAX;
  }
}
__global__ void kSetDt(Scalars *sc, double dt) {
  sc->dtMin = dt;
  sc->finished = 0;
}
// cv(5,nc) in reference order (column-major) -> SoA renumbered
__global__ void kPermuteIn(const double *src, double *dst, const int *refId, int nc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  int o = refId[i];
#pragma unroll
  for (int k = 0; k < 5; ++k) dst[(size_t)k * nc + i] = src[5 * (size_t)o + k];
}
// Renumbered per-cell data (component k of cell i at src[k*kStride +
// i*iStride]) -> reference column-major double
template <typename T>
__global__ void kPermuteOut(const T *src, double *dst, const int *refId, int nc, int ncomp, size_t kStride,
                            size_t iStride) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  int o = refId[i];
  for (int k = 0; k < ncomp; ++k) dst[(size_t)ncomp * o + k] = (double)src[k * kStride + i * iStride];
}

inline int nblk(long long n) { return (int)((n + 255) / 256); }

// Reverse sweep of the RK combination (time-unrolled adjoint): the seed of
// stage s's residual VJP, sigma = sum_t coef_t / vol * lambda_t, per cell in
// the reference layout (5 per cell); coef_t = ark_t * dt * W[t][s].
struct SeedTerms {
  const double *lam[5];
  double coef[5];
  int n;
};
__global__ void kStageSeed(double *sigma, SeedTerms T, const double *vol, const int *refId, int nc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const size_t o = (size_t)refId[i];
  const double iv = 1.0 / vol[i];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    double s = 0.0;
    for (int t = 0; t < T.n; ++t) s += T.coef[t] * T.lam[t][5 * o + k];
    sigma[5 * o + k] = s * iv;
  }
}
__global__ void kSubInto(double *out, const double *a, const double *b, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}
__global__ void kAxpyInPlace(double *y, double a, const double *x, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}
__global__ void kAccumJ(double *acc, const double *j, double dt) { *acc += dt * *j; }

// Download: renumbered SoA (ncomp rows) -> reference order and layout, one
// thread per reference cell o0 .. o1-1 so that the writes to `dst` are
// contiguous.
__global__ void kGatherOut(const double *src, double *dst, const int *newId, int nc, int ncomp, int o0, int o1) {
  const int o = o0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= o1) return;
  const int i = newId[o];
  for (int k = 0; k < ncomp; ++k) dst[(size_t)ncomp * o + k] = src[(size_t)k * nc + i];
}

// T and c of RFLU_SetDependentVars (TCPERF) from cv and p, for a mixed-mode
// context whose steps store p only.
__global__ void kDvFill(const double *cv, double *dv, int nc, double gcR, double gRT) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const double r = cv[i], p = dv[i];
  const double t = p / (r * gcR);
  dv[(size_t)nc + i] = t;
  dv[2 * (size_t)nc + i] = sqrt(gRT * gcR * t);
}

// Scratch of rflu_gpu_residual_static: a fixed device array in this file, so
// that the call allocates nothing.  Every GPU that loads the library keeps
// these 64 MiB until the process exits.  All calls share it (see the header).
constexpr size_t kStaticScratchBytes = size_t(64) << 20;
__device__ __align__(256) unsigned char gStaticScratch[kStaticScratchBytes];

// Device address of gStaticScratch, looked up once per device with that
// device current (host code cannot use the symbol itself as an address).
int staticScratchAddress(void **out) {
  static std::mutex mu;
  static void *addr[128] = {};
  int dev = 0;
  RFLU_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return fail(RFLU_ERR_ARG, "rflu_gpu_residual_static: device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    RFLU_CUDA(cudaGetSymbolAddress(&p, gStaticScratch));
    addr[dev] = p;
  }
  *out = addr[dev];
  return RFLU_OK;
}

// The kind of memory p points to and the device it lives on.
ArgMem pointerKind(const void *p, int *device) {
  cudaPointerAttributes a;
  *device = -1;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return ArgMem::Unknown;
  }
  *device = a.device;
  if (a.type == cudaMemoryTypeDevice) return ArgMem::Device;
  if (a.type == cudaMemoryTypeManaged) return ArgMem::Managed;
  if (a.type == cudaMemoryTypeHost) return ArgMem::Host;
  return ArgMem::Unknown;
}

// FP64 FMA throughput probe: 8 independent chains per thread.
__device__ double gFmaSink;
// Self-check of f2d/d2f against the hardware conversions.  Value k of the
// sample: a 64-bit hash of (seed, k); by k mod 4 its bits as a double, a
// double with an exponent near the float range (normal, denormal and
// overflowing results), the same with the 29 bits dropped by the rounding set
// to a tie, or a float (its hash bits) widened, plus the midpoint between it
// and the next float up.
__device__ inline unsigned long long mix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__device__ inline bool sameFloat(float a, float b) {
  return __float_as_uint(a) == __float_as_uint(b) || (isnan(a) && isnan(b));
}
__global__ void kCvtCheck(long long n, unsigned long long seed, unsigned long long *bad) {
  unsigned long long miss = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const unsigned long long h = mix64(seed ^ mix64((unsigned long long)k));
    const int mode = (int)(k & 3);
    if (mode < 3) {
      unsigned long long bits = h;
      if (mode >= 1) {
        const unsigned long long e = (h >> 40) % 340 + (1023 - 190);
        bits = (h & 0x800FFFFFFFFFFFFFull) | (e << 52);
        if (mode == 2) bits = (bits & ~0x1FFFFFFFull) | 0x10000000ull;
      }
      const double d = __longlong_as_double((long long)bits);
      if (!sameFloat(d2f(d), __double2float_rn(d))) ++miss;
    } else {
      const float f = __uint_as_float((unsigned)(h >> 32));
      const double w = f2d(f);
      if (__double_as_longlong(w) != __double_as_longlong((double)f) && !(isnan(f) && isnan(w))) ++miss;
      if (isfinite(f) && fabsf(f) < 3.0e38f) {
        const double up = (double)__uint_as_float(__float_as_uint(f) + (f >= 0.f ? 1u : 0u) - (f < 0.f ? 1u : 0u));
        const double mid = (double)f + (up - (double)f) * 0.5;
        if (!sameFloat(d2f(mid), __double2float_rn(mid))) ++miss;
        if (!sameFloat(d2f(w), f)) ++miss;
      }
    }
  }
  if (miss) atomicAdd(bad, miss);
}

__global__ void kFp64Fma(int iters, double seed) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed * (threadIdx.x + k);
  const double b = 0.9999999999, c = 1.0e-12;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 12345.678) gFmaSink = s;  // keeps the chains alive
}

// Morton (Z-order) key of a point in the unit box of the mesh, 21 bits/axis.
inline uint64_t spread3(uint64_t x) {
  x &= 0x1fffff;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

}  // namespace

// Base of the per-precision contexts; the C ABI calls these.
struct CtxBase {
  virtual ~CtxBase() {}
  virtual int upload(const double *cv) = 0;
  virtual int download(double *cv, double *dv) = 0;
  virtual int timestep(double t, double *dt) = 0;
  virtual int rkStage(int iStage, double dt) = 0;
  virtual int rungeKutta(double dt) = 0;
  virtual int step(int nSteps, double *time, double endTime, int *done) = 0;
  virtual int runFixedDt(int nSteps, double dt) = 0;
  virtual int residual(const double *cv, double *rhs, double *grad) = 0;
  virtual int vjp(const double *cv, const double *rhsBar, double *cvBar) = 0;
  virtual int jvp(const double *cv, const double *cvDot, double *rhsDot) = 0;
  virtual int patchPressure(const double *cv, int iPatch, double *J, double *cvBar) = 0;
  virtual int status(rflu_status *s) = 0;
  virtual int kernelTimes(int nIter, double *ms) = 0;
  virtual int residualStatic(const double *cvDev, double *rhsDev) = 0;
  virtual int cellGradients() = 0;
  virtual int convectiveFluxes() = 0;
  virtual int addRhs(const double *src, int onDevice) = 0;
  virtual int rkUpdate(int iStage, double dt) = 0;
  virtual int getRhs(double *rhs, int onDevice) = 0;
  virtual int getGrad(double *grad, int onDevice) = 0;
  virtual int limiterBranches(const double *cv, int *branches) = 0;
  virtual int adjointTimes(int nIter, double *ms) = 0;
  virtual int unrolledAdjoint(const double *cv0, int nSteps, double dt, int every, int iPatch, double *J,
                              double *cvBar0, double *stats) = 0;
  cudaStream_t stream = nullptr;
  int device = -1;  // the device the context was created on
  // host transfers: the copy stream and one event per chunk (+ one)
  static constexpr int kMaxChunks = 8;
  cudaStream_t copyStream = nullptr;
  cudaEvent_t chunkEv[kMaxChunks + 1] = {};
};

template <typename R>
struct Ctx : CtxBase {
  View<R> V{};
  const Ops<R> *ops = nullptr;
  std::vector<void *> allocs;
  double *staging = nullptr;     // (15, nc) doubles: transfers in reference order
  bool imageMesh = false;        // the grid came with periodic or symmetry images (fc2 / c2csShift / c2csXf)
  bool constrBurning = false;    // a constrained gradient (CRECONSTC 1) holds a burning injection face's row (cpOff/cpEnt)
  double *work = nullptr;        // adjoint workspace (allocated by the first adjoint call)
  int tsWidthLazy = 0;           // ... and the width of its transposed-stencil weights
  size_t workBytes = 0;
  // scratch state (allocated by the first call that needs it): master cv,
  // dependent variables, primitive records, RK accumulator and scalars of the
  // states that the residual, tangent, adjoint, functional and diagnostic
  // calls evaluate, so that those calls leave the context's own state as it
  // was, bit for bit
  double *sCv = nullptr, *sDv = nullptr;
  R *sPrim = nullptr, *sRhsSum = nullptr;
  Scalars *sSc = nullptr;
  cudaGraphExec_t stepGraph = nullptr, fixedGraph = nullptr;
  long long lastNan = 0;

  ~Ctx() override {
    if (stepGraph) cudaGraphExecDestroy(stepGraph);
    if (fixedGraph) cudaGraphExecDestroy(fixedGraph);
    for (void *p : allocs) cudaFree(p);
    for (auto &e : chunkEv)
      if (e) cudaEventDestroy(e);
    if (copyStream) cudaStreamDestroy(copyStream);
    if (stream) cudaStreamDestroy(stream);
  }

  size_t bytesHeld = 0;          // device bytes of the context's own arrays

  template <typename T>
  int alloc(T **p, size_t n) {
    void *q = nullptr;
    RFLU_CUDA(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
    bytesHeld += std::max<size_t>(n, 1) * sizeof(T);
    allocs.push_back(q);
    *p = (T *)q;
    return RFLU_OK;
  }
  template <typename T, typename S>
  int put(const T **dst, const std::vector<S> &src) {
    std::vector<T> tmp(src.begin(), src.end());
    T *d = nullptr;
    int rc = alloc(&d, tmp.size());
    if (rc) return rc;
    if (!tmp.empty()) RFLU_CUDA(cudaMemcpy(d, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice));
    *dst = d;
    return RFLU_OK;
  }

  int create(const rflu_grid_desc *g, const rflu_num_desc *num);
  int patchConstants(const rflu_grid_desc *g, int ip, const rflu_num_desc *num, int *bcOpt, double *K);
  int buildTiles(const std::vector<int> &cfOff, const std::vector<int> &cfEnt, const std::vector<int> &stOff,
                 const std::vector<int> &stIdx, const std::vector<int> &fc1, const std::vector<int> &fc2,
                 const std::vector<double> &fnx, const std::vector<double> &fny, const std::vector<double> &fnz,
                 const std::vector<double> &fnm, const std::vector<double> &dL, const std::vector<double> &dR,
                 const std::vector<double> &bnx, const std::vector<double> &bny, const std::vector<double> &bnz,
                 const std::vector<double> &bnm, const std::vector<double> &bd);
  int checkLaunch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(RFLU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return RFLU_OK;
  }
  int syncEvents(bool events) {
    RFLU_CUDA(cudaStreamSynchronize(stream));
    if (!events) return RFLU_OK;
    Scalars s;
    RFLU_CUDA(cudaMemcpy(&s, V.sc, sizeof(Scalars), cudaMemcpyDeviceToHost));
    if ((long long)s.nanCells > lastNan) {
      lastNan = (long long)s.nanCells;
      return RFLU_EVENT_NAN;
    }
    return RFLU_OK;
  }
  void stageKernels(int iStage) { stageKernelsOf(V, iStage); }
  void stageKernelsOf(const View<R> &X, int iStage) {
    ops->gradLimit(X, stream);
    ops->faceFlux(X, stream);
    ops->gatherUpdate(X, iStage, &X.sc->dtMin, stream);
  }
  // A view on the scratch state (its arrays allocated on first use); the
  // mesh, geometry and the between-kernel arrays (gradients, face fluxes,
  // residual) are the context's.  copyState: start from a copy of the
  // context's state and scalars.
  int scratchView(View<R> *W, bool copyState) {
    const size_t nc = V.nc;
    if (!sCv) {
      int rc = 0;
      if ((rc = alloc(&sCv, 5 * nc)) || (rc = alloc(&sDv, 3 * nc)) || (rc = alloc(&sPrim, Layout<R>::prim * nc)) ||
          (rc = alloc(&sRhsSum, 5 * nc)) || (rc = alloc(&sSc, 1)))
        return rc;
    }
    *W = V;
    W->cv = sCv;
    W->dv = sDv;
    W->prim = sPrim;
    W->rhsSum = sRhsSum;
    W->sc = sSc;
    RFLU_CUDA(cudaMemcpyAsync(sSc, V.sc, sizeof(Scalars), cudaMemcpyDeviceToDevice, stream));
    if (copyState) {
      RFLU_CUDA(cudaMemcpyAsync(sCv, V.cv, sizeof(double) * 5 * nc, cudaMemcpyDeviceToDevice, stream));
      RFLU_CUDA(cudaMemcpyAsync(sDv, V.dv, sizeof(double) * 3 * nc, cudaMemcpyDeviceToDevice, stream));
      RFLU_CUDA(cudaMemcpyAsync(sPrim, V.prim, sizeof(R) * Layout<R>::prim * nc, cudaMemcpyDeviceToDevice, stream));
      RFLU_CUDA(cudaMemcpyAsync(sRhsSum, V.rhsSum, sizeof(R) * 5 * nc, cudaMemcpyDeviceToDevice, stream));
    }
    return RFLU_OK;
  }
  // Host <-> device transfers in reference order go through the staging
  // buffer in chunks of reference cells: chunk c's copy runs on copyStream
  // while the kernel of chunk c-1 (permute + state set-up, or the reference-
  // order gather) runs on the stream, so that only one chunk's kernel is
  // not hidden behind the copies (the copy engines move pinned buffers at
  // ~200 GB/s; kernels reading the host buffer directly measured 2x slower).
  int nChunks() const { return V.nc >= (1 << 18) ? kMaxChunks : 1; }
  int chunkBegin(int c) const { return (int)(((long long)V.nc * c) / nChunks()); }
  int setState(const double *cv) { return setStateOf(V, cv); }
  int setStateOf(const View<R> &X, const double *cv) {
    const int K = nChunks();
    // staging is free once the work queued on the stream so far is done
    RFLU_CUDA(cudaEventRecord(chunkEv[kMaxChunks], stream));
    RFLU_CUDA(cudaStreamWaitEvent(copyStream, chunkEv[kMaxChunks], 0));
    for (int c = 0; c < K; ++c) {
      const int o0 = chunkBegin(c), o1 = chunkBegin(c + 1);
      RFLU_CUDA(cudaMemcpyAsync(staging + 5 * (size_t)o0, cv + 5 * (size_t)o0, sizeof(double) * 5 * (size_t)(o1 - o0),
                                cudaMemcpyHostToDevice, copyStream));
      RFLU_CUDA(cudaEventRecord(chunkEv[c], copyStream));
      RFLU_CUDA(cudaStreamWaitEvent(stream, chunkEv[c], 0));
      ops->initFromRef(X, staging, o0, o1, stream);
    }
    return checkLaunch("upload");
  }
  // the reference-order gather of ncomp rows of src into staging + off and
  // the copy to the host, chunk by chunk
  int gatherToHost(const double *src, int ncomp, size_t off, double *host) {
    const int K = nChunks();
    for (int c = 0; c < K; ++c) {
      const int o0 = chunkBegin(c), o1 = chunkBegin(c + 1);
      if (o1 <= o0) continue;
      kGatherOut<<<nblk(o1 - o0), 256, 0, stream>>>(src, staging + off, V.newId, V.nc, ncomp, o0, o1);
      RFLU_CUDA(cudaEventRecord(chunkEv[c], stream));
      RFLU_CUDA(cudaStreamWaitEvent(copyStream, chunkEv[c], 0));
      RFLU_CUDA(cudaMemcpyAsync(host + (size_t)ncomp * o0, staging + off + (size_t)ncomp * o0,
                                sizeof(double) * ncomp * (size_t)(o1 - o0), cudaMemcpyDeviceToHost, copyStream));
    }
    // later work on the stream may overwrite staging: it waits for the copies
    RFLU_CUDA(cudaEventRecord(chunkEv[kMaxChunks], copyStream));
    RFLU_CUDA(cudaStreamWaitEvent(stream, chunkEv[kMaxChunks], 0));
    return RFLU_OK;
  }

  int upload(const double *cv) override {
    invalidate();
    if (!cv) return fail(RFLU_ERR_ARG, "rflu_gpu_upload_state: null cv");
    int rc = setState(cv);
    if (rc) return rc;
    return syncEvents(false);
  }
  int download(double *cv, double *dv) override {
    if (dv && V.p.dvPOnly) kDvFill<<<nblk(V.nc), 256, 0, stream>>>(V.cv, V.dv, V.nc, V.p.gcR, V.p.gRT);
    int rcg = RFLU_OK;
    if (cv && (rcg = gatherToHost(V.cv, 5, 0, cv))) return rcg;
    if (dv && (rcg = gatherToHost(V.dv, 3, 5 * (size_t)V.nc, dv))) return rcg;
    int rc = checkLaunch("download");
    if (rc) return rc;
    return syncEvents(false);
  }
  int timestep(double t, double *dt) override {
    kSetScalars<<<1, 1, 0, stream>>>(V.sc, t, 0.0, 0);
    ops->timestep(V, stream);
    int rc = checkLaunch("timestep");
    if (rc) return rc;
    Scalars s;
    RFLU_CUDA(cudaMemcpyAsync(&s, V.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
    RFLU_CUDA(cudaStreamSynchronize(stream));
    if (dt) *dt = s.dtMin;
    return RFLU_OK;
  }
  int rkStage(int iStage, double dt) override {
    invalidate();
    if (iStage < 1 || iStage > V.p.nrkSteps) return fail(RFLU_ERR_ARG, "rflu_gpu_rk_stage: stage out of range");
    kSetDt<<<1, 1, 0, stream>>>(V.sc, dt);
    stageKernels(iStage);
    int rc = checkLaunch("rk_stage");
    if (rc) return rc;
    return syncEvents(true);
  }
  int rungeKutta(double dt) override {
    invalidate();
    kSetDt<<<1, 1, 0, stream>>>(V.sc, dt);
    for (int s = 1; s <= V.p.nrkSteps; ++s) stageKernels(s);
    int rc = checkLaunch("runge_kutta");
    if (rc) return rc;
    return syncEvents(true);
  }
  // One time step (dt + all stages + time advance) captured once as a graph.
  int ensureStepGraph() {
    if (stepGraph) return RFLU_OK;
    cudaGraph_t graph;
    RFLU_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    ops->stepStart(V, stream);  // dt reduction + gradients of stage 1
    ops->faceFlux(V, stream);
    ops->gatherUpdate(V, 1, &V.sc->dtMin, stream);
    for (int s = 2; s <= V.p.nrkSteps; ++s) stageKernels(s);
    ops->stepEnd(V, stream);
    RFLU_CUDA(cudaStreamEndCapture(stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&stepGraph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(RFLU_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return RFLU_OK;
  }
  int ensureFixedGraph() {
    if (fixedGraph) return RFLU_OK;
    cudaGraph_t graph;
    RFLU_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 1; s <= V.p.nrkSteps; ++s) stageKernels(s);
    RFLU_CUDA(cudaStreamEndCapture(stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&fixedGraph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(RFLU_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return RFLU_OK;
  }
  int step(int nSteps, double *time, double endTime, int *done) override {
    invalidate();
    if (!time || nSteps < 0) return fail(RFLU_ERR_ARG, "rflu_gpu_step: bad arguments");
    int rc = ensureStepGraph();
    if (rc) return rc;
    kSetScalars<<<1, 1, 0, stream>>>(V.sc, *time, endTime, 0);
    Scalars s{};
    const int chunk = 64;
    for (int n0 = 0; n0 < nSteps; n0 += chunk) {
      int m = std::min(chunk, nSteps - n0);
      for (int k = 0; k < m; ++k) RFLU_CUDA(cudaGraphLaunch(stepGraph, stream));
      if (endTime > 0.0) {
        RFLU_CUDA(cudaMemcpyAsync(&s, V.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
        RFLU_CUDA(cudaStreamSynchronize(stream));
        if (s.finished != 0) break;
      }
    }
    RFLU_CUDA(cudaMemcpyAsync(&s, V.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, stream));
    rc = syncEvents(true);
    *time = s.time;
    if (done) *done = s.stepsDone;
    return rc;
  }
  int runFixedDt(int nSteps, double dt) override {
    invalidate();
    int rc = ensureFixedGraph();
    if (rc) return rc;
    kSetDt<<<1, 1, 0, stream>>>(V.sc, dt);
    for (int k = 0; k < nSteps; ++k) RFLU_CUDA(cudaGraphLaunch(fixedGraph, stream));
    return syncEvents(true);
  }
  int residual(const double *cv, double *rhs, double *grad) override {
    invalidate();
    if (!cv || !rhs) return fail(RFLU_ERR_ARG, "rflu_gpu_residual: null argument");
    const size_t nc = V.nc;
    View<R> W;
    int rc = scratchView(&W, false);
    if (rc || (rc = setStateOf(W, cv))) return rc;
    ops->gradLimit(W, stream);
    ops->faceFlux(W, stream);
    ops->gatherRhs(W, stream);
    kPermuteOut<R><<<nblk(V.nc), 256, 0, stream>>>(V.rhs, staging, V.refId, V.nc, 5, V.nc, 1);
    RFLU_CUDA(cudaMemcpyAsync(rhs, staging, sizeof(double) * 5 * nc, cudaMemcpyDeviceToHost, stream));
    if (grad) {
      if (V.p.spaceOrder > 1) {
        if (Layout<R>::packed)
          kPermuteOut<R><<<nblk(V.nc), 256, 0, stream>>>(V.grad, staging, V.refId, V.nc, 15, 1, 16);
        else
          kPermuteOut<R><<<nblk(V.nc), 256, 0, stream>>>(V.grad, staging, V.refId, V.nc, 15, V.nc, 1);
        RFLU_CUDA(cudaMemcpyAsync(grad, staging, sizeof(double) * 15 * nc, cudaMemcpyDeviceToHost, stream));
      } else {
        RFLU_CUDA(cudaStreamSynchronize(stream));
        std::memset(grad, 0, sizeof(double) * 15 * nc);
      }
    }
    rc = checkLaunch("residual");
    if (rc) return rc;
    return syncEvents(false);
  }
  // The adjoint's device memory (workspace; mixed mode: the transposed-
  // stencil weights) is allocated on the first adjoint call, so that a
  // context that only steps does not hold it.
  int ensureAdjoint() {
    if (work) return RFLU_OK;
    int rc = alloc((char **)&work, workBytes);
    if (rc) return rc;
    if (tsWidthLazy > 0) {
      if ((rc = alloc(&V.tsW, 4 * (size_t)tsWidthLazy * V.nc))) return rc;
      V.tsWidth = tsWidthLazy;
      ops->adjointSetup(V, stream);
    }
    return checkLaunch("adjoint set-up");
  }
  // the host state cv in the scratch state W (the adjoint kernels then run on W)
  int adjointPrep(const double *cv, View<R> *W) {
    if (!ops->vjp) return fail(RFLU_ERR_UNSUPPORTED, "no adjoint kernels in this precision mode");
    int rc = ensureAdjoint();
    if (rc || (rc = scratchView(W, false))) return rc;
    return setStateOf(*W, cv);
  }
  int adjointDone() {
    int rc = checkLaunch("adjoint");
    if (rc) return rc;
    return syncEvents(false);
  }
  int vjp(const double *cv, const double *rhsBar, double *cvBar) override {
    invalidate();
    if (!cv || !rhsBar || !cvBar) return fail(RFLU_ERR_ARG, "rflu_gpu_vjp: null argument");
    View<R> W;
    int rc = adjointPrep(cv, &W);
    if (rc) return rc;
    const size_t nc = V.nc;
    RFLU_CUDA(cudaMemcpyAsync(staging, rhsBar, sizeof(double) * 5 * nc, cudaMemcpyHostToDevice, stream));
    ops->vjp(W, staging, staging + 5 * nc, work, stream);
    RFLU_CUDA(cudaMemcpyAsync(cvBar, staging + 5 * nc, sizeof(double) * 5 * nc, cudaMemcpyDeviceToHost, stream));
    return adjointDone();
  }
  int jvp(const double *cv, const double *cvDot, double *rhsDot) override {
    invalidate();
    if (!cv || !cvDot || !rhsDot) return fail(RFLU_ERR_ARG, "rflu_gpu_jvp: null argument");
    View<R> W;
    int rc = adjointPrep(cv, &W);
    if (rc) return rc;
    const size_t nc = V.nc;
    RFLU_CUDA(cudaMemcpyAsync(staging, cvDot, sizeof(double) * 5 * nc, cudaMemcpyHostToDevice, stream));
    ops->jvp(W, staging, staging + 5 * nc, work, stream);
    RFLU_CUDA(cudaMemcpyAsync(rhsDot, staging + 5 * nc, sizeof(double) * 5 * nc, cudaMemcpyDeviceToHost, stream));
    return adjointDone();
  }
  int limiterBranches(const double *cv, int *branches) override {
    invalidate();
    if (!cv || !branches) return fail(RFLU_ERR_ARG, "rflu_gpu_limiter_branches: null argument");
    if (V.p.spaceOrder < 2) return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_limiter_branches: first order has no limiter");
    View<R> W;
    int rc = adjointPrep(cv, &W);
    if (rc) return rc;
    int *dev = reinterpret_cast<int *>(staging);  // 10 ints per cell fit in the 15 doubles per cell
    ops->limiterBranches(W, dev, work, stream);
    RFLU_CUDA(cudaMemcpyAsync(branches, dev, sizeof(int) * 10 * (size_t)V.nc, cudaMemcpyDeviceToHost, stream));
    return adjointDone();
  }
  int patchPressure(const double *cv, int iPatch, double *J, double *cvBar) override {
    invalidate();
    if (!cv || !J) return fail(RFLU_ERR_ARG, "rflu_gpu_patch_pressure: null argument");
    if (iPatch < 0 || iPatch >= nPatches) return fail(RFLU_ERR_ARG, "rflu_gpu_patch_pressure: bad patch");
    View<R> W;
    int rc = adjointPrep(cv, &W);
    if (rc) return rc;
    const size_t nc = V.nc;
    ops->patchPressure(W, iPatch, staging + 10 * nc, cvBar ? staging + 5 * nc : nullptr, work, stream);
    RFLU_CUDA(cudaMemcpyAsync(J, staging + 10 * nc, sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (cvBar)
      RFLU_CUDA(cudaMemcpyAsync(cvBar, staging + 5 * nc, sizeof(double) * 5 * nc, cudaMemcpyDeviceToHost, stream));
    return adjointDone();
  }
  // ---- one RK stage at the reference's subroutine granularity --------------
  // Whether V.grad holds the limited gradients of the current state and V.rhs
  // its residual (set by cellGradients / convectiveFluxes); every other call
  // that changes the state or reuses those arrays clears both.
  bool gradValid = false, rhsValid = false;
  void invalidate() { gradValid = rhsValid = false; }
  // A caller's device buffer must live on this context's device, with that
  // device current (args.h).
  int checkDeviceArg(const void *q, const char *who) {
    int cur = -1, qDev = -1;
    RFLU_CUDA(cudaGetDevice(&cur));
    const ArgMem kind = pointerKind(q, &qDev);
    if (const char *why = deviceArgProblem(kind, qDev, device, cur)) return fail(RFLU_ERR_ARG, std::string(who) + ": " + why);
    return RFLU_OK;
  }
  int cellGradients() override {
    invalidate();
    ops->gradLimit(V, stream);
    if (int rc = checkLaunch("rflu_gpu_cell_gradients")) return rc;
    gradValid = true;
    return RFLU_OK;
  }
  int convectiveFluxes() override {
    if (V.p.spaceOrder > 1 && !gradValid)
      return fail(RFLU_ERR_STATE, "rflu_gpu_convective_fluxes: no gradients of this state (call rflu_gpu_cell_gradients)");
    ops->faceFlux(V, stream);
    ops->gatherRhs(V, stream);
    if (int rc = checkLaunch("rflu_gpu_convective_fluxes")) return rc;
    rhsValid = true;
    return RFLU_OK;
  }
  int addRhs(const double *src, int onDevice) override {
    if (!src) return fail(RFLU_ERR_ARG, "rflu_gpu_add_rhs: null src");
    if (!rhsValid) return fail(RFLU_ERR_STATE, "rflu_gpu_add_rhs: no residual (call rflu_gpu_convective_fluxes)");
    const double *d = src;
    if (onDevice) {
      if (int rc = checkDeviceArg(src, "rflu_gpu_add_rhs")) return rc;
    } else {
      RFLU_CUDA(cudaMemcpyAsync(staging, src, sizeof(double) * 5 * (size_t)V.nc, cudaMemcpyHostToDevice, stream));
      d = staging;
    }
    ops->addRhs(V, d, stream);
    if (int rc = checkLaunch("rflu_gpu_add_rhs")) return rc;
    if (!onDevice) RFLU_CUDA(cudaStreamSynchronize(stream));  // src may be reused on return
    return RFLU_OK;
  }
  int rkUpdate(int iStage, double dt) override {
    if (iStage < 1 || iStage > V.p.nrkSteps) return fail(RFLU_ERR_ARG, "rflu_gpu_rk_update: stage out of range");
    if (!rhsValid) return fail(RFLU_ERR_STATE, "rflu_gpu_rk_update: no residual (call rflu_gpu_convective_fluxes)");
    invalidate();
    kSetDt<<<1, 1, 0, stream>>>(V.sc, dt);
    ops->updateFromRhs(V, iStage, &V.sc->dtMin, stream);
    if (int rc = checkLaunch("rflu_gpu_rk_update")) return rc;
    return syncEvents(true);
  }
  // ncomp rows of per-cell data (component k of renumbered cell i at
  // src[k*kStride + i*iStride]) to the reference's layout, on the device
  // (onDevice) or through the staging buffer to the host
  int readOut(const R *src, int ncomp, size_t kStride, size_t iStride, double *dst, int onDevice, const char *who) {
    if (onDevice) {
      if (int rc = checkDeviceArg(dst, who)) return rc;
      kPermuteOut<R><<<nblk(V.nc), 256, 0, stream>>>(src, dst, V.refId, V.nc, ncomp, kStride, iStride);
    } else {
      kPermuteOut<R><<<nblk(V.nc), 256, 0, stream>>>(src, staging, V.refId, V.nc, ncomp, kStride, iStride);
      RFLU_CUDA(cudaMemcpyAsync(dst, staging, sizeof(double) * ncomp * (size_t)V.nc, cudaMemcpyDeviceToHost, stream));
    }
    if (int rc = checkLaunch(who)) return rc;
    RFLU_CUDA(cudaStreamSynchronize(stream));
    return RFLU_OK;
  }
  int getRhs(double *rhs, int onDevice) override {
    if (!rhs) return fail(RFLU_ERR_ARG, "rflu_gpu_get_rhs: null rhs");
    if (!rhsValid) return fail(RFLU_ERR_STATE, "rflu_gpu_get_rhs: no residual (call rflu_gpu_convective_fluxes)");
    return readOut(V.rhs, 5, V.nc, 1, rhs, onDevice, "rflu_gpu_get_rhs");
  }
  int getGrad(double *grad, int onDevice) override {
    if (!grad) return fail(RFLU_ERR_ARG, "rflu_gpu_get_grad: null grad");
    if (!gradValid) return fail(RFLU_ERR_STATE, "rflu_gpu_get_grad: no gradients (call rflu_gpu_cell_gradients)");
    if (V.p.spaceOrder < 2) {
      if (onDevice) {
        if (int rc = checkDeviceArg(grad, "rflu_gpu_get_grad")) return rc;
        RFLU_CUDA(cudaMemsetAsync(grad, 0, sizeof(double) * 15 * (size_t)V.nc, stream));
        RFLU_CUDA(cudaStreamSynchronize(stream));
      } else {
        std::memset(grad, 0, sizeof(double) * 15 * (size_t)V.nc);
      }
      return RFLU_OK;
    }
    if (Layout<R>::packed) return readOut(V.grad, 15, 1, 16, grad, onDevice, "rflu_gpu_get_grad");
    return readOut(V.grad, 15, V.nc, 1, grad, onDevice, "rflu_gpu_get_grad");
  }

  int status(rflu_status *st) override {
    Scalars s;
    RFLU_CUDA(cudaStreamSynchronize(stream));
    RFLU_CUDA(cudaMemcpy(&s, V.sc, sizeof(Scalars), cudaMemcpyDeviceToHost));
    st->nanCells = (long long)s.nanCells;
    st->posFixCells = (long long)s.posFixCells;
    st->negPCells = (long long)s.negPCells;
    st->firstBadCell = (s.firstBadCell == INT_MAX) ? 0 : s.firstBadCell;
    st->stepsDone = s.stepsDone;
    st->time = s.time;
    st->dtMin = s.dtMin;
    return RFLU_OK;
  }
  int kernelTimes(int nIter, double *ms) override {
    invalidate();
    if (nIter <= 0 || !ms) return fail(RFLU_ERR_ARG, "rflu_gpu_kernel_times: bad arguments");
    // on a copy of the state (the same kernels on the same data), so that the
    // context's state, time and accumulator stay as they are
    View<R> W;
    if (int rc0 = scratchView(&W, true)) return rc0;
    cudaEvent_t ev[5];
    for (auto &e : ev) RFLU_CUDA(cudaEventCreate(&e));
    double acc[4] = {0, 0, 0, 0};
    kSetScalars<<<1, 1, 0, stream>>>(W.sc, 1.0, 0.0, 0);
    kSetDt<<<1, 1, 0, stream>>>(W.sc, 0.0);  // dt = 0: the state stays put
    // iteration 0 is an untimed warm-up (the first launch of a kernel also
    // loads its module)
    for (int it = 0; it <= nIter; ++it) {
      cudaEventRecord(ev[0], stream);
      ops->gradLimit(W, stream);
      cudaEventRecord(ev[1], stream);
      ops->faceFlux(W, stream);
      cudaEventRecord(ev[2], stream);
      ops->gatherUpdate(W, 1 + it % V.p.nrkSteps, &W.sc->dtMin, stream);
      cudaEventRecord(ev[3], stream);
      ops->timestep(W, stream);
      cudaEventRecord(ev[4], stream);
      RFLU_CUDA(cudaEventSynchronize(ev[4]));
      for (int k = 0; k < 4 && it > 0; ++k) {
        float t = 0.f;
        cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
        acc[k] += t;
      }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < 4; ++k) ms[k] = acc[k] / nIter;
    return checkLaunch("kernel_times");
  }
  // The residual of rflu_gpu_residual on device buffers, with every
  // intermediate (renumbered state, dependent variables, primitive state,
  // gradients, face fluxes, cell residuals) carved out of gStaticScratch
  // instead of the context's own buffers.  Nothing in the scratch has to
  // start at zero: each element a kernel reads was written earlier in the
  // same call.
  int residualStatic(const double *cvDev, double *rhsDev) override {
    if (!cvDev || !rhsDev) return fail(RFLU_ERR_ARG, "rflu_gpu_residual_static: null argument");
    for (const void *q : {(const void *)cvDev, (const void *)rhsDev})
      if (int rc = checkDeviceArg(q, "rflu_gpu_residual_static")) return rc;
    const size_t nc = V.nc, nT = (size_t)V.nf + V.nb;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t bCv = up(5 * nc * sizeof(double)), bDv = up(3 * nc * sizeof(double));
    const size_t bPrim = up(Layout<R>::prim * nc * sizeof(R)), bGrad = up(Layout<R>::grad * nc * sizeof(R));
    const size_t bFlux = up(5 * nT * sizeof(R)), bRhs = up(5 * nc * sizeof(R));
    const size_t bRaw = V.gradRaw ? bGrad : 0;
    const size_t need = bCv + bDv + bPrim + bGrad + bRaw + bFlux + bRhs;
    if (need > kStaticScratchBytes)
      return fail(RFLU_ERR_ARG, "rflu_gpu_residual_static: this mesh needs " + std::to_string(need) +
                                    " bytes of scratch; the static scratch holds " +
                                    std::to_string(kStaticScratchBytes) + " bytes");
    void *base = nullptr;
    int rc = staticScratchAddress(&base);
    if (rc) return rc;
    unsigned char *p = (unsigned char *)base;
    View<R> W = V;
    W.cv = (double *)p;            p += bCv;
    W.dv = (double *)p;            p += bDv;
    W.prim = (R *)p;               p += bPrim;
    W.grad = (R *)p;               p += bGrad;
    if (V.gradRaw) { W.gradRaw = (R *)p; p += bRaw; }
    W.flux = (R *)p;               p += bFlux;
    W.rhs = (R *)p;
    kPermuteIn<<<nblk(W.nc), 256, 0, stream>>>(cvDev, W.cv, W.refId, W.nc);
    ops->initState(W, stream);
    ops->gradLimit(W, stream);
    ops->faceFlux(W, stream);
    ops->gatherRhs(W, stream);
    kPermuteOut<R><<<nblk(W.nc), 256, 0, stream>>>(W.rhs, rhsDev, W.refId, W.nc, 5, W.nc, 1);
    rc = checkLaunch("residual_static");
    if (rc) return rc;
    RFLU_CUDA(cudaStreamSynchronize(stream));
    return RFLU_OK;
  }
  // rflu_gpu_unrolled_adjoint.  Stage map of every scheme:
  //   cv(s) = cv(s-1) - (ark_s dt / vol) sum_{m<=s} W[s][m] R(cv(m-1))
  // (Wray: W[s][s] = 1, W[s][s-1] = -grk_s; the reference's RK4: W[s][s] = 1,
  // last stage also W[4][1] = 1, W[4][m] = grk_m; Euler: W[1][1] = 1), so
  //   lambda(s-1) = lambda(s) - R'(cv(s-1))^T sum_{t>=s} (ark_t dt W[t][s]/vol) lambda(t).
  int unrolledAdjoint(const double *cv0, int nSteps, double dt, int every, int iPatch, double *Jout, double *cvBar0,
                      double *stats) override {
    invalidate();
    if (!cv0 || !Jout || nSteps < 1 || every < 1 || !(dt > 0.0))
      return fail(RFLU_ERR_ARG, "rflu_gpu_unrolled_adjoint: bad arguments");
    if (!ops->vjp) return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_unrolled_adjoint: no adjoint kernels in this precision mode");
    if (iPatch < 0 || iPatch >= nPatches) return fail(RFLU_ERR_ARG, "rflu_gpu_unrolled_adjoint: bad patch");
    if (int rc0 = ensureAdjoint()) return rc0;
    // the whole forward and reverse sweep runs on the scratch state X
    View<R> X;
    if (int rc0 = scratchView(&X, false)) return rc0;
    const int nrk = V.p.nrkSteps;
    double W[6][6] = {};
    for (int t = 1; t <= nrk; ++t) W[t][t] = 1.0;
    if (V.p.rkScheme == 2) {
      W[2][1] = -V.p.grk[1];
      W[3][2] = -V.p.grk[2];
    } else if (V.p.rkScheme == 1) {
      W[nrk][1] = 1.0;
      for (int m = 2; m < nrk; ++m) W[nrk][m] = V.p.grk[m - 1];
    }
    const size_t nc = V.nc, n5 = 5 * nc, b5 = n5 * sizeof(double);
    const int nCk = (nSteps + every - 1) / every;
    const bool grad = cvBar0 != nullptr;
    const size_t nSeg = grad ? (size_t)every * nrk + 1 : 0;
    // device buffers of the call: checkpoints, segment stage states, the
    // stage adjoints lambda(0..nrk), seed, VJP result, functional gradient
    const size_t nVec = (size_t)nCk + nSeg + (grad ? (size_t)nrk + 1 + 3 : 0);
    double *buf = nullptr, *jd = nullptr;
    RFLU_CUDA(cudaMalloc(&buf, std::max<size_t>(nVec, 1) * b5));
    if (cudaMalloc(&jd, 3 * sizeof(double)) != cudaSuccess) {
      cudaFree(buf);
      return fail(RFLU_ERR_CUDA, "rflu_gpu_unrolled_adjoint: cudaMalloc");
    }
    auto vec = [&](size_t k) { return buf + k * n5; };
    cudaError_t err = cudaSuccess;  // first failed copy; checked before returning
    auto cp = [&](void *d, const void *src, size_t bytes, cudaMemcpyKind kind) {
      const cudaError_t e = cudaMemcpyAsync(d, src, bytes, kind, stream);
      if (e != cudaSuccess && err == cudaSuccess) err = e;
    };
    auto zero = [&](void *d, size_t bytes) {
      const cudaError_t e = cudaMemsetAsync(d, 0, bytes, stream);
      if (e != cudaSuccess && err == cudaSuccess) err = e;
    };
    double *ck = vec(0), *seg = vec(nCk);
    double *lam = grad ? vec(nCk + nSeg) : nullptr;
    double *sigma = grad ? vec(nCk + nSeg + nrk + 1) : nullptr;
    double *wv = grad ? sigma + n5 : nullptr, *pg = grad ? sigma + 2 * n5 : nullptr;
    double *jStep = jd, *jAcc = jd + 1;
    cudaEvent_t ev[3];
    for (auto &e : ev) cudaEventCreate(&e);
    int rc = RFLU_OK;
    auto finish = [&](int r) {
      for (auto &e : ev) cudaEventDestroy(e);
      cudaFree(buf);
      cudaFree(jd);
      return r;
    };
    const int nb = nblk((long long)n5);
    if ((rc = setStateOf(X, cv0))) return finish(rc);
    zero(jd, 3 * sizeof(double));
    kSetDt<<<1, 1, 0, stream>>>(X.sc, dt);
    // forward sweep: checkpoints (and J when no gradient is asked for)
    cudaEventRecord(ev[0], stream);
    for (int n = 0; n < nSteps; ++n) {
      if (n % every == 0)
        cp(ck + (size_t)(n / every) * n5, X.cv, b5, cudaMemcpyDeviceToDevice);
      for (int st = 1; st <= nrk; ++st) stageKernelsOf(X, st);
      if (!grad) {
        ops->patchPressure(X, iPatch, jStep, nullptr, work, stream);
        kAccumJ<<<1, 1, 0, stream>>>(jAcc, jStep, dt);
      }
    }
    cudaEventRecord(ev[1], stream);
    if (grad) {
      double *lamTop = lam + (size_t)nrk * n5;  // lambda at the end of the current step
      zero(lamTop, b5);
      auto loadState = [&](const double *src) {
        cp(X.cv, src, b5, cudaMemcpyDeviceToDevice);
        ops->initState(X, stream);
      };
      for (int sg = nCk - 1; sg >= 0; --sg) {
        const int n0 = sg * every, n1 = std::min(nSteps, n0 + every);
        loadState(ck + (size_t)sg * n5);
        for (int n = n0; n < n1; ++n)
          for (int st = 1; st <= nrk; ++st) {
            cp(seg + ((size_t)(n - n0) * nrk + st - 1) * n5, X.cv, b5, cudaMemcpyDeviceToDevice);
            stageKernelsOf(X, st);
          }
        cp(seg + (size_t)(n1 - n0) * nrk * n5, X.cv, b5, cudaMemcpyDeviceToDevice);
        for (int n = n1 - 1; n >= n0; --n) {
          // the functional's term at the state after step n
          loadState(seg + (size_t)(n + 1 - n0) * nrk * n5);
          ops->patchPressure(X, iPatch, jStep, pg, work, stream);
          kAccumJ<<<1, 1, 0, stream>>>(jAcc, jStep, dt);
          kAxpyInPlace<<<nb, 256, 0, stream>>>(lamTop, dt, pg, n5);
          for (int st = nrk; st >= 1; --st) {
            SeedTerms T{};
            for (int t = st; t <= nrk; ++t)
              if (W[t][st] != 0.0) {
                T.lam[T.n] = lam + (size_t)t * n5;
                T.coef[T.n] = V.p.ark[t - 1] * dt * W[t][st];
                ++T.n;
              }
            kStageSeed<<<nblk(V.nc), 256, 0, stream>>>(sigma, T, V.vol, V.refId, V.nc);
            loadState(seg + ((size_t)(n - n0) * nrk + st - 1) * n5);
            ops->vjp(X, sigma, wv, work, stream);
            kSubInto<<<nb, 256, 0, stream>>>(lam + (size_t)(st - 1) * n5, lam + (size_t)st * n5, wv, n5);
          }
          cp(lamTop, lam, b5, cudaMemcpyDeviceToDevice);
        }
      }
      cp(cvBar0, lamTop, b5, cudaMemcpyDeviceToHost);
    }
    cudaEventRecord(ev[2], stream);
    cp(Jout, jAcc, sizeof(double), cudaMemcpyDeviceToHost);
    if ((rc = checkLaunch("rflu_gpu_unrolled_adjoint"))) return finish(rc);
    const cudaError_t es = cudaStreamSynchronize(stream);
    if (err == cudaSuccess) err = es;
    if (err != cudaSuccess)
      return finish(fail(RFLU_ERR_CUDA, std::string("rflu_gpu_unrolled_adjoint: ") + cudaGetErrorString(err)));
    if (stats) {
      float f = 0.f, b = 0.f;
      cudaEventElapsedTime(&f, ev[0], ev[1]);
      cudaEventElapsedTime(&b, ev[1], ev[2]);
      stats[0] = f;
      stats[1] = grad ? b : 0.0;
      stats[2] = (double)(bytesHeld + std::max<size_t>(nVec, 1) * b5 + 3 * sizeof(double));
      stats[3] = nCk;
    }
    return finish(syncEvents(false));
  }
  int adjointTimes(int nIter, double *ms) override {
    invalidate();
    if (nIter <= 0 || !ms) return fail(RFLU_ERR_ARG, "rflu_gpu_adjoint_times: bad arguments");
    if (!ops->vjp)
      return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_adjoint_times: no adjoint here");
    if (int rc0 = ensureAdjoint()) return rc0;
    const size_t nc = V.nc;
    RFLU_CUDA(cudaMemsetAsync(staging, 0, sizeof(double) * 5 * nc, stream));
    cudaEvent_t ev[3];
    for (auto &e : ev) RFLU_CUDA(cudaEventCreate(&e));
    double acc[2] = {0, 0};
    for (int it = 0; it <= nIter; ++it) {  // iteration 0: untimed warm-up
      cudaEventRecord(ev[0], stream);
      ops->gradLimit(V, stream);
      ops->faceFlux(V, stream);
      ops->gatherRhs(V, stream);
      cudaEventRecord(ev[1], stream);
      ops->vjp(V, staging, staging + 5 * nc, work, stream);
      cudaEventRecord(ev[2], stream);
      RFLU_CUDA(cudaEventSynchronize(ev[2]));
      for (int k = 0; k < 2 && it > 0; ++k) {
        float t = 0.f;
        cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
        acc[k] += t;
      }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    ms[0] = acc[0] / nIter;
    ms[1] = acc[1] / nIter;
    return checkLaunch("adjoint_times");
  }
  int nPatches = 0;
};

// The per-patch constants of the device's patch fluxes (physics.cuh:
// kPatchK) from the patch's boundary values, in the reference's operation
// order: the parts of RFLU_SetRindStateFarfieldPerf
// (modflu/RFLU_ModRindStates.F90:272-290) and BcondInflowPerf
// (libfloflu/BcondInflowPerf.F90: the supersonic branch) that depend on the
// patch alone, with gas constants MixtPerf_R_M and MixtPerf_G_CpR
// (libfloflu/MixtPerf_R.F90:93, MixtPerf_G.F90:78).  *bcOpt receives the
// patch's BCOPT type switch (outflow: patchOutflowType; inflow:
// BCSWI_INFLOW_TYPE).
template <typename R>
int Ctx<R>::patchConstants(const rflu_grid_desc *g, int ip, const rflu_num_desc *num, int *bcOpt, double *K) {
  const int type = g->patchBcType[ip];
  // the gas constants of the device's Params (cp, and the molecular mass
  // MixtPerf_M_R(MixtPerf_R_CpG(cp, gamma)))
  const double gcp = num->cp, gmol = 8314.3 / (num->cp - num->cp / num->gamma);
  const double Rg = 8314.3 / gmol, gam = gcp / (gcp - Rg);
  const double *vals = g->patchVals ? g->patchVals + (size_t)RFLU_BCDAT_N * ip : nullptr;
  const int *sw = g->patchSwitches ? g->patchSwitches + (size_t)RFLU_BCSWI_N * ip : nullptr;
  auto need = [&](bool withSwitches) {
    if (!vals || (withSwitches && !sw))
      return fail(RFLU_ERR_ARG, "rflu_gpu_create: inflow, farfield and injection patches need patchVals/patchSwitches");
    return RFLU_OK;
  };
  switch (type) {
    case RFLU_BC_SLIPWALL:
    case RFLU_BC_NOSLIPWALL_HFLUX:
    case RFLU_BC_NOSLIPWALL_TEMP:
      return RFLU_OK;
    case RFLU_BC_SYMMETRY: {
      // the reflection across the patch's plane, from its first face's
      // normal (RFLU_RELP_TransformMatrix, modflu/RFLU_ModRelatedPatches.F90:
      // 449-514; rflu_setup_build checks that the patch is planar)
      if (g->patchFaceOff[ip + 1] == g->patchFaceOff[ip]) return RFLU_OK;
      const double *n = g->bfn + 4 * (size_t)g->patchFaceOff[ip];
      const double nx = n[0], ny = n[1], nz = n[2];
      const double Q[9] = {1.0 - 2.0 * nx * nx, -2.0 * nx * ny, -2.0 * nx * nz,
                           -2.0 * nx * ny, 1.0 - 2.0 * ny * ny, -2.0 * ny * nz,
                           -2.0 * nx * nz, -2.0 * ny * nz, 1.0 - 2.0 * nz * nz};
      for (int k = 0; k < 9; ++k) K[k] = Q[k];
      return RFLU_OK;
    }
    case RFLU_BC_PERIODIC:  // its faces are interior faces of the identified mesh (fc2, c2csShift)
      if (g->patchFaceOff[ip + 1] != g->patchFaceOff[ip])
        return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_create: a periodic patch must hold no boundary faces (its faces are "
                                          "interior faces of the identified mesh, rflu_setup_build)");
      return RFLU_OK;
    case RFLU_BC_OUTFLOW:
      K[0] = g->patchPout[ip];
      return RFLU_OK;
    case RFLU_BC_FARFIELD: {
      if (int rc = need(true)) return rc;
      if (sw[0] != 0)
        return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_create: the farfield vortex correction (CORR 1) is not on this path");
      const double mf = vals[0], aoa = vals[1], aos = vals[2], pf = vals[3], tf = vals[4];
      const double ri = pf / (Rg * tf);                                  // MixtPerf_D_PRT
      const double qi = mf * std::sqrt(gam * Rg * tf);                   // MixtPerf_C_GRT
      const double ui = qi * std::cos(aoa) * std::cos(aos), vi = qi * std::sin(aoa) * std::cos(aos),
                   wi = qi * std::sin(aos);
      const double k[8] = {mf, ri, pf, qi, ui, vi, wi, ri * (pf / (ri * (gam - 1.0)) + 0.5 * qi * qi)};
      std::memcpy(K, k, sizeof(k));
      return RFLU_OK;
    }
    case RFLU_BC_INFLOW_TOTANG: {
      if (int rc = need(true)) return rc;
      *bcOpt = sw[0];
      if (sw[0] < 0 || sw[0] > 2 || sw[1] < 0 || sw[1] > 1)
        return fail(RFLU_ERR_ARG, "rflu_gpu_create: bad inflow TYPE or FIXED switch");
      const double ptot = vals[0], ttot = vals[1], bh = vals[2], bv = vals[3];
      const double k[7] = {ptot, ttot, std::cos(bh), std::sin(bh), std::cos(bv), std::sin(bv), (double)sw[1]};
      std::memcpy(K, k, sizeof(k));
      if (sw[0] != 1) {  // the supersonic state (BCOPT_SUPERSONIC, and MIXED beyond the sound speed)
        const double mach = vals[4];
        const double pr = ptot / std::pow(1.0 + 0.5 * (gam - 1.0) * mach * mach, gam / (gam - 1.0));  // MixtPerf_P_GMaPo
        const double tr = ttot / (1.0 + 0.5 * (gam - 1.0) * mach * mach);                              // MixtPerf_T_GMaTo
        const double rr = pr / (Rg * tr);
        const double ar = std::sqrt(gam * Rg * tr);
        const double ur = mach * ar * std::cos(bh) * std::cos(bv), vr = mach * ar * std::sin(bh),
                     wr = mach * ar * std::cos(bh) * std::sin(bv);
        const double rer = rr * (pr / (rr * (gam - 1.0)) + 0.5 * (ur * ur + vr * vr + wr * wr));  // MixtPerf_Eo_DGPUVW
        const double s[6] = {rr, rr * ur, rr * vr, rr * wr, rer, pr};
        std::memcpy(K + 7, s, sizeof(s));
      }
      return RFLU_OK;
    }
    case RFLU_BC_INFLOW_VELTEMP: {
      if (int rc = need(true)) return rc;
      *bcOpt = sw[0];
      if (sw[0] < 0 || sw[0] > 2) return fail(RFLU_ERR_ARG, "rflu_gpu_create: bad inflow TYPE switch");
      const double k[6] = {vals[0], vals[1], vals[2], vals[3], vals[4], vals[4] / (Rg * vals[3])};
      std::memcpy(K, k, sizeof(k));
      return RFLU_OK;
    }
    case RFLU_BC_INJECTION: {
      if (int rc = need(false)) return rc;
      K[0] = vals[0];
      K[1] = vals[1];
      return RFLU_OK;
    }
    default:
      return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_create: patch type " + std::to_string(type) + " is not on this path");
  }
}

// Tiles of the mixed-mode gradient kernel (ctx.h): per tile of kTile
// consecutive cells, its halo cells in slots (planTiles, tiles.h: aligned to
// the shared-memory banks where that costs no occupancy); the local id of
// every stencil member; and the entry-major face arrays feD/feN with the
// neighbour's local id as the tag.  Left untiled (V.tiled = 0) when a tile
// would stage more records than shared memory or a 16-bit id holds.
template <typename R>
int Ctx<R>::buildTiles(const std::vector<int> &cfOff, const std::vector<int> &cfEnt, const std::vector<int> &stOff,
                       const std::vector<int> &stIdx, const std::vector<int> &fc1, const std::vector<int> &fc2,
                       const std::vector<double> &fnx, const std::vector<double> &fny,
                       const std::vector<double> &fnz, const std::vector<double> &fnm,
                       const std::vector<double> &dL, const std::vector<double> &dR,
                       const std::vector<double> &bnx, const std::vector<double> &bny,
                       const std::vector<double> &bnz, const std::vector<double> &bnm,
                       const std::vector<double> &bd) {
  const int nc = V.nc, nf = V.nf, nb = V.nb;
  int cfW = 0;
  for (int i = 0; i < nc; ++i) cfW = std::max(cfW, cfOff[i + 1] - cfOff[i]);
  int dev = 0, optin = 0, perSm = 0, reserved = 0;
  RFLU_CUDA(cudaGetDevice(&dev));
  RFLU_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  RFLU_CUDA(cudaDeviceGetAttribute(&perSm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  RFLU_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
  // shared memory of a CTA of the gradient kernel: two tile buffers, and the
  // face-offset cache of the Venkatakrishnan variant
  auto smemOf = [&](int recs, int maxTileSt, bool venkat) {
    return sizeof(float) * (2 * tileBufFloatsFor(recs, maxTileSt) + (venkat ? 3 * 6 * kTile : 0));
  };
  auto ctasPerSm = [&](int recs, int maxTileSt, bool venkat) {
    return (size_t)perSm / (smemOf(recs, maxTileSt, venkat) + (size_t)reserved);
  };
  TilePlan plan;
  if (!planTiles(nc, kTile, cfOff, cfEnt, stOff, stIdx, fc1, fc2, ctasPerSm, plan)) return RFLU_OK;  // stays untiled
  if (smemOf(plan.maxRecs, plan.maxTileSt, true) > (size_t)optin) return RFLU_OK;
  const int maxRecs = plan.maxRecs, maxTileSt = plan.maxTileSt;
  const std::vector<int> &haloOff = plan.haloOff, &haloIdx = plan.haloIdx, &entLoc = plan.entLoc;
  std::vector<unsigned short> &stLoc = plan.stLoc;
  stLoc.resize(stLoc.size() + 16, 0);  // whole 16-byte words past the last tile
  std::vector<float> feD(4 * (size_t)cfW * nc, 0.f), feN(4 * (size_t)cfW * nc, 0.f);
  for (int i = 0; i < nc; ++i)
    for (int k = 0; k < cfW; ++k) {
      float *d = &feD[4 * ((size_t)k * nc + i)], *nn = &feN[4 * ((size_t)k * nc + i)];
      int tag = INT_MIN;
      const int e = cfOff[i] + k;
      if (e < cfOff[i + 1]) {
        const int code = cfEnt[e];
        if (code >= 0) {
          const int f = code >> 1;
          const std::vector<double> &dd = (code & 1) ? dR : dL;
          d[0] = (float)dd[f]; d[1] = (float)dd[(size_t)nf + f]; d[2] = (float)dd[2 * (size_t)nf + f];
          nn[0] = (float)fnx[f]; nn[1] = (float)fny[f]; nn[2] = (float)fnz[f]; nn[3] = (float)fnm[f];
          tag = entLoc[e];
        } else {
          const int b = -code - 1;
          // the boundary face's offset fc - cofg (the WENO pass's positivity
          // check reads it; the gradient kernel reads interior entries only)
          d[0] = (float)bd[b]; d[1] = (float)bd[(size_t)nb + b]; d[2] = (float)bd[2 * (size_t)nb + b];
          nn[0] = (float)bnx[b]; nn[1] = (float)bny[b]; nn[2] = (float)bnz[b]; nn[3] = (float)bnm[b];
          tag = code;
        }
      }
      std::memcpy(&d[3], &tag, sizeof(int));
    }
  (void)nb;
  int rc = 0;
  // per tile {halo list start, its slots, stLoc words [w0, w1)}: one 16-byte
  // load gives the gradient kernel what it needs to stage the tile
  const int nTiles = (nc + kTile - 1) / kTile;
  std::vector<int> desc(4 * (size_t)nTiles);
  for (int t = 0; t < nTiles; ++t) {
    const int b0 = t * kTile, b1 = std::min(nc, b0 + kTile);
    desc[4 * t] = haloOff[t];
    desc[4 * t + 1] = haloOff[t + 1] - haloOff[t];
    desc[4 * t + 2] = stOff[b0] >> 3;
    desc[4 * t + 3] = (stOff[b1] + 7) >> 3;
  }
  std::vector<int> haloPadded(haloIdx);
  haloPadded.resize(haloPadded.size() + 4, -1);
  if ((rc = put<int>(&V.haloOff, haloOff))) return rc;
  if ((rc = put<int>(&V.haloIdx, haloPadded))) return rc;
  {
    const int *d = nullptr;
    if ((rc = put<int>(&d, desc))) return rc;
    V.tileDesc = reinterpret_cast<const int4 *>(d);
  }
  if ((rc = put<unsigned short>(&V.stLoc, stLoc))) return rc;
  if ((rc = put<float>(&V.feD, feD))) return rc;
  if ((rc = put<float>(&V.feN, feN))) return rc;
  V.maxRecs = maxRecs;
  V.maxTileSt = maxTileSt;
  V.cfW = cfW;
  V.tiled = 1;
  return RFLU_OK;
}

template <typename R>
int Ctx<R>::create(const rflu_grid_desc *g, const rflu_num_desc *num) {
  const int nc = g->nCells, nf = g->nFaces, np = g->nPatches;
  const int nb = np > 0 ? g->patchFaceOff[np] : 0;
  nPatches = np;
  RFLU_CUDA(cudaGetDevice(&device));
  RFLU_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  RFLU_CUDA(cudaStreamCreateWithFlags(&copyStream, cudaStreamNonBlocking));
  for (auto &e : chunkEv) RFLU_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));

  // ---- renumbering: Morton order of the cell centroids --------------------
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < nc; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], g->cofg[3 * (size_t)i + d]);
      hi[d] = std::max(hi[d], g->cofg[3 * (size_t)i + d]);
    }
  double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  if (!(ext > 0)) ext = 1.0;
  std::vector<uint64_t> key(nc);
  for (int i = 0; i < nc; ++i) {
    uint64_t q[3];
    for (int d = 0; d < 3; ++d)
      q[d] = (uint64_t)std::min(2097151.0, std::floor((g->cofg[3 * (size_t)i + d] - lo[d]) / ext * 2097151.0));
    key[i] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
  }
  std::vector<int> refId(nc), newId(nc);
  std::iota(refId.begin(), refId.end(), 0);
  std::stable_sort(refId.begin(), refId.end(), [&](int a, int b) { return key[a] < key[b]; });
  for (int i = 0; i < nc; ++i) newId[refId[i]] = i;

  // ---- interior faces: stored in order of their renumbered first cell -----
  std::vector<int> store(nf);
  std::iota(store.begin(), store.end(), 0);
  auto c1of = [&](int f) { return newId[g->f2c[2 * (size_t)f] - 1]; };
  std::stable_sort(store.begin(), store.end(), [&](int a, int b) { return c1of(a) < c1of(b); });
  std::vector<int> slotOf(nf);
  for (int s = 0; s < nf; ++s) slotOf[store[s]] = s;
  std::vector<int> fc1(nf), fc2(nf);
  std::vector<double> fnx(nf), fny(nf), fnz(nf), fnm(nf), dL(3 * (size_t)nf), dR(3 * (size_t)nf);
  for (int s = 0; s < nf; ++s) {
    const int f = store[s];
    const int o1 = g->f2c[2 * (size_t)f] - 1, o2 = g->f2c[2 * (size_t)f + 1] - 1;
    if (o1 < 0 || o1 >= nc || o2 < 0 || o2 >= nc) return fail(RFLU_ERR_ARG, "rflu_gpu_create: f2c out of range");
    fc1[s] = newId[o1];
    fc2[s] = newId[o2];
    const double *fn = g->fn + 4 * (size_t)f, *fcp = g->fc + 3 * (size_t)f;
    // a periodic mesh's second side sees the face centroid in its own frame
    const double *fcq = g->fc2 ? g->fc2 + 3 * (size_t)f : fcp;
    fnx[s] = fn[0]; fny[s] = fn[1]; fnz[s] = fn[2]; fnm[s] = fn[3];
    for (int d = 0; d < 3; ++d) {
      // dx = xc - pGrid%cofg(XCOORD,c1), as the 2nd-order flux routines form it
      dL[(size_t)d * nf + s] = fcp[d] - g->cofg[3 * (size_t)o1 + d];
      dR[(size_t)d * nf + s] = fcq[d] - g->cofg[3 * (size_t)o2 + d];
    }
  }
  // ---- boundary faces --------------------------------------------------------
  std::vector<int> bcell(nb), bpatch(nb);
  std::vector<double> bnx(nb), bny(nb), bnz(nb), bnm(nb), bd(3 * (size_t)nb);
  std::vector<int> pType(std::max(np, 1)), pOut(std::max(np, 1)), pOrder(std::max(np, 1));
  std::vector<double> pK((size_t)kPatchK * std::max(np, 1), 0.0);
  for (int ip = 0; ip < np; ++ip) {
    pType[ip] = g->patchBcType[ip];
    pOut[ip] = g->patchOutflowType[ip];
    pOrder[ip] = g->patchOrder[ip];
    if (int rc = patchConstants(g, ip, num, &pOut[ip], &pK[(size_t)kPatchK * ip])) return rc;
    if (pOrder[ip] == 2 && num->spaceOrder < 2)
      return fail(RFLU_ERR_ARG, "rflu_gpu_create: 2nd-order patch needs ORDER 2");
    for (int b = g->patchFaceOff[ip]; b < g->patchFaceOff[ip + 1]; ++b) {
      const int o = g->bf2c[b] - 1;
      if (o < 0 || o >= nc) return fail(RFLU_ERR_ARG, "rflu_gpu_create: bf2c out of range");
      bcell[b] = newId[o];
      bpatch[b] = ip;
      const double *fn = g->bfn + 4 * (size_t)b, *fcp = g->bfc + 3 * (size_t)b;
      bnx[b] = fn[0]; bny[b] = fn[1]; bnz[b] = fn[2]; bnm[b] = fn[3];
      for (int d = 0; d < 3; ++d) bd[(size_t)d * nb + b] = fcp[d] - g->cofg[3 * (size_t)o + d];
    }
  }
  // ---- cell -> face CSR in the reference's summation order ------------------
  std::vector<int> cnt(nc + 1, 0);
  for (int f = 0; f < nf; ++f) { cnt[g->f2c[2 * (size_t)f] - 1 + 1]++; cnt[g->f2c[2 * (size_t)f + 1] - 1 + 1]++; }
  for (int b = 0; b < nb; ++b) cnt[g->bf2c[b] - 1 + 1]++;
  std::vector<int> offRef(nc + 1, 0);
  for (int o = 0; o < nc; ++o) offRef[o + 1] = offRef[o] + cnt[o + 1];
  std::vector<int> entRef(offRef[nc]);
  {
    std::vector<int> fill(offRef.begin(), offRef.end() - 1);
    for (int f = 0; f < nf; ++f) {
      entRef[fill[g->f2c[2 * (size_t)f] - 1]++] = slotOf[f] << 1;
      entRef[fill[g->f2c[2 * (size_t)f + 1] - 1]++] = (slotOf[f] << 1) | 1;
    }
    for (int b = 0; b < nb; ++b) entRef[fill[g->bf2c[b] - 1]++] = -(b + 1);
  }
  std::vector<int> cfOff(nc + 1, 0), cfEnt;
  cfEnt.reserve(entRef.size());
  for (int i = 0; i < nc; ++i) {
    const int o = refId[i];
    for (int e = offRef[o]; e < offRef[o + 1]; ++e) cfEnt.push_back(entRef[e]);
    cfOff[i + 1] = (int)cfEnt.size();
  }
  // ---- stencils and least-squares weights --------------------------------------
  // per member: RFLU_ComputeGradCellsFast_3D weights (modflu/
  // RFLU_ModDifferentiationCells.F90:983-1044) from the R factor and the
  // unit offset, in FP64 and in the reference's order of operations
  std::vector<int> stOff(nc + 1, 0), stIdx;
  std::vector<double> wx, wy, wz, epsq(nc, 0.0), lsq;
  std::vector<float> stShift;  // mixed mode on a periodic mesh: the members' translations
  imageMesh = g->c2csShift != nullptr || g->fc2 != nullptr || g->c2csXf != nullptr;
  std::vector<int> stXf;  // symmetry meshes: the members' reflections
  const bool mixed = num->precision == RFLU_PREC_MIXED;
  if (mixed && num->spaceOrder > 1) lsq.resize(6 * (size_t)nc);
  if (num->spaceOrder > 1) {
    if (!g->c2csOff || !g->c2csMembs || !g->xyzMoms) return fail(RFLU_ERR_ARG, "rflu_gpu_create: ORDER 2 needs stencils");
    for (int i = 0; i < nc; ++i) {
      const int o = refId[i];
      const double *m = g->xyzMoms + 10 * (size_t)o;
      const double r11 = m[0], r12 = m[1], r22 = m[2], r13 = m[3], r23 = m[4], r33 = m[5];
      const double c11 = 1.0 / r11, c22 = 1.0 / r22, c33 = 1.0 / r33;
      const double c12 = -c11 * r12;
      const double c13 = -(c11 * r13 + c12 * c22 * r23);
      const double c23 = -c22 * r23;
      const double c1111 = c11 * c11, c2222 = c22 * c22, c3333 = c33 * c33;
      if (mixed) {
        // w = L d / |d|^2 with the symmetric L of the weights' linear map
        lsq[i] = c1111 + c12 * c12 * c2222 + c13 * c13 * c3333;
        lsq[(size_t)nc + i] = c12 * c2222 + c13 * c23 * c3333;
        lsq[2 * (size_t)nc + i] = c13 * c3333;
        lsq[3 * (size_t)nc + i] = c2222 + c23 * c23 * c3333;
        lsq[4 * (size_t)nc + i] = c23 * c3333;
        lsq[5 * (size_t)nc + i] = c3333;
      }
      const double *xi = g->cofg + 3 * (size_t)o;
      for (int e = g->c2csOff[o]; e < g->c2csOff[o + 1]; ++e) {
        const int j = g->c2csMembs[e] - 1;
        if (j < 0 || j >= nc) return fail(RFLU_ERR_ARG, "rflu_gpu_create: stencil member out of range");
        double dx = g->cofg[3 * (size_t)j] - xi[0], dy = g->cofg[3 * (size_t)j + 1] - xi[1],
               dz = g->cofg[3 * (size_t)j + 2] - xi[2];
        if (g->c2csXf) {
          const int x = g->c2csXf[e];
          if (x < -1 || x >= g->nXf) return fail(RFLU_ERR_ARG, "rflu_gpu_create: c2csXf out of range");
          stXf.push_back(x);
        }
        if (g->c2csShift) {  // the member's periodic or symmetry image
          const double *sh = g->c2csShift + 3 * (size_t)e;
          dx = dx + sh[0]; dy = dy + sh[1]; dz = dz + sh[2];
          if (mixed) { stShift.push_back((float)sh[0]); stShift.push_back((float)sh[1]); stShift.push_back((float)sh[2]); }
        }
        const double term = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
        dx = term * dx; dy = term * dy; dz = term * dz;
        const double t1 = c1111 * (dx);
        const double t2 = c2222 * (dy + c12 * dx);
        const double t3 = c3333 * (dz + c23 * dy + c13 * dx);
        if (!mixed) {
          wx.push_back(term * (t1 + c12 * t2 + c13 * t3));
          wy.push_back(term * (t2 + c23 * t3));
          wz.push_back(term * (t3));
        }
        stIdx.push_back(newId[j]);
      }
      stOff[i + 1] = (int)stIdx.size();
      // Venkatakrishnan: ds = vol**(1/3), eps^2 = (K ds)^3, K = 1
      // (modflu/RFLU_ModLimiters.F90:457-460)
      const double ds = std::pow(g->vol[o], 1.0 / 3.0);
      epsq[i] = (1.0 * ds) * (1.0 * ds) * (1.0 * ds);
    }
  }
  std::vector<double> vol(nc), ivol(nc), cgx(nc), cgy(nc), cgz(nc);
  for (int i = 0; i < nc; ++i) {
    vol[i] = g->vol[refId[i]];
    ivol[i] = 1.0 / vol[i];
    cgx[i] = g->cofg[3 * (size_t)refId[i]];
    cgy[i] = g->cofg[3 * (size_t)refId[i] + 1];
    cgz[i] = g->cofg[3 * (size_t)refId[i] + 2];
  }
  // transposed stencil for the adjoint of the LSQ gradient (FP64 modes)
  std::vector<int> tsOff(nc + 1, 0), tsCell(stIdx.size()), tsEnt(stIdx.size());
  for (size_t s = 0; s < stIdx.size(); ++s) tsOff[stIdx[s] + 1]++;
  for (int j = 0; j < nc; ++j) tsOff[j + 1] += tsOff[j];
  {
    std::vector<int> fill(tsOff.begin(), tsOff.end() - 1);
    for (int i = 0; i < nc; ++i)
      for (int s = stOff[i]; s < stOff[i + 1]; ++s) {
        const int e = fill[stIdx[s]]++;
        tsCell[e] = i;
        tsEnt[e] = s;
      }
  }

  // ---- device upload -----------------------------------------------------------
  V.nc = nc; V.nf = nf; V.nb = nb;
  int rc = 0;
#define PUT(dst, src, T) if ((rc = put<T>(&(dst), src))) return rc
  if (mixed) {
    // one 48-byte record per interior face (ctx.h)
    for (int i = 0; i < nc; ++i)
      if (cfOff[i + 1] - cfOff[i] > 6)
        return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_create: the mixed mode takes cells of at most 6 faces");
    std::vector<float> fpk(12 * (size_t)nf);
    for (int s = 0; s < nf; ++s) {
      float *r = &fpk[12 * (size_t)s];
      r[0] = (float)fnx[s]; r[1] = (float)fny[s]; r[2] = (float)fnz[s]; r[3] = (float)fnm[s];
      r[4] = (float)dL[s]; r[5] = (float)dL[(size_t)nf + s]; r[6] = (float)dL[2 * (size_t)nf + s];
      r[7] = (float)dR[s]; r[8] = (float)dR[(size_t)nf + s]; r[9] = (float)dR[2 * (size_t)nf + s];
      std::memcpy(&r[10], &fc1[s], sizeof(int));
      std::memcpy(&r[11], &fc2[s], sizeof(int));
    }
    PUT(V.fpk, fpk, float);
  } else {
    PUT(V.fc1, fc1, int); PUT(V.fc2, fc2, int);
    PUT(V.fnx, fnx, R); PUT(V.fny, fny, R); PUT(V.fnz, fnz, R); PUT(V.fnm, fnm, R);
    PUT(V.dL, dL, R); PUT(V.dR, dR, R);
  }
  PUT(V.bcell, bcell, int); PUT(V.bpatch, bpatch, int);
  PUT(V.bnx, bnx, R); PUT(V.bny, bny, R); PUT(V.bnz, bnz, R); PUT(V.bnm, bnm, R);
  PUT(V.bd, bd, R);
  PUT(V.patchType, pType, int); PUT(V.patchOutflow, pOut, int); PUT(V.patchOrder, pOrder, int);
  PUT(V.patchK, pK, double);
  PUT(V.cfOff, cfOff, int); PUT(V.cfEnt, cfEnt, int);
  PUT(V.stOff, stOff, int); PUT(V.stIdx, stIdx, int);
  PUT(V.vol, vol, double); PUT(V.epsq, epsq, R);
  PUT(V.refId, refId, int); PUT(V.newId, newId, int);
  if (mixed) {
    // weights formed in the gradient kernel from the R factor and centroids
    PUT(V.cgx, cgx, R); PUT(V.cgy, cgy, R); PUT(V.cgz, cgz, R);
    PUT(V.lsq, lsq, R); PUT(V.ivol, ivol, R);
    if (!stShift.empty()) PUT(V.stShift, stShift, float);
    if (g->c2csXf && !g->c2csShift)
      return fail(RFLU_ERR_ARG, "rflu_gpu_create: c2csXf needs c2csShift (the reflected members' offsets)");
    // the tile plan stages records with their own centroids; a periodic
    // mesh's members need their images' (the gather kernel adds stShift)
    if (num->spaceOrder > 1 && !(num->options & RFLU_OPT_UNTILED) && stShift.empty()) {
      if ((rc = buildTiles(cfOff, cfEnt, stOff, stIdx, fc1, fc2, fnx, fny, fnz, fnm, dL, dR, bnx, bny, bnz, bnm, bd)))
        return rc;
    }
    if (num->spaceOrder > 1) {
      // the width of the adjoint's transposed-stencil weights, allocated and
      // filled with the adjoint workspace on the first adjoint call
      int w = 0;
      for (int j = 0; j < nc; ++j) w = std::max(w, tsOff[j + 1] - tsOff[j]);
      tsWidthLazy = w;
    }
  } else {
    PUT(V.wx, wx, R); PUT(V.wy, wy, R); PUT(V.wz, wz, R);
  }
  // transposed stencil (adjoint of the LSQ gradient, every mode)
  PUT(V.tsOff, tsOff, int); PUT(V.tsCell, tsCell, int); PUT(V.tsEnt, tsEnt, int);
  if (!stXf.empty()) {
    if (!g->xfQ || g->nXf <= 0) return fail(RFLU_ERR_ARG, "rflu_gpu_create: c2csXf needs xfQ");
    std::vector<R> q(g->xfQ, g->xfQ + 9 * (size_t)g->nXf);
    PUT(V.stXf, stXf, int);
    PUT(V.xfQ, q, R);
  }
  // constrained gradients (CRECONSTC 1): the plan in the reference's cell
  // numbering (constr.h), moved to the renumbered cells; the stencil rows
  // keep the reference's member order, which the device's stencil keeps too
  // (a mesh with periodic or symmetry images and no wall or injection patch
  // has no constrained cell)
  bool constrPatches = false;
  for (int ip = 0; ip < np; ++ip)
    if ((pType[ip] == RFLU_BC_SLIPWALL || pType[ip] == RFLU_BC_NOSLIPWALL_HFLUX || pType[ip] == RFLU_BC_NOSLIPWALL_TEMP ||
         pType[ip] == RFLU_BC_INJECTION) && g->patchFaceOff[ip + 1] > g->patchFaceOff[ip])
      constrPatches = true;
  if (num->cReconstCells == 1 && num->spaceOrder > 1 && imageMesh && constrPatches)
    return fail(RFLU_ERR_UNSUPPORTED,
                "rflu_gpu_create: constrained gradients (CRECONSTC 1) on a mesh with periodic or symmetry patches");
  if (num->cReconstCells == 1 && num->spaceOrder > 1 && !imageMesh) {
    std::vector<int> stOffRef(g->c2csOff, g->c2csOff + nc + 1), stIdxRef(g->c2csOff[nc]);
    for (int e = 0; e < g->c2csOff[nc]; ++e) stIdxRef[e] = g->c2csMembs[e] - 1;
    std::vector<int> bf2cRef(nb);
    for (int b = 0; b < nb; ++b) bf2cRef[b] = g->bf2c[b] - 1;
    std::vector<double> minj(std::max(np, 1), 0.0);
    for (int ip = 0; ip < np; ++ip)
      if (pType[ip] == RFLU_BC_INJECTION) minj[ip] = pK[(size_t)kPatchK * ip];
    ConstrInput in{nc, g->cofg, stOffRef.data(), stIdxRef.data(), np, g->patchFaceOff, pType.data(), minj.data(),
                   bf2cRef.data(), g->bfn, g->bfc, num->cReconstCellsWeight};
    ConstrPlan plan;
    int bad = -1;
    if (planConstrained(in, plan, &bad) != 0)
      return fail(RFLU_ERR_ARG, "rflu_gpu_create: the constrained gradient matrix of cell " + std::to_string(bad + 1) +
                                    " is singular (RFLU_ComputeGradCellsConstr stops there)");
    std::vector<int> slot(nc, -1);
    for (size_t k = 0; k < plan.cells.size(); ++k) slot[newId[plan.cells[k]]] = (int)k;
    // a burning injection face's constraint values follow the pressure of
    // its cell: per cell the (constrained cell, row, variable) entries it
    // feeds, for the adjoint's gather (kAdjCell2)
    std::vector<std::vector<int>> cpList(nc);
    for (size_t sl = 0; sl < plan.cells.size(); ++sl) {
      const int ci = newId[plan.cells[sl]];
      const int nst = g->c2csOff[plan.cells[sl] + 1] - g->c2csOff[plan.cells[sl]];
      int r = plan.rowOff[sl];
      for (int k = 0; k < 5; ++k) {
        const int ncon = plan.nCon[5 * sl + k];
        if (!ncon) continue;
        r += nst;
        for (int c = 0; c < ncon; ++c, ++r) {
          const int b = plan.rowFace[r];
          if (b < 0) continue;
          int ip = 0;
          while (ip + 1 < np && b >= g->patchFaceOff[ip + 1]) ++ip;
          if (!(pType[ip] == RFLU_BC_INJECTION && minj[ip] > 0.0) || k > 3) continue;
          constrBurning = true;
          cpList[newId[g->bf2c[b] - 1]].push_back(ci);
          cpList[newId[g->bf2c[b] - 1]].push_back(8 * r + k);
        }
      }
    }
    if (constrBurning) {
      std::vector<int> cpOff(nc + 1, 0), cpEnt;
      for (int i = 0; i < nc; ++i) {
        cpEnt.insert(cpEnt.end(), cpList[i].begin(), cpList[i].end());
        cpOff[i + 1] = (int)cpEnt.size() / 2;
      }
      PUT(V.cpOff, cpOff, int);
      PUT(V.cpEnt, cpEnt, int);
    }
    std::vector<R> w(plan.w.begin(), plan.w.end());
    if (plan.cells.empty()) plan.rowFace.push_back(-1);
    PUT(V.cSlot, slot, int); PUT(V.cNcon, plan.nCon, int); PUT(V.cRowOff, plan.rowOff, int);
    PUT(V.cRowFace, plan.rowFace, int); PUT(V.cW, w, R);
  }
#undef PUT
  if ((rc = alloc(&V.cv, 5 * (size_t)nc))) return rc;
  if ((rc = alloc(&V.dv, 3 * (size_t)nc))) return rc;
  if ((rc = alloc(&V.prim, Layout<R>::prim * (size_t)nc))) return rc;
  if ((rc = alloc(&V.grad, Layout<R>::grad * (size_t)nc))) return rc;
  if ((num->reconst == 1 || num->reconst == 2) && num->spaceOrder > 1 &&
      (rc = alloc(&V.gradRaw, Layout<R>::grad * (size_t)nc)))
    return rc;
  if ((rc = alloc(&V.rhsSum, 5 * (size_t)nc))) return rc;
  if ((rc = alloc(&V.flux, 5 * ((size_t)nf + nb)))) return rc;
  if ((rc = alloc(&V.rhs, 5 * (size_t)nc))) return rc;
  if ((rc = alloc(&V.sc, 1))) return rc;
  if ((rc = alloc(&staging, 15 * (size_t)nc + 16))) return rc;
  RFLU_CUDA(cudaMemset(V.grad, 0, sizeof(R) * Layout<R>::grad * (size_t)nc));
  RFLU_CUDA(cudaMemset(V.rhsSum, 0, sizeof(R) * 5 * (size_t)nc));
  RFLU_CUDA(cudaMemset(V.cv, 0, sizeof(double) * 5 * (size_t)nc));
  Scalars s0{};
  s0.dtBits = 0x7fefffffffffffffull;
  s0.firstBadCell = INT_MAX;
  RFLU_CUDA(cudaMemcpy(V.sc, &s0, sizeof(Scalars), cudaMemcpyHostToDevice));

  // ---- numerics (libflu/RFLU_DerivedInputValues.F90:309-410) ----------------
  Params &P = V.p;
  P.spaceOrder = num->spaceOrder; P.spaceDiscr = num->spaceDiscr; P.reconst = num->reconst;
  P.rkScheme = num->rkScheme; P.piclBuild = num->piclBuild; P.precision = num->precision;
  P.refCp = num->cp; P.refGamma = num->gamma;
  P.gvCp = num->cp;
  P.gvMol = 8314.3 / (num->cp - num->cp / num->gamma);  // MixtPerf_M_R(MixtPerf_R_CpG(cp,gamma))
  P.gcR = 8314.3 / P.gvMol;                             // MixtPerf_R_M(M), the round trip
  P.gRT = P.gvCp / (P.gvCp - P.gcR);                    // MixtPerf_G_CpR(cp,R)
  P.igcR = 1.0 / P.gcR;
  P.refCpF = (float)P.refCp; P.refGammaF = (float)P.refGamma; P.epsEntrF = (float)num->epsEntr;
  P.dissFactF = (float)num->dissFact; P.gvCpF = (float)P.gvCp; P.gvMolF = (float)P.gvMol;
  P.epsEntr = num->epsEntr; P.dissFact = num->dissFact;
  P.cfl = num->cfl; P.dtImposed = num->dtImposed; P.dtMinLimit = num->dtMinLimit;
  for (int k = 0; k < 5; ++k) P.ark[k] = P.grk[k] = 0.0;
  if (num->rkScheme == 1) {
    P.nrkSteps = 4;
    P.ark[0] = 0.5; P.ark[1] = 0.5; P.ark[2] = 1.0; P.ark[3] = 1.0 / 6.0;
    P.grk[0] = 1.0; P.grk[1] = 2.0; P.grk[2] = 2.0; P.grk[3] = 1.0;
  } else if (num->rkScheme == 2) {
    P.nrkSteps = 3;
    P.ark[0] = 8.0 / 15.0; P.ark[1] = 5.0 / 12.0; P.ark[2] = 0.75;
    P.grk[0] = 0.0; P.grk[1] = 17.0 / 25.0; P.grk[2] = 5.0 / 9.0;
  } else {
    P.nrkSteps = 1;
    P.ark[0] = 1.0; P.grk[0] = 1.0;
  }
  for (int k = 0; k < 5; ++k) { P.arkF[k] = (float)P.ark[k]; P.grkF[k] = (float)P.grk[k]; }
  P.dvPOnly = (num->precision == RFLU_PREC_MIXED && num->spaceOrder > 1) ? 1 : 0;
  // adjoint workspace (adjoint.cuh: carveAdjWork): gradients, limiter
  // factors and branches, face adjoints of one residual, in the mode's type
  workBytes = sizeof(R) * (size_t)(130 * (size_t)nc + 24 * ((size_t)nf + nb) + 64) + sizeof(int) * 10 * (size_t)nc + 256;
  ops->configure(V);
  RFLU_CUDA(cudaDeviceSynchronize());
  V.tileGrid = ops->tileGrid(V, 0);
  V.tileGridDt = ops->tileGrid(V, 1);
  return checkLaunch("rflu_gpu_create");
}

}  // namespace rflu

struct rflu_gpu_ctx {
  std::unique_ptr<rflu::CtxBase> impl;
};

using rflu::fail;

extern "C" {

const char *rflu_gpu_last_error(void) { return rflu::lastError().c_str(); }

int rflu_gpu_create(const rflu_grid_desc *grid, const rflu_num_desc *num, rflu_gpu_ctx **ctx) {
  if (!grid || !num || !ctx) return fail(RFLU_ERR_ARG, "rflu_gpu_create: null argument");
  *ctx = nullptr;
  if (grid->nCells <= 0 || grid->nFaces < 0 || !grid->f2c || !grid->fn || !grid->fc || !grid->vol || !grid->cofg)
    return fail(RFLU_ERR_ARG, "rflu_gpu_create: incomplete grid description");
  if (num->spaceOrder != 1 && num->spaceOrder != 2) return fail(RFLU_ERR_ARG, "rflu_gpu_create: ORDER must be 1 or 2");
  if (num->spaceDiscr != 1 && num->spaceDiscr != 3 && num->spaceDiscr != 4)
    return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_create: DISCR must be 1 (Roe), 3 (HLLC) or 4 (AUSM+)");
  if (num->reconst != 0 && num->reconst != 1 && num->reconst != 2 && num->reconst != 10 && num->reconst != 11 &&
      num->reconst != 100)
    return fail(RFLU_ERR_UNSUPPORTED, "rflu_gpu_create: RECONST must be 0, 1, 2, 10, 11 or 100");
  if (num->rkScheme < 1 || num->rkScheme > 3) return fail(RFLU_ERR_ARG, "rflu_gpu_create: RKSCHEME must be 1, 2 or 3");
  if (num->precision < 0 || num->precision > 2) return fail(RFLU_ERR_ARG, "rflu_gpu_create: bad precision");
  if (num->options & ~RFLU_OPT_UNTILED) return fail(RFLU_ERR_ARG, "rflu_gpu_create: unknown option bits");
  if (num->cReconstCells != 0 && num->cReconstCells != 1)
    return fail(RFLU_ERR_ARG, "rflu_gpu_create: CRECONSTC must be 0 or 1");
  if (num->cReconstCells == 1 && !(num->cReconstCellsWeight >= 0.0))
    return fail(RFLU_ERR_ARG, "rflu_gpu_create: CRECONSTCW must be >= 0");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(RFLU_ERR_CUDA, "rflu_gpu_create: no CUDA device");
  rflu_gpu_ctx *c = new (std::nothrow) rflu_gpu_ctx();
  if (!c) return fail(RFLU_ERR_ARG, "rflu_gpu_create: out of host memory");
  int rc;
  if (num->precision == RFLU_PREC_MIXED) {
    auto *p = new rflu::Ctx<float>();
    p->ops = rflu::opsMixed();
    c->impl.reset(p);
    rc = p->create(grid, num);
  } else {
    auto *p = new rflu::Ctx<double>();
    p->ops = (num->precision == RFLU_PREC_FP64_EXACT) ? rflu::opsFp64Exact() : rflu::opsFp64();
    c->impl.reset(p);
    rc = p->create(grid, num);
  }
  if (rc) {
    delete c;
    return rc;
  }
  *ctx = c;
  return RFLU_OK;
}

int rflu_gpu_destroy(rflu_gpu_ctx *ctx) {
  delete ctx;
  return RFLU_OK;
}

void *rflu_gpu_stream(rflu_gpu_ctx *ctx) { return ctx ? (void *)ctx->impl->stream : nullptr; }

#define CTX_CHECK(name) \
  if (!ctx) return fail(RFLU_ERR_ARG, name ": null context")

int rflu_gpu_upload_state(rflu_gpu_ctx *ctx, const double *cv) {
  CTX_CHECK("rflu_gpu_upload_state");
  return ctx->impl->upload(cv);
}
int rflu_gpu_download_state(rflu_gpu_ctx *ctx, double *cv, double *dv) {
  CTX_CHECK("rflu_gpu_download_state");
  return ctx->impl->download(cv, dv);
}
int rflu_gpu_timestep(rflu_gpu_ctx *ctx, double currentTime, double *dtMin) {
  CTX_CHECK("rflu_gpu_timestep");
  return ctx->impl->timestep(currentTime, dtMin);
}
int rflu_gpu_rk_stage(rflu_gpu_ctx *ctx, int iStage, double dtMin) {
  CTX_CHECK("rflu_gpu_rk_stage");
  return ctx->impl->rkStage(iStage, dtMin);
}
int rflu_gpu_runge_kutta(rflu_gpu_ctx *ctx, double dtMin) {
  CTX_CHECK("rflu_gpu_runge_kutta");
  return ctx->impl->rungeKutta(dtMin);
}
int rflu_gpu_step(rflu_gpu_ctx *ctx, int nSteps, double *time, double endTime, int *stepsDone) {
  CTX_CHECK("rflu_gpu_step");
  return ctx->impl->step(nSteps, time, endTime, stepsDone);
}
int rflu_gpu_run_fixed_dt(rflu_gpu_ctx *ctx, int nSteps, double dtMin) {
  CTX_CHECK("rflu_gpu_run_fixed_dt");
  return ctx->impl->runFixedDt(nSteps, dtMin);
}
int rflu_gpu_residual(rflu_gpu_ctx *ctx, const double *cv, double *rhs, double *grad) {
  CTX_CHECK("rflu_gpu_residual");
  return ctx->impl->residual(cv, rhs, grad);
}
int rflu_gpu_vjp(rflu_gpu_ctx *ctx, const double *cv, const double *rhsBar, double *cvBar) {
  CTX_CHECK("rflu_gpu_vjp");
  return ctx->impl->vjp(cv, rhsBar, cvBar);
}
int rflu_gpu_jvp(rflu_gpu_ctx *ctx, const double *cv, const double *cvDot, double *rhsDot) {
  CTX_CHECK("rflu_gpu_jvp");
  return ctx->impl->jvp(cv, cvDot, rhsDot);
}
int rflu_gpu_patch_pressure(rflu_gpu_ctx *ctx, const double *cv, int iPatch, double *J, double *cvBar) {
  CTX_CHECK("rflu_gpu_patch_pressure");
  return ctx->impl->patchPressure(cv, iPatch, J, cvBar);
}
int rflu_gpu_unrolled_adjoint(rflu_gpu_ctx *ctx, const double *cv0, int nSteps, double dtMin, int every, int iPatch,
                              double *J, double *cvBar0, double *stats) {
  CTX_CHECK("rflu_gpu_unrolled_adjoint");
  return ctx->impl->unrolledAdjoint(cv0, nSteps, dtMin, every, iPatch, J, cvBar0, stats);
}
int rflu_gpu_status(rflu_gpu_ctx *ctx, rflu_status *status) {
  CTX_CHECK("rflu_gpu_status");
  if (!status) return fail(RFLU_ERR_ARG, "rflu_gpu_status: null status");
  return ctx->impl->status(status);
}

int rflu_gpu_kernel_times(rflu_gpu_ctx *ctx, int nIter, double *ms) {
  CTX_CHECK("rflu_gpu_kernel_times");
  return ctx->impl->kernelTimes(nIter, ms);
}

int rflu_gpu_adjoint_times(rflu_gpu_ctx *ctx, int nIter, double *ms) {
  CTX_CHECK("rflu_gpu_adjoint_times");
  return ctx->impl->adjointTimes(nIter, ms);
}

int rflu_gpu_fp64_rate(double *tflops) {
  if (!tflops) return fail(RFLU_ERR_ARG, "rflu_gpu_fp64_rate: null argument");
  int dev = 0, sms = 0;
  RFLU_CUDA(cudaGetDevice(&dev));
  RFLU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t s;
  RFLU_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = 8192, threads = 256, blocksPerSm = 8;
  rflu::kFp64Fma<<<sms * blocksPerSm, threads, 0, s>>>(iters / 8, 1e-3);  // warm-up
  cudaEventRecord(e0, s);
  rflu::kFp64Fma<<<sms * blocksPerSm, threads, 0, s>>>(iters, 1e-3);
  cudaEventRecord(e1, s);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  if (err != cudaSuccess) return fail(RFLU_ERR_CUDA, std::string("rflu_gpu_fp64_rate: ") + cudaGetErrorString(err));
  const double flops = 2.0 * 8.0 * iters * (double)threads * sms * blocksPerSm;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return RFLU_OK;
}

int rflu_gpu_check_conversions(long long n, unsigned long long seed, unsigned long long *mismatches) {
  if (!mismatches || n < 0) return fail(RFLU_ERR_ARG, "rflu_gpu_check_conversions: bad argument");
  unsigned long long *bad = nullptr;
  RFLU_CUDA(cudaMalloc(&bad, sizeof(unsigned long long)));
  cudaError_t err = cudaMemset(bad, 0, sizeof(unsigned long long));
  if (err == cudaSuccess) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    rflu::kCvtCheck<<<sms * 8, 256>>>(n, seed, bad);
    err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaMemcpy(mismatches, bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  }
  cudaFree(bad);
  if (err != cudaSuccess) return fail(RFLU_ERR_CUDA, std::string("rflu_gpu_check_conversions: ") + cudaGetErrorString(err));
  return RFLU_OK;
}

int rflu_gpu_cell_gradients(rflu_gpu_ctx *ctx) {
  CTX_CHECK("rflu_gpu_cell_gradients");
  return ctx->impl->cellGradients();
}
int rflu_gpu_convective_fluxes(rflu_gpu_ctx *ctx) {
  CTX_CHECK("rflu_gpu_convective_fluxes");
  return ctx->impl->convectiveFluxes();
}
int rflu_gpu_add_rhs(rflu_gpu_ctx *ctx, const double *src, int onDevice) {
  CTX_CHECK("rflu_gpu_add_rhs");
  return ctx->impl->addRhs(src, onDevice);
}
int rflu_gpu_rk_update(rflu_gpu_ctx *ctx, int iStage, double dtMin) {
  CTX_CHECK("rflu_gpu_rk_update");
  return ctx->impl->rkUpdate(iStage, dtMin);
}
int rflu_gpu_get_rhs(rflu_gpu_ctx *ctx, double *rhs, int onDevice) {
  CTX_CHECK("rflu_gpu_get_rhs");
  return ctx->impl->getRhs(rhs, onDevice);
}
int rflu_gpu_get_grad(rflu_gpu_ctx *ctx, double *grad, int onDevice) {
  CTX_CHECK("rflu_gpu_get_grad");
  return ctx->impl->getGrad(grad, onDevice);
}

int rflu_gpu_limiter_branches(rflu_gpu_ctx *ctx, const double *cv, int *branches) {
  CTX_CHECK("rflu_gpu_limiter_branches");
  return ctx->impl->limiterBranches(cv, branches);
}

int rflu_gpu_check_refinements(long long n, unsigned long long seed, double *maxRelErr) {
  if (!maxRelErr || n < 0) return fail(RFLU_ERR_ARG, "rflu_gpu_check_refinements: bad argument");
  const cudaError_t e = rflu::mixedRefineCheck(n, seed, maxRelErr);
  if (e != cudaSuccess) return fail(RFLU_ERR_CUDA, std::string("rflu_gpu_check_refinements: ") + cudaGetErrorString(e));
  return RFLU_OK;
}

int rflu_gpu_residual_static(rflu_gpu_ctx *ctx, const double *cvDev, double *rhsDev) {
  CTX_CHECK("rflu_gpu_residual_static");
  return ctx->impl->residualStatic(cvDev, rhsDev);
}

}  // extern "C"
