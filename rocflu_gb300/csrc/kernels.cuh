// Kernels of one RK stage and of the time step, templated on the state type
// R (double or float).  Included by one translation unit per precision mode;
// RFLU_NS names the namespace of the instantiation.
//
// Per stage (RungeKuttaMP, libfloflu/RungeKuttaMP.F90:148-508):
//   gradLimit   cell-centric: LSQ gradient + limiter  (CellGradientsMP)
//   faceFlux    face-centric: reconstruction + Riemann flux per face, patch
//               fluxes per boundary face                (ConvectiveFluxesMP)
//   gatherUpdate cell-centric: deterministic CSR gather of the face fluxes in
//               the reference's summation order, RK update, dependent
//               variables, validity/bounds/positivity   (RKUpdateMP,
//               RFLU_SetVarsContWrapper, AfterUpdateMP)
// Per step: cellDt (RFLU_TimeStepInviscid) + dtFinalize (RFLU_MinimumTimeStep).
#pragma once
#include <algorithm>
#include <climits>
#include <type_traits>
#include <cuda_runtime.h>

#include "convert.cuh"
#include "ctx.h"
#include "dual.cuh"
#include "physics.cuh"

namespace rflu {
namespace RFLU_NS {

constexpr int kBlock = 256;
inline int blocks(long long n) { return (int)((n + kBlock - 1) / kBlock); }

// Reference arithmetic (the FP64 modes) reproduces the cons -> prim -> cons
// round trip of CellGradientsMP on the fly; the mixed mode uses the
// primitive velocity directly.
template <typename R> struct Ref { static constexpr bool on = false; };
template <> struct Ref<double> { static constexpr bool on = true; };
// Resident blocks requested from the register allocator: the FP32 gather
// kernels are latency-bound and need the occupancy; the FP64 ones are
// FP64-pipe-bound and keep their registers.
template <typename R> struct MinBlocks { static constexpr int v = 1; };
template <> struct MinBlocks<float> { static constexpr int v = 4; };
template <typename R> struct MinBlocksFlux { static constexpr int v = 1; };
template <> struct MinBlocksFlux<float> { static constexpr int v = 4; };

// ---------------------------------------------------------------------------
// Dependent variables of one cell from cv: RFLU_SetDependentVars, TCPERF
// (libflu/RFLU_SetDependentVars.F90:254-287), always in FP64.
// ---------------------------------------------------------------------------
__device__ inline void dependentVars(const Params &p, const double *cv, double &pres, double &temp, double &snd) {
  const double gc = p.gcR;  // MixtPerf_R_M(gv(GV_MIXT_MOL)), computed once
  const double g = p.gRT;   // MixtPerf_G_CpR(gv(GV_MIXT_CP), gc)
  double r = cv[0];
  double ir = 1.0 / r;
  double Eo = ir * cv[4];
  double Vm2 = ir * ir * (cv[1] * cv[1] + cv[2] * cv[2] + cv[3] * cv[3]);
  pres = (g - 1.0) * r * (Eo - 0.5 * Vm2);
  temp = pres / (r * gc);
  snd = sqrt(g * gc * temp);
}

template <typename R>
__device__ inline void loadCv(const View<R> &V, int i, double *cv) {
#pragma unroll
  for (int k = 0; k < 5; ++k) cv[k] = V.cv[(size_t)k * V.nc + i];
}

// ---------------------------------------------------------------------------
// Cell data as the stage code reads it.  PlainLoad reads the primal arrays
// (S = R, the state type; H = double, the type of the first-order paths,
// FP64 in every mode); the tangent kernels use a loader whose S and H are
// dual numbers carrying the directional derivatives.
// ---------------------------------------------------------------------------
__device__ inline float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ inline void st4(float *p, float a, float b, float c, float d) {
  *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}
// One 32-byte record in a single 256-bit load (sm_100 and later; the address
// is 32-byte aligned: records are 8 floats from a 256-byte aligned base).
// Only for data no thread of the running kernel writes.
__device__ inline void ld8(const float *p, float *v) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
      : "l"(p));
}

// Interior face f in either layout: cells, unit normal and area, and the
// offset fc - cofg of side 0 (c1) or side 1 (c2).
template <typename R>
__device__ inline void faceCells(const View<R> &V, int f, int &c1, int &c2) {
  if constexpr (Layout<R>::packed) {
    const float4 F2 = ld4(V.fpk + 12 * (size_t)f + 8);
    c1 = __float_as_int(F2.z);
    c2 = __float_as_int(F2.w);
  } else {
    c1 = V.fc1[f];
    c2 = V.fc2[f];
  }
}
template <typename R>
__device__ inline void faceNormal(const View<R> &V, int f, R &nx, R &ny, R &nz, R &nm) {
  if constexpr (Layout<R>::packed) {
    const float4 F0 = ld4(V.fpk + 12 * (size_t)f);
    nx = F0.x; ny = F0.y; nz = F0.z; nm = F0.w;
  } else {
    nx = V.fnx[f]; ny = V.fny[f]; nz = V.fnz[f]; nm = V.fnm[f];
  }
}
template <typename R>
__device__ inline void faceOffset(const View<R> &V, int f, int side, R *d) {
  if constexpr (Layout<R>::packed) {
    const float4 F1 = ld4(V.fpk + 12 * (size_t)f + 4);
    if (side) {
      const float4 F2 = ld4(V.fpk + 12 * (size_t)f + 8);
      d[0] = F1.w; d[1] = F2.x; d[2] = F2.y;
    } else {
      d[0] = F1.x; d[1] = F1.y; d[2] = F1.z;
    }
  } else {
    const R *a = side ? V.dR : V.dL;
    const size_t nf = V.nf;
    d[0] = a[f]; d[1] = a[nf + f]; d[2] = a[2 * nf + f];
  }
}

template <typename R>
struct PlainLoad {
  using S = R;
  using H = double;
  const View<R> &V;
  __device__ S prim(int k, int c) const {
    if constexpr (Layout<R>::packed) return V.prim[8 * (size_t)c + k];
    else return V.prim[(size_t)k * V.nc + c];
  }
  __device__ S grad(int k, int c) const {
    if constexpr (Layout<R>::packed) return V.grad[16 * (size_t)c + k];
    else return V.grad[(size_t)k * V.nc + c];
  }
  // rho, u, v, w
  __device__ void prim4(int c, S *q) const {
    if constexpr (Layout<R>::packed) {
      const float4 a = ld4(V.prim + 8 * (size_t)c);
      q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = a.w;
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) q[k] = prim(k, c);
    }
  }
  // rho, u, v, w, p
  __device__ void prim5(int c, S *q) const {
    if constexpr (Layout<R>::packed) {
      float r[8];
      ld8(V.prim + 8 * (size_t)c, r);
#pragma unroll
      for (int k = 0; k < 5; ++k) q[k] = r[k];
    } else {
#pragma unroll
      for (int k = 0; k < 5; ++k) q[k] = prim(k, c);
    }
  }
  // rho, u, v, w, p and the centroid (packed layout only)
  __device__ void primCg(int c, S *q, S *x) const {
    float r[8];
    ld8(V.prim + 8 * (size_t)c, r);
#pragma unroll
    for (int k = 0; k < 5; ++k) q[k] = r[k];
    x[0] = r[5]; x[1] = r[6]; x[2] = r[7];
  }
  __device__ void grad15(int c, S *g) const {
    if constexpr (Layout<R>::packed) {
      float r[16];
      ld8(V.grad + 16 * (size_t)c, r);
      ld8(V.grad + 16 * (size_t)c + 8, r + 8);
#pragma unroll
      for (int k = 0; k < 15; ++k) g[k] = r[k];
    } else {
#pragma unroll
      for (int k = 0; k < 15; ++k) g[k] = grad(k, c);
    }
  }
  __device__ H cv(int k, int c) const { return V.cv[(size_t)k * V.nc + c]; }
  __device__ H dv(int k, int c) const { return V.dv[(size_t)k * V.nc + c]; }
};

// Least-squares weight of stencil member s (cell j) of cell i
// (RFLU_ComputeGradCellsFast_3D, :983-1044): the FP64 modes read the
// precomputed weights; the mixed mode forms w = L d / |d|^2 from the cell's
// matrix L and the centroid offset d = x_j - x_i of the packed records.
template <typename R>
__device__ inline void lsqWeight(const View<R> &V, int i, int s, R &wx, R &wy, R &wz) {
  if constexpr (Layout<R>::packed) {
    const int j = V.stIdx[s];
    const size_t n = V.nc;
    float dx = V.prim[8 * (size_t)j + 5] - V.prim[8 * (size_t)i + 5];
    float dy = V.prim[8 * (size_t)j + 6] - V.prim[8 * (size_t)i + 6];
    float dz = V.prim[8 * (size_t)j + 7] - V.prim[8 * (size_t)i + 7];
    if (V.stShift) {  // a periodic mesh: the member's image
      dx = dx + V.stShift[3 * (size_t)s];
      dy = dy + V.stShift[3 * (size_t)s + 1];
      dz = dz + V.stShift[3 * (size_t)s + 2];
    }
    const float inv = 1.f / (dx * dx + dy * dy + dz * dz);
    const float sx = inv * dx, sy = inv * dy, sz = inv * dz;
    const float lxx = V.lsq[i], lxy = V.lsq[n + i], lxz = V.lsq[2 * n + i];
    const float lyy = V.lsq[3 * n + i], lyz = V.lsq[4 * n + i], lzz = V.lsq[5 * n + i];
    wx = lxx * sx + lxy * sy + lxz * sz;
    wy = lxy * sx + lyy * sy + lyz * sz;
    wz = lxz * sx + lyz * sy + lzz * sz;
  } else {
    wx = V.wx[s];
    wy = V.wy[s];
    wz = V.wz[s];
  }
}

// Store of one cell's gradient record.
template <typename R>
__device__ inline void storeGradTo(const View<R> &V, R *base, int i, const R *g) {
  if constexpr (Layout<R>::packed) {
    float *p = base + 16 * (size_t)i;
    st4(p, g[0], g[1], g[2], g[3]);
    st4(p + 4, g[4], g[5], g[6], g[7]);
    st4(p + 8, g[8], g[9], g[10], g[11]);
    st4(p + 12, g[12], g[13], g[14], 0.f);
  } else {
    const size_t n = V.nc;
#pragma unroll
    for (int k = 0; k < 15; ++k) base[k * n + i] = g[k];
  }
}
template <typename R>
__device__ inline void storeGrad(const View<R> &V, int i, const R *g) {
  storeGradTo(V, V.grad, i, g);
}

// Store of one cell's primitive record (the packed layout carries the centroid).
template <typename R>
__device__ inline void storePrimRec(const View<R> &V, int i, R r, R u, R v, R w, R p) {
  if constexpr (Layout<R>::packed) {
    float *q = V.prim + 8 * (size_t)i;
    st4(q, r, u, v, w);
    st4(q + 4, p, V.cgx[i], V.cgy[i], V.cgz[i]);
  } else {
    const size_t n = V.nc;
    V.prim[i] = r;
    V.prim[n + i] = u;
    V.prim[2 * n + i] = v;
    V.prim[3 * n + i] = w;
    V.prim[4 * n + i] = p;
  }
}

// Flux of face t: SoA in the FP64 modes; in the packed layout one float4
// (mass, momentum) per face followed by the nT energy fluxes.
template <typename R>
__device__ inline void storeFluxAt(R *flux, size_t nT, int t, const R *f) {
  if constexpr (Layout<R>::packed) {
    st4(flux + 4 * (size_t)t, f[0], f[1], f[2], f[3]);
    flux[4 * nT + t] = f[4];
  } else {
#pragma unroll
    for (int k = 0; k < 5; ++k) flux[k * nT + t] = f[k];
  }
}
template <typename R>
__device__ inline void storeFlux(const View<R> &V, size_t nT, int t, const R *f) {
  storeFluxAt(V.flux, nT, t, f);
}
template <typename R, typename T>
__device__ inline void loadFlux(const T *flux, size_t nT, int t, T *f) {
  if constexpr (Layout<R>::packed) {
    const float4 a = ld4(flux + 4 * (size_t)t);
    f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w;
    f[4] = flux[4 * nT + t];
  } else {
#pragma unroll
    for (int k = 0; k < 5; ++k) f[k] = flux[k * nT + t];
  }
}


// FP64 reciprocal of x from an FP32 seed y ~ 1/x: one Newton-Raphson step
// y + y*(1 - x*y).  The error of the seed (rounding x to FP32 and the
// approximate FP32 division, ~2^-22 relative) is squared: ~2^-44.
__device__ inline double refinedRecip(double x, float seed) {
  const double y = f2d(seed);
  return fma(y, fma(-x, y, 1.0), y);
}
// FP64 square root of x > 0 from an FP32 reciprocal-square-root seed y: h =
// x*y, then h + h*(1 - h*y)/2 (relative error 1.5 e^2 for a seed error e).
__device__ inline double refinedSqrt(double x) {
  const double y = f2d(rsqrtf(d2f(x)));
  const double h = x * y;
  return fma(0.5 * h, fma(-h, y, 1.0), h);
}

// Mixed mode: primitive state from the FP64 master cv.  1/rho from an FP32
// seed (also the FP32 velocities' reciprocal) refined once in FP64
// (refinedRecip), and the pressure in FP64 from the kinetic energy (the
// cancellation at strong shocks).
struct MixedPrim {
  float rf, irf, uf, vf, wf;
  double ir, ke, pr;
  __device__ MixedPrim(const Params &P, const double *cv) {
    rf = d2f(cv[0]);
    irf = 1.0f / rf;
    ir = refinedRecip(cv[0], irf);
    // explicit fused multiply-adds: the same bits wherever the compiler
    // inlines this (the update and the state set-up agree)
    const double msq = fma(cv[3], cv[3], fma(cv[2], cv[2], cv[1] * cv[1]));
    ke = 0.5 * msq * ir;
    pr = (P.gRT - 1.0) * (cv[4] - ke);
    uf = d2f(cv[1]) * irf;
    vf = d2f(cv[2]) * irf;
    wf = d2f(cv[3]) * irf;
  }
};

// prim = (rho, u, v, w, p) as RFLU_ConvertCvCons2Prim DUVWP builds it
// (modflu/RFLU_ModConvertCv.F90:214-224)
template <typename R>
__device__ inline void storePrim(const View<R> &V, int i, const double *cv, double pres) {
  double ir = 1.0 / cv[0];
  storePrimRec(V, i, (R)cv[0], (R)(ir * cv[1]), (R)(ir * cv[2]), (R)(ir * cv[3]), (R)pres);
}

// Dependent variables and primitive state of every cell from cv
// (RFLU_SetVarsContWrapper after upload).
template <typename R>
__device__ inline void initCell(const View<R> &V, int i, const double *cv) {
  if constexpr (Layout<R>::packed) {
    // the primitive record exactly as the mixed update forms it, so that a
    // state restarted from cv continues bit for bit; T and c only when a
    // kernel of the step reads them (else formed at read-out)
    const MixedPrim m(V.p, cv);
    V.dv[i] = m.pr;
    if (!V.p.dvPOnly) {
      // T and c with the mixed update's formulas
      V.dv[(size_t)V.nc + i] = m.pr * m.ir * V.p.igcR;
      V.dv[2 * (size_t)V.nc + i] = refinedSqrt(V.p.gRT * m.pr * m.ir);
    }
    storePrimRec(V, i, m.rf, m.uf, m.vf, m.wf, (float)m.pr);
  } else {
    double pr, t, c;
    dependentVars(V.p, cv, pr, t, c);
    V.dv[i] = pr;
    V.dv[(size_t)V.nc + i] = t;
    V.dv[2 * (size_t)V.nc + i] = c;
    storePrim(V, i, cv, pr);
  }
}

template <typename R>
__global__ void kInitState(View<R> V) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  double cv[5];
  loadCv(V, i, cv);
  initCell(V, i, cv);
}

// Upload in one pass: cv(5,nCells) in the reference's order and layout
// (staged on the device) -> the renumbered master cv, primitive state and
// dependent variables; one thread per reference cell o0 .. o1-1 (contiguous
// reads).
template <typename R>
__global__ void kInitFromRef(View<R> V, const double *ref, int o0, int o1) {
  const int o = o0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= o1) return;
  const int i = V.newId[o];
  double cv[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    cv[k] = ref[5 * (size_t)o + k];
    V.cv[(size_t)k * V.nc + i] = cv[k];
  }
  initCell(V, i, cv);
}

// ---------------------------------------------------------------------------
// Constraint value of primitive variable k at boundary face b
// (RFLU_GetConstrValue, modflu/RFLU_ModConstraintUtils.F90:366-745, TCPERF,
// static grid): 0 for the velocity at walls; at an injection face, fsu * n
// (fsu = 0) when it does not burn, else the density and velocity of
// RFLU_SetRindStateInjectPerf (modflu/RFLU_ModRindStates.F90:459-501) from
// the face cell's pressure.
template <typename S, typename R, typename L>
__device__ inline S constrValue(const View<R> &V, const L &ld, int b, int k) {
  const int ip = V.bpatch[b];
  if (V.patchType[ip] != 90) return S(0);
  const double *K = V.patchK + kPatchK * ip;
  const S n = (k == 1) ? S(V.bnx[b]) : (k == 2) ? S(V.bny[b]) : S(V.bnz[b]);
  if (!(K[0] > 0.0)) return S(0) * n;
  const S rgas = S(8314.3) / S(V.p.gvMol);
  // the face's cell pressure through the loader (the tangent's carries its
  // derivative)
  const S rl = S(ld.dv(0, V.bcell[b])) / (rgas * S(K[1]));  // MixtPerf_D_PRT(pl, rGas, tInj)
  if (k == 0) return rl;
  const S ql = -S(K[0]) / rl + S(0);
  return ql * n;
}

// The constrained gradients of cell i (slot sl) for CRECONSTC 1
// (RFLU_ComputeGradCellsConstr, modflu/RFLU_ModDifferentiationCells.F90:
// 1180-1563): every variable some face of the cell's boundary-face stencil
// constrains gets the fit to its stencil differences and constraint values
// through the planned weights (constr.h), rows in the reference's order;
// the others keep their least-squares gradient.
template <typename R, typename L>
__device__ inline void constrainedGrad(const View<R> &V, const L &ld, int i, int sl, const typename L::S *q,
                                       typename L::S *g) {
  using S = typename L::S;
  int r = V.cRowOff[sl];
  const int sb = V.stOff[i], se = V.stOff[i + 1];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int nCon = V.cNcon[5 * sl + k];
    if (nCon == 0) continue;
    S gx = S(0), gy = S(0), gz = S(0);
    for (int s = sb; s < se; ++s, ++r) {
      const S d = ld.prim(k, V.stIdx[s]) - q[k];
      gx = gx + S(V.cW[3 * (size_t)r]) * d;
      gy = gy + S(V.cW[3 * (size_t)r + 1]) * d;
      gz = gz + S(V.cW[3 * (size_t)r + 2]) * d;
    }
    for (int c = 0; c < nCon; ++c, ++r) {
      const S d = constrValue<S>(V, ld, V.cRowFace[r], k) - q[k];
      gx = gx + S(V.cW[3 * (size_t)r]) * d;
      gy = gy + S(V.cW[3 * (size_t)r + 1]) * d;
      gz = gz + S(V.cW[3 * (size_t)r + 2]) * d;
    }
    g[3 * k] = gx;
    g[3 * k + 1] = gy;
    g[3 * k + 2] = gz;
  }
}

// Symmetry patches (RFLU_BC_SYMMETRY): a face on one is an interior face to
// the cell's reflection across it (the reference's virtual cell, modflu/
// RFLU_ModSymmetryPeriodic.F90:471-787, whose momentum is reflected,
// modflu/RFLU_ModRelatedPatches.F90:268-353), and a stencil member may be
// seen reflected (V.stXf).  y = Q x for a row-major 3x3 Q, summed in index
// order.
template <typename S, typename Qt>
__device__ inline void reflect3(const Qt *Q, const S *x, S *y) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    S t = S(Q[3 * a]) * x[0];
    t = t + S(Q[3 * a + 1]) * x[1];
    t = t + S(Q[3 * a + 2]) * x[2];
    y[a] = t;
  }
}
// The reflection of a boundary face entry (code < 0) on a symmetry patch,
// else null.
template <typename R>
__device__ inline const double *symmetryQ(const View<R> &V, int code) {
  if (code >= 0) return nullptr;
  const int ip = V.bpatch[-code - 1];
  return V.patchType[ip] == kBcSymmetry ? V.patchK + kPatchK * ip : nullptr;
}
// The offset fc - cofg of a cell's face entry for the limiters' face loops:
// an interior face's, a symmetry face's (an interior face to the cell's
// reflection); false for the other boundary faces.
template <typename R>
__device__ inline bool limiterFaceOffset(const View<R> &V, int code, R *d) {
  if (code >= 0) {
    faceOffset(V, code >> 1, code & 1, d);
    return true;
  }
  if (!symmetryQ(V, code)) return false;
  const int b = -code - 1;
  const size_t nb = V.nb;
  d[0] = V.bd[b];
  d[1] = V.bd[nb + b];
  d[2] = V.bd[2 * nb + b];
  return true;
}
// A reflected stencil member's raw gradient (15 components, 3 * var + dir):
// Q g for density and pressure, Q G Q^T for the velocity gradient
// (RFLU_RELP_TransformGradWrapper, modflu/RFLU_ModRelatedPatches.F90:380-435).
template <typename S, typename Qt>
__device__ inline void reflectGrad(const Qt *Q, S *g) {
  S t[3];
  reflect3(Q, g, t);
  g[0] = t[0]; g[1] = t[1]; g[2] = t[2];
  reflect3(Q, g + 12, t);
  g[12] = t[0]; g[13] = t[1]; g[14] = t[2];
  S T[9];
#pragma unroll
  for (int b = 0; b < 3; ++b)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      S x = g[3 * (1 + b)] * S(Q[3 * c]);
      x = x + g[3 * (1 + b) + 1] * S(Q[3 * c + 1]);
      x = x + g[3 * (1 + b) + 2] * S(Q[3 * c + 2]);
      T[3 * b + c] = x;
    }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      S x = S(Q[3 * a]) * T[c];
      x = x + S(Q[3 * a + 1]) * T[3 + c];
      x = x + S(Q[3 * a + 2]) * T[6 + c];
      g[3 * (1 + a) + c] = x;
    }
}

// Gradient + limiter of one cell.
// LSQ gradient: RFLU_ComputeGradCellsFast_3D (modflu/RFLU_ModDifferentiationCells.F90:
// 931-1178) with the per-member weights precomputed at set-up.
// Limiters: RFLU_ComputeLimiterBarthJesp (modflu/RFLU_ModLimiters.F90:132-322),
// RFLU_ComputeLimiterVenkat (:353-587), RFLU_LimitGradVelocityBarthJesp
// (:588-790), RFLU_LimitGradCells (:1061-1146).  Each cell's limiter needs
// only its own gradient and its face neighbours' values, so the reference's
// two face sweeps become two loops over the cell's own faces.
// ---------------------------------------------------------------------------
template <typename R, typename L>
__device__ inline void gradLimitCell(const View<R> &V, const L &ld, int i, typename L::S *g) {
  using S = typename L::S;
  S q[5];
  ld.prim5(i, q);
#pragma unroll
  for (int k = 0; k < 15; ++k) g[k] = S(0);
  const int sb = V.stOff[i], se = V.stOff[i + 1];
  if constexpr (Ref<R>::on) {
#pragma unroll 2
    for (int s = sb; s < se; ++s) {
      const int j = V.stIdx[s];
      const S wx = S(V.wx[s]), wy = S(V.wy[s]), wz = S(V.wz[s]);
      S qj[5];
      ld.prim5(j, qj);
      if (V.stXf) {  // a member seen reflected across symmetry patches
        const int x = V.stXf[s];
        if (x >= 0) {
          const S u[3] = {qj[1], qj[2], qj[3]};
          reflect3(V.xfQ + 9 * x, u, qj + 1);
        }
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        S d = qj[k] - q[k];
        g[3 * k] = g[3 * k] + wx * d;
        g[3 * k + 1] = g[3 * k + 1] + wy * d;
        g[3 * k + 2] = g[3 * k + 2] + wz * d;
      }
    }
    if (V.cSlot) {
      const int sl = V.cSlot[i];
      if (sl >= 0) constrainedGrad(V, ld, i, sl, q, g);
    }
  } else {
    // mixed mode (the tangent kernels): G = L sum_j (q_j - q_i) d_j/|d_j|^2,
    // the formulation of gradLimitPacked; centroids carry no derivative
    S qi[5], xi[3];
    ld.primCg(i, qi, xi);
#pragma unroll 2
    for (int s = sb; s < se; ++s) {
      S qj[5], xj[3];
      ld.primCg(V.stIdx[s], qj, xj);
      S dx = xj[0] - xi[0], dy = xj[1] - xi[1], dz = xj[2] - xi[2];
      if (V.stShift) {  // a periodic or symmetry mesh: the member's image
        dx = dx + S(V.stShift[3 * (size_t)s]);
        dy = dy + S(V.stShift[3 * (size_t)s + 1]);
        dz = dz + S(V.stShift[3 * (size_t)s + 2]);
        if (V.stXf && V.stXf[s] >= 0) {
          const S u[3] = {qj[1], qj[2], qj[3]};
          reflect3(V.xfQ + 9 * V.stXf[s], u, qj + 1);
        }
      }
      const S inv = S(1) / (dx * dx + dy * dy + dz * dz);
      const S sx = inv * dx, sy = inv * dy, sz = inv * dz;
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const S d = qj[k] - q[k];
        g[3 * k] = g[3 * k] + sx * d;
        g[3 * k + 1] = g[3 * k + 1] + sy * d;
        g[3 * k + 2] = g[3 * k + 2] + sz * d;
      }
    }
    const size_t n = V.nc;
    const S lxx = S(V.lsq[i]), lxy = S(V.lsq[n + i]), lxz = S(V.lsq[2 * n + i]);
    const S lyy = S(V.lsq[3 * n + i]), lyz = S(V.lsq[4 * n + i]), lzz = S(V.lsq[5 * n + i]);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const S x = g[3 * k], y = g[3 * k + 1], z = g[3 * k + 2];
      g[3 * k] = lxx * x + lxy * y + lxz * z;
      g[3 * k + 1] = lxy * x + lyy * y + lyz * z;
      g[3 * k + 2] = lxz * x + lyz * y + lzz * z;
    }
    if (V.cSlot) {
      const int sl = V.cSlot[i];
      if (sl >= 0) constrainedGrad(V, ld, i, sl, q, g);
    }
  }
  const int rc = V.p.reconst;
  const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
  if (rc == 10 || rc == 100 || rc == 11) {
    // scalar limiters: min/max over face neighbours, then per face side
    S vmin[5], vmax[5], lim[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) { vmin[k] = q[k]; vmax[k] = q[k]; lim[k] = S(1); }
    for (int e = cb; e < ce; ++e) {
      const int code = V.cfEnt[e];
      S x[5];
      if (code < 0) {
        // a symmetry face: the neighbour is the cell's reflection
        const double *Q = symmetryQ(V, code);
        if (!Q) continue;
        x[0] = q[0];
        reflect3(Q, q + 1, x + 1);
        x[4] = q[4];
      } else {
        const int f = code >> 1;
        int c1, c2;
        faceCells(V, f, c1, c2);
        const int nb = (code & 1) ? c1 : c2;
        ld.prim5(nb, x);
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        vmin[k] = fmin2(vmin[k], x[k]);
        vmax[k] = fmax2(vmax[k], x[k]);
      }
    }
    S epsq = (rc == 11) ? S(V.epsq[i]) : S(0);
    // Barth-Jespersen on plain floating-point types: the minimum over faces
    // of dmax/d2 (d2 > 0) is dmax over the largest d2, because correctly
    // rounded division is monotone and dmax >= 0, and likewise dmin over the
    // most negative d2: one division per variable and sign instead of one
    // per face, with the same values (signed zeros aside).  The tangent
    // types keep the per-face form, whose ties pick the first face.
    constexpr bool kOnePass = std::is_floating_point<S>::value;
    S pmx[5], nmn[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) { pmx[k] = S(0); nmn[k] = S(0); }
    for (int e = cb; e < ce; ++e) {
      const int code = V.cfEnt[e];
      R d[3];
      if (!limiterFaceOffset(V, code, d)) continue;
      const S dx = S(d[0]), dy = S(d[1]), dz = S(d[2]);
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        if (rc == 10 && k >= 1 && k <= 3) continue;
        // d2 = grad . (cofg - fc), the reference's sign
        S d2 = -(g[3 * k] * dx + g[3 * k + 1] * dy + g[3 * k + 2] * dz);
        S dmax = vmax[k] - q[k], dmin = vmin[k] - q[k];
        if (kOnePass && rc != 11) {
          if (d2 > S(0)) pmx[k] = fmax2(pmx[k], d2);
          else if (d2 < S(0)) nmn[k] = fmin2(nmn[k], d2);
        } else if (rc == 11) {
          const S tiny = S(1.0e-12);
          if (d2 > S(0)) {
            S numer = (dmax * dmax + epsq) * d2 + S(2) * d2 * d2 * dmax;
            S denom = d2 * (dmax * dmax + S(2) * d2 * d2 + dmax * d2 + epsq);
            lim[k] = fmin2(numer / (denom + tiny), lim[k]);
          } else if (d2 < S(0)) {
            S numer = (dmin * dmin + epsq) * d2 + S(2) * d2 * d2 * dmin;
            S denom = d2 * (dmin * dmin + S(2) * d2 * d2 + dmin * d2 + epsq);
            lim[k] = fmin2(numer / (denom + tiny), lim[k]);
          }
        } else {
          if (d2 > S(0)) lim[k] = fmin2(fmin2(S(1), dmax / d2), lim[k]);
          else if (d2 < S(0)) lim[k] = fmin2(fmin2(S(1), dmin / d2), lim[k]);
        }
      }
    }
    if (kOnePass && rc != 11) {
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        if (rc == 10 && k >= 1 && k <= 3) continue;
        const S dmax = vmax[k] - q[k], dmin = vmin[k] - q[k];
        if (pmx[k] > S(0)) lim[k] = fmin2(fmin2(S(1), dmax / pmx[k]), lim[k]);
        if (nmn[k] < S(0)) lim[k] = fmin2(fmin2(S(1), dmin / nmn[k]), lim[k]);
      }
    }
    if (rc == 10) {
      // frame-invariant velocity limiting along the strain-rate eigenvectors
      S G[9], Sy[9], A[9], ev[3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) G[a + 3 * b] = g[3 * (1 + a) + b];  // G(iComp, dir)
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) Sy[a + 3 * b] = S(0.5) * (G[a + 3 * b] + G[b + 3 * a]);
      symmetricEigen3(Sy, A, ev);
      S dmn[3] = {S(0), S(0), S(0)}, dmx[3] = {S(0), S(0), S(0)}, al[3] = {S(1), S(1), S(1)};
      S spx[3] = {S(0), S(0), S(0)}, snx[3] = {S(0), S(0), S(0)};  // extreme projections (one pass)
      for (int e = cb; e < ce; ++e) {
        const int code = V.cfEnt[e];
        S du[3];
        int side = 0;
        if (code < 0) {
          // a symmetry face: the cell's reflection as the second cell
          const double *Q = symmetryQ(V, code);
          if (!Q) continue;
          S um[3];
          reflect3(Q, q + 1, um);
#pragma unroll
          for (int k = 0; k < 3; ++k) du[k] = um[k] - q[1 + k];
        } else {
          const int f = code >> 1;
          side = code & 1;
          int c1, c2;
          faceCells(V, f, c1, c2);
          S a1[4], a2[4];
          ld.prim4(c1, a1);
          ld.prim4(c2, a2);
#pragma unroll
          for (int k = 0; k < 3; ++k) du[k] = a2[1 + k] - a1[1 + k];
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          S pr = S(0);
          pr = pr + A[3 * j] * du[0];
          pr = pr + A[3 * j + 1] * du[1];
          pr = pr + A[3 * j + 2] * du[2];
          if (side) pr = -pr;
          dmn[j] = fmin2(dmn[j], pr);
          dmx[j] = fmax2(dmx[j], pr);
        }
      }
      for (int e = cb; e < ce; ++e) {
        const int code = V.cfEnt[e];
        R d[3];
        if (!limiterFaceOffset(V, code, d)) continue;
        const S off[3] = {-S(d[0]), -S(d[1]), -S(d[2])};
        S sh[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          S s = S(0);
          s = s + G[a] * off[0];
          s = s + G[a + 3] * off[1];
          s = s + G[a + 6] * off[2];
          sh[a] = s;
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          S pr = S(0);
          pr = pr + A[3 * j] * sh[0];
          pr = pr + A[3 * j + 1] * sh[1];
          pr = pr + A[3 * j + 2] * sh[2];
          if (kOnePass) {
            if (pr > S(0)) spx[j] = fmax2(spx[j], pr);
            else if (pr < S(0)) snx[j] = fmin2(snx[j], pr);
          } else {
            if (pr > S(0)) al[j] = fmin2(al[j], dmx[j] / pr);
            else if (pr < S(0)) al[j] = fmin2(al[j], dmn[j] / pr);
          }
        }
      }
      if (kOnePass) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          if (spx[j] > S(0)) al[j] = fmin2(al[j], dmx[j] / spx[j]);
          if (snx[j] < S(0)) al[j] = fmin2(al[j], dmn[j] / snx[j]);
        }
      }
      holdIdleAxes(A, G, al);
      S mx = fabs_(ev[0]);
      mx = fmax2(mx, fabs_(ev[1]));
      mx = fmax2(mx, fabs_(ev[2]));
      const S scale = S(1.0e-3) * mx;
      const bool e12 = (ev[1] - ev[0] <= scale), e23 = (ev[2] - ev[1] <= scale);
      if (e12 && e23) {
        S m = fmin2(fmin2(al[0], al[1]), al[2]);
        al[0] = al[1] = al[2] = m;
      } else if (e12) {
        S m = fmin2(al[0], al[1]);
        al[0] = al[1] = m;
      } else if (e23) {
        S m = fmin2(al[1], al[2]);
        al[1] = al[2] = m;
      }
      // G <- A diag(alpha) A^T G
      S Rm[9];
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          S s = S(0);
          s = s + A[3 * j] * G[3 * c];
          s = s + A[3 * j + 1] * G[1 + 3 * c];
          s = s + A[3 * j + 2] * G[2 + 3 * c];
          Rm[j + 3 * c] = al[j] * s;
        }
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          S s = S(0);
          s = s + A[a] * Rm[3 * c];
          s = s + A[a + 3] * Rm[1 + 3 * c];
          s = s + A[a + 6] * Rm[2 + 3 * c];
          g[3 * (1 + a) + c] = s;
        }
      lim[1] = lim[2] = lim[3] = S(1);
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      g[3 * k] = lim[k] * g[3 * k];
      g[3 * k + 1] = lim[k] * g[3 * k + 1];
      g[3 * k + 2] = lim[k] * g[3 * k + 2];
    }
  }
}

// The mixed-mode cell kernel: the same gradient and limiter as gradLimitCell
// (and, with kDt, the spectral-radius sum of RFLU_TimeStepInviscid) in one
// pass over the cell's faces instead of five.  The strain-rate eigenframe
// needs only the unlimited gradient, so the velocity projections are taken in
// the same pass as the neighbour min/max.  Venkatakrishnan keeps each face's
// offset fc - cofg in shared memory (dc, stride kBlock) for its second pass;
// at most kMaxCellFaces faces per cell (tetrahedra 4, prisms and pyramids 5,
// hexahedra 6).  With kTiled the cell's, its stencil members' and its face
// neighbours' prim records come from the CTA's staged tile (recs, local ids)
// and its faces from the entry-major arrays feD/feN; otherwise they are
// gathered from global memory.  kRc is the limiter (RECONST) when fixed at
// compile time, -1 to read it from the parameters.  Returns the
// spectral-radius sum (kDt) or 0.
//
// LSQ gradient (RFLU_ComputeGradCellsFast_3D, modflu/
// RFLU_ModDifferentiationCells.F90:983-1044): the reference's per-member
// weights are w_j = L d_j / |d_j|^2 with L the cell's symmetric matrix of
// R-factor products, so G = L * sum_j (q_j - q_i) d_j / |d_j|^2.
constexpr int kMaxCellFaces = 6;

// A staged record's two 16-byte halves are swapped when bit 2 of its local id
// is set: the first halves of 8 consecutive records then cover all eight
// 16-byte bank groups of a 128-byte row instead of four, and a quarter-warp's
// 16-byte loads of neighbouring records do not conflict.
__device__ inline int recHalf0(int l) { return 8 * l + (l & 4); }

// One approximate reciprocal (rcp.approx.ftz.f32) where the argument is a
// squared distance between cell centroids: a normal float for any mesh whose
// cells are wider than ~1e-19 in its length unit, so the flush of denormals
// never acts and the compiler's general reciprocal sequence is not needed.
__device__ inline float rcpDist2(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ inline void ldRec(const float *recs, int l, float *v) {
  const int o = recHalf0(l);
  const float4 a = *reinterpret_cast<const float4 *>(recs + o);
  const float4 b = *reinterpret_cast<const float4 *>(recs + (o ^ 4));
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

// Spectral-radius sum of RFLU_TimeStepInviscid (rocflu/
// RFLU_TimeStepInviscid.F90:165-293) for cell i of a tile staged in shared
// memory, in FP32: its face entries and normals are all loaded first, then
// the neighbours' records are read from the tile.  q, ai: the cell's
// primitive state and sound speed.
__device__ inline float tileDtSum(const View<float> &V, int i, const float *recs, const float *q, float ai) {
  const size_t n = V.nc;
  const float gam = V.p.refGammaF;
  float sum = 0.f;
  float4 Dt[kMaxCellFaces], Nt[kMaxCellFaces];
#pragma unroll
  for (int k = 0; k < kMaxCellFaces; ++k) {
    if (k < V.cfW) {
      Dt[k] = ld4(V.feD + 4 * (k * n + i));
      Nt[k] = ld4(V.feN + 4 * (k * n + i));
    } else {
      Dt[k].w = __int_as_float(INT_MIN);
    }
  }
#pragma unroll
  for (int k = 0; k < kMaxCellFaces; ++k) {
    const int tag = __float_as_int(Dt[k].w);
    if (tag >= 0) {
      float x[8];
      ldRec(recs, tag, x);
      const float aj = sqrtf(gam * x[4] / x[0]);
      const float vc = 0.5f * ((q[1] + x[1]) * Nt[k].x + (q[2] + x[2]) * Nt[k].y + (q[3] + x[3]) * Nt[k].z);
      sum += (fabsf(vc) + 0.5f * (ai + aj)) * Nt[k].w;
    } else if (tag != INT_MIN) {
      const float vc = q[1] * Nt[k].x + q[2] * Nt[k].y + q[3] * Nt[k].z;
      sum += (fabsf(vc) + ai) * Nt[k].w;
    }
  }
  return sum;
}

template <bool kDt, bool kTiled, int kRc>
__device__ inline float gradLimitPacked(const View<float> &V, int i, float *g, float *dc, const float *recs,
                                        int li, const unsigned short *stSm = nullptr,
                                        const int *stOffSm = nullptr) {
  const Params &P = V.p;
  const size_t n = V.nc;
  const int rc = kRc >= 0 ? kRc : P.reconst;
  const bool second = P.spaceOrder > 1;
  const bool lim = second && (rc == 10 || rc == 100 || rc == 11);
  // The tiled path issues its per-cell global loads (LSQ matrix,
  // Venkatakrishnan epsilon) before the stencil loop, which runs from shared
  // memory and hides their latency, and all of its face entries at once after
  // it.  Every cell has V.cfW entries in feD/feN; the unused ones carry the
  // tag INT_MIN.
  float4 De[kMaxCellFaces];
  float lq[6];
  float epsq = 0.f;
  if (kTiled) {
    if (second) {
#pragma unroll
      for (int c = 0; c < 6; ++c) lq[c] = V.lsq[c * n + i];
    }
    if (lim && rc == 11) epsq = V.epsq[i];
  }
  float rec[8];
  if (kTiled) ldRec(recs, li, rec);
  else ld8(V.prim + 8 * (size_t)i, rec);
  const float q[5] = {rec[0], rec[1], rec[2], rec[3], rec[4]};
  const float gam = P.refGammaF;
  const float ai = kDt ? sqrtf(gam * q[4] / q[0]) : 0.f;
  float sum = 0.f;
  // the spectral-radius sum of the time step first, while no gradient state
  // is live
  if (kTiled && kDt) sum = tileDtSum(V, i, recs, q, ai);
#pragma unroll
  for (int k = 0; k < 15; ++k) g[k] = 0.f;
  if (second) {
    // tiled: s counts from the first staged 16-byte word of stencil ids
    const int s0 = kTiled ? 8 * (stOffSm[0] >> 3) : 0;
    const int sb = (kTiled ? stOffSm[li] : V.stOff[i]) - s0, se = (kTiled ? stOffSm[li + 1] : V.stOff[i + 1]) - s0;
    if (kTiled) {
      // Packed FP32 pairs (f32x2): the record's register pairs (rho, u),
      // (v, w), (p, xc), (yc, zc) give the eight differences in four adds,
      // and the sums of (rho, u) and (v, w) advance in pairs per direction.
      // Each lane rounds as the scalar loop below does.
      const float2 n01 = make_float2(-rec[0], -rec[1]), n23 = make_float2(-rec[2], -rec[3]);
      const float2 n4x = make_float2(-rec[4], -rec[5]), nyz = make_float2(-rec[6], -rec[7]);
      float2 gx01 = make_float2(0.f, 0.f), gx23 = gx01, gy01 = gx01, gy23 = gx01, gz01 = gx01, gz23 = gx01;
      float gx4 = 0.f, gy4 = 0.f, gz4 = 0.f;
#pragma unroll 4
      for (int s = sb; s < se; ++s) {
        const int o = recHalf0(stSm[s]);
        const float4 a = *reinterpret_cast<const float4 *>(recs + o);
        const float4 b = *reinterpret_cast<const float4 *>(recs + (o ^ 4));
        const float2 d01 = __fadd2_rn(make_float2(a.x, a.y), n01);
        const float2 d23 = __fadd2_rn(make_float2(a.z, a.w), n23);
        const float2 d4x = __fadd2_rn(make_float2(b.x, b.y), n4x);
        const float2 dyz = __fadd2_rn(make_float2(b.z, b.w), nyz);
        const float dx = d4x.y, dy = dyz.x, dz = dyz.y;
        const float inv = rcpDist2(dx * dx + dy * dy + dz * dz);
        const float sx = inv * dx, sy = inv * dy, sz = inv * dz;
        const float2 sx2 = make_float2(sx, sx), sy2 = make_float2(sy, sy), sz2 = make_float2(sz, sz);
        gx01 = __ffma2_rn(sx2, d01, gx01);
        gx23 = __ffma2_rn(sx2, d23, gx23);
        gy01 = __ffma2_rn(sy2, d01, gy01);
        gy23 = __ffma2_rn(sy2, d23, gy23);
        gz01 = __ffma2_rn(sz2, d01, gz01);
        gz23 = __ffma2_rn(sz2, d23, gz23);
        gx4 = fmaf(sx, d4x.x, gx4);
        gy4 = fmaf(sy, d4x.x, gy4);
        gz4 = fmaf(sz, d4x.x, gz4);
      }
      g[0] = gx01.x; g[1] = gy01.x; g[2] = gz01.x;
      g[3] = gx01.y; g[4] = gy01.y; g[5] = gz01.y;
      g[6] = gx23.x; g[7] = gy23.x; g[8] = gz23.x;
      g[9] = gx23.y; g[10] = gy23.y; g[11] = gz23.y;
      g[12] = gx4; g[13] = gy4; g[14] = gz4;
    } else {
#pragma unroll 2
      for (int s = sb; s < se; ++s) {
        float r[8];
        ld8(V.prim + 8 * (size_t)V.stIdx[s], r);
        float dx = r[5] - rec[5], dy = r[6] - rec[6], dz = r[7] - rec[7];
        if (V.stShift) {  // a periodic or symmetry mesh: the member's image
          dx = dx + V.stShift[3 * (size_t)s];
          dy = dy + V.stShift[3 * (size_t)s + 1];
          dz = dz + V.stShift[3 * (size_t)s + 2];
          if (V.stXf) {
            const int x = V.stXf[s];
            if (x >= 0) {
              const float u[3] = {r[1], r[2], r[3]};
              reflect3(V.xfQ + 9 * x, u, r + 1);
            }
          }
        }
        const float inv = 1.f / (dx * dx + dy * dy + dz * dz);
        const float sx = inv * dx, sy = inv * dy, sz = inv * dz;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const float d = r[k] - q[k];
          g[3 * k] = g[3 * k] + sx * d;
          g[3 * k + 1] = g[3 * k + 1] + sy * d;
          g[3 * k + 2] = g[3 * k + 2] + sz * d;
        }
      }
    }
  }
  if (kTiled) {
#pragma unroll
    for (int k = 0; k < kMaxCellFaces; ++k) {
      if (lim && k < V.cfW) De[k] = ld4(V.feD + 4 * (k * n + i));
      else De[k] = make_float4(0.f, 0.f, 0.f, __int_as_float(INT_MIN));
    }
  }
  if (second) {
    if (!kTiled) {
#pragma unroll
      for (int c = 0; c < 6; ++c) lq[c] = V.lsq[c * n + i];
    }
    const float lxx = lq[0], lxy = lq[1], lxz = lq[2], lyy = lq[3], lyz = lq[4], lzz = lq[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const float x = g[3 * k], y = g[3 * k + 1], z = g[3 * k + 2];
      g[3 * k] = lxx * x + lxy * y + lxz * z;
      g[3 * k + 1] = lxy * x + lyy * y + lyz * z;
      g[3 * k + 2] = lxz * x + lyz * y + lzz * z;
    }
    if (V.cSlot) {  // constrained cells (CRECONSTC 1) read their members from global memory
      const int sl = V.cSlot[i];
      if (sl >= 0) constrainedGrad(V, PlainLoad<float>{V}, i, sl, q, g);
    }
  }
  const bool velo = lim && rc == 10;
  const bool venkat = lim && rc == 11;
  // velocity limiter frame: eigenvectors A(:, j) = A[3j..3j+2] of the
  // strain rate, and B = A^T G with G(comp, dir) the velocity gradient
  float A[9], B[9];
  bool e12 = false, e23 = false;  // eigenvalues merged (within 1e-3 of the largest magnitude)
  if (velo) {
    float G[9], Sy[9], ev[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) G[a + 3 * b] = g[3 * (1 + a) + b];  // G(iComp, dir)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) Sy[a + 3 * b] = 0.5f * (G[a + 3 * b] + G[b + 3 * a]);
    symmetricEigen3(Sy, A, ev);
    float mx = fabsf(ev[0]);
    mx = fmax2(mx, fabsf(ev[1]));
    mx = fmax2(mx, fabsf(ev[2]));
    const float scale = 1.0e-3f * mx;
    e12 = (ev[1] - ev[0] <= scale);
    e23 = (ev[2] - ev[1] <= scale);
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int c = 0; c < 3; ++c) B[3 * j + c] = A[3 * j] * G[3 * c] + A[3 * j + 1] * G[1 + 3 * c] + A[3 * j + 2] * G[2 + 3 * c];
  }
  // Barth-Jespersen in one pass: min over faces of dmax/d2 (d2 > 0) is
  // dmax / (largest positive d2), and likewise dmin / (most negative d2), so
  // the pass keeps the extreme d2 per component (pmx, nmn) next to the
  // neighbour extremes; the velocity limiter keeps the extreme projections of
  // the face increments (smx, smn) next to those of the neighbour differences
  // (dmx, dmn).  Venkatakrishnan needs the final extremes per face and takes
  // a second pass over the offsets kept in dc.
  float vmin[5], vmax[5], pmx[5], nmn[5];
  float dmn[3] = {0.f, 0.f, 0.f}, dmx[3] = {0.f, 0.f, 0.f}, smn[3] = {0.f, 0.f, 0.f}, smx[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 5; ++k) { vmin[k] = q[k]; vmax[k] = q[k]; pmx[k] = 0.f; nmn[k] = 0.f; }
  int nfc = 0;
  // one face of the pass: neighbour record x, offset d = fc - cofg of this side
  auto face = [&](const float *x, float d0, float d1, float d2) {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      if (velo && k >= 1 && k <= 3) continue;
      vmin[k] = fmin2(vmin[k], x[k]);
      vmax[k] = fmax2(vmax[k], x[k]);
      if (!venkat) {
        // grad . (cofg - fc), the reference's sign
        const float dd = -(g[3 * k] * d0 + g[3 * k + 1] * d1 + g[3 * k + 2] * d2);
        if (dd > 0.f) pmx[k] = fmax2(pmx[k], dd);
        else if (dd < 0.f) nmn[k] = fmin2(nmn[k], dd);
      }
    }
    if (velo) {
      // A^T (u(c2) - u(c1)) seen from this cell = A^T (u(nb) - u(i))
      const float du0 = x[1] - q[1], du1 = x[2] - q[2], du2 = x[3] - q[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        float pr = 0.f;
        pr = pr + A[3 * j] * du0;
        pr = pr + A[3 * j + 1] * du1;
        pr = pr + A[3 * j + 2] * du2;
        dmn[j] = fmin2(dmn[j], pr);
        dmx[j] = fmax2(dmx[j], pr);
        // A^T G (cofg - fc)
        const float ps = -(B[3 * j] * d0 + B[3 * j + 1] * d1 + B[3 * j + 2] * d2);
        if (ps > 0.f) smx[j] = fmax2(smx[j], ps);
        else if (ps < 0.f) smn[j] = fmin2(smn[j], ps);
      }
    }
    if (venkat) {
      float *slot = dc + 3 * nfc * kBlock;
      slot[0] = d0;
      slot[kBlock] = d1;
      slot[2 * kBlock] = d2;
      ++nfc;
    }
  };
  if (kTiled) {
    if (lim) {
#pragma unroll
      for (int k = 0; k < kMaxCellFaces; ++k) {
        const int tag = __float_as_int(De[k].w);
        if (tag >= 0) {
          float x[8];
          ldRec(recs, tag, x);
          face(x, De[k].x, De[k].y, De[k].z);
        }
      }
    }
  } else {
    const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
    for (int e = cb; e < ce; ++e) {
      const int code = V.cfEnt[e];
      if (code >= 0) {
        if (!lim && !kDt) continue;
        const int f = code >> 1, side = code & 1;
        const float *fr = V.fpk + 12 * (size_t)f;
        const float4 F1 = ld4(fr + 4), F2 = ld4(fr + 8);
        const int nb = side ? __float_as_int(F2.z) : __float_as_int(F2.w);
        float x[8];
        ld8(V.prim + 8 * (size_t)nb, x);
        if (lim) face(x, side ? F1.w : F1.x, side ? F2.x : F1.y, side ? F2.y : F1.z);
        if (kDt) {
          const float4 F0 = ld4(fr);
          const float aj = sqrtf(gam * x[4] / x[0]);
          const float vc = 0.5f * ((q[1] + x[1]) * F0.x + (q[2] + x[2]) * F0.y + (q[3] + x[3]) * F0.z);
          sum += (fabsf(vc) + 0.5f * (ai + aj)) * F0.w;
        }
      } else if (const double *Q = symmetryQ(V, code)) {
        // a symmetry face: an interior face to the cell's reflection
        const int b = -code - 1;
        const size_t nb = V.nb;
        float x[8];
        x[0] = q[0];
        reflect3(Q, q + 1, x + 1);
        x[4] = q[4];
        if (lim) face(x, V.bd[b], V.bd[nb + b], V.bd[2 * nb + b]);
        if (kDt) {
          const float vc = 0.5f * ((q[1] + x[1]) * V.bnx[b] + (q[2] + x[2]) * V.bny[b] + (q[3] + x[3]) * V.bnz[b]);
          sum += (fabsf(vc) + 0.5f * (ai + ai)) * V.bnm[b];
        }
      } else if (kDt) {
        const int b = -code - 1;
        const float vc = q[1] * V.bnx[b] + q[2] * V.bny[b] + q[3] * V.bnz[b];
        sum += (fabsf(vc) + ai) * V.bnm[b];
      }
    }
  }
  if (!lim) return sum;
  float lm[5] = {1.f, 1.f, 1.f, 1.f, 1.f};
  if (venkat) {
    if (!kTiled) epsq = V.epsq[i];
    const float tiny = 1.0e-12f;
    for (int c = 0; c < nfc; ++c) {
      const float *slot = dc + 3 * c * kBlock;
      const float dx = slot[0], dy = slot[kBlock], dz = slot[2 * kBlock];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const float d2 = -(g[3 * k] * dx + g[3 * k + 1] * dy + g[3 * k + 2] * dz);
        const float dmax = vmax[k] - q[k], dmin = vmin[k] - q[k];
        if (d2 > 0.f) {
          const float numer = (dmax * dmax + epsq) * d2 + 2.f * d2 * d2 * dmax;
          const float denom = d2 * (dmax * dmax + 2.f * d2 * d2 + dmax * d2 + epsq);
          lm[k] = fmin2(numer / (denom + tiny), lm[k]);
        } else if (d2 < 0.f) {
          const float numer = (dmin * dmin + epsq) * d2 + 2.f * d2 * d2 * dmin;
          const float denom = d2 * (dmin * dmin + 2.f * d2 * d2 + dmin * d2 + epsq);
          lm[k] = fmin2(numer / (denom + tiny), lm[k]);
        }
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      if (velo && k >= 1 && k <= 3) continue;
      if (pmx[k] > 0.f) lm[k] = fmin2(fmin2(1.f, (vmax[k] - q[k]) / pmx[k]), lm[k]);
      if (nmn[k] < 0.f) lm[k] = fmin2(fmin2(1.f, (vmin[k] - q[k]) / nmn[k]), lm[k]);
    }
  }
  if (velo) {
    float al[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      al[j] = 1.f;
      if (smx[j] > 0.f) al[j] = fmin2(al[j], dmx[j] / smx[j]);
      if (smn[j] < 0.f) al[j] = fmin2(al[j], dmn[j] / smn[j]);
    }
    if (e12 && e23) {
      const float m = fmin2(fmin2(al[0], al[1]), al[2]);
      al[0] = al[1] = al[2] = m;
    } else if (e12) {
      const float m = fmin2(al[0], al[1]);
      al[0] = al[1] = m;
    } else if (e23) {
      const float m = fmin2(al[1], al[2]);
      al[1] = al[2] = m;
    }
    // G <- A diag(alpha) A^T G = A diag(alpha) B
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        g[3 * (1 + a) + c] = A[a] * (al[0] * B[c]) + A[a + 3] * (al[1] * B[3 + c]) + A[a + 6] * (al[2] * B[6 + c]);
    lm[1] = lm[2] = lm[3] = 1.f;
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    g[3 * k] = lm[k] * g[3 * k];
    g[3 * k + 1] = lm[k] * g[3 * k + 1];
    g[3 * k + 2] = lm[k] * g[3 * k + 2];
  }
  return sum;
}

template <typename R>
__global__ void __launch_bounds__(kBlock, MinBlocks<R>::v) kGradLimit(View<R> V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  R g[15];
  if constexpr (Layout<R>::packed) {
    __shared__ float dc[3 * kMaxCellFaces * kBlock];
    gradLimitPacked<false, false, -1>(V, i, g, dc + threadIdx.x, nullptr, 0);
  } else {
    gradLimitCell(V, PlainLoad<R>{V}, i, g);
  }
  storeGrad(V, i, g);
}

// Block minimum of a per-thread dt (warp shuffles, then one warp over the
// warp minima) folded into one atomicMin on the bit pattern of the positive
// double (IEEE order of positive doubles = order of their bit patterns).
__device__ inline void blockMinDt(Scalars *sc, double dt) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) dt = fmin(dt, __shfl_xor_sync(0xffffffffu, dt, o));
  __shared__ double wmin[kBlock / 32];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = dt;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = wmin[0];
    for (int w = 1; w < kBlock / 32; ++w) m = fmin(m, wmin[w]);
    if (m > 0.0) atomicMin(&sc->dtBits, (unsigned long long)__double_as_longlong(m));
    else atomicMin(&sc->dtBits, 0ull);
  }
}

// Tiled mixed-mode gradient + limiter (+ time step with kDt), persistent:
// each CTA walks the tiles t = blockIdx.x, + gridDim.x, ... of kTile
// consecutive cells.  A tile's prim records (its own cells, contiguous, and
// its halo) and its stencil ids are copied into shared memory with cp.async,
// double-buffered: the copies of the next tile are in flight while the CTA
// computes the current one.  Each record leaves L2 once per tile instead of
// once per stencil reference.  Three CTAs fit per SM by shared memory; the
// variant with the time-step sum holds more per-cell state and runs at two
// (up to 128 registers) instead of spilling at three.
static_assert(kTile == kBlock, "one thread per cell of a tile");

__device__ inline void cpAsync16(void *smemDst, const void *gSrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smemDst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gSrc) : "memory");
}
__device__ inline void cpAsync4(void *smemDst, const void *gSrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smemDst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gSrc) : "memory");
}
__device__ inline void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ inline void cpAsyncWait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// One tile buffer: 8 floats per staged record, then the tile's stencil ids
// as whole 16-byte words of stLoc (maxTileSt ids plus the misalignment of
// the first word), then the tile's kTile + 1 stencil offsets stOff (padded to
// kTileOffInts).  Two buffers per CTA, then the Venkatakrishnan face-offset
// cache.
template <typename R>
__host__ __device__ inline size_t tileIdWords(const View<R> &V) {
  return tileIdWordsFor(V.maxTileSt);
}
template <typename R>
__host__ __device__ inline size_t tileBufFloats(const View<R> &V) {
  return tileBufFloatsFor(V.maxRecs, V.maxTileSt);
}
template <typename R>
inline size_t tileSmemBytes(const View<R> &V, bool venkat) {
  return sizeof(float) * (2 * tileBufFloats(V) + (venkat ? 3 * kMaxCellFaces * kBlock : 0));
}
// The standalone time-step kernel stages the records only.
template <typename R>
inline size_t dtTileSmemBytes(const View<R> &V) {
  return sizeof(float) * 8 * (size_t)V.maxRecs;
}

// L2 prefetch of the per-cell arrays the compute phase of tile t reads from
// global memory (face entries, LSQ matrix, volumes, Venkatakrishnan epsilon),
// issued for the next tile while the CTA computes the current one.  Each
// array is read per tile as chunks of kTile consecutive elements (feD/feN: one
// chunk per face slot, lsq: one per matrix entry) of at most 4 KB: warp w
// takes chunks w, w + 8, ... and its lanes one 128-byte line each.
template <typename R, bool kDt, int kRc>
__device__ inline void prefetchTile(const View<R> &V, int t) {
  const size_t n = V.nc;
  const int lane = threadIdx.x & 31;
  const int nFe = V.cfW, nN = kDt ? V.cfW : 0;
  const int nChunks = nFe + nN + 6 + (kDt ? 1 : 0) + (kRc == 11 ? 1 : 0);
  for (int c = threadIdx.x >> 5; c < nChunks; c += kBlock / 32) {
    const char *arr;
    unsigned esz;
    size_t off = 0;
    if (c < nFe) { arr = reinterpret_cast<const char *>(V.feD); esz = 16; off = (size_t)c * n; }
    else if (c < nFe + nN) { arr = reinterpret_cast<const char *>(V.feN); esz = 16; off = (size_t)(c - nFe) * n; }
    else if (c < nFe + nN + 6) { arr = reinterpret_cast<const char *>(V.lsq); esz = 4; off = (size_t)(c - nFe - nN) * n; }
    else if (kDt && c == nFe + nN + 6) { arr = reinterpret_cast<const char *>(V.vol); esz = 8; }
    else { arr = reinterpret_cast<const char *>(V.epsq); esz = 4; }
    // bytes of this chunk's part of the array from the tile's first element
    const size_t first = (size_t)t * kTile;
    const size_t avail = esz * (n - first);
    const unsigned bytes = esz * kTile;
    const unsigned at = 128u * lane;
    if (at < bytes && at < avail) {
      const char *a = arr + esz * (off + first) + at;
      asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
    }
  }
}

// Tile staging, in two steps a tile apart so that no thread waits on a
// global load before it computes: stageHalo copies the halo cell ids of a
// tile into its buffer's id area (given the tile's descriptor, a plain load
// one tile earlier still), and stageRecs, once those ids have landed, copies
// the tile's own records, its halo records (addresses from shared memory),
// stencil ids and offsets.  Both are this thread's share of cp.async copies.
template <typename R>
__device__ inline int *tileHaloIds(const View<R> &V, float *buf) {
  return reinterpret_cast<int *>(buf + 8 * (size_t)V.maxRecs + 4 * tileIdWords(V) + kTileOffInts);
}
template <typename R>
__device__ inline int4 loadTileDesc(const View<R> &V, int t, int nTiles) {
  return t < nTiles ? __ldg(V.tileDesc + t) : make_int4(0, 0, 0, 0);
}
template <typename R>
__device__ inline void stageHalo(const View<R> &V, int4 d, float *buf) {
  int *ids = tileHaloIds(V, buf);
  const int nw = (d.y + 3) >> 2;
  for (int w = threadIdx.x; w < nw; w += kBlock) cpAsync16(ids + 4 * w, V.haloIdx + d.x + 4 * w);
}
template <typename R>
__device__ inline void stageRecs(const View<R> &V, int t, int4 d, float *buf) {
  const int base = t * kTile, nIn = min(kTile, V.nc - base);
  uint4 *ids = reinterpret_cast<uint4 *>(buf + 8 * (size_t)V.maxRecs);
  const uint4 *src4 = reinterpret_cast<const uint4 *>(V.stLoc);
  for (int w = d.z + (int)threadIdx.x; w < d.w; w += kBlock) cpAsync16(ids + (w - d.z), src4 + w);
  int *offs = reinterpret_cast<int *>(ids + tileIdWords(V));
  for (int r = threadIdx.x; r <= nIn; r += kBlock) cpAsync4(offs + r, V.stOff + base + r);
  const int *halo = tileHaloIds(V, buf);
  for (int r = threadIdx.x; r < nIn + d.y; r += kBlock) {
    const int src = r < nIn ? base + r : halo[r - nIn];
    if (src < 0) continue;  // an unused halo slot
    const int dst = r < nIn ? r : kTile + (r - nIn);
    const float *g = V.prim + 8 * (size_t)src;
    const int o = recHalf0(dst);
    cpAsync16(buf + o, g);
    cpAsync16(buf + (o ^ 4), g + 4);
  }
}

// The pipeline over a CTA's tiles t = blockIdx.x, + G, ... (G = gridDim.x):
// while tile t is computed from buffer b, the records of t + G are in flight
// into buffer b ^ 1 and the halo ids of t + 2 G into buffer b's id area
// (free: t's ids were read when t was staged), and the descriptor of t + 3 G
// is loading into registers.
template <typename R, bool kDt, int kRc>
__global__ void __launch_bounds__(kBlock, kDt ? 2 : 3) kGradTile(View<R> V) {
  if constexpr (Layout<R>::packed) {
    extern __shared__ float4 tileSmem[];
    const size_t bufFloats = tileBufFloats(V);
    float *const smem = reinterpret_cast<float *>(tileSmem);
    float *dc = smem + 2 * bufFloats;
    const int nTiles = (V.nc + kTile - 1) / kTile;
    const int G = gridDim.x;
    // a step after the clipped last step does nothing (uniform over the CTA)
    const bool live = !kDt || V.sc->finished >= 0;
    double dt = 1.79769313486231571e308;
    int t = blockIdx.x, b = 0;
    if (live && t < nTiles) {
      const int4 d0 = loadTileDesc(V, t, nTiles);
      stageHalo(V, d0, smem);
      cpAsyncCommit();
      cpAsyncWait<0>();
      __syncthreads();
      int4 d1 = loadTileDesc(V, t + G, nTiles);
      stageRecs(V, t, d0, smem);
      if (t + G < nTiles) stageHalo(V, d1, smem + bufFloats);
      cpAsyncCommit();
      prefetchTile<R, kDt, kRc>(V, t);
      int4 d2 = loadTileDesc(V, t + 2 * G, nTiles);
      for (; t < nTiles; t += G, b ^= 1) {
        cpAsyncWait<0>();  // this thread's copies of tile t and of t + G's halo ids have landed
        __syncthreads();   // and everyone else's
        const int tn = t + G;
        float *buf = smem + b * bufFloats;
        if (tn < nTiles) {
          stageRecs(V, tn, d1, smem + (b ^ 1) * bufFloats);
          prefetchTile<R, kDt, kRc>(V, tn);
        }
        if (tn + G < nTiles) stageHalo(V, d2, buf);
        cpAsyncCommit();
        d1 = d2;
        d2 = loadTileDesc(V, tn + 2 * G, nTiles);
        const int base = t * kTile;
        const int i = base + threadIdx.x;
        if (i < V.nc) {
          const float *ids = buf + 8 * (size_t)V.maxRecs;
          float g[15];
          const float sum = gradLimitPacked<kDt, true, kRc>(
              V, i, g, dc + threadIdx.x, buf, threadIdx.x, reinterpret_cast<const unsigned short *>(ids),
              reinterpret_cast<const int *>(ids + 4 * tileIdWords(V)));
          storeGrad(V, i, g);
          if (kDt) dt = fmin(dt, V.vol[i] / (double)sum);
        }
        __syncthreads();  // buffer b is free for the tile after next
      }
    }
    cpAsyncWait<0>();
    if (kDt) blockMinDt(V.sc, dt);
  }
}

// RFLU_TimeStepInviscid's per-cell spectral-radius sum in FP32 from the
// primitive state (mixed mode; the sound speed from the FP64-recovered p).
template <typename R>
__device__ inline double cellDtPrim(const View<R> &V, int i) {
  const PlainLoad<R> ld{V};
  const float g = (float)V.p.refGamma;
  R qi[5];
  ld.prim5(i, qi);
  const float ri = (float)qi[0];
  const float ui = (float)qi[1], vi = (float)qi[2], wi = (float)qi[3];
  const float ai = sqrtf(g * (float)qi[4] / ri);
  float sum = 0.f;
  const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
  for (int e = cb; e < ce; ++e) {
    const int code = V.cfEnt[e];
    if (code >= 0) {
      const int f = code >> 1;
      int c1, c2;
      faceCells(V, f, c1, c2);
      const int nb = (code & 1) ? c1 : c2;
      R qj[5];
      ld.prim5(nb, qj);
      const float rj = (float)qj[0];
      const float uj = (float)qj[1], vj = (float)qj[2], wj = (float)qj[3];
      const float aj = sqrtf(g * (float)qj[4] / rj);
      R nx, ny, nz, nm;
      faceNormal(V, f, nx, ny, nz, nm);
      const float vc = 0.5f * ((ui + uj) * (float)nx + (vi + vj) * (float)ny + (wi + wj) * (float)nz);
      sum += (fabsf(vc) + 0.5f * (ai + aj)) * (float)nm;
    } else if (const double *Q = symmetryQ(V, code)) {
      const int b = -code - 1;
      const float u[3] = {ui, vi, wi};
      float m[3];
      reflect3(Q, u, m);
      const float vc = 0.5f * ((ui + m[0]) * (float)V.bnx[b] + (vi + m[1]) * (float)V.bny[b] + (wi + m[2]) * (float)V.bnz[b]);
      sum += (fabsf(vc) + 0.5f * (ai + ai)) * (float)V.bnm[b];
    } else {
      const int b = -code - 1;
      const float vc = ui * (float)V.bnx[b] + vi * (float)V.bny[b] + wi * (float)V.bnz[b];
      sum += (fabsf(vc) + ai) * (float)V.bnm[b];
    }
  }
  return V.vol[i] / (double)sum;
}

// First stage of a mixed-mode step: gradient + limiter and the time-step
// reduction in one pass over the cell's neighbours.
template <typename R>
__global__ void __launch_bounds__(kBlock, MinBlocks<R>::v) kGradLimitDt(View<R> V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double dt = 1.79769313486231571e308;
  if constexpr (Layout<R>::packed) {
    __shared__ float dc[3 * kMaxCellFaces * kBlock];
    if (i < V.nc && V.sc->finished >= 0) {
      R g[15];
      const float sum = gradLimitPacked<true, false, -1>(V, i, g, dc + threadIdx.x, nullptr, 0);
      if (V.p.spaceOrder > 1) storeGrad(V, i, g);
      dt = V.vol[i] / (double)sum;
    }
  } else {
    if (i < V.nc && V.sc->finished >= 0) {
      if (V.p.spaceOrder > 1) {
        R g[15];
        gradLimitCell(V, PlainLoad<R>{V}, i, g);
        storeGrad(V, i, g);
      }
      dt = cellDtPrim(V, i);
    }
  }
  blockMinDt(V.sc, dt);
}

// WENO smoothing of the cell gradients and the simple limiter, one thread
// per cell (CellGradientsMP, libfloflu/CellGradientsMP.F90:184-200):
// RECONST 2 = RFLU_WENOGradCellsXYZFast_3D (modflu/RFLU_ModWENO.F90:
// 1366-1572), RECONST 1 = RFLU_WENOGradCells_3D (:298-452), then
// RFLU_LimitGradCellsSimple (modflu/RFLU_ModLimiters.F90:1147-1300).  The
// unsmoothed gradients (raw, written by the gradient kernels) of the cell and
// its stencil members are averaged, the cell first and the members in
// stencil order, with weights 1/(t^2 + 1e-15): XYZ per component, sum(w g) /
// sum(w); the simple form one weight per variable from |gx|+|gy|+|gz|,
// normalised before it is applied.  Then the density and pressure gradients
// (the positive variables, libflu/RFLU_SetVarInfo.F90:140-144) are zeroed
// where the cell's value reconstructed at one of its faces,
// ((q + gx dx) + gy dy) + gz dz with d = fc - cofg, is <= 0; that any face
// does is independent of the reference's face order.
// The WENO averages of one cell from its own unsmoothed gradient and its
// stencil members' (fetch(s, t) fills member s's 15 components into t).
// Mixed mode, XYZ: packed f32x2 pairs of components, one approximate
// reciprocal per weight (its argument t^2 + 1e-15 is a normal float, its
// result at most 1e15).
template <typename Fetch>
__device__ inline void wenoXyzPacked(const float *own, int sb, int se, Fetch fetch, float *g) {
  auto rcp = [](float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  };
  const float2 e2 = make_float2(1.0e-15f, 1.0e-15f);
  float2 sum[8], gl[8];
  auto add = [&](const float *t, bool first) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float2 tq = make_float2(t[2 * q], q < 7 ? t[2 * q + 1] : 0.f);
      const float2 a = __ffma2_rn(tq, tq, e2);
      const float2 w = make_float2(rcp(a.x), rcp(a.y));
      if (first) {
        sum[q] = w;
        gl[q] = __fmul2_rn(w, tq);
      } else {
        sum[q] = __fadd2_rn(sum[q], w);
        gl[q] = __ffma2_rn(w, tq, gl[q]);
      }
    }
  };
  add(own, true);
  for (int s = sb; s < se; ++s) {
    float r[16];
    fetch(s, r);
    add(r, false);
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    g[2 * q] = gl[q].x * rcp(sum[q].x);
    if (q < 7) g[2 * q + 1] = gl[q].y * rcp(sum[q].y);
  }
}
// Every mode, XYZ in the reference's operation order; sum receives the
// weight sums (the reverse pass divides by them).  Generic in R so that the
// tangent kernels run it on dual numbers.
template <typename R, typename Fetch>
__device__ inline void wenoXyz(const R *own, int sb, int se, Fetch fetch, R *g, R *sum) {
  const R eps = R(1.0e-15);
#pragma unroll
  for (int k = 0; k < 15; ++k) {
    sum[k] = R(1) / (own[k] * own[k] + eps);
    g[k] = sum[k] * own[k];
  }
  for (int s = sb; s < se; ++s) {
    R t[16];
    fetch(s, t);
#pragma unroll
    for (int k = 0; k < 15; ++k) {
      const R w = R(1) / (t[k] * t[k] + eps);
      sum[k] = sum[k] + w;
      g[k] = g[k] + w * t[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 15; ++k) g[k] = g[k] / sum[k];
}
template <typename R, typename Fetch>
__device__ inline void wenoXyz(const R *own, int sb, int se, Fetch fetch, R *g) {
  R sum[15];
  wenoXyz(own, sb, se, fetch, g, sum);
}
// Every mode, the simple form (one weight per variable from |gx|+|gy|+|gz|,
// normalised before it is applied) in the reference's operation order; sum
// receives the five weight sums.
template <typename R, typename Fetch>
__device__ inline void wenoSimple(const R *own, int sb, int se, Fetch fetch, R *g, R *sum) {
  const R eps = R(1.0e-15);
  R w0[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const R t = fabs_(own[3 * v]) + fabs_(own[3 * v + 1]) + fabs_(own[3 * v + 2]);
    w0[v] = R(1) / (t * t + eps);
    sum[v] = w0[v];
  }
  for (int s = sb; s < se; ++s) {
    R t[16];
    fetch(s, t);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const R m = fabs_(t[3 * v]) + fabs_(t[3 * v + 1]) + fabs_(t[3 * v + 2]);
      sum[v] = sum[v] + R(1) / (m * m + eps);
    }
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const R term = w0[v] / sum[v];
#pragma unroll
    for (int d = 0; d < 3; ++d) g[3 * v + d] = term * own[3 * v + d];
  }
  for (int s = sb; s < se; ++s) {
    R t[16];
    fetch(s, t);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const R m = fabs_(t[3 * v]) + fabs_(t[3 * v + 1]) + fabs_(t[3 * v + 2]);
      const R term = (R(1) / (m * m + eps)) / sum[v];
#pragma unroll
      for (int d = 0; d < 3; ++d) g[3 * v + d] = g[3 * v + d] + term * t[3 * v + d];
    }
  }
}
template <typename R, typename Fetch>
__device__ inline void wenoSimple(const R *own, int sb, int se, Fetch fetch, R *g) {
  R sum[5];
  wenoSimple(own, sb, se, fetch, g, sum);
}
// RFLU_LimitGradCellsSimple on one cell: face(k, d) gives the cell's k-th
// face offset d = fc - cofg and returns false past its last face.  Returns
// which gradients it zeroed (1: density, 2: pressure).
template <typename R, typename Face>
__device__ inline int simplePositivity(R q0, R q4, int nFaces, Face face, R *g) {
  bool z0 = false, z4 = false;
  for (int k = 0; k < nFaces; ++k) {
    R d[3];
    if (!face(k, d)) continue;
    if (q0 + g[0] * d[0] + g[1] * d[1] + g[2] * d[2] <= R(0)) z0 = true;
    if (q4 + g[12] * d[0] + g[13] * d[1] + g[14] * d[2] <= R(0)) z4 = true;
  }
  if (z0) g[0] = g[1] = g[2] = R(0);
  if (z4) g[12] = g[13] = g[14] = R(0);
  return (z0 ? 1 : 0) | (z4 ? 2 : 0);
}

template <typename R>
__global__ void __launch_bounds__(kBlock) kWenoSmooth(View<R> V, const R *raw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const size_t n = V.nc, nb = V.nb;
  auto rawRow = [&](int c, R *t) {
    if constexpr (Layout<R>::packed) {
      ld8(raw + 16 * (size_t)c, t);
      ld8(raw + 16 * (size_t)c + 8, t + 8);
    } else {
#pragma unroll
      for (int k = 0; k < 15; ++k) t[k] = raw[k * n + c];
    }
  };
  auto fetch = [&](int s, R *t) {
    rawRow(V.stIdx[s], t);
    if (V.stXf) {  // a member seen reflected across symmetry patches
      const int x = V.stXf[s];
      if (x >= 0) reflectGrad(V.xfQ + 9 * x, t);
    }
  };
  const int sb = V.stOff[i], se = V.stOff[i + 1];
  R g[15], own[16];
  rawRow(i, own);
  if (V.p.reconst == 2) {
    if constexpr (Layout<R>::packed) wenoXyzPacked(own, sb, se, fetch, g);
    else wenoXyz(own, sb, se, fetch, g);
  } else {
    wenoSimple(own, sb, se, fetch, g);
  }
  const PlainLoad<R> ld{V};
  const int cb = V.cfOff[i];
  simplePositivity(ld.prim(0, i), ld.prim(4, i), V.cfOff[i + 1] - cb,
                   [&](int k, R *d) {
                     const int code = V.cfEnt[cb + k];
                     if (code >= 0) {
                       faceOffset(V, code >> 1, code & 1, d);
                     } else {
                       const int b = -code - 1;
                       d[0] = V.bd[b];
                       d[1] = V.bd[nb + b];
                       d[2] = V.bd[2 * nb + b];
                     }
                     return true;
                   },
                   g);
  storeGrad(V, i, g);
}

// Tiled WENO smoothing for the mixed mode: one tile of kTile Morton cells per
// CTA.  The unsmoothed 64-byte gradient records of the tile's cells and of
// its halo, its stencil ids and its stencil offsets are staged in shared
// memory (the gradient kernel's tiles and 16-bit local ids), so the members'
// records are read from shared memory instead of gathered through L2; the
// positivity check reads the entry-major face offsets feD.  The four 16-byte
// quarters of record l are stored rotated by (l >> 1) & 3, so that the same
// quarter of eight consecutive records lies in eight different bank groups.
__device__ inline int wenoQuad(int l, int q) { return 16 * l + 4 * (q ^ ((l >> 1) & 3)); }

template <typename R>
inline size_t wenoTileSmemBytes(const View<R> &V) {
  return sizeof(float) * (16 * (size_t)V.maxRecs + 4 * tileIdWords(V) + kTileOffInts);
}

template <typename R>
__global__ void __launch_bounds__(kBlock) kWenoTile(View<R> V, const R *raw) {
  if constexpr (Layout<R>::packed) {
    extern __shared__ float4 wenoSmem[];
    float *recs = reinterpret_cast<float *>(wenoSmem);
    uint4 *ids = reinterpret_cast<uint4 *>(recs + 16 * (size_t)V.maxRecs);
    int *offs = reinterpret_cast<int *>(ids + tileIdWords(V));
    const size_t n = V.nc;
    const int t = blockIdx.x, base = t * kTile, nIn = min(kTile, V.nc - base);
    const int hb = V.haloOff[t], nh = V.haloOff[t + 1] - hb;
    const int w0 = V.stOff[base] >> 3, w1 = (V.stOff[base + nIn] + 7) >> 3;
    const uint4 *src4 = reinterpret_cast<const uint4 *>(V.stLoc);
    for (int w = w0 + (int)threadIdx.x; w < w1; w += kBlock) cpAsync16(ids + (w - w0), src4 + w);
    for (int r = threadIdx.x; r <= nIn; r += kBlock) cpAsync4(offs + r, V.stOff + base + r);
    for (int x = threadIdx.x; x < 4 * (nIn + nh); x += kBlock) {
      const int r = x >> 2, q = x & 3;
      const int src = r < nIn ? base + r : V.haloIdx[hb + r - nIn];
      if (src < 0) continue;  // an unused halo slot
      const int dst = r < nIn ? r : kTile + (r - nIn);
      cpAsync16(recs + wenoQuad(dst, q), raw + 16 * (size_t)src + 4 * q);
    }
    cpAsyncCommit();
    cpAsyncWait<0>();
    __syncthreads();
    const int i = base + threadIdx.x;
    if (i >= V.nc) return;
    const unsigned short *st = reinterpret_cast<const unsigned short *>(ids);
    const int s0 = 8 * (offs[0] >> 3);
    const int sb = offs[threadIdx.x] - s0, se = offs[threadIdx.x + 1] - s0;
    auto rec = [&](int l, float *v) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 a = *reinterpret_cast<const float4 *>(recs + wenoQuad(l, q));
        v[4 * q] = a.x;
        v[4 * q + 1] = a.y;
        v[4 * q + 2] = a.z;
        v[4 * q + 3] = a.w;
      }
    };
    auto fetch = [&](int s, float *v) { rec(st[s], v); };
    float own[16], g[15];
    rec(threadIdx.x, own);
    if (V.p.reconst == 2) wenoXyzPacked(own, sb, se, fetch, g);
    else wenoSimple(own, sb, se, fetch, g);
    float pr[8];
    ld8(V.prim + 8 * (size_t)i, pr);
    simplePositivity(pr[0], pr[4], V.cfW,
                     [&](int k, float *d) {
                       const float4 D = ld4(V.feD + 4 * (k * n + i));
                       d[0] = D.x;
                       d[1] = D.y;
                       d[2] = D.z;
                       return __float_as_int(D.w) != INT_MIN;
                     },
                     g);
    storeGrad(V, i, g);
  }
}

// The transposed-stencil weights of the mixed adjoint (View::tsW), formed
// with the expression the gradient kernels use for the same pair of cells.
template <typename R>
__global__ void kTsWeights(View<R> V) {
  if constexpr (Layout<R>::packed) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= V.nc) return;
    const size_t n = V.nc;
    const float xj = V.cgx[j], yj = V.cgy[j], zj = V.cgz[j];
    const int b = V.tsOff[j], c = V.tsOff[j + 1] - b;
    for (int k = 0; k < V.tsWidth; ++k) {
      float4 w = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
      if (k < c) {
        const int i = V.tsCell[b + k];
        float dx = xj - V.cgx[i], dy = yj - V.cgy[i], dz = zj - V.cgz[i];
        int tag = i;
        if (V.stShift) {  // a periodic or symmetry mesh: j seen from i as its image
          const size_t e = V.tsEnt[b + k];
          dx = dx + V.stShift[3 * e];
          dy = dy + V.stShift[3 * e + 1];
          dz = dz + V.stShift[3 * e + 2];
          if (V.stXf && V.stXf[e] >= 0) tag |= kTsReflected;  // seen reflected
        }
        const float inv = 1.f / (dx * dx + dy * dy + dz * dz);
        w = make_float4(inv * dx, inv * dy, inv * dz, __int_as_float(tag));
      }
      *reinterpret_cast<float4 *>(V.tsW + 4 * (k * n + j)) = w;
    }
  }
}

// Time step alone from the primitive state (mixed mode).
template <typename R>
__global__ void __launch_bounds__(kBlock) kCellDtPrim(View<R> V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double dt = 1.79769313486231571e308;
  if (i < V.nc) dt = cellDtPrim(V, i);
  blockMinDt(V.sc, dt);
}

// Time step alone on a tiled mesh (mixed mode), one CTA per tile: the tile's
// and halo's prim records are staged in shared memory and each cell takes
// the spectral-radius sum of the first stage of a step (tileDtSum), so this
// entry and the step's own time step agree.
template <typename R>
__global__ void __launch_bounds__(kBlock) kCellDtTile(View<R> V) {
  if constexpr (Layout<R>::packed) {
    extern __shared__ float4 dtSmem[];
    float *recs = reinterpret_cast<float *>(dtSmem);
    const int t = blockIdx.x, base = t * kTile, nIn = min(kTile, V.nc - base);
    const int hb = V.haloOff[t], nh = V.haloOff[t + 1] - hb;
    for (int r = threadIdx.x; r < nIn + nh; r += kBlock) {
      const int src = r < nIn ? base + r : V.haloIdx[hb + r - nIn];
      if (src < 0) continue;  // an unused halo slot
      const int dst = r < nIn ? r : kTile + (r - nIn);
      const float *g = V.prim + 8 * (size_t)src;
      const int o = recHalf0(dst);
      cpAsync16(recs + o, g);
      cpAsync16(recs + (o ^ 4), g + 4);
    }
    cpAsyncCommit();
    cpAsyncWait<0>();
    __syncthreads();
    const int i = base + threadIdx.x;
    double dt = 1.79769313486231571e308;
    if (i < V.nc) {
      float rec[8];
      ldRec(recs, threadIdx.x, rec);
      const float q[5] = {rec[0], rec[1], rec[2], rec[3], rec[4]};
      const float ai = sqrtf(V.p.refGammaF * q[4] / q[0]);
      dt = V.vol[i] / (double)tileDtSum(V, i, recs, q, ai);
    }
    blockMinDt(V.sc, dt);
  }
}

// ---------------------------------------------------------------------------
// Face state for the 2nd-order routines (*_ComputeFlux2_TCP):
// cell primitive (with the reference's momentum round trip in the FP64 modes)
// plus grad . (fc - cofg).
// ---------------------------------------------------------------------------
template <typename R, typename L>
__device__ inline void faceState(const View<R> &V, const L &ld, int c, typename L::S dx, typename L::S dy,
                                 typename L::S dz, typename L::S *s, typename L::S &irCell) {
  using S = typename L::S;
  S q[5], gr[15];
  ld.prim5(c, q);
  ld.grad15(c, gr);
  S r = q[0];
  S ir = S(1) / r;
  S u = q[1], v = q[2], w = q[3];
  if (Ref<R>::on) {
    // ul = pCv(CV_MIXT_XMOM,c1)*irl with pCv(XMOM) = r*u after RFLU_ConvertCvPrim2Cons
    u = (r * u) * ir;
    v = (r * v) * ir;
    w = (r * w) * ir;
  }
  S p = q[4];
  s[0] = r + gr[0] * dx + gr[1] * dy + gr[2] * dz;
  s[1] = u + gr[3] * dx + gr[4] * dy + gr[5] * dz;
  s[2] = v + gr[6] * dx + gr[7] * dy + gr[8] * dz;
  s[3] = w + gr[9] * dx + gr[10] * dy + gr[11] * dz;
  s[4] = p + gr[12] * dx + gr[13] * dy + gr[14] * dz;
  irCell = ir;
}

// A numerics parameter in the arithmetic type S (the FP32 copy in the mixed mode).
template <typename S> __device__ inline S prm(double d, float) { return S(d); }
template <> __device__ inline float prm<float>(double, float f) { return f; }

template <typename S>
__device__ inline void riemann2(const Params &P, S nx, S ny, S nz, S nm, const S *L, S irl, const S *Rt, S irr, S *flx) {
  const S cp = prm<S>(P.refCp, P.refCpF), g = prm<S>(P.refGamma, P.refGammaF);
  if (P.spaceDiscr == 1) {
    S gc = cp - cp / g;
    S tl = L[4] / (L[0] * gc), tr = Rt[4] / (Rt[0] * gc);
    S Hl = perfHo(cp, tl, L[1], L[2], L[3]), Hr = perfHo(cp, tr, Rt[1], Rt[2], Rt[3]);
    roeFlux(g, prm<S>(P.epsEntr, P.epsEntrF), prm<S>(P.dissFact, P.dissFactF), nx, ny, nz, nm, L[0], L[1], L[2], L[3],
            L[4], Hl, Rt[0], Rt[1], Rt[2], Rt[3], Rt[4], Hr, flx);
  } else if (P.spaceDiscr == 3) {
    S el = perfEo(L[0], g, L[4], L[1], L[2], L[3]), al = sqrt_(g * L[4] / L[0]);
    S er = perfEo(Rt[0], g, Rt[4], Rt[1], Rt[2], Rt[3]), ar = sqrt_(g * Rt[4] / Rt[0]);
    S Hl = el + irl * L[4], Hr = er + irr * Rt[4];
    hllcFlux(g, nx, ny, nz, nm, L[0], L[1], L[2], L[3], L[4], el, al, Hl, Rt[0], Rt[1], Rt[2], Rt[3], Rt[4], er, ar,
             Hr, flx);
  } else {
    S gc = cp - cp / g;
    S tl = L[4] / (L[0] * gc), tr = Rt[4] / (Rt[0] * gc);
    S al = sqrt_(g * gc * tl), ar = sqrt_(g * gc * tr);
    S Hl = perfHo(cp, tl, L[1], L[2], L[3]), Hr = perfHo(cp, tr, Rt[1], Rt[2], Rt[3]);
    ausmFlux(nx, ny, nz, nm, L[0], L[1], L[2], L[3], L[4], Hl, al, Rt[0], Rt[1], Rt[2], Rt[3], Rt[4], Hr, ar, flx);
  }
}

// First-order interior flux from cv and dv (type H: FP64 in every mode).
template <typename H>
__device__ inline void riemann1(const Params &P, const H *cl, const H *dvl, const H *cr, const H *dvr, H nx, H ny,
                                H nz, H nm, H *flx) {
  H rl = cl[0], irl = H(1) / rl, ul = cl[1] * irl, vl = cl[2] * irl, wl = cl[3] * irl;
  H rr = cr[0], irr = H(1) / rr, ur = cr[1] * irr, vr = cr[2] * irr, wr = cr[3] * irr;
  H pl = dvl[0], pr = dvr[0];
  const H cp = H(P.refCp), g = H(P.refGamma);
  if (P.spaceDiscr == 1) {
    H Hl = perfHo(cp, dvl[1], ul, vl, wl), Hr = perfHo(cp, dvr[1], ur, vr, wr);
    roeFlux(g, H(P.epsEntr), H(P.dissFact), nx, ny, nz, nm, rl, ul, vl, wl, pl, Hl, rr, ur, vr, wr, pr, Hr, flx);
  } else if (P.spaceDiscr == 3) {
    H el = cl[4] * irl, er = cr[4] * irr;
    H Hl = el + irl * pl, Hr = er + irr * pr;
    hllcFlux(g, nx, ny, nz, nm, rl, ul, vl, wl, pl, el, dvl[2], Hl, rr, ur, vr, wr, pr, er, dvr[2], Hr, flx);
  } else {
    H Hl = cl[4] * irl + pl / rl, Hr = cr[4] * irr + pr / rr;
    ausmFlux(nx, ny, nz, nm, rl, ul, vl, wl, pl, Hl, dvl[2], rr, ur, vr, wr, pr, Hr, dvr[2], flx);
  }
}

// First-order patch flux (rocflu/RFLU_CentralFirstPatch.F90: inflow :228-570,
// outflow :571-784, slip wall :785-911, no-slip walls :912-947, farfield
// :948-1042, injection :1043-1127) from the cell's cv and p; K: the patch's
// constants (physics.cuh: kPatchK).  RFLU_CentralFirstPatch reads cv as
// CellGradientsMP left it: in a 2nd-order run the momentum went through the
// prim round trip and, in the PICL build, the energy slot holds the
// pressure.
template <typename H>
__device__ inline void patch1(const Params &P, int type, int bcOpt, const double *K, const H *cvIn, H pl, H nx, H ny,
                              H nz, H nm, H *fd) {
  H cv[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) cv[k] = cvIn[k];
  if (P.spaceOrder == 2) {
    const H ir = H(1) / cv[0];
    const H up = ir * cv[1], vp = ir * cv[2], wp = ir * cv[3];
    cv[1] = cv[0] * up;
    cv[2] = cv[0] * vp;
    cv[3] = cv[0] * wp;
    if (P.piclBuild) {
      cv[4] = pl;
    } else {
      const H g = H(P.gvCp) / (H(P.gvCp) - H(8314.3) / H(P.gvMol));
      cv[4] = cv[0] * perfEo(cv[0], g, pl, up, vp, wp);
    }
  }
  if (patchLeavesDensity(type)) {
    fd[0] = H(0);
    fd[1] = pl * nx * nm;
    fd[2] = pl * ny * nm;
    fd[3] = pl * nz * nm;
    fd[4] = pl * H(0) * nm;
    return;
  }
  if (type == 20) {
    outflowPatchFlux(bcOpt, H(K[0]), H(P.gvCp), H(P.gvMol), nx, ny, nz, nm, cv[0], cv[1], cv[2], cv[3], cv[4], pl,
                     fd);
    return;
  }
  const H cp = H(P.gvCp), rgas = H(8314.3) / H(P.gvMol);
  const H g = cp / (cp - rgas);
  if (type == 90) {
    injectionPatchFlux(K, g, cp, rgas, nx, ny, nz, nm, cv[0], cv[1], cv[2], cv[3], pl, fd);
    return;
  }
  H rr, rur, rvr, rwr, rer, pr;
  if (type == 80) farfieldRindPerf(K, g, nx, ny, nz, cv[0], cv[1], cv[2], cv[3], cv[4], rr, rur, rvr, rwr, rer, pr);
  else if (type == 10) inflowTotAngPerf(bcOpt, K, g, rgas, nx, ny, nz, cv[0], cv[1], cv[2], cv[3], rr, rur, rvr, rwr, rer, pr);
  else inflowVelTempPerf(bcOpt, K, g, rgas, cv[0], rr, rur, rvr, rwr, rer, pr);
  centralPatchFlux(nx, ny, nz, nm, cv[0], cv[1], cv[2], cv[3], cv[4], pl, rr, rur, rvr, rwr, rer, pr, fd);
}

// Second-order patch flux (rocflu/RFLU_CentralSecondPatch.F90: inflow
// :239-633, outflow :634-857, slip wall :858-1029, no-slip walls :1030-1087,
// farfield :1088-1228, injection :1229-1343) from the reconstructed face
// state L = (rho, u, v, w, p).
template <typename S>
__device__ inline void patch2(const Params &P, int type, int bcOpt, const double *K, const S *L, S nx, S ny, S nz,
                              S nm, S *flx) {
  if (patchLeavesDensity(type)) {
    flx[0] = S(0);
    flx[1] = L[4] * nx * nm;
    flx[2] = L[4] * ny * nm;
    flx[3] = L[4] * nz * nm;
    flx[4] = L[4] * S(0) * nm;
    return;
  }
  const S cp = prm<S>(P.gvCp, P.gvCpF), mol = prm<S>(P.gvMol, P.gvMolF);
  S rgas = S(8314.3) / mol;
  S g = cp / (cp - rgas);
  S rul = L[0] * L[1], rvl = L[0] * L[2], rwl = L[0] * L[3];
  if (type == 90) {
    injectionPatchFlux(K, g, cp, rgas, nx, ny, nz, nm, L[0], rul, rvl, rwl, L[4], flx);
    return;
  }
  S rel = L[0] * perfEo(L[0], g, L[4], L[1], L[2], L[3]);
  if (type == 20) {
    outflowPatchFlux(bcOpt, S(K[0]), cp, mol, nx, ny, nz, nm, L[0], rul, rvl, rwl, rel, L[4], flx);
    return;
  }
  S rr, rur, rvr, rwr, rer, pr;
  if (type == 80) farfieldRindPerf(K, g, nx, ny, nz, L[0], rul, rvl, rwl, rel, rr, rur, rvr, rwr, rer, pr);
  else if (type == 10) inflowTotAngPerf(bcOpt, K, g, rgas, nx, ny, nz, L[0], rul, rvl, rwl, rr, rur, rvr, rwr, rer, pr);
  else inflowVelTempPerf(bcOpt, K, g, rgas, L[0], rr, rur, rvr, rwr, rer, pr);
  centralPatchFlux(nx, ny, nz, nm, L[0], rul, rvl, rwl, rel, L[4], rr, rur, rvr, rwr, rer, pr, flx);
}

template <typename To, typename From> __device__ inline To cvt(const From &x) { return To(x); }

// Flux of face t (interior faces [0,nf), then boundary faces).
template <typename R, typename L>
__device__ inline void faceFluxEval(const View<R> &V, const L &ld, int t, typename L::S *flx) {
  using S = typename L::S;
  using H = typename L::H;
  const Params &P = V.p;
  if (t < V.nf) {
    const int f = t;
    int c1, c2;
    faceCells(V, f, c1, c2);
    R nx, ny, nz, nm;
    faceNormal(V, f, nx, ny, nz, nm);
    if (P.spaceOrder == 1) {
      H cl[5], cr[5], dl[3], dr[3], fd[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) { cl[k] = ld.cv(k, c1); cr[k] = ld.cv(k, c2); }
#pragma unroll
      for (int k = 0; k < 3; ++k) { dl[k] = ld.dv(k, c1); dr[k] = ld.dv(k, c2); }
      riemann1(P, cl, dl, cr, dr, H((double)nx), H((double)ny), H((double)nz), H((double)nm), fd);
#pragma unroll
      for (int k = 0; k < 5; ++k) flx[k] = cvt<S>(fd[k]);
    } else {
      S Lf[5], Rt[5], irl, irr;
      R dl[3], dr[3];
      faceOffset(V, f, 0, dl);
      faceOffset(V, f, 1, dr);
      faceState(V, ld, c1, S(dl[0]), S(dl[1]), S(dl[2]), Lf, irl);
      faceState(V, ld, c2, S(dr[0]), S(dr[1]), S(dr[2]), Rt, irr);
      riemann2(P, S(nx), S(ny), S(nz), S(nm), Lf, irl, Rt, irr, flx);
    }
  } else {
    const int b = t - V.nf, c = V.bcell[b], ip = V.bpatch[b];
    const int type = V.patchType[ip], order = V.patchOrder[ip];
    if (type == kBcSymmetry) {
      // an interior face to the cell's reflection, at the interior order:
      // first order the cell against its reflected state, second order the
      // reconstructed face state against its own reflection
      const double *Q = V.patchK + kPatchK * ip;
      if (P.spaceOrder == 1) {
        H cl[5], cr[5], dl[3], fd[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) cl[k] = ld.cv(k, c);
#pragma unroll
        for (int k = 0; k < 3; ++k) dl[k] = ld.dv(k, c);
        cr[0] = cl[0];
        reflect3(Q, cl + 1, cr + 1);
        cr[4] = cl[4];
        riemann1(P, cl, dl, cr, dl, H((double)V.bnx[b]), H((double)V.bny[b]), H((double)V.bnz[b]),
                 H((double)V.bnm[b]), fd);
#pragma unroll
        for (int k = 0; k < 5; ++k) flx[k] = cvt<S>(fd[k]);
      } else {
        const size_t nb = V.nb;
        S Lf[5], Rt[5], irl;
        faceState(V, ld, c, S(V.bd[b]), S(V.bd[nb + b]), S(V.bd[2 * nb + b]), Lf, irl);
        Rt[0] = Lf[0];
        reflect3(Q, Lf + 1, Rt + 1);
        Rt[4] = Lf[4];
        riemann2(P, S(V.bnx[b]), S(V.bny[b]), S(V.bnz[b]), S(V.bnm[b]), Lf, irl, Rt, irl, flx);
      }
      return;
    }
    if (order == 1) {
      H cv[5], fd[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) cv[k] = ld.cv(k, c);
      patch1(P, type, V.patchOutflow[ip], V.patchK + kPatchK * ip, cv, ld.dv(0, c), H((double)V.bnx[b]),
             H((double)V.bny[b]), H((double)V.bnz[b]), H((double)V.bnm[b]), fd);
#pragma unroll
      for (int k = 0; k < 5; ++k) flx[k] = cvt<S>(fd[k]);
    } else {
      const size_t nb = V.nb;
      S Lf[5], irl;
      faceState(V, ld, c, S(V.bd[b]), S(V.bd[nb + b]), S(V.bd[2 * nb + b]), Lf, irl);
      patch2(P, type, V.patchOutflow[ip], V.patchK + kPatchK * ip, Lf, S(V.bnx[b]), S(V.bny[b]), S(V.bnz[b]),
             S(V.bnm[b]), flx);
    }
  }
}

// One thread per face: interior faces [0,nf), then boundary faces.
template <typename R>
__global__ void __launch_bounds__(kBlock, MinBlocksFlux<R>::v) kFaceFlux(View<R> V) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nfT = V.nf + V.nb;
  if (t >= nfT) return;
  R flx[5];
  if constexpr (Layout<R>::packed) {
    if (t < V.nf && V.p.spaceOrder > 1) {
      // one 48-byte face record, one 32-byte prim and one 64-byte gradient
      // record per side
      const float *fr = V.fpk + 12 * (size_t)t;
      const float4 F0 = ld4(fr), F1 = ld4(fr + 4), F2 = ld4(fr + 8);
      const PlainLoad<R> ld{V};
      float Lf[5], Rt[5], irl, irr;
      faceState(V, ld, __float_as_int(F2.z), F1.x, F1.y, F1.z, Lf, irl);
      faceState(V, ld, __float_as_int(F2.w), F1.w, F2.x, F2.y, Rt, irr);
      riemann2(V.p, F0.x, F0.y, F0.z, F0.w, Lf, irl, Rt, irr, flx);
      storeFlux(V, (size_t)nfT, t, flx);
      return;
    }
  }
  faceFluxEval(V, PlainLoad<R>{V}, t, flx);
  storeFlux(V, (size_t)nfT, t, flx);
}

// ---------------------------------------------------------------------------
// Residual gather (ConvectiveFluxes, libfloflu/ConvectiveFluxes.F90:133-175):
// rhs(c) = -diss(c) + sum over the cell's faces in reference order of +-F.
// ---------------------------------------------------------------------------
template <typename R, typename T>
__device__ inline void gatherRhs(const View<R> &V, const T *flux, int i, T *rhs) {
  const size_t nT = (size_t)V.nf + V.nb;
#pragma unroll
  for (int k = 0; k < 5; ++k) rhs[k] = -T(0);
  const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
  for (int e = cb; e < ce; ++e) {
    const int code = V.cfEnt[e];
    if (code >= 0) {
      const int f = code >> 1;
      T fl[5];
      loadFlux<R>(flux, nT, f, fl);
      if (code & 1) {
#pragma unroll
        for (int k = 0; k < 5; ++k) rhs[k] = rhs[k] - fl[k];
      } else {
#pragma unroll
        for (int k = 0; k < 5; ++k) rhs[k] = rhs[k] + fl[k];
      }
    } else {
      const int b = -code - 1;
      const int k0 = patchLeavesDensity(V.patchType[V.bpatch[b]]) ? 1 : 0;  // walls leave rhs(DENS)
      T fl[5];
      loadFlux<R>(flux, nT, V.nf + b, fl);
#pragma unroll
      for (int k = 0; k < 5; ++k)
        if (k >= k0) rhs[k] = rhs[k] + fl[k];
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) kGatherRhs(View<R> V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  R rhs[5];
  gatherRhs(V, (const R *)V.flux, i, rhs);
#pragma unroll
  for (int k = 0; k < 5; ++k) V.rhs[(size_t)k * V.nc + i] = rhs[k];
}

// rhs += src, src(5,nCells) in the reference's cell order and layout (the
// SourceTermsMP / PICL_Runge slot of RungeKuttaMP, libfloflu/
// RungeKuttaMP.F90:274-290); the sum in FP64, stored in the residual's type.
template <typename R>
__global__ void __launch_bounds__(kBlock) kAddRhs(View<R> V, const double *src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const size_t o = (size_t)V.refId[i];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    R &r = V.rhs[(size_t)k * V.nc + i];
    r = (R)((double)r + src[5 * o + k]);
  }
}

// RFLU_CheckValidity / RFLU_EnforceBounds / RFLU_CheckPositivity for one cell
// (libflu/RFLU_CheckValidity.F90:165-214, RFLU_EnforceBounds.F90:165-230,
// RFLU_CheckPositivity.F90:173-193); cv and dv updated in place.
template <typename R>
__device__ inline void afterUpdate(const View<R> &V, int i, double *cv, double &pr, double &tp, double &cs) {
  const Params &P = V.p;
  {
    double rho = cv[0], rrho = 1.0 / rho;
    double u = rrho * cv[1], v = rrho * cv[2], w = rrho * cv[3];
    if (isnan(rho) || isnan(u) || isnan(v) || isnan(w) || isnan(pr) || isnan(tp)) {
      atomicAdd(&V.sc->nanCells, 1ull);
      atomicMin(&V.sc->firstBadCell, V.refId[i] + 1);
    }
  }
  const double gamma = P.gRT;
  {
    double r = cv[0], ir = 1.0 / r;
    double u = ir * cv[1], v = ir * cv[2], w = ir * cv[3];
    double Eo = ir * cv[4];
    double Vm2 = u * u + v * v + w * w;
    double p = (gamma - 1.0) * r * (Eo - 0.5 * Vm2);
    if (p <= 0.0 && fabs(p) <= 1.0e-12) {
      atomicAdd(&V.sc->negPCells, 1ull);
      cv[4] = r * perfEo(r, gamma, 1.0e-12, u, v, w);
    }
  }
  if (pr <= 0.0) {
    double rho = cv[0], rrho = 1.0 / rho;
    double u = rrho * cv[1], v = rrho * cv[2], w = rrho * cv[3];
    double Vm2 = u * u + v * v + w * w;
    atomicAdd(&V.sc->posFixCells, 1ull);
    cv[4] = rho * (1.0e4 + 0.5 * Vm2);
    dependentVars(P, cv, pr, tp, cs);
  }
}

// Which stages read and which write the accumulated residual rhsSum
// (RkUpdateGeneric: classical RK4 sums the stage residuals, Wray's scheme
// keeps the previous one).  All five components are loaded before any is
// stored, so the loads are not ordered behind the stores.
struct RkAccess {
  bool rd, wr;
  __device__ RkAccess(const Params &P, int iStage) {
    if (P.rkScheme == 1) { rd = iStage > 1; wr = iStage < P.nrkSteps; }
    else if (P.rkScheme == 2) { rd = iStage > 1; wr = iStage < 3; }
    else { rd = false; wr = false; }
  }
};

// Mixed-mode RKUpdateMP + RFLU_SetVarsContWrapper + AfterUpdateMP of one cell
// (T and c only when a kernel of the step reads them, P.dvPOnly == 0).
// The increment adtv*(rhs - grk*rhsSum) is formed in FP32 (the rhs is FP32)
// and added to the FP64 master cv; p is recovered in FP64 (it is a difference
// of two nearly equal energies at high Mach numbers).  The FP64 reciprocal of
// rho and the sound speed start from FP32 seeds refined by one Newton-Raphson
// step (quadratic convergence: a 2^-22 seed ends near 2^-44), so the cell
// costs a few dozen FP64 instructions instead of two IEEE divisions and a
// square root.  A cell with p <= 0 gets the energy floor of
// RFLU_CheckPositivity (libflu/RFLU_CheckPositivity.F90:173-193), which also
// overrides the tiny-pressure clamp of RFLU_EnforceBounds.
template <typename R>
__device__ inline void mixedUpdate(const View<R> &V, int i, int iStage, float fac, float grk, const R *rhs,
                                   double *cv) {
  const Params &P = V.p;
  const size_t n = V.nc;
  const float adtv = fac * (float)V.ivol[i];
  RkAccess ra(P, iStage);
  float rs[5];
  if (ra.rd) {
#pragma unroll
    for (int k = 0; k < 5; ++k) rs[k] = (float)V.rhsSum[k * n + i];
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const float r = (float)rhs[k];
    float inc;
    switch (P.rkScheme) {
      case 1:
        if (iStage == 1) { inc = adtv * r; rs[k] = r; }
        else if (iStage == P.nrkSteps) inc = adtv * (r + rs[k]);
        else { inc = adtv * r; rs[k] = rs[k] + grk * r; }
        break;
      case 2:
        if (iStage == 1) { inc = adtv * r; rs[k] = r; }
        else if (iStage == 2) { inc = adtv * (r - grk * rs[k]); rs[k] = r; }
        else inc = adtv * (r - grk * rs[k]);
        break;
      default:
        inc = adtv * r;
    }
    cv[k] = cv[k] - f2d(inc);
  }
  if (ra.wr) {
#pragma unroll
    for (int k = 0; k < 5; ++k) V.rhsSum[k * n + i] = (R)rs[k];
  }
  const MixedPrim m(P, cv);
  const float rf = m.rf, uf = m.uf, vf = m.vf, wf = m.wf;
  const double ir = m.ir, ke = m.ke;
  double pr = m.pr;
  const float prf = d2f(pr);
  if (isnan(rf) || isnan(uf) || isnan(vf) || isnan(wf) || isnan(prf)) {
    atomicAdd(&V.sc->nanCells, 1ull);
    atomicMin(&V.sc->firstBadCell, V.refId[i] + 1);
  }
  if (pr <= 0.0) {
    if (fabs(pr) <= 1.0e-12) atomicAdd(&V.sc->negPCells, 1ull);
    atomicAdd(&V.sc->posFixCells, 1ull);
    cv[4] = 1.0e4 * cv[0] + ke;
    pr = (P.gRT - 1.0) * (cv[4] - ke);
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) V.cv[k * n + i] = cv[k];
  V.dv[i] = pr;
  if (!P.dvPOnly) {
    V.dv[n + i] = pr * ir * P.igcR;
    V.dv[2 * n + i] = refinedSqrt(P.gRT * pr * ir);
  }
  storePrimRec(V, i, (R)rf, (R)uf, (R)vf, (R)wf, (R)d2f(pr));
}

// Gather + RKUpdateMP (RkUpdateGeneric, static grid, libfloflu/
// RkUpdateGeneric.F90:257-322) + RFLU_SetVarsContWrapper + AfterUpdateMP.
// cvOld of RkInitGeneric is cv itself: nothing writes cv before this kernel.
// kFromRhs: the residual is read from V.rhs (formed by kGatherRhs and
// perhaps changed by the caller's source terms) instead of gathered here.
template <typename R, bool kFromRhs>
__global__ void __launch_bounds__(kBlock) kGatherUpdate(View<R> V, int iStage, const double *dtp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc || V.sc->finished < 0) return;
  const Params &P = V.p;
  const size_t n = V.nc;
  R rhs[5];
  if constexpr (kFromRhs) {
#pragma unroll
    for (int k = 0; k < 5; ++k) rhs[k] = V.rhs[k * n + i];
  } else {
    gatherRhs(V, (const R *)V.flux, i, rhs);
  }
  double cv[5];
  loadCv(V, i, cv);
  if constexpr (!Ref<R>::on) {
    mixedUpdate(V, i, iStage, P.arkF[iStage - 1] * d2f(*dtp), P.grkF[iStage - 1], rhs, cv);
    return;
  }
  const double fac = P.ark[iStage - 1] * (*dtp);
  const double grk = P.grk[iStage - 1];
  const double adtv = fac / V.vol[i];
  RkAccess ra(P, iStage);
  R rs[5];
  if (ra.rd) {
#pragma unroll
    for (int k = 0; k < 5; ++k) rs[k] = V.rhsSum[k * n + i];
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const double r = (double)rhs[k];
    switch (P.rkScheme) {
      case 1:
        if (iStage == 1) { cv[k] = cv[k] - adtv * r; rs[k] = rhs[k]; }
        else if (iStage == P.nrkSteps) cv[k] = cv[k] - adtv * (r + (double)rs[k]);
        else { cv[k] = cv[k] - adtv * r; rs[k] = (R)((double)rs[k] + grk * r); }
        break;
      case 2:
        if (iStage == 1) { cv[k] = cv[k] - adtv * r; rs[k] = rhs[k]; }
        else if (iStage == 2) { cv[k] = cv[k] - adtv * (r - grk * (double)rs[k]); rs[k] = rhs[k]; }
        else cv[k] = cv[k] - adtv * (r - grk * (double)rs[k]);
        break;
      default:
        cv[k] = cv[k] - adtv * r;
    }
  }
  if (ra.wr) {
#pragma unroll
    for (int k = 0; k < 5; ++k) V.rhsSum[k * n + i] = rs[k];
  }
  double pr, tp, cs;
  dependentVars(P, cv, pr, tp, cs);
  afterUpdate(V, i, cv, pr, tp, cs);
#pragma unroll
  for (int k = 0; k < 5; ++k) V.cv[k * n + i] = cv[k];
  V.dv[i] = pr;
  V.dv[n + i] = tp;
  V.dv[2 * n + i] = cs;
  storePrim(V, i, cv, pr);
}

// ---------------------------------------------------------------------------
// Time step: RFLU_TimeStepInviscid (rocflu/RFLU_TimeStepInviscid.F90:120-333)
// per cell in face order, then a warp-shuffle + block minimum folded into one
// atomicMin on the bit pattern of the (positive) dt.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kBlock) kCellDt(View<R> V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double dt = 1.79769313486231571e308;
  if (i < V.nc) {
    const size_t n = V.nc;
    double sum = 0.0;
    const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
    for (int e = cb; e < ce; ++e) {
      const int code = V.cfEnt[e];
      if (code >= 0) {
        const int f = code >> 1, c1 = V.fc1[f], c2 = V.fc2[f];
        const double nx = V.fnx[f], ny = V.fny[f], nz = V.fnz[f], nm = V.fnm[f];
        const double ir1 = 1.0 / V.cv[c1], ir2 = 1.0 / V.cv[c2];
        const double u1 = V.cv[n + c1] * ir1, v1 = V.cv[2 * n + c1] * ir1, w1 = V.cv[3 * n + c1] * ir1;
        const double u2 = V.cv[n + c2] * ir2, v2 = V.cv[2 * n + c2] * ir2, w2 = V.cv[3 * n + c2] * ir2;
        const double a1 = V.dv[2 * n + c1], a2 = V.dv[2 * n + c2];
        const double vc = 0.5 * ((u1 + u2) * nx + (v1 + v2) * ny + (w1 + w2) * nz);
        const double as = 0.5 * (a1 + a2);
        sum = sum + (fabs(vc - 0.0) + as) * nm;
      } else {
        const int b = -code - 1;
        const double nx = V.bnx[b], ny = V.bny[b], nz = V.bnz[b], nm = V.bnm[b];
        const double ir1 = 1.0 / V.cv[i];
        const double u1 = V.cv[n + i] * ir1, v1 = V.cv[2 * n + i] * ir1, w1 = V.cv[3 * n + i] * ir1;
        if (const double *Q = symmetryQ(V, code)) {
          // an interior face to the cell's reflection (momentum reflected)
          const double m1[3] = {V.cv[n + i], V.cv[2 * n + i], V.cv[3 * n + i]};
          double m2[3];
          reflect3(Q, m1, m2);
          const double u2 = m2[0] * ir1, v2 = m2[1] * ir1, w2 = m2[2] * ir1;
          const double a1 = V.dv[2 * n + i];
          const double vc = 0.5 * ((u1 + u2) * nx + (v1 + v2) * ny + (w1 + w2) * nz);
          const double as = 0.5 * (a1 + a1);
          sum = sum + (fabs(vc - 0.0) + as) * nm;
          continue;
        }
        const double vc = u1 * nx + v1 * ny + w1 * nz;
        sum = sum + (fabs(vc - 0.0) + V.dv[2 * n + i]) * nm;
      }
    }
    dt = V.vol[i] / sum;
  }
  blockMinDt(V.sc, dt);
}

// RFLU_MinimumTimeStep (rocflu/RFLU_MinimumTimeStep.F90:100-245) and the
// endTime clip of RFLU_TimeStepping (rocflu/RFLU_TimeStepping.F90:444-446).
__device__ inline void finalizeDt(const Params &P, Scalars *sc) {
  double dtMin = __longlong_as_double((long long)sc->dtBits);
  double cfl = P.cfl;
  if (P.rkScheme == 1) cfl = fmin2(cfl, 3.0);
  else if (P.rkScheme == 2) cfl = fmin2(cfl, 2.0);
  else cfl = fmin2(cfl, 1.0);
  dtMin = cfl * dtMin;
  double wtI = 0.0, wtC = 0.0;
  if (sc->time <= 1.0e-8) wtI = 1.0; else wtC = 1.0;
  dtMin = wtI / P.dtImposed + wtC / dtMin;
  dtMin = 1.0 / dtMin;
  if (dtMin <= 0.0) dtMin = 6.0e-12;
  dtMin = fmax2(dtMin, P.dtMinLimit);
  if (sc->endTime > 0.0 && sc->time + dtMin > sc->endTime) {
    dtMin = sc->endTime - sc->time;
    sc->finished = 1;
  }
  sc->dtMin = dtMin;
}

template <typename R>
__global__ void kStepBegin(View<R> V) {
  // a step after the clipped last step does nothing (finished < 0)
  if (V.sc->finished > 0) V.sc->finished = -1;
  V.sc->dtBits = 0x7fefffffffffffffull;
}

template <typename R>
__global__ void kDtFinalize(View<R> V) {
  if (V.sc->finished < 0) return;
  finalizeDt(V.p, V.sc);
}

template <typename R>
__global__ void kStepEnd(View<R> V) {
  if (V.sc->finished < 0) return;
  V.sc->time = V.sc->time + V.sc->dtMin;
  V.sc->stepsDone += 1;
}

// Self-check of refinedRecip and refinedSqrt against IEEE FP64 division and
// square root, compiled with this translation unit's flags (the FP32 seeds of
// the mixed mode use its approximate division): x = 2^e * m with m uniform in
// [1, 2) and e uniform in [-emax, emax] from a 64-bit hash of (seed, k); the
// largest relative error of each, as the bits of a positive double
// (monotone in the value), in out[0] and out[1].
__device__ inline unsigned long long refineHash(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__global__ void kRefineCheck(long long n, unsigned long long seed, int emax, unsigned long long *out) {
  double eR = 0.0, eS = 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const unsigned long long h = refineHash(seed ^ refineHash((unsigned long long)k));
    const int e = (int)((h >> 52) % (unsigned long long)(2 * emax + 1)) - emax;
    const double x = ldexp(1.0 + (double)(h & 0xFFFFFFFFFFFFFull) * 0x1p-52, e);
    const double r = refinedRecip(x, 1.0f / d2f(x));
    eR = fmax(eR, fabs(r - 1.0 / x) * x);
    const double sx = sqrt(x);
    eS = fmax(eS, fabs(refinedSqrt(x) - sx) / sx);
  }
  atomicMax(&out[0], (unsigned long long)__double_as_longlong(eR));
  atomicMax(&out[1], (unsigned long long)__double_as_longlong(eS));
}

// ---------------------------------------------------------------------------
// Host launchers of this precision
// ---------------------------------------------------------------------------
template <typename R>
struct Launch {
  static void initState(const View<R> &V, cudaStream_t s) { kInitState<R><<<blocks(V.nc), kBlock, 0, s>>>(V); }
  static void initFromRef(const View<R> &V, const double *ref, int o0, int o1, cudaStream_t s) {
    if (o1 > o0) kInitFromRef<R><<<blocks(o1 - o0), kBlock, 0, s>>>(V, ref, o0, o1);
  }
  // WENO smoothing (RECONST 1, 2): the gradient kernels write the
  // unsmoothed gradients into gradRaw (a copy of the view), kWenoSmooth the
  // final ones into grad
  static bool weno(const View<R> &V) { return V.p.reconst == 1 || V.p.reconst == 2; }
  static View<R> rawView(const View<R> &V) {
    View<R> W = V;
    if (weno(V)) W.grad = V.gradRaw;
    return W;
  }
  static void gradLimit(const View<R> &V, cudaStream_t s) {
    if (V.p.spaceOrder < 2) return;
    const View<R> W = rawView(V);
    if (V.tiled) launchTile<false>(W, s);
    else kGradLimit<R><<<blocks(V.nc), kBlock, 0, s>>>(W);
    if (weno(V)) smooth(V, s);
  }
  static void smooth(const View<R> &V, cudaStream_t s) {
    if (Layout<R>::packed && V.tiled)
      kWenoTile<R><<<(V.nc + kTile - 1) / kTile, kBlock, wenoTileSmemBytes(V), s>>>(V, V.gradRaw);
    else
      kWenoSmooth<R><<<blocks(V.nc), kBlock, 0, s>>>(V, V.gradRaw);
  }
  // the tiled kernel specialised for the limiter (RECONST 10, 100, 11; other
  // values: unlimited)
  template <bool kDt>
  static void launchTile(const View<R> &V, cudaStream_t s) {
    const int rc = V.p.reconst;
    const size_t b = tileSmemBytes(V, rc == 11);
    const int nTiles = (V.nc + kTile - 1) / kTile;
    const int g = kDt ? V.tileGridDt : V.tileGrid;
    const int grid = g > 0 ? std::min(nTiles, g) : nTiles;
    if (rc == 10) kGradTile<R, kDt, 10><<<grid, kBlock, b, s>>>(V);
    else if (rc == 100) kGradTile<R, kDt, 100><<<grid, kBlock, b, s>>>(V);
    else if (rc == 11) kGradTile<R, kDt, 11><<<grid, kBlock, b, s>>>(V);
    else kGradTile<R, kDt, 0><<<grid, kBlock, b, s>>>(V);
  }
  // CTAs of the persistent tiled kernels: the resident CTAs per SM of the
  // variant the mesh's limiter selects (with the time-step sum when withDt),
  // times the SMs (0 when untiled)
  template <bool kDt, int kRc>
  static int residentTiles(const View<R> &V) {
    int per = 0, dev = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kGradTile<R, kDt, kRc>, kBlock, tileSmemBytes(V, kRc == 11));
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(per, 1) * sms;
  }
  static int tileGrid(const View<R> &V, int withDt) {
    if (!V.tiled) return 0;
    const int rc = V.p.reconst;
    if (rc == 10) return withDt ? residentTiles<true, 10>(V) : residentTiles<false, 10>(V);
    if (rc == 100) return withDt ? residentTiles<true, 100>(V) : residentTiles<false, 100>(V);
    if (rc == 11) return withDt ? residentTiles<true, 11>(V) : residentTiles<false, 11>(V);
    return withDt ? residentTiles<true, 0>(V) : residentTiles<false, 0>(V);
  }
  template <bool kDt, int kRc>
  static void setTileSmem(const View<R> &V) {
    cudaFuncSetAttribute(kGradTile<R, kDt, kRc>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)tileSmemBytes(V, kRc == 11));
  }
  // Kernel attributes that depend on the mesh (shared memory of the tiled
  // kernels); called once at set-up, outside any stream capture.
  static void adjointSetup(const View<R> &V, cudaStream_t s) {
    if (V.tsW) kTsWeights<R><<<blocks(V.nc), kBlock, 0, s>>>(V);
  }
  static void configure(const View<R> &V) {
    if (V.tiled) {
      setTileSmem<false, 0>(V); setTileSmem<false, 10>(V); setTileSmem<false, 100>(V); setTileSmem<false, 11>(V);
      setTileSmem<true, 0>(V); setTileSmem<true, 10>(V); setTileSmem<true, 100>(V); setTileSmem<true, 11>(V);
    }
    if (Layout<R>::packed && V.tiled && V.gradRaw)
      cudaFuncSetAttribute(kWenoTile<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wenoTileSmemBytes(V));
    if (Layout<R>::packed && V.tiled)
      cudaFuncSetAttribute(kCellDtTile<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dtTileSmemBytes(V));
  }
  static void faceFlux(const View<R> &V, cudaStream_t s) {
    kFaceFlux<R><<<blocks((long long)V.nf + V.nb), kBlock, 0, s>>>(V);
  }
  static void gatherRhs(const View<R> &V, cudaStream_t s) { kGatherRhs<R><<<blocks(V.nc), kBlock, 0, s>>>(V); }
  static void gatherUpdate(const View<R> &V, int iStage, const double *dtp, cudaStream_t s) {
    kGatherUpdate<R, false><<<blocks(V.nc), kBlock, 0, s>>>(V, iStage, dtp);
  }
  static void updateFromRhs(const View<R> &V, int iStage, const double *dtp, cudaStream_t s) {
    kGatherUpdate<R, true><<<blocks(V.nc), kBlock, 0, s>>>(V, iStage, dtp);
  }
  static void addRhs(const View<R> &V, const double *src, cudaStream_t s) {
    kAddRhs<R><<<blocks(V.nc), kBlock, 0, s>>>(V, src);
  }
  // The FP64 modes: RFLU_TimeStepInviscid in FP64 from cv and dv; the mixed
  // mode: the FP32 sum from the primitive state, as its steps take it.
  static void timestep(const View<R> &V, cudaStream_t s) {
    kStepBegin<R><<<1, 1, 0, s>>>(V);
    if (Ref<R>::on) kCellDt<R><<<blocks(V.nc), kBlock, 0, s>>>(V);
    else if (Layout<R>::packed && V.tiled)
      kCellDtTile<R><<<(V.nc + kTile - 1) / kTile, kBlock, dtTileSmemBytes(V), s>>>(V);
    else kCellDtPrim<R><<<blocks(V.nc), kBlock, 0, s>>>(V);
    kDtFinalize<R><<<1, 1, 0, s>>>(V);
  }
  // Time-step reduction + gradients of the first stage of a step.  The FP64
  // modes keep the reference's separate FP64 sweep (bit-exact dt); the mixed
  // mode folds an FP32 sweep into the gradient kernel, which gathers the
  // same neighbours.
  static void stepStart(const View<R> &V, cudaStream_t s) {
    if (Ref<R>::on) {
      timestep(V, s);
      gradLimit(V, s);
    } else {
      kStepBegin<R><<<1, 1, 0, s>>>(V);
      const View<R> W = rawView(V);
      if (V.tiled) launchTile<true>(W, s);
      else kGradLimitDt<R><<<blocks(V.nc), kBlock, 0, s>>>(W);
      if (weno(V) && V.p.spaceOrder > 1) smooth(V, s);
      kDtFinalize<R><<<1, 1, 0, s>>>(V);
    }
  }
  static void stepEnd(const View<R> &V, cudaStream_t s) { kStepEnd<R><<<1, 1, 0, s>>>(V); }
};

}  // namespace RFLU_NS
}  // namespace rflu
