// Tangent (JVP) and discrete adjoint (VJP) of the residual of one region,
// R(cv) = CellGradientsMP + ConvectiveFluxesMP, for every precision mode:
// templated on the state type R of the View (double: FP64 modes, float: the
// mixed mode).  In the mixed mode the flux, reconstruction, limiter and
// prim/dv -> cv Jacobians are evaluated in FP32 (the arithmetic of the mixed
// primal's fluxes; the Jacobian of the pressure recovery has no cancellation,
// unlike the recovery itself).
//
// Tangent: the primal cell/face code of kernels.cuh evaluated on Dual<1>
// (value + one directional derivative), so every branch the primal takes
// (limiter minima, eigen-frame merging, flux cases) is differentiated as
// taken.
//
// Adjoint, for rhsBar = lambda(5,nCells):
//   1. forward: primitive state, unlimited LSQ gradient G, limiter factors
//      with their active face and active extremum neighbour per variable,
//      limited gradient G~;
//   2. face adjoint (one thread per face): Fbar = lambda(c1) - lambda(c2)
//      (boundary: lambda(c)); the transposed flux Jacobian applied to Fbar
//      from the face's local Jacobian (Dual<6>/Dual<8> seeds on the
//      reconstructed left/right states; the Roe flux has a hand-written
//      reverse sweep), stored per face side;
//   3. cell adjoint (one thread per cell, gather over the same CSR): side
//      adjoints -> primitive and limited-gradient adjoints; limiter reverse
//      through its active branch; own-term of the gradient transpose;
//   4. cell adjoint (gather over the transposed stencil and the face
//      neighbours): neighbour terms of the gradient and limiter transposes,
//      then prim/dv -> cv through the local Jacobian (Dual<5> in FP64; the
//      mixed mode's closed form in FP32).
// No atomics: every sum is a gather in a fixed order.  The adjoint covers
// RECONST 0, 11 (Venkatakrishnan), 100 (componentwise BJ) and 10 (BJ with the
// eigen-frame velocity limiter, whose eigenvectors are differentiated by
// first-order perturbation in the tangent and the adjoint alike).
#pragma once
#include "dual.cuh"
#include "roe_adjoint.cuh"

namespace rflu {
namespace RFLU_NS {

template <typename R>
struct AdjWork {
  R *cvd, *primd, *dvd, *gradd, *fluxd;  // tangent state / lambda in cvd
  R *G, *lim, *faceAdj, *Gbar, *qbar, *nbBar, *cvbarD, *dvbar;
  R *nbVel;                              // FP64 layouts, RECONST 10: per axis the neighbour's velocity share (9 Nc)
  int *estar, *jstar;                    // 5 per cell each
  // packed layout: per cell i a 16-float record (L_i Gbar_i for the five
  // variables, 15 floats; pad), so that a transposed stencil entry of cell j
  // costs two 256-bit loads next to its weights from View::tsW:
  // w_s . Gbar_i = (d/|d|^2) . (L_i Gbar_i), d = x_j - x_i (L symmetric)
  R *adjRec;
  // packed layout: per cell a 20-word record of the limiter's extreme-
  // neighbour terms: for each variable the neighbour that receives one (-1:
  // none; int bits; RECONST 10: the eigen-frame axes in slots 1-3), then the
  // variables' values, then the axes' velocity vectors, then pad
  R *nbRec;
  // packed layout: per cell the sum over its stencil of d/|d|^2 (3 Nc, SoA),
  // so that the gradient's own term in the adjoint is one dot product
  R *ssum;
};

// The workspace carved from the context's adjoint buffer: 90 Nc + 21 (Nf+Nb)
// values of R, 10 Nc ints and (packed layout) 16 + 20 + 3 Nc floats on a 32-byte
// boundary (the context allocates sizeof(R)*(130 Nc + 24 (Nf+Nb) + 64) +
// 4*10 Nc + 256 bytes).
template <typename R>
inline AdjWork<R> carveAdjWork(double *work, size_t nc, size_t nT) {
  char *p = reinterpret_cast<char *>(work);
  auto take = [&](size_t count) {
    R *r = reinterpret_cast<R *>(p);
    p += count * sizeof(R);
    return r;
  };
  AdjWork<R> a;
  a.cvd = take(5 * nc);
  a.primd = take(5 * nc);
  a.dvd = take(3 * nc);
  a.gradd = take(15 * nc);
  a.fluxd = take(5 * nT);
  a.G = take(15 * nc);
  a.lim = take(5 * nc);
  a.faceAdj = take(16 * nT);
  a.Gbar = take(15 * nc);
  a.qbar = take(5 * nc);
  a.nbBar = take(5 * nc);
  a.cvbarD = take(5 * nc);
  a.dvbar = take(3 * nc);
  a.nbVel = take(9 * nc);
  a.estar = reinterpret_cast<int *>(p);
  p += sizeof(int) * 5 * nc;
  a.jstar = reinterpret_cast<int *>(p);
  p += sizeof(int) * 5 * nc;
  p = reinterpret_cast<char *>((reinterpret_cast<size_t>(p) + 31) & ~size_t(31));
  a.adjRec = reinterpret_cast<R *>(p);
  a.nbRec = a.adjRec + 16 * nc;
  a.ssum = a.nbRec + 20 * nc;
  return a;
}

// WENO smoothing of the gradients (RECONST 1, 2) on a second-order run.
__host__ __device__ inline bool isWeno(const Params &P) {
  return P.spaceOrder > 1 && (P.reconst == 1 || P.reconst == 2);
}

// Constrained gradients (CRECONSTC 1) in the tangent and the adjoint: the
// fit of a constrained variable is linear in its rows' differences (the
// stencil members' and the constraint values, constant at the walls; a
// burning injection face's follow its cell's pressure, whose adjoint gathers
// them through the per-cell lists V.cpOff/V.cpEnt), so its transpose takes
// the plan's weights where the least-squares fit takes the members' weights.
// The plan's rows per constrained variable: its stencil rows in stencil
// order, then its constraint rows.
template <typename R>
__device__ inline int constrMask(const View<R> &V, int i, int &sl) {
  sl = V.cSlot ? V.cSlot[i] : -1;
  if (sl < 0) return 0;
  int m = 0;
#pragma unroll
  for (int k = 0; k < 5; ++k)
    if (V.cNcon[5 * sl + k]) m |= 1 << k;
  return m;
}
// the first row of constrained variable k of slot sl (nst stencil members)
template <typename R>
__device__ inline int constrRow0(const View<R> &V, int sl, int k, int nst) {
  int r = V.cRowOff[sl];
  for (int kk = 0; kk < k; ++kk) {
    const int nc = V.cNcon[5 * sl + kk];
    if (nc) r += nst + nc;
  }
  return r;
}
// the own term of cell i's constrained variables: every row's difference
// subtracts the cell's value
template <typename R>
__device__ inline void constrOwnTerm(const View<R> &V, int i, int sl, const R *gb, R *qb) {
  const int nst = V.stOff[i + 1] - V.stOff[i];
  int r = V.cRowOff[sl];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int nc = V.cNcon[5 * sl + k];
    for (int t = 0; t < (nc ? nst + nc : 0); ++t, ++r)
      qb[k] -= V.cW[3 * (size_t)r] * gb[3 * k] + V.cW[3 * (size_t)r + 1] * gb[3 * k + 1] +
               V.cW[3 * (size_t)r + 2] * gb[3 * k + 2];
  }
}

// Symmetry patches in the tangent and the adjoint: a reflected stencil
// member's velocity is Q u (memberReflection), and a face on a symmetry
// patch is a face to the cell's own reflection, which the limiters' branch
// records mark as the neighbour kMirrorNb - b (b the boundary face): its
// extreme value's derivative goes back to the cell itself through Q.
constexpr int kMirrorNb = -2;

// Threads per cell of the packed layout's WENO gathers (kAdjWeno over the
// transposed stencil, kAdjWenoFwdLanes over the stencil): each lane every
// second entry, the sums joined by shuffles.  (Measured: the same split of
// kAdjCell2's and kAdjGradFwd's gathers, by entries or by record halves,
// made them slower.)
template <typename R>
__host__ __device__ constexpr int adjLanes() {
  return Layout<R>::packed ? 2 : 1;
}
template <typename R>
__device__ inline const R *memberReflection(const View<R> &V, int s) {
  if (!V.stXf) return nullptr;
  const int x = V.stXf[s];
  return x >= 0 ? V.xfQ + 9 * x : nullptr;
}

// Primitive state and dependent variables of one cell as functions of cv:
// RFLU_ConvertCvCons2Prim (DUVWP) and RFLU_SetDependentVars.
template <typename S>
__device__ inline void primFromCv(const Params &P, const S *cv, S *q, S *dv) {
  const S gc = S(8314.3 / P.gvMol);
  const S g = S(P.gvCp / (P.gvCp - 8314.3 / P.gvMol));
  S r = cv[0];
  S ir = S(1) / r;
  S Eo = ir * cv[4];
  S Vm2 = ir * ir * (cv[1] * cv[1] + cv[2] * cv[2] + cv[3] * cv[3]);
  S p = (g - S(1)) * r * (Eo - S(0.5) * Vm2);
  S t = p / (r * gc);
  dv[0] = p;
  dv[1] = t;
  dv[2] = sqrt_(g * gc * t);
  q[0] = r;
  q[1] = ir * cv[1];
  q[2] = ir * cv[2];
  q[3] = ir * cv[3];
  q[4] = p;
}

// Cell data of the tangent: primal values (layout of the mode) with the
// directional derivatives of the workspace (structure of arrays).
template <typename R>
struct TanLoad {
  using S = Dual<1, R>;
  using H = Dual<1, double>;
  const View<R> &V;
  const AdjWork<R> &W;
  __device__ S prim(int k, int c) const {
    S x(PlainLoad<R>{V}.prim(k, c));
    x.d[0] = W.primd[(size_t)k * V.nc + c];
    return x;
  }
  __device__ S grad(int k, int c) const {
    S x(PlainLoad<R>{V}.grad(k, c));
    x.d[0] = W.gradd[(size_t)k * V.nc + c];
    return x;
  }
  __device__ void prim4(int c, S *q) const {
    for (int k = 0; k < 4; ++k) q[k] = prim(k, c);
  }
  __device__ void prim5(int c, S *q) const {
    for (int k = 0; k < 5; ++k) q[k] = prim(k, c);
  }
  // packed layout only: prim and the centroid (no derivative)
  __device__ void primCg(int c, S *q, S *x) const {
    prim5(c, q);
    for (int k = 0; k < 3; ++k) x[k] = S(V.prim[8 * (size_t)c + 5 + k]);
  }
  __device__ void grad15(int c, S *g) const {
    for (int k = 0; k < 15; ++k) g[k] = grad(k, c);
  }
  __device__ H cv(int k, int c) const {
    size_t o = (size_t)k * V.nc + c;
    H x(V.cv[o]);
    x.d[0] = W.cvd[o];
    return x;
  }
  __device__ H dv(int k, int c) const {
    size_t o = (size_t)k * V.nc + c;
    H x(V.dv[o]);
    x.d[0] = W.dvd[o];
    return x;
  }
};

// ---------------------------------------------------------------------------
// Tangent kernels
// ---------------------------------------------------------------------------
template <typename R>
__global__ void kTanInit(View<R> V, AdjWork<R> W, const double *cvDotRef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const size_t n = V.nc;
  const int o = V.refId[i];
  using D1 = Dual<1>;
  D1 cv[5], q[5], dv[3];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    cv[k] = D1(V.cv[k * n + i]);
    cv[k].d[0] = cvDotRef[5 * (size_t)o + k];
    W.cvd[k * n + i] = (R)cv[k].d[0];
  }
  primFromCv(V.p, cv, q, dv);
#pragma unroll
  for (int k = 0; k < 5; ++k) W.primd[k * n + i] = (R)q[k].d[0];
#pragma unroll
  for (int k = 0; k < 3; ++k) W.dvd[k * n + i] = (R)dv[k].d[0];
}

template <typename R>
__global__ void __launch_bounds__(kBlock) kTanGrad(View<R> V, AdjWork<R> W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  Dual<1, R> g[15];
  gradLimitCell(V, TanLoad<R>{V, W}, i, g);
  const size_t n = V.nc;
  if (isWeno(V.p)) {
    // the unsmoothed gradient and its derivative, for kTanWeno
#pragma unroll
    for (int k = 0; k < 15; ++k) {
      W.G[k * n + i] = g[k].v;
      W.Gbar[k * n + i] = g[k].d[0];
    }
    return;
  }
  R gv[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) {
    gv[k] = g[k].v;
    W.gradd[k * n + i] = g[k].d[0];
  }
  storeGrad(V, i, gv);
}

// The simple limiter after the WENO smoothing (RFLU_LimitGradCellsSimple,
// modflu/RFLU_ModLimiters.F90:1147-1300) on one cell's smoothed gradient g,
// generic in its scalar type: the zeroing is a branch, so a zeroed
// gradient's derivative is zero too.  Returns the factors (0 or 1) of
// density and pressure.
template <typename R, typename S>
__device__ inline void wenoPositivity(const View<R> &V, int i, S *g, R *f0, R *f4) {
  const PlainLoad<R> ld{V};
  const int cb = V.cfOff[i];
  const size_t nb = V.nb;
  const int z = simplePositivity(S(ld.prim(0, i)), S(ld.prim(4, i)), V.cfOff[i + 1] - cb,
                   [&](int k, S *d) {
                     const int code = V.cfEnt[cb + k];
                     R e[3];
                     if (code >= 0) {
                       faceOffset(V, code >> 1, code & 1, e);
                     } else {
                       const int b = -code - 1;
                       e[0] = V.bd[b];
                       e[1] = V.bd[nb + b];
                       e[2] = V.bd[2 * nb + b];
                     }
                     d[0] = S(e[0]);
                     d[1] = S(e[1]);
                     d[2] = S(e[2]);
                     return true;
                   },
                   g);
  *f0 = (z & 1) ? R(0) : R(1);
  *f4 = (z & 2) ? R(0) : R(1);
}

// Tangent of the WENO smoothing (RECONST 1, 2): the averages of kWenoSmooth
// on dual numbers from the unsmoothed gradients and their derivatives
// (W.G, W.Gbar, written by kTanGrad), then the simple limiter.
template <typename R>
__global__ void __launch_bounds__(kBlock) kTanWeno(View<R> V, AdjWork<R> W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  using S = Dual<1, R>;
  const size_t n = V.nc;
  auto row = [&](int c, S *t) {
#pragma unroll
    for (int k = 0; k < 15; ++k) {
      t[k] = S(W.G[k * n + c]);
      t[k].d[0] = W.Gbar[k * n + c];
    }
  };
  auto fetch = [&](int s, S *t) {
    row(V.stIdx[s], t);
    if (const R *Q = memberReflection(V, s)) reflectGrad(Q, t);
  };
  const int sb = V.stOff[i], se = V.stOff[i + 1];
  S own[16], g[15];
  row(i, own);
  if (V.p.reconst == 2) wenoXyz(own, sb, se, fetch, g);
  else wenoSimple(own, sb, se, fetch, g);
  R f0, f4;
  wenoPositivity(V, i, g, &f0, &f4);
  R gv[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) {
    gv[k] = g[k].v;
    W.gradd[k * n + i] = g[k].d[0];
  }
  storeGrad(V, i, gv);
}

template <typename R>
__global__ void __launch_bounds__(kBlock) kTanFlux(View<R> V, AdjWork<R> W) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nT = V.nf + V.nb;
  if (t >= nT) return;
  Dual<1, R> flx[5];
  faceFluxEval(V, TanLoad<R>{V, W}, t, flx);
  R fd[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) fd[k] = flx[k].d[0];
  storeFluxAt(W.fluxd, (size_t)nT, t, fd);
}

template <typename R>
__global__ void kTanGather(View<R> V, AdjWork<R> W, double *outRef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  R r[5];
  gatherRhs(V, (const R *)W.fluxd, i, r);
  const int o = V.refId[i];
#pragma unroll
  for (int k = 0; k < 5; ++k) outRef[5 * (size_t)o + k] = (double)r[k];
}

// ---------------------------------------------------------------------------
// Adjoint kernels
// ---------------------------------------------------------------------------
template <typename R>
__global__ void kAdjLambda(View<R> V, AdjWork<R> W, const double *lamRef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const int o = V.refId[i];
#pragma unroll
  for (int k = 0; k < 5; ++k) W.cvd[(size_t)k * V.nc + i] = (R)lamRef[5 * (size_t)o + k];
}

// Venkatakrishnan factor (RFLU_ModLimiters.F90:494-516) of one face side.
template <typename S>
__device__ inline S venkat(S dext, S d2, S epsq) {
  S numer = (dext * dext + epsq) * d2 + S(2) * d2 * d2 * dext;
  S denom = d2 * (dext * dext + S(2) * d2 * d2 + dext * d2 + epsq);
  return numer / (denom + S(1.0e-12));
}

// The eigen-frame velocity limiter of one cell (RECONST 10,
// RFLU_LimitGradVelocityBarthJesp, modflu/RFLU_ModLimiters.F90:588-790) as
// the tangent kernels evaluate it (gradLimitCell on dual numbers: per-face
// minima, eigenpairs of the strain rate with perturbation derivatives), with
// the branch each axis's factor takes, for the reverse pass.  G is the
// unlimited velocity gradient, G[a + 3c] = d u_a / d x_c.
template <typename R>
struct VelFrame {
  R A[9], ev[3];   // eigenvectors (component r of axis j at A[r + 3j]) and eigenvalues
  R B[9];          // A^T G: B[j + 3c] = sum_a A[a + 3j] G[a + 3c]
  R alRaw[3];      // each axis's factor before the merge of equal eigenvalues
  R al[3];         // after it
  int src[3];      // the axis whose raw factor al[j] equals
  int side[3];     // 0: alRaw = 1; 1: dmx / pr; 2: dmn / pr
  int face[3];     // cell-face entry of the active projection pr
  int nb[3];       // neighbour of the active extreme dmx or dmn (-1: the extreme is the initial 0)
  bool held[3];    // idle axis (physics.cuh: idleAxis): the factor is held at its value
  R dext[3], pext[3];
};

template <typename R, typename L>
__device__ inline void velFrameForward(const View<R> &V, const L &ld, int i, const R *G, VelFrame<R> &F) {
  R Sy[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) Sy[a + 3 * b] = R(0.5) * (G[a + 3 * b] + G[b + 3 * a]);
  symmetricEigen3(Sy, F.A, F.ev);
  const R *A = F.A;
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      R s = R(0);
      s = s + A[3 * j] * G[3 * c];
      s = s + A[3 * j + 1] * G[1 + 3 * c];
      s = s + A[3 * j + 2] * G[2 + 3 * c];
      F.B[j + 3 * c] = s;
    }
  R dmn[3] = {R(0), R(0), R(0)}, dmx[3] = {R(0), R(0), R(0)};
  int nmn[3] = {-1, -1, -1}, nmx[3] = {-1, -1, -1};
  const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
  R ui[4];
  ld.prim4(i, ui);
  for (int e = cb; e < ce; ++e) {
    const int code = V.cfEnt[e];
    R du[3];
    int other;
    if (code < 0) {
      // a symmetry face: the cell's reflection as the second cell
      const double *Q = symmetryQ(V, code);
      if (!Q) continue;
      R um[3];
      reflect3(Q, ui + 1, um);
#pragma unroll
      for (int k = 0; k < 3; ++k) du[k] = um[k] - ui[1 + k];
      other = kMirrorNb - (-code - 1);
    } else {
      int c1, c2;
      faceCells(V, code >> 1, c1, c2);
      R a1[4], a2[4];
      ld.prim4(c1, a1);
      ld.prim4(c2, a2);
#pragma unroll
      for (int k = 0; k < 3; ++k) du[k] = a2[1 + k] - a1[1 + k];
      other = (code & 1) ? c1 : c2;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      R pr = R(0);
      pr = pr + A[3 * j] * du[0];
      pr = pr + A[3 * j + 1] * du[1];
      pr = pr + A[3 * j + 2] * du[2];
      if (code >= 0 && (code & 1)) pr = -pr;
      if (pr < dmn[j]) { dmn[j] = pr; nmn[j] = other; }
      if (pr > dmx[j]) { dmx[j] = pr; nmx[j] = other; }
    }
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    F.alRaw[j] = R(1); F.side[j] = 0; F.face[j] = -1; F.nb[j] = -1; F.dext[j] = R(0); F.pext[j] = R(1);
  }
  for (int e = cb; e < ce; ++e) {
    const int code = V.cfEnt[e];
    R d[3];
    if (!limiterFaceOffset(V, code, d)) continue;
    const R off[3] = {-d[0], -d[1], -d[2]};
    R sh[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      R s = R(0);
      s = s + G[a] * off[0];
      s = s + G[a + 3] * off[1];
      s = s + G[a + 6] * off[2];
      sh[a] = s;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      R pr = R(0);
      pr = pr + A[3 * j] * sh[0];
      pr = pr + A[3 * j + 1] * sh[1];
      pr = pr + A[3 * j + 2] * sh[2];
      if (pr > R(0)) {
        const R t = dmx[j] / pr;
        if (t < F.alRaw[j]) { F.alRaw[j] = t; F.side[j] = 1; F.face[j] = e; F.nb[j] = nmx[j]; F.dext[j] = dmx[j]; F.pext[j] = pr; }
      } else if (pr < R(0)) {
        const R t = dmn[j] / pr;
        if (t < F.alRaw[j]) { F.alRaw[j] = t; F.side[j] = 2; F.face[j] = e; F.nb[j] = nmn[j]; F.dext[j] = dmn[j]; F.pext[j] = pr; }
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) F.held[j] = idleAxis(A, G, j);
  // merge the factors of equal eigenvalues (within 1e-3 of the largest magnitude)
  R mx = fabs_(F.ev[0]);
  mx = fmax2(mx, fabs_(F.ev[1]));
  mx = fmax2(mx, fabs_(F.ev[2]));
  const R scale = R(1.0e-3) * mx;
  const bool e12 = (F.ev[1] - F.ev[0] <= scale), e23 = (F.ev[2] - F.ev[1] <= scale);
#pragma unroll
  for (int j = 0; j < 3; ++j) { F.al[j] = F.alRaw[j]; F.src[j] = j; }
  // fmin2's choice (the first of equal values), by selects only (no
  // run-time array index)
  if (e12 && e23) {
    const bool b01 = F.alRaw[1] < F.alRaw[0];
    const R v01 = b01 ? F.alRaw[1] : F.alRaw[0];
    const bool b2 = F.alRaw[2] < v01;
    const R v = b2 ? F.alRaw[2] : v01;
    const int m = b2 ? 2 : (b01 ? 1 : 0);
#pragma unroll
    for (int j = 0; j < 3; ++j) { F.al[j] = v; F.src[j] = m; }
  } else if (e12) {
    const bool b = F.alRaw[1] < F.alRaw[0];
    F.al[0] = F.al[1] = b ? F.alRaw[1] : F.alRaw[0];
    F.src[0] = F.src[1] = b ? 1 : 0;
  } else if (e23) {
    const bool b = F.alRaw[2] < F.alRaw[1];
    F.al[1] = F.al[2] = b ? F.alRaw[2] : F.alRaw[1];
    F.src[1] = F.src[2] = b ? 2 : 1;
  }
}

// Limited velocity gradient from the frame: A diag(al) A^T G, in the
// primal's operation order; gl[3 * (1 + a) + c].
template <typename R>
__device__ inline void velFrameApply(const VelFrame<R> &F, R *gl) {
  R Rm[9];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int c = 0; c < 3; ++c) Rm[j + 3 * c] = F.al[j] * F.B[j + 3 * c];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      R s = R(0);
      s = s + F.A[a] * Rm[3 * c];
      s = s + F.A[a + 3] * Rm[1 + 3 * c];
      s = s + F.A[a + 6] * Rm[2 + 3 * c];
      gl[3 * (1 + a) + c] = s;
    }
}

// Reverse of the limiter: from glb (adjoint of the limited velocity
// gradient, glb[a + 3c]) to Gb (of the unlimited one), ub (of the cell's
// own velocity) and, per axis j, the velocity adjoint nbv[3j..3j+2] that
// neighbour F.nb[j] receives (when F.side[j], not F.held[j], and
// F.nb[j] >= 0).  The
// transpose of the tangent's linear map: Gl = sum_j al_j A_j B_j with
// B = A^T G; the active factor al = dext / pr, dext = A_j . (u_nb - u_i),
// pr = A_j . G (cofg - fc); the eigenvectors' perturbation
// da_j = sum_{k != j} a_k (a_k' dS a_j) / (l_j - l_k), S = sym(G), without
// the pairs the limiter merges (physics.cuh: mergedPair).
template <typename R, typename L>
__device__ inline void velFrameReverse(const View<R> &V, const L &ld, int i, const R *G, const VelFrame<R> &F,
                                       const R *glb, R *Gb, R *ub, R *nbv) {
  const R *A = F.A;
  R Ab[9], Bb[9], alb[3] = {R(0), R(0), R(0)};
#pragma unroll
  for (int k = 0; k < 9; ++k) { Ab[k] = R(0); Gb[k] = R(0); nbv[k] = R(0); }
  ub[0] = ub[1] = ub[2] = R(0);
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      // M = diag(al) B, Gl = A M
      R mb = R(0);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        mb += A[a + 3 * j] * glb[a + 3 * c];
        Ab[a + 3 * j] += glb[a + 3 * c] * F.al[j] * F.B[j + 3 * c];
      }
      Bb[j + 3 * c] = F.al[j] * mb;
      alb[j] += mb * F.B[j + 3 * c];
    }
  R albRaw[3] = {R(0), R(0), R(0)};
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int t = 0; t < 3; ++t)
      if (F.src[j] == t) albRaw[t] += alb[j];
  R ui[4];
  ld.prim4(i, ui);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    if (F.side[j] == 0 || F.held[j] || albRaw[j] == R(0)) continue;
    // alRaw = dext / pr: the same guarded form as the scalar limiter's
    const R r = albRaw[j] / F.pext[j];
    const R dextb = r, prb = -r * (F.dext[j] / F.pext[j]);
    if (F.nb[j] >= 0) {
      R un[4];
      ld.prim4(F.nb[j], un);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        Ab[a + 3 * j] += dextb * (un[1 + a] - ui[1 + a]);
        nbv[3 * j + a] = dextb * A[a + 3 * j];
        ub[a] -= dextb * A[a + 3 * j];
      }
    } else if (F.nb[j] <= kMirrorNb) {
      // the extreme is the cell's reflection Q u across a symmetry face:
      // dext = A_j . (Q u - u), its derivative (Q - I) A_j (Q symmetric)
      const int ip = V.bpatch[kMirrorNb - F.nb[j]];
      const double *Q = V.patchK + kPatchK * ip;
      R un[3], qa[3];
      reflect3(Q, ui + 1, un);
      const R aj[3] = {A[3 * j], A[3 * j + 1], A[3 * j + 2]};
      reflect3(Q, aj, qa);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        Ab[a + 3 * j] += dextb * (un[a] - ui[1 + a]);
        ub[a] += dextb * (qa[a] - A[a + 3 * j]);
      }
    }
    // pr = A_j . G off, off = cofg - fc of the active face
    const int code = V.cfEnt[F.face[j]];
    R d[3];
    limiterFaceOffset(V, code, d);
    const R off[3] = {-d[0], -d[1], -d[2]};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const R sh = G[a] * off[0] + G[a + 3] * off[1] + G[a + 6] * off[2];
      Ab[a + 3 * j] += prb * sh;
#pragma unroll
      for (int c = 0; c < 3; ++c) Gb[a + 3 * c] += prb * A[a + 3 * j] * off[c];
    }
  }
  // B = A^T G
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        Ab[a + 3 * j] += G[a + 3 * c] * Bb[j + 3 * c];
        Gb[a + 3 * c] += A[a + 3 * j] * Bb[j + 3 * c];
      }
  // eigenvectors of S = sym(G): Sb = sum_{j<k} coef_jk sym(a_k a_j')
  R Sb[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Sb[k] = R(0);
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int k = j + 1; k < 3; ++k) {
      if (F.ev[j] == F.ev[k] || mergedPair(F.ev, j, k)) continue;
      R ajk = R(0), akj = R(0);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        ajk += Ab[a + 3 * j] * A[a + 3 * k];
        akj += Ab[a + 3 * k] * A[a + 3 * j];
      }
      const R coef = (ajk - akj) / (F.ev[j] - F.ev[k]);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) Sb[a + 3 * b] += coef * R(0.5) * (A[a + 3 * k] * A[b + 3 * j] + A[a + 3 * j] * A[b + 3 * k]);
    }
  // S = (G + G') / 2
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) Gb[a + 3 * b] += R(0.5) * (Sb[a + 3 * b] + Sb[b + 3 * a]);
}

// Forward pass of the limited gradient with the limiter's active branch;
// with lamRef, also kAdjLambda's copy of the cell's adjoint seed.
// kVel: compiled with the eigen-frame velocity limiter (RECONST 10), so that
// the other limiters keep their smaller register allocation.
template <typename R, bool kVel>
__global__ void __launch_bounds__(kBlock) kAdjGradFwd(View<R> V, AdjWork<R> W, const double *lamRef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const size_t n = V.nc;
  if (lamRef) {
    const int o = V.refId[i];
#pragma unroll
    for (int k = 0; k < 5; ++k) W.cvd[(size_t)k * n + i] = (R)lamRef[5 * (size_t)o + k];
  }
  const PlainLoad<R> ld{V};
  R q[5], g[15];
  ld.prim5(i, q);
#pragma unroll
  for (int k = 0; k < 15; ++k) g[k] = R(0);
  if constexpr (Layout<R>::packed) {
    // the primal's formulation (one record per member, L applied to the
    // sums), so G is the primal's gradient; with it the sum of the members'
    // d/|d|^2 for the own term of the reverse pass
    float rec[8];
    ld8(V.prim + 8 * (size_t)i, rec);
    float sx0 = 0.f, sy0 = 0.f, sz0 = 0.f;
#pragma unroll 4
    for (int s = V.stOff[i]; s < V.stOff[i + 1]; ++s) {
      float r[8];
      ld8(V.prim + 8 * (size_t)V.stIdx[s], r);
      float dx = r[5] - rec[5], dy = r[6] - rec[6], dz = r[7] - rec[7];
      if (V.stShift) {  // a periodic or symmetry mesh: the member's image
        dx = dx + V.stShift[3 * (size_t)s];
        dy = dy + V.stShift[3 * (size_t)s + 1];
        dz = dz + V.stShift[3 * (size_t)s + 2];
        if (const float *Q = memberReflection(V, s)) {
          const float u[3] = {r[1], r[2], r[3]};
          reflect3(Q, u, r + 1);
        }
      }
      const float inv = 1.f / (dx * dx + dy * dy + dz * dz);
      const float sx = inv * dx, sy = inv * dy, sz = inv * dz;
      sx0 += sx;
      sy0 += sy;
      sz0 += sz;
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const float d = r[k] - q[k];
        g[3 * k] = g[3 * k] + sx * d;
        g[3 * k + 1] = g[3 * k + 1] + sy * d;
        g[3 * k + 2] = g[3 * k + 2] + sz * d;
      }
    }
    const float lxx = V.lsq[i], lxy = V.lsq[n + i], lxz = V.lsq[2 * n + i];
    const float lyy = V.lsq[3 * n + i], lyz = V.lsq[4 * n + i], lzz = V.lsq[5 * n + i];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const float x = g[3 * k], y = g[3 * k + 1], z = g[3 * k + 2];
      g[3 * k] = lxx * x + lxy * y + lxz * z;
      g[3 * k + 1] = lxy * x + lyy * y + lyz * z;
      g[3 * k + 2] = lxz * x + lyz * y + lzz * z;
    }
    W.ssum[i] = sx0;
    W.ssum[n + i] = sy0;
    W.ssum[2 * n + i] = sz0;
    if (V.cSlot) {
      const int sl = V.cSlot[i];
      if (sl >= 0) constrainedGrad(V, ld, i, sl, q, g);
    }
  } else {
    for (int s = V.stOff[i]; s < V.stOff[i + 1]; ++s) {
      const int j = V.stIdx[s];
      R wx, wy, wz;
      lsqWeight(V, i, s, wx, wy, wz);
      R qj[5];
      ld.prim5(j, qj);
      if (const R *Q = memberReflection(V, s)) {
        const R u[3] = {qj[1], qj[2], qj[3]};
        reflect3(Q, u, qj + 1);
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        R d = qj[k] - q[k];
        g[3 * k] = g[3 * k] + wx * d;
        g[3 * k + 1] = g[3 * k + 1] + wy * d;
        g[3 * k + 2] = g[3 * k + 2] + wz * d;
      }
    }
    if (V.cSlot) {
      const int sl = V.cSlot[i];
      if (sl >= 0) constrainedGrad(V, ld, i, sl, q, g);
    }
  }
#pragma unroll
  for (int k = 0; k < 15; ++k) W.G[k * n + i] = g[k];
  const int rc = V.p.reconst;
  R lim[5] = {R(1), R(1), R(1), R(1), R(1)};
  int es[5] = {-1, -1, -1, -1, -1}, js[5] = {-1, -1, -1, -1, -1};
  if (rc == 11 || rc == 100 || rc == 10) {
    R vmin[5], vmax[5];
    int jmin[5], jmax[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) { vmin[k] = vmax[k] = q[k]; jmin[k] = jmax[k] = -1; }
    const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
    for (int e = cb; e < ce; ++e) {
      const int code = V.cfEnt[e];
      int nb;
      R x[5];
      if (code < 0) {
        const double *Q = symmetryQ(V, code);
        if (!Q) continue;
        nb = kMirrorNb - (-code - 1);  // the cell's reflection across this face
        x[0] = q[0];
        reflect3(Q, q + 1, x + 1);
        x[4] = q[4];
      } else {
        int c1, c2;
        faceCells(V, code >> 1, c1, c2);
        nb = (code & 1) ? c1 : c2;
        ld.prim5(nb, x);
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        if (x[k] < vmin[k]) { vmin[k] = x[k]; jmin[k] = nb; }
        if (x[k] > vmax[k]) { vmax[k] = x[k]; jmax[k] = nb; }
      }
    }
    const R epsq = V.epsq[i];
    for (int e = cb; e < ce; ++e) {
      const int code = V.cfEnt[e];
      R d[3];
      if (!limiterFaceOffset(V, code, d)) continue;
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        if (rc == 10 && k >= 1 && k <= 3) continue;  // the eigen-frame limiter below
        const R d2 = -(g[3 * k] * d[0] + g[3 * k + 1] * d[1] + g[3 * k + 2] * d[2]);
        if (!(d2 > R(0)) && !(d2 < R(0))) continue;
        const bool up = d2 > R(0);
        const R dext = up ? vmax[k] - q[k] : vmin[k] - q[k];
        R t;
        bool active;
        if (rc == 11) {
          t = venkat(dext, d2, epsq);
          active = true;
        } else {
          const R x = dext / d2;
          t = fmin2(R(1), x);
          active = x < R(1);
        }
        if (t < lim[k]) {
          lim[k] = t;
          es[k] = active ? e : -1;
          js[k] = up ? jmax[k] : jmin[k];
        }
      }
    }
  }
  R gl[15];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    W.lim[k * n + i] = lim[k];
    W.estar[k * n + i] = es[k];
    W.jstar[k * n + i] = js[k];
#pragma unroll
    for (int c = 0; c < 3; ++c) gl[3 * k + c] = lim[k] * g[3 * k + c];
  }
  if constexpr (kVel) {
    R G[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) G[a + 3 * c] = g[3 * (1 + a) + c];
    VelFrame<R> F;
    velFrameForward(V, ld, i, G, F);
    velFrameApply(F, gl);
  }
  // packed layout with WENO smoothing: the unsmoothed gradient as a record
  // in gradRaw (free outside the primal's gradient phase) for kAdjWenoFwd's
  // member fetches
  if (Layout<R>::packed && isWeno(V.p)) storeGradTo(V, V.gradRaw, i, gl);
  else storeGrad(V, i, gl);
}

// the simple positivity limiter, the factors, the weight sums and the
// smoothed gradient of cell i
template <typename R>
__device__ inline void wenoFwdFinish(const View<R> &V, AdjWork<R> &W, int i, R *g, const R *sum, bool xyz) {
  const size_t n = V.nc;
  R f0, f4;
  wenoPositivity(V, i, g, &f0, &f4);
  W.lim[i] = f0;
  W.lim[4 * n + i] = f4;
#pragma unroll
  for (int k = 0; k < 15; ++k)
    if (xyz || k < 5) W.gradd[k * n + i] = sum[k];
  storeGrad(V, i, g);
}

// Forward pass of the WENO smoothing (RECONST 1, 2) for the reverse pass:
// each cell's smoothed and limited gradient from the unsmoothed ones
// (written by kAdjGradFwd: W.G, and in the packed layout records in
// gradRaw) into the view, the simple limiter's factors of density and
// pressure (0: zeroed) in W.lim, and the weight sums in W.gradd (XYZ: 15 per
// cell; simple form: 5).
template <typename R>
__global__ void __launch_bounds__(kBlock) kAdjWenoFwd(View<R> V, AdjWork<R> W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const size_t n = V.nc;
  auto row = [&](int c, R *t) {
    if constexpr (Layout<R>::packed) {
      ld8(V.gradRaw + 16 * (size_t)c, t);
      ld8(V.gradRaw + 16 * (size_t)c + 8, t + 8);
    } else {
#pragma unroll
      for (int k = 0; k < 15; ++k) t[k] = W.G[k * n + c];
    }
  };
  auto fetch = [&](int s, R *t) {
    row(V.stIdx[s], t);
    if (const R *Q = memberReflection(V, s)) reflectGrad(Q, t);
  };
  const int sb = V.stOff[i], se = V.stOff[i + 1];
  R own[16], g[15], sum[15];
  row(i, own);
  const bool xyz = V.p.reconst == 2;
  if (xyz) wenoXyz(own, sb, se, fetch, g, sum);
  else wenoSimple(own, sb, se, fetch, g, sum);
  wenoFwdFinish(V, W, i, g, sum, xyz);
}
// The packed layout: adjLanes threads per cell, each over every
// adjLanes-th member, the sums joined by shuffles (the averages' terms are
// the ones of wenoXyz / wenoSimple, summed in another order).
template <typename R>
__global__ void __launch_bounds__(kBlock) kAdjWenoFwdLanes(View<R> V, AdjWork<R> W) {
  if constexpr (Layout<R>::packed) {
    constexpr int kL = adjLanes<R>();
    const int th = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = th / kL, h = th % kL;
    const bool live = i < V.nc;
    const R eps = R(1.0e-15);
    R own[16], t[16], g[15], sum[15];
#pragma unroll
    for (int k = 0; k < 16; ++k) own[k] = R(0);
    if (live) {
      ld8(V.gradRaw + 16 * (size_t)i, own);
      ld8(V.gradRaw + 16 * (size_t)i + 8, own + 8);
    }
    const int sb = live ? V.stOff[i] : 0, se = live ? V.stOff[i + 1] : 0;
    auto fetch = [&](int s) {
      const int c = V.stIdx[s];
      ld8(V.gradRaw + 16 * (size_t)c, t);
      ld8(V.gradRaw + 16 * (size_t)c + 8, t + 8);
      if (const R *Q = memberReflection(V, s)) reflectGrad(Q, t);
    };
    auto join = [&](R *x, int m) {
#pragma unroll
      for (int o = 1; o < kL; o <<= 1)
#pragma unroll
        for (int k = 0; k < 15; ++k)
          if (k < m) x[k] += __shfl_xor_sync(0xffffffffu, x[k], o);
    };
    const bool xyz = V.p.reconst == 2;
    if (xyz) {
#pragma unroll
      for (int k = 0; k < 15; ++k) {
        const R w = h == 0 ? R(1) / (own[k] * own[k] + eps) : R(0);
        sum[k] = w;
        g[k] = w * own[k];
      }
      for (int s = sb + h; s < se; s += kL) {
        fetch(s);
#pragma unroll
        for (int k = 0; k < 15; ++k) {
          const R w = R(1) / (t[k] * t[k] + eps);
          sum[k] = sum[k] + w;
          g[k] = g[k] + w * t[k];
        }
      }
      join(sum, 15);
      join(g, 15);
#pragma unroll
      for (int k = 0; k < 15; ++k) g[k] = g[k] / sum[k];
    } else {
      R w0[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const R m = fabs_(own[3 * v]) + fabs_(own[3 * v + 1]) + fabs_(own[3 * v + 2]);
        w0[v] = R(1) / (m * m + eps);
        sum[v] = h == 0 ? w0[v] : R(0);
      }
      for (int s = sb + h; s < se; s += kL) {
        fetch(s);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          const R m = fabs_(t[3 * v]) + fabs_(t[3 * v + 1]) + fabs_(t[3 * v + 2]);
          sum[v] = sum[v] + R(1) / (m * m + eps);
        }
      }
      join(sum, 5);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const R term = h == 0 ? w0[v] / sum[v] : R(0);
#pragma unroll
        for (int d = 0; d < 3; ++d) g[3 * v + d] = term * own[3 * v + d];
      }
      for (int s = sb + h; s < se; s += kL) {
        fetch(s);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          const R m = fabs_(t[3 * v]) + fabs_(t[3 * v + 1]) + fabs_(t[3 * v + 2]);
          const R term = (R(1) / (m * m + eps)) / sum[v];
#pragma unroll
          for (int d = 0; d < 3; ++d) g[3 * v + d] = g[3 * v + d] + term * t[3 * v + d];
        }
      }
      join(g, 15);
    }
    if (!live || h) return;
    wenoFwdFinish(V, W, i, g, sum, xyz);
  }
}

// Transposed flux Jacobian of one face applied to Fbar.
template <int N, typename T>
__device__ inline void contract(const Dual<N, T> *flx, const T *fbar, T *out) {
#pragma unroll
  for (int m = 0; m < N; ++m) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < 5; ++k) s += fbar[k] * flx[k].d[m];
    out[m] = s;
  }
}

// Face adjoints of faces t0 .. t1-1 (interior faces first, then boundary
// faces).  kRoe2 compiles only the second-order Roe interior path (its
// hand-written reverse sweep), so that the common case is not held to the
// register allocation of the dual-number paths; the launcher gives it the
// interior faces of such runs and the generic kernel the rest.
template <typename R, bool kRoe2>
__global__ void __launch_bounds__(kBlock) kAdjFace(View<R> V, AdjWork<R> W, int t0, int t1) {
  const int t = t0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= t1) return;
  const Params &P = V.p;
  const size_t n = V.nc;
  const PlainLoad<R> ld{V};
  R *out = W.faceAdj + 16 * (size_t)t;
  R fbar[5];
  if (t < V.nf) {
    const int f = t;
    int c1, c2;
    faceCells(V, f, c1, c2);
    R nx, ny, nz, nm;
    faceNormal(V, f, nx, ny, nz, nm);
#pragma unroll
    for (int k = 0; k < 5; ++k) fbar[k] = W.cvd[k * n + c1] - W.cvd[k * n + c2];
    if (!kRoe2 && P.spaceOrder == 1) {
      // first order: FP64 from cv and dv in every mode (as the primal)
      using D8 = Dual<8>;
      D8 cl[5], dl[3], cr[5], dr[3], flx[5];
      double fb[5], o8[8];
#pragma unroll
      for (int k = 0; k < 5; ++k) fb[k] = (double)fbar[k];
      for (int side = 0; side < 2; ++side) {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          cl[k] = side ? D8(V.cv[k * n + c1]) : D8::seed(V.cv[k * n + c1], k);
          cr[k] = side ? D8::seed(V.cv[k * n + c2], k) : D8(V.cv[k * n + c2]);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          dl[k] = side ? D8(V.dv[k * n + c1]) : D8::seed(V.dv[k * n + c1], 5 + k);
          dr[k] = side ? D8::seed(V.dv[k * n + c2], 5 + k) : D8(V.dv[k * n + c2]);
        }
        riemann1(P, cl, dl, cr, dr, D8((double)nx), D8((double)ny), D8((double)nz), D8((double)nm), flx);
        contract(flx, fb, o8);
#pragma unroll
        for (int m = 0; m < 8; ++m) out[8 * side + m] = (R)o8[m];
      }
    } else {
      R L[5], Rt[5], irl, irr, dl[3], dr[3];
      faceOffset(V, f, 0, dl);
      faceOffset(V, f, 1, dr);
      faceState(V, ld, c1, dl[0], dl[1], dl[2], L, irl);
      faceState(V, ld, c2, dr[0], dr[1], dr[2], Rt, irr);
      if (kRoe2 || P.spaceDiscr == 1) {
        // Roe: hand-written reverse sweep in the mode's arithmetic (no
        // dependence on the cell 1/rho)
        roe2Adjoint(P.refGamma, P.refCp, P.epsEntr, P.dissFact, nx, ny, nz, nm, L, Rt, fbar, out, out + 6);
        out[5] = R(0);
        out[11] = R(0);
        return;
      }
      using D6 = Dual<6, R>;
      D6 a[5], b[5], ia, ib, flx[5];
      for (int side = 0; side < 2; ++side) {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          a[k] = side ? D6(L[k]) : D6::seed(L[k], k);
          b[k] = side ? D6::seed(Rt[k], k) : D6(Rt[k]);
        }
        ia = side ? D6(irl) : D6::seed(irl, 5);
        ib = side ? D6::seed(irr, 5) : D6(irr);
        if constexpr (!kRoe2) {
          riemann2(P, D6(nx), D6(ny), D6(nz), D6(nm), a, ia, b, ib, flx);
          contract(flx, fbar, out + 6 * side);
        }
      }
    }
  } else if constexpr (!kRoe2) {
    const int b = t - V.nf, c = V.bcell[b], ip = V.bpatch[b];
    const int type = V.patchType[ip], order = V.patchOrder[ip];
#pragma unroll
    for (int k = 0; k < 5; ++k) fbar[k] = W.cvd[k * n + c];
    if (patchLeavesDensity(type)) fbar[0] = R(0);  // walls leave rhs(DENS)
    if (type == kBcSymmetry) {
      // the interior flux against the cell's own reflection (faceFluxEval):
      // both sides follow the cell, so the seeds are on its side only and
      // the reflected side carries them through Q.  First order: (cv, dv)
      // of the cell, 8 values; second order: the face state and the cell's
      // 1/rho, 6 values, as an interior face's first side
      const double *Q = V.patchK + kPatchK * ip;
      if (P.spaceOrder == 1) {
        using D8 = Dual<8>;
        D8 cl[5], dl[3], cr[5], flx[5];
        double fb[5], o8[8];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          cl[k] = D8::seed(V.cv[k * n + c], k);
          fb[k] = (double)fbar[k];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) dl[k] = D8::seed(V.dv[k * n + c], 5 + k);
        cr[0] = cl[0];
        reflect3(Q, cl + 1, cr + 1);
        cr[4] = cl[4];
        riemann1(P, cl, dl, cr, dl, D8((double)V.bnx[b]), D8((double)V.bny[b]), D8((double)V.bnz[b]),
                 D8((double)V.bnm[b]), flx);
        contract(flx, fb, o8);
#pragma unroll
        for (int m = 0; m < 8; ++m) out[m] = (R)o8[m];
      } else {
        using D6 = Dual<6, R>;
        const size_t nb = V.nb;
        R L[5], irl;
        faceState(V, ld, c, V.bd[b], V.bd[nb + b], V.bd[2 * nb + b], L, irl);
        D6 a[5], r[5], ia, flx[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) a[k] = D6::seed(L[k], k);
        ia = D6::seed(irl, 5);
        r[0] = a[0];
        reflect3(Q, a + 1, r + 1);
        r[4] = a[4];
        riemann2(P, D6(V.bnx[b]), D6(V.bny[b]), D6(V.bnz[b]), D6(V.bnm[b]), a, ia, r, ia, flx);
        contract(flx, fbar, out);
      }
      return;
    }
    if (order == 1) {
      using D6 = Dual<6>;
      D6 cv[5], flx[5];
      double fb[5], o6[6];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        cv[k] = D6::seed(V.cv[k * n + c], k);
        fb[k] = (double)fbar[k];
      }
      D6 pl = D6::seed(V.dv[c], 5);
      patch1(P, type, V.patchOutflow[ip], V.patchK + kPatchK * ip, cv, pl, D6((double)V.bnx[b]),
             D6((double)V.bny[b]), D6((double)V.bnz[b]), D6((double)V.bnm[b]), flx);
      contract(flx, fb, o6);
#pragma unroll
      for (int m = 0; m < 6; ++m) out[m] = (R)o6[m];
    } else {
      using D5 = Dual<5, R>;
      const size_t nb = V.nb;
      R L[5], irl;
      faceState(V, ld, c, V.bd[b], V.bd[nb + b], V.bd[2 * nb + b], L, irl);
      D5 a[5], flx[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) a[k] = D5::seed(L[k], k);
      patch2(P, type, V.patchOutflow[ip], V.patchK + kPatchK * ip, a, D5(V.bnx[b]), D5(V.bny[b]), D5(V.bnz[b]),
             D5(V.bnm[b]), flx);
      contract(flx, fbar, out);
    }
  }
}

// Side adjoints -> primitive / gradient adjoints of the cell, limiter reverse,
// gradient own-term.  kVel: with the eigen-frame velocity limiter (RECONST 10).
// FP64 layouts: the own term of the LSQ gradient's transpose (or, for a
// constrained variable, of its rows) on the cell's primitive adjoint.
template <typename R>
__device__ inline void adjOwnTermFp64(const View<R> &V, int i, const R *gb, R *qb) {
  int sl;
  const int cm = constrMask(V, i, sl);
  for (int s = V.stOff[i]; s < V.stOff[i + 1]; ++s) {
    R wx, wy, wz;
    lsqWeight(V, i, s, wx, wy, wz);
#pragma unroll
    for (int k = 0; k < 5; ++k)
      if (!((cm >> k) & 1)) qb[k] -= wx * gb[3 * k] + wy * gb[3 * k + 1] + wz * gb[3 * k + 2];
  }
  if (cm) constrOwnTerm(V, i, sl, gb, qb);
}

// Packed layout: the own term of the LSQ gradient's transpose on the cell's
// primitive adjoint, and the cell's record L_i Gbar_i for the neighbour terms
// (kAdjCell2).  w_s = L_i d_s/|d_s|^2 with L_i symmetric: sum_s w_s . Gbar_k
// = (sum_s d_s/|d_s|^2) . (L_i Gbar_k).
// A constrained variable's record entries are zero (its rows' weights are
// not of that form): its own term is taken here and its neighbour terms by
// kAdjCell2's constrained pass.
template <typename R>
__device__ inline void adjOwnTerm(const View<R> &V, const AdjWork<R> &W, int i, const float *gb, float *qb) {
  const size_t n = V.nc;
  const float lxx = V.lsq[i], lxy = V.lsq[n + i], lxz = V.lsq[2 * n + i];
  const float lyy = V.lsq[3 * n + i], lyz = V.lsq[4 * n + i], lzz = V.lsq[5 * n + i];
  int sl;
  const int cm = constrMask(V, i, sl);
  float h[16];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const float x = gb[3 * k], y = gb[3 * k + 1], z = gb[3 * k + 2];
    const bool con = (cm >> k) & 1;
    h[3 * k] = con ? 0.f : lxx * x + lxy * y + lxz * z;
    h[3 * k + 1] = con ? 0.f : lxy * x + lyy * y + lyz * z;
    h[3 * k + 2] = con ? 0.f : lxz * x + lyz * y + lzz * z;
  }
  if (cm) constrOwnTerm(V, i, sl, gb, qb);
  if (V.p.spaceOrder > 1) {
    const float sx = W.ssum[i], sy = W.ssum[n + i], sz = W.ssum[2 * n + i];
#pragma unroll
    for (int k = 0; k < 5; ++k) qb[k] -= sx * h[3 * k] + sy * h[3 * k + 1] + sz * h[3 * k + 2];
  }
  h[15] = 0.f;
  float *rec = W.adjRec + 16 * (size_t)i;
#pragma unroll
  for (int q = 0; q < 4; ++q) st4(rec + 4 * q, h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
}

template <typename R, bool kVel>
__global__ void __launch_bounds__(kBlock) kAdjCell1(View<R> V, AdjWork<R> W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const Params &P = V.p;
  const size_t n = V.nc, nb = V.nb;
  const PlainLoad<R> ld{V};
  R qb[5] = {0, 0, 0, 0, 0}, gtb[15], cvb[5] = {0, 0, 0, 0, 0}, dvb[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < 15; ++k) gtb[k] = R(0);
  R rbar = R(0);
  const R rho = ld.prim(0, i);
  const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
  for (int e = cb; e < ce; ++e) {
    const int code = V.cfEnt[e];
    if (code >= 0) {
      const int f = code >> 1, side = code & 1;
      const R *a = W.faceAdj + 16 * (size_t)f;
      if (P.spaceOrder == 1) {
        a += 8 * side;
#pragma unroll
        for (int k = 0; k < 5; ++k) cvb[k] += a[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) dvb[k] += a[5 + k];
      } else {
        a += 6 * side;
        R d[3];
        faceOffset(V, f, side, d);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          qb[k] += a[k];
          gtb[3 * k] += a[k] * d[0];
          gtb[3 * k + 1] += a[k] * d[1];
          gtb[3 * k + 2] += a[k] * d[2];
        }
        rbar += a[5];
      }
    } else {
      const int b = -code - 1;
      const R *a = W.faceAdj + 16 * (size_t)(V.nf + b);
      if (symmetryQ(V, code)) {
        // an interior face to the cell's reflection, at the interior order:
        // first order (cv, dv) adjoints, second order the face state's and
        // the cell 1/rho's (kAdjFace)
        if (P.spaceOrder == 1) {
#pragma unroll
          for (int k = 0; k < 5; ++k) cvb[k] += a[k];
#pragma unroll
          for (int k = 0; k < 3; ++k) dvb[k] += a[5 + k];
        } else {
          const R dx = V.bd[b], dy = V.bd[nb + b], dz = V.bd[2 * nb + b];
#pragma unroll
          for (int k = 0; k < 5; ++k) {
            qb[k] += a[k];
            gtb[3 * k] += a[k] * dx;
            gtb[3 * k + 1] += a[k] * dy;
            gtb[3 * k + 2] += a[k] * dz;
          }
          rbar += a[5];
        }
      } else if (V.patchOrder[V.bpatch[b]] == 1) {
#pragma unroll
        for (int k = 0; k < 5; ++k) cvb[k] += a[k];
        dvb[0] += a[5];
      } else {
        const R dx = V.bd[b], dy = V.bd[nb + b], dz = V.bd[2 * nb + b];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          qb[k] += a[k];
          gtb[3 * k] += a[k] * dx;
          gtb[3 * k + 1] += a[k] * dy;
          gtb[3 * k + 2] += a[k] * dz;
        }
      }
    }
  }
  // irl = 1/rho of the cell (HLLC: Hl = el + irl*pl)
  qb[0] += rbar * (R(-1) / (rho * rho));
  R gb[15], nbb[5] = {0, 0, 0, 0, 0};
  int nbt[5] = {-1, -1, -1, -1, -1};  // the neighbour receiving nbb[k]
#pragma unroll
  for (int k = 0; k < 15; ++k) gb[k] = R(0);
  const int rc = P.reconst;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    if (P.spaceOrder < 2) break;
    if (rc == 10 && k >= 1 && k <= 3) continue;  // the eigen-frame limiter below
    const R l = W.lim[k * n + i];
    R lb = R(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      gb[3 * k + c] = l * gtb[3 * k + c];
      lb += gtb[3 * k + c] * W.G[(3 * k + c) * n + i];
    }
    const int es = W.estar[k * n + i];
    if ((rc == 11 || rc == 100 || rc == 10) && es >= 0) {
      const int code = V.cfEnt[es];
      R dxyz[3];
      limiterFaceOffset(V, code, dxyz);
      R g3[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) g3[c] = W.G[(3 * k + c) * n + i];
      const R d2 = -(g3[0] * dxyz[0] + g3[1] * dxyz[1] + g3[2] * dxyz[2]);
      const int js = W.jstar[k * n + i];
      const R qi = ld.prim(k, i);
      // the extreme: a neighbour's value, none (the cell's own), or the
      // cell's reflection across a symmetry face (velocity: (Q u)_k)
      const double *Qm = (js <= kMirrorNb) ? V.patchK + kPatchK * V.bpatch[kMirrorNb - js] : nullptr;
      R qm = qi;
      if (Qm && k >= 1 && k <= 3) {
        R u[3], um[3];
        u[0] = ld.prim(1, i); u[1] = ld.prim(2, i); u[2] = ld.prim(3, i);
        reflect3(Qm, u, um);
        qm = um[k - 1];
      }
      const R dext = (js >= 0 ? ld.prim(k, js) : qm) - qi;
      R db, d2b;
      if (rc == 11) {
        using D2 = Dual<2, R>;
        D2 phi = venkat(D2::seed(dext, 0), D2::seed(d2, 1), D2(V.epsq[i]));
        db = lb * phi.d[0];
        d2b = lb * phi.d[1];
      } else {
        // lim = dext/d2: d lim/d dext = 1/d2, d lim/d d2 = -(dext/d2)/d2, taken
        // as (lb/d2) and -(lb/d2)*(dext/d2) so that a tiny d2 (differences of
        // ~1e-200 ahead of a wave) neither squares into 0 nor makes 0/0 at a
        // local extreme (dext = 0)
        const R r = lb / d2;
        db = r;
        d2b = -r * (dext / d2);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) gb[3 * k + c] += d2b * (-dxyz[c]);
      if (js >= 0) {
        qb[k] -= db;
        nbb[k] = db;
        nbt[k] = js;
      } else if (Qm && k >= 1 && k <= 3) {
        // d((Q u)_k - u_k)/du = Q(k, :) - e_k
        qb[k] -= db;
#pragma unroll
        for (int a = 0; a < 3; ++a) qb[1 + a] += db * R(Qm[3 * (k - 1) + a]);
      }
    }
  }
  // the eigen-frame velocity limiter in reverse; the neighbours' shares go
  // out per axis (velocity vectors), gathered by kAdjCell2
  R nbv[9];
  int nbAx[3] = {-1, -1, -1};
#pragma unroll
  for (int k = 0; k < 9; ++k) nbv[k] = R(0);
  if (kVel && P.spaceOrder > 1) {
    R G[9], glb[9], Gb[9], ub[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        G[a + 3 * c] = W.G[(3 * (1 + a) + c) * n + i];
        glb[a + 3 * c] = gtb[3 * (1 + a) + c];
      }
    VelFrame<R> F;
    velFrameForward(V, ld, i, G, F);
    velFrameReverse(V, ld, i, G, F, glb, Gb, ub, nbv);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      qb[1 + a] += ub[a];
#pragma unroll
      for (int c = 0; c < 3; ++c) gb[3 * (1 + a) + c] = Gb[a + 3 * c];
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (F.side[j] != 0 && !F.held[j] && F.nb[j] >= 0) nbAx[j] = F.nb[j];
  }
  const bool weno = isWeno(P);
  if (weno) {
    // WENO smoothing: gb is the adjoint of the smoothed gradient; its terms
    // over the weight sums go to kAdjWeno, which gathers them over the cells
    // whose averages hold a cell and applies the gradient's own term there
    // (packed layout: as a record in gradRaw, whose unsmoothed gradients
    // kAdjWenoFwd has consumed)
    R sw[15], a[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) sw[k] = W.gradd[(rc == 2 ? k : k / 3) * n + i];
#pragma unroll
    for (int k = 0; k < 15; ++k) a[k] = gb[k] / sw[k];
    if constexpr (Layout<R>::packed) storeGradTo(V, V.gradRaw, i, a);
    else storeGradTo(V, W.gradd, i, a);
  }
  // gradient own-term: G_i = sum_s w_s (q_{m_s} - q_i)
  if constexpr (!Layout<R>::packed) {
    if (P.spaceOrder > 1 && !weno) adjOwnTermFp64(V, i, gb, qb);
  }
  // the raw gradient's adjoint: the FP64 layouts' neighbour terms read it,
  // the packed layout's only for constrained cells (its records carry L Gbar)
  if (!weno && (!Layout<R>::packed || V.cSlot)) {
#pragma unroll
    for (int k = 0; k < 15; ++k) W.Gbar[k * n + i] = gb[k];
  }
  if constexpr (Layout<R>::packed) {
    if (!weno) adjOwnTerm(V, W, i, gb, qb);
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    W.qbar[k * n + i] = qb[k];
    W.cvbarD[k * n + i] = cvb[k];
  }
  if constexpr (Layout<R>::packed) {
    // 20-word record: the variables' receiving neighbours (the eigen-frame
    // limiter's axes in slots 1-3), their values, the axes' vectors
    float *nr = W.nbRec + 20 * (size_t)i;
    if (kVel) {
#pragma unroll
      for (int j = 0; j < 3; ++j) nbt[1 + j] = nbAx[j];
    }
    st4(nr, __int_as_float(nbt[0]), __int_as_float(nbt[1]), __int_as_float(nbt[2]), __int_as_float(nbt[3]));
    st4(nr + 4, __int_as_float(nbt[4]), nbb[0], nbb[1], nbb[2]);
    st4(nr + 8, nbb[3], nbb[4], nbv[0], nbv[1]);
    if (kVel) {  // the axes' vectors: read by kAdjCell2 for RECONST 10 only
      st4(nr + 12, nbv[2], nbv[3], nbv[4], nbv[5]);
      st4(nr + 16, nbv[6], nbv[7], nbv[8], 0.f);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 5; ++k) W.nbBar[k * n + i] = nbb[k];
    if (kVel) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        W.jstar[(1 + j) * n + i] = nbAx[j];
#pragma unroll
        for (int a = 0; a < 3; ++a) W.nbVel[(3 * j + a) * n + i] = nbv[3 * j + a];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) W.dvbar[k * n + i] = dvb[k];
}

// Reverse of the WENO smoothing (RECONST 1, 2) for cell m, after kAdjCell1:
// the cell's unsmoothed gradient t enters its own average and those of the
// cells whose stencils hold it (the transposed stencil).  With a_i cell i's
// smoothed-gradient adjoint over its weight sums (kAdjCell1, in W.gradd;
// packed layout: records in gradRaw) and
// g_i its smoothed gradient, summed over those cells i (m first):
//   XYZ, per component, w = 1/(t^2 + eps), w' = -2 t w^2:
//     tbar = (w + w' t) sum a_i - w' sum a_i g_i;
//   simple form, per variable, W = 1/(T^2 + eps), T = |tx| + |ty| + |tz|,
//   W' = -2 T W^2:
//     tbar_d = W sum a_i,d + W' (t . sum a_i - sum a_i . g_i) sgn(t_d)
//   (sgn(0) = +1, as the tangent's |.|).
// A gradient the simple limiter zeroed has a_i = 0 there, so the view's
// limited gradient serves as g_i.  Then the LSQ gradient's own term on the
// cell's primitive adjoint, and tbar for kAdjCell2's neighbour terms.
template <typename R>
__global__ void __launch_bounds__(kBlock) kAdjWeno(View<R> V, AdjWork<R> W) {
  constexpr int kL = adjLanes<R>();  // lanes per cell for the gather
  const int th = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = th / kL, h = th % kL;
  if (kL == 1 && m >= V.nc) return;
  const bool live = m < V.nc;
  const size_t n = V.nc;
  const PlainLoad<R> ld{V};
  R A[15], B[15], A2[15], B2[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) A[k] = B[k] = R(0);
  // the a-terms and a g of cell i into (Ac, Bc)
  auto addTo = [&](int i, R *Ac, R *Bc) {
    if constexpr (Layout<R>::packed) {
      float a[16], g[16];
      ld8(V.gradRaw + 16 * (size_t)i, a);
      ld8(V.gradRaw + 16 * (size_t)i + 8, a + 8);
      ld8(V.grad + 16 * (size_t)i, g);
      ld8(V.grad + 16 * (size_t)i + 8, g + 8);
#pragma unroll
      for (int k = 0; k < 15; ++k) {
        Ac[k] += a[k];
        Bc[k] += a[k] * g[k];
      }
    } else {
#pragma unroll
      for (int k = 0; k < 15; ++k) {
        const R a = W.gradd[k * n + i];
        Ac[k] += a;
        Bc[k] += a * ld.grad(k, i);
      }
    }
  };
  auto add2 = [&](int i) { addTo(i, A2, B2); };
  auto add = [&](int i) { addTo(i, A, B); };

  R t[15], tb[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) t[k] = live ? W.G[k * n + m] : R(0);
  const R eps = R(1.0e-15);
  const bool xyz = V.p.reconst == 2;
  // the adjoint of a member gradient tt from (sums of) the averages' terms
  // a and a g that hold it: linear in (a, a g) for a fixed tt
  auto reverse = [&](const R *tt, const R *a, const R *ag, R *out) {
    if (xyz) {
#pragma unroll
      for (int k = 0; k < 15; ++k) {
        const R w = R(1) / (tt[k] * tt[k] + eps);
        const R wp = R(-2) * tt[k] * w * w;
        out[k] = (w + wp * tt[k]) * a[k] - wp * ag[k];
      }
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const R *tv = tt + 3 * v, *av = a + 3 * v, *bv = ag + 3 * v;
        const R T = fabs_(tv[0]) + fabs_(tv[1]) + fabs_(tv[2]);
        const R w = R(1) / (T * T + eps);
        const R c = R(-2) * T * w * w * (tv[0] * av[0] + tv[1] * av[1] + tv[2] * av[2] - (bv[0] + bv[1] + bv[2]));
#pragma unroll
        for (int d = 0; d < 3; ++d) out[3 * v + d] = w * av[d] + (tv[d] < R(0) ? -c : c);
      }
    }
  };
  // symmetry meshes: a cell whose average holds m reflected sees Q(t); its
  // share is evaluated there and goes back through the (symmetric) transform
  R tr[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) tr[k] = R(0);
  if (live && h == 0) add(m);
  for (int e = live ? V.tsOff[m] + h : 0, ee = live ? V.tsOff[m + 1] : 0; e < ee; e += kL) {
    const R *Q = memberReflection(V, V.tsEnt[e]);
    if (!Q) {
      add(V.tsCell[e]);
      continue;
    }
#pragma unroll
    for (int k = 0; k < 15; ++k) A2[k] = B2[k] = R(0);
    add2(V.tsCell[e]);
    R tq[16], c[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) tq[k] = t[k];
    reflectGrad(Q, tq);
    reverse(tq, A2, B2, c);
    reflectGrad(Q, c);
#pragma unroll
    for (int k = 0; k < 15; ++k) tr[k] += c[k];
  }
  if constexpr (kL > 1) {
#pragma unroll
    for (int k = 0; k < 15; ++k)
#pragma unroll
      for (int o = 1; o < kL; o <<= 1) {
        A[k] += __shfl_xor_sync(0xffffffffu, A[k], o);
        B[k] += __shfl_xor_sync(0xffffffffu, B[k], o);
        tr[k] += __shfl_xor_sync(0xffffffffu, tr[k], o);
      }
    if (!live || h) return;
  }
  reverse(t, A, B, tb);
#pragma unroll
  for (int k = 0; k < 15; ++k) tb[k] += tr[k];
  R qb[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) qb[k] = W.qbar[k * n + m];
  if constexpr (Layout<R>::packed) {
    adjOwnTerm(V, W, m, tb, qb);
  } else {
    adjOwnTermFp64(V, m, tb, qb);
  }
  // the raw gradient's adjoint (the FP64 layouts' neighbour terms, and the
  // constrained cells' in every layout)
  if (!Layout<R>::packed || V.cSlot) {
#pragma unroll
    for (int k = 0; k < 15; ++k) W.Gbar[k * n + m] = tb[k];
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) W.qbar[k * n + m] = qb[k];
}

// Neighbour terms, then (prim, dv) -> cv; output in reference order.
template <typename R>
__global__ void __launch_bounds__(kBlock) kAdjCell2(View<R> V, AdjWork<R> W, double *outRef) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= V.nc) return;
  const size_t n = V.nc;
  R qb[5], pcon = R(0);
#pragma unroll
  for (int k = 0; k < 5; ++k) qb[k] = W.qbar[k * n + j];
  if (V.tsOff && V.p.spaceOrder > 1) {
    if constexpr (Layout<R>::packed) {
#pragma unroll 2
      for (int k = 0; k < V.tsWidth; ++k) {
        const float4 w = ld4(V.tsW + 4 * (k * n + j));
        const int tag = __float_as_int(w.w);
        if (tag < 0) break;
        const int i = tag & ~kTsReflected;
        float h[16];
        const float *rec = W.adjRec + 16 * (size_t)i;
        ld8(rec, h);
        ld8(rec + 8, h + 8);
        float cb[5];
#pragma unroll
        for (int c = 0; c < 5; ++c) cb[c] = w.x * h[3 * c] + w.y * h[3 * c + 1] + w.z * h[3 * c + 2];
        if (tag & kTsReflected) {
          // j entered i's gradient reflected: its velocity's share goes back
          // through Q (symmetric)
          const float *Q = memberReflection(V, V.tsEnt[V.tsOff[j] + k]);
          float u[3];
          reflect3(Q, cb + 1, u);
          cb[1] = u[0]; cb[2] = u[1]; cb[3] = u[2];
        }
#pragma unroll
        for (int c = 0; c < 5; ++c) qb[c] += cb[c];
      }
    } else {
      for (int e = V.tsOff[j]; e < V.tsOff[j + 1]; ++e) {
        const int i = V.tsCell[e], s = V.tsEnt[e];
        R wx, wy, wz;
        lsqWeight(V, i, s, wx, wy, wz);
        int sl;
        const int cm = V.cSlot ? constrMask(V, i, sl) : 0;
        R cb[5];
#pragma unroll
        for (int k = 0; k < 5; ++k)
          cb[k] = ((cm >> k) & 1) ? R(0)
                                  : wx * W.Gbar[(3 * k) * n + i] + wy * W.Gbar[(3 * k + 1) * n + i] +
                                        wz * W.Gbar[(3 * k + 2) * n + i];
        if (const R *Q = memberReflection(V, s)) {  // j entered i's gradient reflected
          R u[3];
          reflect3(Q, cb + 1, u);
          cb[1] = u[0]; cb[2] = u[1]; cb[3] = u[2];
        }
#pragma unroll
        for (int k = 0; k < 5; ++k) qb[k] += cb[k];
      }
    }
    // constrained cells holding j: their constrained variables' rows
    if (V.cSlot) {
      for (int e = V.tsOff[j]; e < V.tsOff[j + 1]; ++e) {
        const int i = V.tsCell[e];
        int sl;
        const int cm = constrMask(V, i, sl);
        if (!cm) continue;
        const int nst = V.stOff[i + 1] - V.stOff[i], so = V.tsEnt[e] - V.stOff[i];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          if (!((cm >> k) & 1)) continue;
          const int r = constrRow0(V, sl, k, nst) + so;
          qb[k] += V.cW[3 * (size_t)r] * W.Gbar[(3 * k) * n + i] + V.cW[3 * (size_t)r + 1] * W.Gbar[(3 * k + 1) * n + i] +
                   V.cW[3 * (size_t)r + 2] * W.Gbar[(3 * k + 2) * n + i];
        }
      }
    }
    // burning injection faces of j: their constraint rows' values follow j's
    // pressure (constrValue: rho = p/(rgas T_inj), v = -(minj/rho) n), and
    // their share reaches j as an adjoint of its pressure
    if (V.cpOff) {
      const double rgas = 8314.3 / V.p.gvMol;
      const double p = V.dv[j];
      for (int e = V.cpOff[j]; e < V.cpOff[j + 1]; ++e) {
        const int i = V.cpEnt[2 * e], rk = V.cpEnt[2 * e + 1];
        const int r = rk >> 3, k = rk & 7, b = V.cRowFace[r];
        const double *K = V.patchK + kPatchK * V.bpatch[b];
        const double rt = rgas * K[1];
        double dval = 1.0 / rt;  // d rho / dp
        if (k > 0) {
          const double rl = p / rt, nk = (k == 1) ? V.bnx[b] : (k == 2) ? V.bny[b] : V.bnz[b];
          dval = K[0] * nk / (rl * rl) * dval;
        }
        const R dot = V.cW[3 * (size_t)r] * W.Gbar[(3 * k) * n + i] + V.cW[3 * (size_t)r + 1] * W.Gbar[(3 * k + 1) * n + i] +
                      V.cW[3 * (size_t)r + 2] * W.Gbar[(3 * k + 2) * n + i];
        pcon += dot * (R)dval;
      }
    }
  }
  const int cb = V.cfOff[j], ce = (V.p.spaceOrder > 1) ? V.cfOff[j + 1] : cb;
  for (int e = cb; e < ce; ++e) {
    const int code = V.cfEnt[e];
    if (code < 0) continue;
    int c1, c2;
    faceCells(V, code >> 1, c1, c2);
    const int i = (code & 1) ? c1 : c2;
    if constexpr (Layout<R>::packed) {
      const float *nr = W.nbRec + 20 * (size_t)i;
      const float4 a = ld4(nr), b = ld4(nr + 4), c = ld4(nr + 8);
      const int t[5] = {__float_as_int(a.x), __float_as_int(a.y), __float_as_int(a.z), __float_as_int(a.w),
                        __float_as_int(b.x)};
      if (V.p.reconst == 10) {
        if (t[0] == j) qb[0] += b.y;
        if (t[4] == j) qb[4] += c.y;
        if (t[1] == j || t[2] == j || t[3] == j) {
          const float4 d = ld4(nr + 12), e = ld4(nr + 16);
          const float vv[9] = {c.z, c.w, d.x, d.y, d.z, d.w, e.x, e.y, e.z};
#pragma unroll
          for (int ax = 0; ax < 3; ++ax)
            if (t[1 + ax] == j) {
              qb[1] += vv[3 * ax];
              qb[2] += vv[3 * ax + 1];
              qb[3] += vv[3 * ax + 2];
            }
        }
      } else {
        const float v[5] = {b.y, b.z, b.w, c.x, c.y};
#pragma unroll
        for (int k = 0; k < 5; ++k)
          if (t[k] == j) qb[k] += v[k];
      }
    } else {
      const bool velo = V.p.reconst == 10;
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        if (velo && k >= 1 && k <= 3) continue;
        if (W.jstar[k * n + i] == j && W.estar[k * n + i] >= 0) qb[k] += W.nbBar[k * n + i];
      }
      if (velo) {
#pragma unroll
        for (int ax = 0; ax < 3; ++ax)
          if (W.jstar[(1 + ax) * n + i] == j) {
#pragma unroll
            for (int a = 0; a < 3; ++a) qb[1 + a] += W.nbVel[(3 * ax + a) * n + i];
          }
      }
    }
  }
  const int o = V.refId[j];
  if constexpr (Layout<R>::packed) {
    // (prim, dv) -> cv in FP32 from the primitive record: the Jacobian has no
    // cancellation (dp/dcv = (g-1)(|u|^2/2, -u, -v, -w, 1)); only the
    // primal's recovery of p itself needs FP64
    const float *rec = V.prim + 8 * (size_t)j;
    const float r = rec[0], u = rec[1], v = rec[2], w = rec[3], pr = rec[4];
    const float g = V.p.refGammaF, gc = (float)V.p.gcR;
    const float ir = 1.f / r;
    const float dp[5] = {(g - 1.f) * 0.5f * (u * u + v * v + w * w), -(g - 1.f) * u, -(g - 1.f) * v, -(g - 1.f) * w,
                         g - 1.f};
    float out[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) out[m] = W.cvbarD[m * n + j] + qb[4] * dp[m];
    out[0] += qb[0] - ir * (qb[1] * u + qb[2] * v + qb[3] * w);
    out[1] += ir * qb[1];
    out[2] += ir * qb[2];
    out[3] += ir * qb[3];
    // dv = (p, T, c): T = p/(r gc), c = sqrt(g gc T)
    const float b0 = W.dvbar[j] + pcon, b1 = W.dvbar[n + j], b2 = W.dvbar[2 * n + j];
    if (b0 != 0.f || b1 != 0.f || b2 != 0.f) {
      const float t = pr * ir / gc, c = sqrtf(g * gc * t);
      const float tb = b1 + b2 * 0.5f * g * gc / c;  // adjoint of T
      const float pb = b0 + tb * ir / gc;            // of p through T
#pragma unroll
      for (int m = 0; m < 5; ++m) out[m] += pb * dp[m];
      out[0] += -tb * t * ir;                        // dT/drho at fixed p
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) outRef[5 * (size_t)o + m] = (double)out[m];
  } else {
    using D5 = Dual<5>;
    D5 cv[5], q[5], dv[3];
#pragma unroll
    for (int k = 0; k < 5; ++k) cv[k] = D5::seed(V.cv[k * n + j], k);
    primFromCv(V.p, cv, q, dv);
    double dvb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dvb[k] = W.dvbar[k * n + j];
    dvb[0] += pcon;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      double s = W.cvbarD[m * n + j];
#pragma unroll
      for (int k = 0; k < 5; ++k) s += (double)qb[k] * q[k].d[m];
#pragma unroll
      for (int k = 0; k < 3; ++k) s += dvb[k] * dv[k].d[m];
      outRef[5 * (size_t)o + m] = s;
    }
  }
}

// The limiter's active branches of every cell after kAdjGradFwd, in the
// reference's cell order: per variable k, out[10 o + 2k] = the active face as
// the index of the cell's face entry (-1: the factor is 1, not limited), and
// out[10 o + 2k + 1] = the reference id of the neighbour whose value is the
// active extreme (-1: none or the cell itself).  The eigen-frame limiter
// (RECONST 10) reports its axes in k = 1..3, the face index times 4 plus the
// side (1: the largest increment, 2: the smallest).  The WENO smoothing
// (RECONST 1, 2) reports -2 as the face of density and pressure where its
// simple limiter zeroed the gradient.  A residual whose every cell keeps
// these branches is a smooth function of the state.
template <typename R>
__global__ void kLimiterBranches(View<R> V, AdjWork<R> W, int *outRef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const size_t n = V.nc;
  int *out = outRef + 10 * (size_t)V.refId[i];
  const int cb = V.cfOff[i];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int es = W.estar[k * n + i], js = W.jstar[k * n + i];
    out[2 * k] = es >= 0 ? es - cb : -1;
    out[2 * k + 1] = (es >= 0 && js >= 0) ? V.refId[js] : -1;
  }
  if (isWeno(V.p)) {
    // the simple limiter after the WENO smoothing: -2 where it zeroed the
    // density (k = 0) or the pressure (k = 4) gradient
    if (W.lim[i] == R(0)) out[0] = -2;
    if (W.lim[4 * n + i] == R(0)) out[8] = -2;
  }
  if (V.p.reconst == 10 && V.p.spaceOrder > 1) {
    const PlainLoad<R> ld{V};
    R G[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) G[a + 3 * c] = W.G[(3 * (1 + a) + c) * n + i];
    VelFrame<R> F;
    velFrameForward(V, ld, i, G, F);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      out[2 * (1 + j)] = F.side[j] ? 4 * (F.face[j] - cb) + F.side[j] : -1;
      out[2 * (1 + j) + 1] = (F.side[j] && F.nb[j] >= 0) ? V.refId[F.nb[j]] : -1;
    }
  }
}

// Boundary-pressure functional: per-face p_f |A_f| on patch ip and the seed
// of the face adjoint (dJ/dp_f = |A_f|); the sum is a fixed-order block
// reduction.
template <typename R>
__global__ void kPatchSeed(View<R> V, AdjWork<R> W, int ip, double *Jout) {
  __shared__ double part[kBlock];
  const size_t nb = V.nb;
  const PlainLoad<R> ld{V};
  double acc = 0.0;
  for (int b = threadIdx.x; b < V.nb; b += blockDim.x) {
    if (V.bpatch[b] != ip) continue;
    const int c = V.bcell[b];
    const R nm = V.bnm[b];
    R *a = W.faceAdj + 16 * (size_t)(V.nf + b);
    double pf;
    if (V.patchOrder[ip] == 1) {
      pf = V.dv[c];
      a[5] = nm;
    } else {
      R L[5], irl;
      faceState(V, ld, c, V.bd[b], V.bd[nb + b], V.bd[2 * nb + b], L, irl);
      pf = (double)L[4];
      a[4] = nm;
    }
    acc += pf * (double)nm;
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *Jout = part[0];
}

// A second stream of the adjoint's launches, with the events that fork it
// from and join it to the calling stream (created once per process).
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
inline SideStream &sideStream() {
  static SideStream ss = [] {
    SideStream x;
    cudaStreamCreateWithFlags(&x.stream, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&x.fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&x.join, cudaEventDisableTiming);
    return x;
  }();
  return ss;
}

template <typename R>
struct AdjointOps {
  static void jvp(const View<R> &V, const double *cvDotRef, double *rhsDotRef, double *work, cudaStream_t s) {
    const size_t nT = (size_t)V.nf + V.nb;
    AdjWork<R> W = carveAdjWork<R>(work, V.nc, nT);
    kTanInit<R><<<blocks(V.nc), kBlock, 0, s>>>(V, W, cvDotRef);
    if (V.p.spaceOrder > 1) kTanGrad<R><<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    if (isWeno(V.p)) kTanWeno<R><<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    kTanFlux<R><<<blocks((long long)nT), kBlock, 0, s>>>(V, W);
    kTanGather<R><<<blocks(V.nc), kBlock, 0, s>>>(V, W, rhsDotRef);
  }
  static void gradFwd(const View<R> &V, const AdjWork<R> &W, const double *lamRef, cudaStream_t s) {
    if (V.p.reconst == 10) kAdjGradFwd<R, true><<<blocks(V.nc), kBlock, 0, s>>>(V, W, lamRef);
    else kAdjGradFwd<R, false><<<blocks(V.nc), kBlock, 0, s>>>(V, W, lamRef);
    if (isWeno(V.p)) {
      if constexpr (Layout<R>::packed)
        kAdjWenoFwdLanes<R><<<blocks((long long)V.nc * adjLanes<R>()), kBlock, 0, s>>>(V, W);
      else
        kAdjWenoFwd<R><<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    }
  }
  static void cellAdjoint(const View<R> &V, AdjWork<R> &W, double *cvBarRef, cudaStream_t s) {
    if (V.p.reconst == 10 && V.p.spaceOrder > 1) kAdjCell1<R, true><<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    else kAdjCell1<R, false><<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    if (isWeno(V.p)) kAdjWeno<R><<<blocks((long long)V.nc * adjLanes<R>()), kBlock, 0, s>>>(V, W);
    kAdjCell2<R><<<blocks(V.nc), kBlock, 0, s>>>(V, W, cvBarRef);
  }
  // The boundary faces' kernel (dual numbers through the patch fluxes; few
  // faces, a small grid) runs on a second stream beside the interior faces'
  // (they write disjoint face-adjoint entries), forked from and joined
  // back to s by events, so that it fills the SMs the interior kernel's
  // last wave leaves idle.
  static void faceAdjoint(const View<R> &V, const AdjWork<R> &W, cudaStream_t s) {
    const int nT = V.nf + V.nb;
    const bool roe2 = V.p.spaceOrder > 1 && V.p.spaceDiscr == 1;
    if (V.nf == 0 || V.nb == 0) {
      if (nT > 0 && !(roe2 && V.nb == 0)) kAdjFace<R, false><<<blocks((long long)nT), kBlock, 0, s>>>(V, W, 0, nT);
      else if (nT > 0) kAdjFace<R, true><<<blocks((long long)nT), kBlock, 0, s>>>(V, W, 0, nT);
      return;
    }
    SideStream &ss = sideStream();
    cudaEventRecord(ss.fork, s);
    cudaStreamWaitEvent(ss.stream, ss.fork, 0);
    kAdjFace<R, false><<<blocks((long long)V.nb), kBlock, 0, ss.stream>>>(V, W, V.nf, nT);
    cudaEventRecord(ss.join, ss.stream);
    if (roe2) kAdjFace<R, true><<<blocks((long long)V.nf), kBlock, 0, s>>>(V, W, 0, V.nf);
    else kAdjFace<R, false><<<blocks((long long)V.nf), kBlock, 0, s>>>(V, W, 0, V.nf);
    cudaStreamWaitEvent(s, ss.join, 0);
  }
  static void vjp(const View<R> &V, const double *rhsBarRef, double *cvBarRef, double *work, cudaStream_t s) {
    const size_t nT = (size_t)V.nf + V.nb;
    AdjWork<R> W = carveAdjWork<R>(work, V.nc, nT);
    // every face-adjoint entry the cell kernels read is written by the face
    // kernels: no clearing of faceAdj here
    if (V.p.spaceOrder > 1) gradFwd(V, W, rhsBarRef, s);
    else kAdjLambda<R><<<blocks(V.nc), kBlock, 0, s>>>(V, W, rhsBarRef);
    (void)nT;
    faceAdjoint(V, W, s);
    cellAdjoint(V, W, cvBarRef, s);
  }
  static void limiterBranches(const View<R> &V, int *outRef, double *work, cudaStream_t s) {
    const size_t nT = (size_t)V.nf + V.nb;
    AdjWork<R> W = carveAdjWork<R>(work, V.nc, nT);
    gradFwd(V, W, nullptr, s);
    kLimiterBranches<R><<<blocks(V.nc), kBlock, 0, s>>>(V, W, outRef);
  }
  static void patchPressure(const View<R> &V, int ip, double *J, double *cvBarRef, double *work, cudaStream_t s) {
    const size_t nT = (size_t)V.nf + V.nb;
    AdjWork<R> W = carveAdjWork<R>(work, V.nc, nT);
    if (V.p.spaceOrder > 1) gradFwd(V, W, nullptr, s);
    cudaMemsetAsync(W.faceAdj, 0, sizeof(R) * 16 * nT, s);
    kPatchSeed<R><<<1, kBlock, 0, s>>>(V, W, ip, J);
    if (cvBarRef) cellAdjoint(V, W, cvBarRef, s);
  }
};

}  // namespace RFLU_NS
}  // namespace rflu
