// Tangent (JVP) and discrete adjoint (VJP) of the residual of one region,
// R(cv) = CellGradientsMP + ConvectiveFluxesMP, in the FP64 modes.
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
//      reconstructed left/right states), stored per face side;
//   3. cell adjoint (one thread per cell, gather over the same CSR): side
//      adjoints -> primitive and limited-gradient adjoints; limiter reverse
//      through its active branch; own-term of the gradient transpose;
//   4. cell adjoint (gather over the transposed stencil and the face
//      neighbours): neighbour terms of the gradient and limiter transposes,
//      then prim/dv -> cv through the local Jacobian (Dual<5>).
// No atomics: every sum is a gather in a fixed order.  The adjoint covers
// RECONST 0, 11 (Venkatakrishnan) and 100 (componentwise BJ); the
// eigen-frame velocity limiter of RECONST 10 is covered by the tangent only.
#pragma once
#include "dual.cuh"
#include "roe_adjoint.cuh"

namespace rflu {
namespace RFLU_NS {

#ifdef RFLU_WITH_ADJOINT
struct AdjWork {
  double *cvd, *primd, *dvd, *gradd, *fluxd;          // tangent state / lambda in cvd
  double *G, *lim, *faceAdj, *Gbar, *qbar, *nbBar, *cvbarD, *dvbar;
  int *estar, *jstar;
};

inline size_t adjWorkDoubles(size_t nc, size_t nT) { return 96 * nc + 24 * nT + 64; }

inline AdjWork carveAdjWork(double *w, size_t nc, size_t nT) {
  AdjWork a;
  a.cvd = w; w += 5 * nc;
  a.primd = w; w += 5 * nc;
  a.dvd = w; w += 3 * nc;
  a.gradd = w; w += 15 * nc;
  a.fluxd = w; w += 5 * nT;
  a.G = w; w += 15 * nc;
  a.lim = w; w += 5 * nc;
  a.faceAdj = w; w += 16 * nT;
  a.Gbar = w; w += 15 * nc;
  a.qbar = w; w += 5 * nc;
  a.nbBar = w; w += 5 * nc;
  a.cvbarD = w; w += 5 * nc;
  a.dvbar = w; w += 3 * nc;
  a.estar = (int *)w; w += 3 * nc;  // 5 ints per cell
  a.jstar = (int *)w; w += 3 * nc;
  return a;
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

using D1 = Dual<1>;

struct TanLoad {
  using S = D1;
  using H = D1;
  const View<double> &V;
  const AdjWork &W;
  __device__ S mk(double v, double d) const {
    S x(v);
    x.d[0] = d;
    return x;
  }
  __device__ S prim(int k, int c) const {
    size_t o = (size_t)k * V.nc + c;
    return mk(V.prim[o], W.primd[o]);
  }
  __device__ S grad(int k, int c) const {
    size_t o = (size_t)k * V.nc + c;
    return mk(V.grad[o], W.gradd[o]);
  }
  __device__ void prim4(int c, S *q) const {
    for (int k = 0; k < 4; ++k) q[k] = prim(k, c);
  }
  __device__ void prim5(int c, S *q) const {
    for (int k = 0; k < 5; ++k) q[k] = prim(k, c);
  }
  __device__ void grad15(int c, S *g) const {
    for (int k = 0; k < 15; ++k) g[k] = grad(k, c);
  }
  __device__ H cv(int k, int c) const {
    size_t o = (size_t)k * V.nc + c;
    return mk(V.cv[o], W.cvd[o]);
  }
  __device__ H dv(int k, int c) const {
    size_t o = (size_t)k * V.nc + c;
    return mk(V.dv[o], W.dvd[o]);
  }
};

// ---------------------------------------------------------------------------
// Tangent kernels
// ---------------------------------------------------------------------------
__global__ void kTanInit(View<double> V, AdjWork W, const double *cvDotRef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const size_t n = V.nc;
  const int o = V.refId[i];
  D1 cv[5], q[5], dv[3];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    cv[k] = D1(V.cv[k * n + i]);
    cv[k].d[0] = cvDotRef[5 * (size_t)o + k];
    W.cvd[k * n + i] = cv[k].d[0];
  }
  primFromCv(V.p, cv, q, dv);
#pragma unroll
  for (int k = 0; k < 5; ++k) W.primd[k * n + i] = q[k].d[0];
#pragma unroll
  for (int k = 0; k < 3; ++k) W.dvd[k * n + i] = dv[k].d[0];
}

__global__ void __launch_bounds__(kBlock) kTanGrad(View<double> V, AdjWork W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  D1 g[15];
  gradLimitCell(V, TanLoad{V, W}, i, g);
  const size_t n = V.nc;
#pragma unroll
  for (int k = 0; k < 15; ++k) {
    V.grad[k * n + i] = g[k].v;
    W.gradd[k * n + i] = g[k].d[0];
  }
}

__global__ void __launch_bounds__(kBlock) kTanFlux(View<double> V, AdjWork W) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nT = V.nf + V.nb;
  if (t >= nT) return;
  D1 flx[5];
  faceFluxEval(V, TanLoad{V, W}, t, flx);
#pragma unroll
  for (int k = 0; k < 5; ++k) W.fluxd[(size_t)k * nT + t] = flx[k].d[0];
}

__global__ void kTanGather(View<double> V, AdjWork W, double *outRef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  double r[5];
  gatherRhs(V, (const double *)W.fluxd, i, r);
  const int o = V.refId[i];
#pragma unroll
  for (int k = 0; k < 5; ++k) outRef[5 * (size_t)o + k] = r[k];
}

// ---------------------------------------------------------------------------
// Adjoint kernels
// ---------------------------------------------------------------------------
__global__ void kAdjLambda(View<double> V, AdjWork W, const double *lamRef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const int o = V.refId[i];
#pragma unroll
  for (int k = 0; k < 5; ++k) W.cvd[(size_t)k * V.nc + i] = lamRef[5 * (size_t)o + k];
}

// Venkatakrishnan factor (RFLU_ModLimiters.F90:494-516) of one face side.
template <typename S>
__device__ inline S venkat(S dext, S d2, S epsq) {
  S numer = (dext * dext + epsq) * d2 + S(2) * d2 * d2 * dext;
  S denom = d2 * (dext * dext + S(2) * d2 * d2 + dext * d2 + epsq);
  return numer / (denom + S(1.0e-12));
}

// Forward pass of the limited gradient with the limiter's active branch.
__global__ void __launch_bounds__(kBlock) kAdjGradFwd(View<double> V, AdjWork W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const size_t n = V.nc;
  double q[5], g[15];
#pragma unroll
  for (int k = 0; k < 5; ++k) q[k] = V.prim[k * n + i];
#pragma unroll
  for (int k = 0; k < 15; ++k) g[k] = 0.0;
  for (int s = V.stOff[i]; s < V.stOff[i + 1]; ++s) {
    const int j = V.stIdx[s];
    const double wx = V.wx[s], wy = V.wy[s], wz = V.wz[s];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      double d = V.prim[k * n + j] - q[k];
      g[3 * k] = g[3 * k] + wx * d;
      g[3 * k + 1] = g[3 * k + 1] + wy * d;
      g[3 * k + 2] = g[3 * k + 2] + wz * d;
    }
  }
#pragma unroll
  for (int k = 0; k < 15; ++k) W.G[k * n + i] = g[k];
  const int rc = V.p.reconst;
  double lim[5] = {1, 1, 1, 1, 1};
  int es[5] = {-1, -1, -1, -1, -1}, js[5] = {-1, -1, -1, -1, -1};
  if (rc == 11 || rc == 100) {
    double vmin[5], vmax[5];
    int jmin[5], jmax[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) { vmin[k] = vmax[k] = q[k]; jmin[k] = jmax[k] = -1; }
    const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
    for (int e = cb; e < ce; ++e) {
      const int code = V.cfEnt[e];
      if (code < 0) continue;
      const int f = code >> 1, nb = (code & 1) ? V.fc1[f] : V.fc2[f];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        double x = V.prim[k * n + nb];
        if (x < vmin[k]) { vmin[k] = x; jmin[k] = nb; }
        if (x > vmax[k]) { vmax[k] = x; jmax[k] = nb; }
      }
    }
    const double epsq = V.epsq[i];
    for (int e = cb; e < ce; ++e) {
      const int code = V.cfEnt[e];
      if (code < 0) continue;
      const int f = code >> 1;
      const double *d = (code & 1) ? V.dR : V.dL;
      const double dx = d[f], dy = d[(size_t)V.nf + f], dz = d[2 * (size_t)V.nf + f];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const double d2 = -(g[3 * k] * dx + g[3 * k + 1] * dy + g[3 * k + 2] * dz);
        if (!(d2 > 0.0) && !(d2 < 0.0)) continue;
        const bool up = d2 > 0.0;
        const double dext = up ? vmax[k] - q[k] : vmin[k] - q[k];
        double t;
        bool active;
        if (rc == 11) {
          t = venkat(dext, d2, epsq);
          active = true;
        } else {
          const double x = dext / d2;
          t = fmin2(1.0, x);
          active = x < 1.0;
        }
        if (t < lim[k]) {
          lim[k] = t;
          es[k] = active ? e : -1;
          js[k] = up ? jmax[k] : jmin[k];
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    W.lim[k * n + i] = lim[k];
    W.estar[k * n + i] = es[k];
    W.jstar[k * n + i] = js[k];
#pragma unroll
    for (int c = 0; c < 3; ++c) V.grad[(3 * k + c) * n + i] = lim[k] * g[3 * k + c];
  }
}

// Transposed flux Jacobian of one face applied to Fbar.
template <int N>
__device__ inline void contract(const Dual<N> *flx, const double *fbar, double *out) {
#pragma unroll
  for (int m = 0; m < N; ++m) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) s += fbar[k] * flx[k].d[m];
    out[m] = s;
  }
}

__global__ void __launch_bounds__(kBlock) kAdjFace(View<double> V, AdjWork W) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nT = V.nf + V.nb;
  if (t >= nT) return;
  const Params &P = V.p;
  const size_t n = V.nc;
  const PlainLoad<double> ld{V};
  double *out = W.faceAdj + 16 * (size_t)t;
  double fbar[5];
  if (t < V.nf) {
    const int f = t, c1 = V.fc1[f], c2 = V.fc2[f];
#pragma unroll
    for (int k = 0; k < 5; ++k) fbar[k] = W.cvd[k * n + c1] - W.cvd[k * n + c2];
    if (P.spaceOrder == 1) {
      using D8 = Dual<8>;
      D8 cl[5], dl[3], cr[5], dr[3], flx[5];
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
        riemann1(P, cl, dl, cr, dr, D8(V.fnx[f]), D8(V.fny[f]), D8(V.fnz[f]), D8(V.fnm[f]), flx);
        contract(flx, fbar, out + 8 * side);
      }
    } else {
      using D6 = Dual<6>;
      const size_t nf = V.nf;
      double L[5], Rt[5], irl, irr;
      faceState(V, ld, c1, V.dL[f], V.dL[nf + f], V.dL[2 * nf + f], L, irl);
      faceState(V, ld, c2, V.dR[f], V.dR[nf + f], V.dR[2 * nf + f], Rt, irr);
      if (P.spaceDiscr == 1) {
        // Roe: hand-written reverse sweep (no dependence on the cell 1/rho)
        roe2Adjoint(P.refGamma, P.refCp, P.epsEntr, P.dissFact, V.fnx[f], V.fny[f], V.fnz[f], V.fnm[f], L, Rt, fbar,
                    out, out + 6);
        out[5] = 0.0;
        out[11] = 0.0;
        return;
      }
      D6 a[5], b[5], ia, ib, flx[5];
      for (int side = 0; side < 2; ++side) {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          a[k] = side ? D6(L[k]) : D6::seed(L[k], k);
          b[k] = side ? D6::seed(Rt[k], k) : D6(Rt[k]);
        }
        ia = side ? D6(irl) : D6::seed(irl, 5);
        ib = side ? D6::seed(irr, 5) : D6(irr);
        riemann2(P, D6(V.fnx[f]), D6(V.fny[f]), D6(V.fnz[f]), D6(V.fnm[f]), a, ia, b, ib, flx);
        contract(flx, fbar, out + 6 * side);
      }
    }
  } else {
    const int b = t - V.nf, c = V.bcell[b], ip = V.bpatch[b];
    const int type = V.patchType[ip], order = V.patchOrder[ip];
#pragma unroll
    for (int k = 0; k < 5; ++k) fbar[k] = W.cvd[k * n + c];
    if (type == 60) fbar[0] = 0.0;  // slip walls leave rhs(DENS)
    if (order == 1) {
      using D6 = Dual<6>;
      D6 cv[5], flx[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) cv[k] = D6::seed(V.cv[k * n + c], k);
      D6 pl = D6::seed(V.dv[c], 5);
      patch1(P, type, V.patchOutflow[ip], V.patchPout[ip], cv, pl, D6(V.bnx[b]), D6(V.bny[b]), D6(V.bnz[b]),
             D6(V.bnm[b]), flx);
      contract(flx, fbar, out);
    } else {
      using D5 = Dual<5>;
      const size_t nb = V.nb;
      double L[5], irl;
      faceState(V, ld, c, V.bd[b], V.bd[nb + b], V.bd[2 * nb + b], L, irl);
      D5 a[5], flx[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) a[k] = D5::seed(L[k], k);
      patch2(P, type, V.patchOutflow[ip], V.patchPout[ip], a, D5(V.bnx[b]), D5(V.bny[b]), D5(V.bnz[b]), D5(V.bnm[b]),
             flx);
      contract(flx, fbar, out);
    }
  }
}

// Side adjoints -> primitive / gradient adjoints of the cell, limiter reverse,
// gradient own-term.
__global__ void __launch_bounds__(kBlock) kAdjCell1(View<double> V, AdjWork W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V.nc) return;
  const Params &P = V.p;
  const size_t n = V.nc, nf = V.nf, nb = V.nb;
  double qb[5] = {0, 0, 0, 0, 0}, gtb[15], cvb[5] = {0, 0, 0, 0, 0}, dvb[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < 15; ++k) gtb[k] = 0.0;
  double rbar = 0.0;
  const double rho = V.prim[i];
  const int cb = V.cfOff[i], ce = V.cfOff[i + 1];
  for (int e = cb; e < ce; ++e) {
    const int code = V.cfEnt[e];
    if (code >= 0) {
      const int f = code >> 1, side = code & 1;
      const double *a = W.faceAdj + 16 * (size_t)f;
      if (P.spaceOrder == 1) {
        a += 8 * side;
#pragma unroll
        for (int k = 0; k < 5; ++k) cvb[k] += a[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) dvb[k] += a[5 + k];
      } else {
        a += 6 * side;
        const double *d = side ? V.dR : V.dL;
        const double dx = d[f], dy = d[nf + f], dz = d[2 * nf + f];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          qb[k] += a[k];
          gtb[3 * k] += a[k] * dx;
          gtb[3 * k + 1] += a[k] * dy;
          gtb[3 * k + 2] += a[k] * dz;
        }
        rbar += a[5];
      }
    } else {
      const int b = -code - 1;
      const double *a = W.faceAdj + 16 * (size_t)(nf + b);
      if (V.patchOrder[V.bpatch[b]] == 1) {
#pragma unroll
        for (int k = 0; k < 5; ++k) cvb[k] += a[k];
        dvb[0] += a[5];
      } else {
        const double dx = V.bd[b], dy = V.bd[nb + b], dz = V.bd[2 * nb + b];
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
  qb[0] += rbar * (-1.0 / (rho * rho));
  double gb[15], nbb[5] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < 15; ++k) gb[k] = 0.0;
  const int rc = P.reconst;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    if (P.spaceOrder < 2) break;
    const double l = W.lim[k * n + i];
    double lb = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      gb[3 * k + c] = l * gtb[3 * k + c];
      lb += gtb[3 * k + c] * W.G[(3 * k + c) * n + i];
    }
    const int es = W.estar[k * n + i];
    if ((rc == 11 || rc == 100) && es >= 0) {
      const int code = V.cfEnt[es];
      const int f = code >> 1;
      const double *d = (code & 1) ? V.dR : V.dL;
      const double dxyz[3] = {d[f], d[nf + f], d[2 * nf + f]};
      double g3[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) g3[c] = W.G[(3 * k + c) * n + i];
      const double d2 = -(g3[0] * dxyz[0] + g3[1] * dxyz[1] + g3[2] * dxyz[2]);
      const int js = W.jstar[k * n + i];
      const double qi = V.prim[k * n + i];
      const double dext = (js >= 0 ? V.prim[k * n + js] : qi) - qi;
      double db, d2b;
      if (rc == 11) {
        using D2 = Dual<2>;
        D2 phi = venkat(D2::seed(dext, 0), D2::seed(d2, 1), D2(V.epsq[i]));
        db = lb * phi.d[0];
        d2b = lb * phi.d[1];
      } else {
        // lim = dext/d2: d lim/d dext = 1/d2, d lim/d d2 = -(dext/d2)/d2, taken
        // as (lb/d2) and -(lb/d2)*(dext/d2) so that a tiny d2 (differences of
        // ~1e-200 ahead of a wave) neither squares into 0 nor makes 0/0 at a
        // local extreme (dext = 0)
        const double r = lb / d2;
        db = r;
        d2b = -r * (dext / d2);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) gb[3 * k + c] += d2b * (-dxyz[c]);
      if (js >= 0) {
        qb[k] -= db;
        nbb[k] = db;
      }
    }
  }
  // gradient own-term: G_i = sum_s w_s (q_{m_s} - q_i)
  for (int s = V.stOff[i]; s < V.stOff[i + 1] && P.spaceOrder > 1; ++s) {
    const double wx = V.wx[s], wy = V.wy[s], wz = V.wz[s];
#pragma unroll
    for (int k = 0; k < 5; ++k) qb[k] -= wx * gb[3 * k] + wy * gb[3 * k + 1] + wz * gb[3 * k + 2];
  }
#pragma unroll
  for (int k = 0; k < 15; ++k) W.Gbar[k * n + i] = gb[k];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    W.qbar[k * n + i] = qb[k];
    W.nbBar[k * n + i] = nbb[k];
    W.cvbarD[k * n + i] = cvb[k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) W.dvbar[k * n + i] = dvb[k];
}

// Neighbour terms, then (prim, dv) -> cv; output in reference order.
__global__ void __launch_bounds__(kBlock) kAdjCell2(View<double> V, AdjWork W, double *outRef) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= V.nc) return;
  const size_t n = V.nc;
  double qb[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) qb[k] = W.qbar[k * n + j];
  if (V.tsOff && V.p.spaceOrder > 1) {
    for (int e = V.tsOff[j]; e < V.tsOff[j + 1]; ++e) {
      const int i = V.tsCell[e], s = V.tsEnt[e];
      const double wx = V.wx[s], wy = V.wy[s], wz = V.wz[s];
#pragma unroll
      for (int k = 0; k < 5; ++k)
        qb[k] += wx * W.Gbar[(3 * k) * n + i] + wy * W.Gbar[(3 * k + 1) * n + i] + wz * W.Gbar[(3 * k + 2) * n + i];
    }
  }
  const int cb = V.cfOff[j], ce = (V.p.spaceOrder > 1) ? V.cfOff[j + 1] : cb;
  for (int e = cb; e < ce; ++e) {
    const int code = V.cfEnt[e];
    if (code < 0) continue;
    const int f = code >> 1, i = (code & 1) ? V.fc1[f] : V.fc2[f];
#pragma unroll
    for (int k = 0; k < 5; ++k)
      if (W.jstar[k * n + i] == j && W.estar[k * n + i] >= 0) qb[k] += W.nbBar[k * n + i];
  }
  using D5 = Dual<5>;
  D5 cv[5], q[5], dv[3];
#pragma unroll
  for (int k = 0; k < 5; ++k) cv[k] = D5::seed(V.cv[k * n + j], k);
  primFromCv(V.p, cv, q, dv);
  double dvb[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) dvb[k] = W.dvbar[k * n + j];
  const int o = V.refId[j];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    double s = W.cvbarD[m * n + j];
#pragma unroll
    for (int k = 0; k < 5; ++k) s += qb[k] * q[k].d[m];
#pragma unroll
    for (int k = 0; k < 3; ++k) s += dvb[k] * dv[k].d[m];
    outRef[5 * (size_t)o + m] = s;
  }
}

// Boundary-pressure functional: per-face p_f |A_f| on patch ip and the seed
// of the face adjoint (dJ/dp_f = |A_f|); the sum is a fixed-order block
// reduction.
__global__ void kPatchSeed(View<double> V, AdjWork W, int ip, double *Jout) {
  __shared__ double part[kBlock];
  const size_t n = V.nc, nb = V.nb;
  const PlainLoad<double> ld{V};
  double acc = 0.0;
  for (int b = threadIdx.x; b < V.nb; b += blockDim.x) {
    if (V.bpatch[b] != ip) continue;
    const int c = V.bcell[b];
    const double nm = V.bnm[b];
    double *a = W.faceAdj + 16 * (size_t)(V.nf + b);
    double pf;
    if (V.patchOrder[ip] == 1) {
      pf = V.dv[c];
      a[5] = nm;
    } else {
      double L[5], irl;
      faceState(V, ld, c, V.bd[b], V.bd[nb + b], V.bd[2 * nb + b], L, irl);
      pf = L[4];
      a[4] = nm;
    }
    acc += pf * nm;
  }
  (void)n;
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *Jout = part[0];
}

template <typename R>
struct AdjointOps {
  static void jvp(const View<R> &V, const double *cvDotRef, double *rhsDotRef, double *work, cudaStream_t s) {
    const size_t nT = (size_t)V.nf + V.nb;
    AdjWork W = carveAdjWork(work, V.nc, nT);
    kTanInit<<<blocks(V.nc), kBlock, 0, s>>>(V, W, cvDotRef);
    if (V.p.spaceOrder > 1) kTanGrad<<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    kTanFlux<<<blocks((long long)nT), kBlock, 0, s>>>(V, W);
    kTanGather<<<blocks(V.nc), kBlock, 0, s>>>(V, W, rhsDotRef);
  }
  static void cellAdjoint(const View<R> &V, AdjWork &W, double *cvBarRef, cudaStream_t s) {
    kAdjCell1<<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    kAdjCell2<<<blocks(V.nc), kBlock, 0, s>>>(V, W, cvBarRef);
  }
  static void vjp(const View<R> &V, const double *rhsBarRef, double *cvBarRef, double *work, cudaStream_t s) {
    const size_t nT = (size_t)V.nf + V.nb;
    AdjWork W = carveAdjWork(work, V.nc, nT);
    kAdjLambda<<<blocks(V.nc), kBlock, 0, s>>>(V, W, rhsBarRef);
    if (V.p.spaceOrder > 1) kAdjGradFwd<<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    cudaMemsetAsync(W.faceAdj, 0, sizeof(double) * 16 * nT, s);
    kAdjFace<<<blocks((long long)nT), kBlock, 0, s>>>(V, W);
    cellAdjoint(V, W, cvBarRef, s);
  }
  static void patchPressure(const View<R> &V, int ip, double *J, double *cvBarRef, double *work, cudaStream_t s) {
    const size_t nT = (size_t)V.nf + V.nb;
    AdjWork W = carveAdjWork(work, V.nc, nT);
    if (V.p.spaceOrder > 1) kAdjGradFwd<<<blocks(V.nc), kBlock, 0, s>>>(V, W);
    cudaMemsetAsync(W.faceAdj, 0, sizeof(double) * 16 * nT, s);
    kPatchSeed<<<1, kBlock, 0, s>>>(V, W, ip, J);
    if (cvBarRef) cellAdjoint(V, W, cvBarRef, s);
  }
};

#else
// Translation units without the adjoint (the mixed mode): no entries.
template <typename R>
struct AdjointOps {
  static constexpr void (*jvp)(const View<R> &, const double *, double *, double *, cudaStream_t) = nullptr;
  static constexpr void (*vjp)(const View<R> &, const double *, double *, double *, cudaStream_t) = nullptr;
  static constexpr void (*patchPressure)(const View<R> &, int, double *, double *, double *, cudaStream_t) = nullptr;
};
#endif

}  // namespace RFLU_NS
}  // namespace rflu
