// Point-wise physics of the path, generic in the scalar type S (double,
// float, or the dual numbers of the tangent/adjoint kernels).  Each function
// keeps the operation order of the reference routine it cites, so that the
// FP64 build without FMA contraction reproduces the reference bit for bit.
#pragma once
#include <cmath>

#include "dual.cuh"

namespace rflu {

__host__ __device__ inline double sqrt_(double x) { return sqrt(x); }
__host__ __device__ inline float sqrt_(float x) { return sqrtf(x); }
__host__ __device__ inline double fabs_(double x) { return fabs(x); }
__host__ __device__ inline float fabs_(float x) { return fabsf(x); }
__host__ __device__ inline double copysign_(double a, double b) { return copysign(a, b); }
__host__ __device__ inline float copysign_(float a, float b) { return copysignf(a, b); }
// x ** y where the exponent is a gas constant (g / (g - 1) and the like):
// the dual-number overload differentiates in x only
__host__ __device__ inline double powConstExp(double x, double y) { return pow(x, y); }
__host__ __device__ inline float powConstExp(float x, float y) { return powf(x, y); }
// Fortran MIN/MAX of two reals (first argument kept on ties)
template <typename S> __host__ __device__ inline S fmin2(const S &a, const S &b) { return (b < a) ? b : a; }
template <typename S> __host__ __device__ inline S fmax2(const S &a, const S &b) { return (b > a) ? b : a; }

// libfloflu/MixtPerf_*.F90
template <typename S> __host__ __device__ inline S perfEo(S d, S g, S p, S u, S v, S w) {  // MixtPerf_E.F90:79
  return p / (d * (g - S(1))) + S(0.5) * (u * u + v * v + w * w);
}
template <typename S> __host__ __device__ inline S perfHo(S cp, S t, S u, S v, S w) {      // MixtPerf_H.F90:78
  return cp * t + S(0.5) * (u * u + v * v + w * w);
}
template <typename S> __host__ __device__ inline S perfCGHoVm2(S g, S ho, S vm2) {          // MixtPerf_C.F90:110
  return sqrt_((g - S(1)) * (ho - S(0.5) * vm2));
}

// modflu/RFLU_ModEntropyFixes.F90:95-106
template <typename S> __host__ __device__ inline S entropyFixHH(S l, S d) {
  if (l > d) return l;
  return (l * l + d * d) / (S(2) * d);
}

// Roe flux with the Harten-Hyman fix, flxConv - flxDiss:
// RFLU_ROE_ComputeFlux1_TCP / _Flux2_TCP (modflu/RFLU_ModRoeFlux.F90:
// 1683-1942, 2513-2867).
template <typename S>
__host__ __device__ inline void roeFlux(S g, S epsentr, S dissFact, S nx, S ny, S nz, S nm, S rl, S ul, S vl, S wl,
                                        S pl, S Hl, S rr, S ur, S vr, S wr, S pr, S Hr, S *flx) {
  const S fs = S(0);
  S ql = ul * nx + vl * ny + wl * nz - fs;
  S qr = ur * nx + vr * ny + wr * nz - fs;
  S rh = sqrt_(rl * rr);
  S wt = rl / (rl + rh);
  S uh = wt * ul + (S(1) - wt) * ur;
  S vh = wt * vl + (S(1) - wt) * vr;
  S wh = wt * wl + (S(1) - wt) * wr;
  S Hh = wt * Hl + (S(1) - wt) * Hr;
  S qh = uh * nx + vh * ny + wh * nz - fs;
  S sh = S(0.5) * (uh * uh + vh * vh + wh * wh);
  S ah = perfCGHoVm2(g, Hh, S(2) * sh);
  S l1 = fabs_(qh - ah), l2 = fabs_(qh), l5 = fabs_(qh + ah);
  S efc = epsentr * l5;
  l1 = entropyFixHH(l1, efc);
  l2 = entropyFixHH(l2, efc);
  l5 = entropyFixHH(l5, efc);
  S dr = rr - rl, du = ur - ul, de = vr - vl, dw = wr - wl, dp = pr - pl;
  S dq = du * nx + de * ny + dw * nz;
  S dv1 = (dp - rh * ah * dq) / (S(2) * ah * ah);
  S dv5 = (dp + rh * ah * dq) / (S(2) * ah * ah);
  S dv2 = dr - dp / (ah * ah);
  S t1 = l1 * dv1, t2 = l2 * dv2, t3 = l2 * rh, t5 = l5 * dv5;
  S h = S(0.5), hd = S(0.5) * dissFact;
  S fc1 = h * (ql * rl + qr * rr) * nm;
  S fc2 = h * (ql * rl * ul + pl * nx + qr * rr * ur + pr * nx) * nm;
  S fc3 = h * (ql * rl * vl + pl * ny + qr * rr * vr + pr * ny) * nm;
  S fc4 = h * (ql * rl * wl + pl * nz + qr * rr * wr + pr * nz) * nm;
  S fc5 = h * (ql * rl * Hl + pl * fs + qr * rr * Hr + pr * fs) * nm;
  S fd1 = hd * (t1 + t2 + t5) * nm;
  S fd2 = hd * (t1 * (uh - nx * ah) + t2 * uh + t3 * (du - nx * dq) + t5 * (uh + nx * ah)) * nm;
  S fd3 = hd * (t1 * (vh - ny * ah) + t2 * vh + t3 * (de - ny * dq) + t5 * (vh + ny * ah)) * nm;
  S fd4 = hd * (t1 * (wh - nz * ah) + t2 * wh + t3 * (dw - nz * dq) + t5 * (wh + nz * ah)) * nm;
  S fd5 = hd * (t1 * (Hh - qh * ah) + t2 * sh + t3 * (uh * du + vh * de + wh * dw - qh * dq) + t5 * (Hh + qh * ah)) * nm;
  flx[0] = fc1 - fd1; flx[1] = fc2 - fd2; flx[2] = fc3 - fd3; flx[3] = fc4 - fd4; flx[4] = fc5 - fd5;
}

// HLLC: RFLU_HLLC_ComputeFlux1_TCP / _Flux2_TCP (modflu/RFLU_ModHLLCFlux.F90:
// 926-1194, 2131-2434).
template <typename S>
__host__ __device__ inline void hllcFlux(S g, S nx, S ny, S nz, S nm, S rl, S ul, S vl, S wl, S pl, S el, S al, S Hl,
                                         S rr, S ur, S vr, S wr, S pr, S er, S ar, S Hr, S *flx) {
  const S fs = S(0);
  S ql = ul * nx + vl * ny + wl * nz - fs;
  S qr = ur * nx + vr * ny + wr * nz - fs;
  S wt1 = sqrt_(rr / rl);
  S wt2 = S(1) / (S(1) + wt1);
  S us = wt2 * (ul + wt1 * ur);
  S vs = wt2 * (vl + wt1 * vr);
  S ws = wt2 * (wl + wt1 * wr);
  S qs = wt2 * (ql + wt1 * qr);
  S Hs = wt2 * (Hl + wt1 * Hr);
  S Vms = us * us + vs * vs + ws * ws;
  S as = perfCGHoVm2(g, Hs, Vms);
  S sl = fmin2(ql - al, qs - as);
  S sr = fmax2(qr + ar, qs + as);
  if (sl > S(0)) {
    flx[0] = ql * rl * nm;
    flx[1] = (ql * rl * ul + pl * nx) * nm;
    flx[2] = (ql * rl * vl + pl * ny) * nm;
    flx[3] = (ql * rl * wl + pl * nz) * nm;
    flx[4] = (ql * (rl * el + pl) + pl * fs) * nm;
  } else if (sr < S(0)) {
    flx[0] = qr * rr * nm;
    flx[1] = (qr * rr * ur + pr * nx) * nm;
    flx[2] = (qr * rr * vr + pr * ny) * nm;
    flx[3] = (qr * rr * wr + pr * nz) * nm;
    flx[4] = (qr * (rr * er + pr) + pr * fs) * nm;
  } else {
    S sm = (rr * qr * (sr - qr) - rl * ql * (sl - ql) - pr + pl) / (rr * (sr - qr) - rl * (sl - ql));
    S ps = pl + rl * (ql - sl) * (ql - sm);
    S rs, rus, rvs, rws, res;
    if (sm > S(0)) {
      S term = S(1) / (sl - sm);
      rs = term * (sl - ql) * rl;
      rus = term * ((sl - ql) * rl * ul + (ps - pl) * nx);
      rvs = term * ((sl - ql) * rl * vl + (ps - pl) * ny);
      rws = term * ((sl - ql) * rl * wl + (ps - pl) * nz);
      res = term * ((sl - ql) * rl * el + (ps * sm - pl * ql));
    } else {
      S term = S(1) / (sr - sm);
      rs = term * (sr - qr) * rr;
      rus = term * ((sr - qr) * rr * ur + (ps - pr) * nx);
      rvs = term * ((sr - qr) * rr * vr + (ps - pr) * ny);
      rws = term * ((sr - qr) * rr * wr + (ps - pr) * nz);
      res = term * ((sr - qr) * rr * er + (ps * sm - pr * qr));
    }
    flx[0] = sm * rs * nm;
    flx[1] = (sm * rus + ps * nx) * nm;
    flx[2] = (sm * rvs + ps * ny) * nm;
    flx[3] = (sm * rws + ps * nz) * nm;
    flx[4] = (sm * (res + ps) - ps * fs) * nm;
  }
}

// AUSM+: RFLU_AUSM_FluxFunction (modflu/RFLU_ModAUSMFlux.F90:282-416).
template <typename S>
__host__ __device__ inline void ausmFlux(S nx, S ny, S nz, S nm, S rl, S ul, S vl, S wl, S pl, S Hl, S al, S rr, S ur,
                                         S vr, S wr, S pr, S Hr, S ar, S *flx) {
  const S fs = S(0), one = S(1);
  S ql = ul * nx + vl * ny + wl * nz - fs;
  S qr = ur * nx + vr * ny + wr * nz - fs;
  S af = S(0.5) * (al + ar);
  S ml = ql / af, mla = fabs_(ml);
  S mr = qr / af, mra = fabs_(mr);
  S mlp, wtl, mrm, wtr;
  if (mla <= one) {
    mlp = S(0.25) * (ml + one) * (ml + one) + S(0.125) * (ml * ml - one) * (ml * ml - one);
    wtl = S(0.25) * (ml + one) * (ml + one) * (S(2) - ml) + S(0.1875) * ml * (ml * ml - one) * (ml * ml - one);
  } else {
    mlp = S(0.5) * (ml + mla);
    wtl = S(0.5) * (one + ml / mla);
  }
  if (mra <= one) {
    mrm = -S(0.25) * (mr - one) * (mr - one) - S(0.125) * (mr * mr - one) * (mr * mr - one);
    wtr = S(0.25) * (mr - one) * (mr - one) * (S(2) + mr) - S(0.1875) * mr * (mr * mr - one) * (mr * mr - one);
  } else {
    mrm = S(0.5) * (mr - mra);
    wtr = S(0.5) * (one - mr / mra);
  }
  S mf = mlp + mrm, mfa = fabs_(mf);
  S mfp = S(0.5) * (mf + mfa), mfm = S(0.5) * (mf - mfa);
  S pf = wtl * pl + wtr * pr;
  flx[0] = (af * (mfp * rl + mfm * rr)) * nm;
  flx[1] = (af * (mfp * rl * ul + mfm * rr * ur) + pf * nx) * nm;
  flx[2] = (af * (mfp * rl * vl + mfm * rr * vr) + pf * ny) * nm;
  flx[3] = (af * (mfp * rl * wl + mfm * rr * wr) + pf * nz) * nm;
  flx[4] = (af * (mfp * rl * Hl + mfm * rr * Hr) + pf * fs) * nm;
}

// BcondOutflowPerf (libfloflu/BcondOutflowPerf.F90:88-159).
template <typename S>
__host__ __device__ inline void bcondOutflowPerf(int bcOpt, S pout, S sxn, S syn, S szn, S cpgas, S mol, S rho, S rhou,
                                                 S rhov, S rhow, S rhoe, S press, S &rhob, S &rhoub, S &rhovb,
                                                 S &rhowb, S &rhoeb) {
  S rgas = S(8314.3) / mol;
  S gamma = cpgas / (cpgas - rgas);
  S u = rhou / rho, v = rhov / rho, w = rhow / rho;
  S csound = sqrt_(gamma * press / rho);
  S mach = sqrt_(u * u + v * v + w * w) / csound;
  if (mach < S(1) && (bcOpt == 1 || bcOpt == 2)) {
    S rrhoc = S(1) / (rho * csound);
    S deltp = press - pout;
    rhob = rho - deltp / (csound * csound);
    S ub = u + sxn * deltp * rrhoc;
    S vb = v + syn * deltp * rrhoc;
    S wb = w + szn * deltp * rrhoc;
    S vnd = ub * sxn + vb * syn + wb * szn;
    if (vnd < S(0)) {
      ub = copysign_(S(1), u) * fmax2(fabs_(ub), fabs_(u));
      vb = copysign_(S(1), v) * fmax2(fabs_(vb), fabs_(v));
      wb = copysign_(S(1), w) * fmax2(fabs_(wb), fabs_(w));
    }
    rhoub = rhob * ub;
    rhovb = rhob * vb;
    rhowb = rhob * wb;
    rhoeb = rhob * perfEo(rhob, gamma, pout, ub, vb, wb);
  } else {
    rhob = rho; rhoub = rhou; rhovb = rhov; rhowb = rhow; rhoeb = rhoe;
  }
}

// The central patch flux of the inflow, outflow and farfield cases of
// rocflu/RFLU_CentralFirstPatch.F90 (:281-287, :571-784, :1001-1007) and
// RFLU_CentralSecondPatch.F90: the average of the interior state l and the
// boundary state r, static grid (fs = 0).
template <typename S>
__host__ __device__ inline void centralPatchFlux(S nx, S ny, S nz, S nm, S rl, S rul, S rvl, S rwl, S rel, S pl, S rr,
                                                 S rur, S rvr, S rwr, S rer, S pr, S *flx) {
  const S fs = S(0);
  S ql = (rul * nx + rvl * ny + rwl * nz) / rl - fs;
  S qr = (rur * nx + rvr * ny + rwr * nz) / rr - fs;
  S h = S(0.5);
  flx[0] = h * (ql * rl + qr * rr) * nm;
  flx[1] = h * (ql * rul + pl * nx + qr * rur + pr * nx) * nm;
  flx[2] = h * (ql * rvl + pl * ny + qr * rvr + pr * ny) * nm;
  flx[3] = h * (ql * rwl + pl * nz + qr * rwr + pr * nz) * nm;
  flx[4] = h * (ql * (rel + pl) + pl * fs + qr * (rer + pr) + pr * fs) * nm;
}

// Central patch flux on outflow faces (rocflu/RFLU_CentralFirstPatch.F90:
// 571-784, RFLU_CentralSecondPatch.F90:634-857).
template <typename S>
__host__ __device__ inline void outflowPatchFlux(int bcOpt, S pOut, S cp, S mol, S nx, S ny, S nz, S nm, S rl, S rul,
                                                 S rvl, S rwl, S rel, S pl, S *flx) {
  S pr = (bcOpt != 0) ? pOut : pl;
  S rr, rur, rvr, rwr, rer;
  bcondOutflowPerf(bcOpt, pr, nx, ny, nz, cp, mol, rl, rul, rvl, rwl, rel, pl, rr, rur, rvr, rwr, rer);
  centralPatchFlux(nx, ny, nz, nm, rl, rul, rvl, rwl, rel, pl, rr, rur, rvr, rwr, rer, pr, flx);
}

// The boundary types below read their patch's constants K (ctx.h: kPatchK),
// formed on the host by rflu_gpu_create.

// RFLU_SetRindStateFarfieldPerf without the vortex correction
// (modflu/RFLU_ModRindStates.F90:248-420).
template <typename S>
__host__ __device__ inline void farfieldRindPerf(const double *K, S g, S nx, S ny, S nz, S rl, S rul, S rvl, S rwl,
                                                 S rel, S &rr, S &rur, S &rvr, S &rwr, S &rer, S &pr) {
  S ul = rul / rl, vl = rvl / rl, wl = rwl / rl;
  S ql = ul * nx + vl * ny + wl * nz;
  S el = rel / rl;
  S sl2 = ul * ul + vl * vl + wl * wl;
  S pl = (g - S(1)) * rl * (el - S(0.5) * sl2);  // MixtPerf_P_DEoGVm2
  const S ri = S(K[1]), pi = S(K[2]), ui = S(K[4]), vi = S(K[5]), wi = S(K[6]);
  if (K[0] < 1.0) {
    S al = sqrt_(g * pl / rl);  // MixtPerf_C_DGP
    S pb, rb, ub, vb, wb;
    if (ql < S(0)) {
      pb = S(0.5) * (pi + pl - rl * al * ((ui - ul) * nx + (vi - vl) * ny + (wi - wl) * nz));
      rb = ri - (pi - pb) / (al * al);
      ub = ui - nx * (pi - pb) / (rl * al);
      vb = vi - ny * (pi - pb) / (rl * al);
      wb = wi - nz * (pi - pb) / (rl * al);
    } else {
      pb = pi;
      rb = rl - (pl - pi) / (al * al);
      ub = ul + nx * (pl - pi) / (rl * al);
      vb = vl + ny * (pl - pi) / (rl * al);
      wb = wl + nz * (pl - pi) / (rl * al);
    }
    rr = rb;
    rur = rb * ub;
    rvr = rb * vb;
    rwr = rb * wb;
    rer = rb * perfEo(rb, g, pb, ub, vb, wb);
    pr = pb;
  } else if (ql < S(0)) {
    rr = ri;
    rur = ri * ui;
    rvr = ri * vi;
    rwr = ri * wi;
    rer = S(K[7]);
    pr = pi;
  } else {
    rr = rl; rur = rul; rvr = rvl; rwr = rwl; rer = rel; pr = pl;
  }
}

// BcondInflowPerf (libfloflu/BcondInflowPerf.F90): the boundary state of an
// inflow given by total pressure and temperature and flow angles.  A
// subsonic-type patch whose face sees |q| >= c gets no state in the
// reference (its outputs stay unset); here it gets NaN, which the validity
// check reports.
template <typename S>
__host__ __device__ inline void inflowTotAngPerf(int bcOpt, const double *K, S g, S rgas, S nx, S ny, S nz, S rl,
                                                 S rul, S rvl, S rwl, S &rr, S &rur, S &rvr, S &rwr, S &rer,
                                                 S &pr) {
  if (bcOpt == 1 || bcOpt == 2) {  // BCOPT_SUBSONIC, BCOPT_MIXED
    const S ptot = S(K[0]), ttot = S(K[1]);
    S gm1 = g - S(1);
    S ul = rul / rl, vl = rvl / rl, wl = rwl / rl;
    S a02 = g * rgas * ttot;                                           // MixtPerf_C2_GRT
    S al = sqrt_(a02 - S(0.5) * (g - S(1)) * (ul * ul + vl * vl + wl * wl));  // MixtPerf_C_Co2GUVW
    S ql = ul * nx + vl * ny + wl * nz;
    if (fabs_(ql) < al) {
      S sl = sqrt_(ul * ul + vl * vl + wl * wl);
      S eta = S(-1);
      if (K[6] == 0.0 && sl > S(1.0e-6)) eta = ql / sl;  // BCOPT_FIXED_NO, a well-defined angle
      S Rm = al - S(0.5) * gm1 * ql;
      S disc = S(0.5) * gm1 * (eta * eta) * (a02 / (Rm * Rm) * (S(1) + S(0.5) * gm1 * (eta * eta)) - S(1));
      S ar, tr, sr;
      if (disc < S(0)) {
        ar = sqrt_(a02);
        tr = ttot;
        pr = ptot;
        sr = S(0);
      } else {
        ar = Rm / (S(1) + S(0.5) * gm1 * eta * eta) * (S(1) + sqrt_(disc));
        tr = ar * ar / (g * rgas);                              // MixtPerf_T_CGR
        pr = ptot * powConstExp(tr / ttot, g / (g - S(1)));     // MixtPerf_P_GPoTTo
        S c2 = ar * ar;                                          // MixtPerf_Vm_C2Co2G
        sr = (a02 > c2) ? sqrt_(S(2) / (g - S(1)) * (a02 - c2)) : S(0);
      }
      rr = pr / (rgas * tr);  // MixtPerf_D_PRT
      S ur = sr * S(K[2]) * S(K[4]);
      S vr = sr * S(K[3]);
      S wr = sr * S(K[2]) * S(K[5]);
      rer = rr * (pr / (rr * (g - S(1))) + S(0.5) * sr * sr);  // MixtPerf_Eo_DGPVm
      rur = rr * ur;
      rvr = rr * vr;
      rwr = rr * wr;
      return;
    }
    if (bcOpt == 1) {
      rr = rur = rvr = rwr = rer = pr = S(nan(""));
      return;
    }
  }
  rr = S(K[7]); rur = S(K[8]); rvr = S(K[9]); rwr = S(K[10]); rer = S(K[11]); pr = S(K[12]);
}

// The inflow state given by velocity and temperature (RFLU_CentralFirstPatch.
// F90:375-570): prescribed pressure unless subsonic, else the interior
// density.
template <typename S>
__host__ __device__ inline void inflowVelTempPerf(int bcOpt, const double *K, S g, S rgas, S rl, S &rr, S &rur,
                                                  S &rvr, S &rwr, S &rer, S &pr) {
  const S ur = S(K[0]), vr = S(K[1]), wr = S(K[2]), tr = S(K[3]);
  if (bcOpt != 1) {  // not BCOPT_SUBSONIC: rr = MixtPerf_D_PRT(pr, rgas, tr), formed on the host
    pr = S(K[4]);
    rr = S(K[5]);
  } else {
    rr = rl;
    pr = rr * rgas * tr;  // MixtPerf_P_DRT
  }
  rer = rr * perfEo(rr, g, pr, ur, vr, wr);
  rur = rr * ur;
  rvr = rr * vr;
  rwr = rr * wr;
}

// RFLU_SetRindStateSlipWallPerf (modflu/RFLU_ModRindStates.F90:535-584):
// the wall pressure of a non-burning injection face, static grid.
template <typename S>
__host__ __device__ inline S slipWallRindPerf(S g, S nx, S ny, S nz, S rl, S rul, S rvl, S rwl, S pl) {
  const S fs = S(0);
  S irl = S(1) / rl;
  S ul = irl * rul, vl = irl * rvl, wl = irl * rwl;
  S ql = ul * nx + vl * ny + wl * nz - fs;
  S al = sqrt_(g * pl / rl);
  if (ql < S(0)) {
    S term = S(1) + S(0.5) * (g - S(1)) * ql / al;
    return pl * powConstExp(term, S(2) * g / (g - S(1)));
  }
  S term = (g + S(1)) / S(4);
  return pl + term * rl * ql * (ql + sqrt_(al * al + term * term * ql * ql) / term);
}

// Injection patch flux (RFLU_CentralFirstPatch.F90:1043-1127,
// RFLU_CentralSecondPatch.F90:1229-1343): a burning face (mass flux > 0)
// injects gas at T_inj through RFLU_SetRindStateInjectPerf
// (RFLU_ModRindStates.F90:459-501); a non-burning one is a wall with the
// slip-wall rind pressure.  All five components enter rhs.
template <typename S>
__host__ __device__ inline void injectionPatchFlux(const double *K, S g, S cp, S rgas, S nx, S ny, S nz, S nm, S rl,
                                                   S rul, S rvl, S rwl, S pl, S *flx) {
  const S fs = S(0);
  if (K[0] > 0.0) {
    const S minj = S(K[0]), tinj = S(K[1]);
    S rb = pl / (rgas * tinj);  // MixtPerf_D_PRT
    S qb = -minj / rb + fs;
    S ub = qb * nx, vb = qb * ny, wb = qb * nz;
    S hb = perfHo(cp, tinj, ub, vb, wb);
    flx[0] = -minj * nm;
    flx[1] = (-minj * ub + pl * nx) * nm;
    flx[2] = (-minj * vb + pl * ny) * nm;
    flx[3] = (-minj * wb + pl * nz) * nm;
    flx[4] = (-minj * hb + pl * fs) * nm;
  } else {
    S pw = slipWallRindPerf(g, nx, ny, nz, rl, rul, rvl, rwl, pl);
    flx[0] = S(0);
    flx[1] = pw * nx * nm;
    flx[2] = pw * ny * nm;
    flx[3] = pw * nz * nm;
    flx[4] = pw * fs * nm;
  }
}

// Walls (slip, no-slip) leave rhs(DENS) as it is; every other patch adds
// all five components (ConvectiveFluxes' patch loop).
__host__ __device__ inline bool patchLeavesDensity(int type) { return type == 60 || type == 70 || type == 71; }

// Cyclic Jacobi eigen-decomposition of a symmetric 3x3 (RFLU_SymmetricEigen3,
// modflu/RFLU_ModLimiters.F90:791-912): ascending eigenvalues, eigenvectors
// as columns.  m, vec are column-major.
template <typename S>
__host__ __device__ inline void symmetricEigen3(const S m[9], S vec[9], S val[3]) {
  S r[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) { r[k] = m[k]; vec[k] = S(0); }
  vec[0] = vec[4] = vec[8] = S(1);
  S total = S(0);
#pragma unroll
  for (int k = 0; k < 9; ++k) total = total + r[k] * r[k];
  const S tol = S(1.0e-24);
  for (int sweep = 0; sweep < 50; ++sweep) {
    S off = r[3] * r[3] + r[6] * r[6] + r[7] * r[7];
    if (off <= tol * total) break;
#pragma unroll
    for (int ip = 0; ip < 2; ++ip)
#pragma unroll
      for (int iq = ip + 1; iq < 3; ++iq) {
        const int pq = ip + 3 * iq, pp = ip + 3 * ip, qq = iq + 3 * iq;
        if (r[pq] != S(0)) {
          S theta = (r[qq] - r[pp]) / (S(2) * r[pq]);
          S t;
          if (fabs_(theta) > S(1.0e150)) t = S(0.5) / theta;
          else t = copysign_(S(1), theta) / (fabs_(theta) + sqrt_(theta * theta + S(1)));
          S c = S(1) / sqrt_(t * t + S(1));
          S s = t * c;
          const int ir = 3 - ip - iq;
          S arp = r[ir + 3 * ip], arq = r[ir + 3 * iq];
          r[pp] = r[pp] - t * r[pq];
          r[qq] = r[qq] + t * r[pq];
          r[pq] = S(0);
          r[iq + 3 * ip] = S(0);
          r[ir + 3 * ip] = c * arp - s * arq;
          r[ip + 3 * ir] = r[ir + 3 * ip];
          r[ir + 3 * iq] = s * arp + c * arq;
          r[iq + 3 * ir] = r[ir + 3 * iq];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            S vp = vec[i + 3 * ip], vq = vec[i + 3 * iq];
            vec[i + 3 * ip] = c * vp - s * vq;
            vec[i + 3 * iq] = s * vp + c * vq;
          }
        }
      }
  }
  val[0] = r[0]; val[1] = r[4]; val[2] = r[8];
  // selection sort (first strict minimum, swapped into place), written with
  // fixed indices so that val and vec stay in registers
  auto swapCols = [&](int a, int b) {
    S t = val[a]; val[a] = val[b]; val[b] = t;
#pragma unroll
    for (int k = 0; k < 3; ++k) { S x = vec[k + 3 * a]; vec[k + 3 * a] = vec[k + 3 * b]; vec[k + 3 * b] = x; }
  };
  const bool m1 = val[1] < val[0];
  const bool m2 = val[2] < (m1 ? val[1] : val[0]);
  if (m2) swapCols(0, 2);
  else if (m1) swapCols(0, 1);
  if (val[2] < val[1]) swapCols(1, 2);
}

// Whether eigenvalues j < k (ascending) lie in one group of the eigen-frame
// limiter's merge (RFLU_LimitGradVelocityBarthJesp, modflu/
// RFLU_ModLimiters.F90:728-760: neighbours within 1e-3 of the largest
// magnitude share one factor).
template <typename T>
__host__ __device__ inline bool mergedPair(const T *l, int j, int k) {
  T mx = fabs_(l[0]);
  mx = fmax2(mx, fabs_(l[1]));
  mx = fmax2(mx, fabs_(l[2]));
  const T scale = T(1.0e-3) * mx;
  const bool e12 = (l[1] - l[0] <= scale), e23 = (l[2] - l[1] <= scale);
  if (j == 0 && k == 1) return e12;
  if (j == 1 && k == 2) return e23;
  return e12 && e23;
}

// Whether axis j of the eigen-frame carries no velocity gradient: its row
// A_j' G is at the level of the eigenvectors' rounding (the Jacobi
// iteration stops at off-diagonals of 1e-12 |S|, so eigenvectors of
// eigenvalues 1e-3 |S| apart carry errors up to 1e-9; FP32 about 1e-4).  In
// a flow whose velocity varies in fewer than three directions (one velocity
// component zero, a plane or axis of symmetry) the strain rate has such an
// axis, and the limiter's factor on it, dext / pr with dext = A_j . du and
// pr = A_j . G off, is a ratio of two rounding residues: a value anywhere in
// [0, 1] that multiplies A_j' G and so changes the limited gradient only at
// rounding level, but whose derivative is of order 1 / rounding.  The
// tangent and the adjoint hold such a factor at its value (at the exact
// configuration the primal is not differentiable: the factor along a
// perturbation is the ratio of the perturbation's own projections).
template <typename T>
__host__ __device__ inline bool idleAxis(const T *A, const T *G, int j) {
  const T tol = sizeof(T) >= 8 ? T(1.0e-8) : T(1.0e-3);
  T gm = T(0), bm = T(0);
#pragma unroll
  for (int k = 0; k < 9; ++k) gm = fmax2(gm, fabs_(G[k]));
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    T s = T(0);
    s = s + A[3 * j] * G[3 * c];
    s = s + A[3 * j + 1] * G[1 + 3 * c];
    s = s + A[3 * j + 2] * G[2 + 3 * c];
    bm = fmax2(bm, fabs_(s));
  }
  return bm <= tol * gm;
}

// The eigen-frame limiter's factors al[3] on the tangent types: idle axes
// (idleAxis) keep their value and lose their derivative.  A no-op on plain
// floating-point types (the primal).
template <typename S>
__host__ __device__ inline void holdIdleAxes(const S *, const S *, S *) {}
template <int N, typename T>
__host__ __device__ inline void holdIdleAxes(const Dual<N, T> *A, const Dual<N, T> *G, Dual<N, T> *al) {
  T a[9], g[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) { a[k] = A[k].v; g[k] = G[k].v; }
#pragma unroll
  for (int j = 0; j < 3; ++j)
    if (idleAxis(a, g, j)) al[j] = Dual<N, T>(al[j].v);
}

// The same on dual numbers (the tangent kernels): values by the Jacobi
// iteration above, derivatives by first-order perturbation of the computed
// eigenpairs of the symmetric m, dl_j = a_j' dm a_j and
// da_j = sum over k != j of a_k (a_k' dm a_j) / (l_j - l_k).  Pairs the
// limiter merges are one eigenspace to the derivative: their axes are held
// fixed within it (their rotation there is of order 1 for a change of
// order l_j - l_k, a sensitivity of the basis the merged factor follows only
// through its minimum; keeping it would scale rounding by 1/(l_j - l_k) in
// the near-symmetric flows where such pairs arise).  The tangent of the
// eigen-frame limiter is then the linear map whose transpose its adjoint
// applies (adjoint.cuh: velFrameReverse).
template <int N, typename T>
__host__ __device__ inline void symmetricEigen3(const Dual<N, T> m[9], Dual<N, T> vec[9], Dual<N, T> val[3]) {
  T mv[9], a[9], l[3];
#pragma unroll
  for (int k = 0; k < 9; ++k) mv[k] = m[k].v;
  symmetricEigen3(mv, a, l);
#pragma unroll
  for (int k = 0; k < 9; ++k) vec[k] = Dual<N, T>(a[k]);
#pragma unroll
  for (int j = 0; j < 3; ++j) val[j] = Dual<N, T>(l[j]);
#pragma unroll
  for (int q = 0; q < N; ++q) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T sa[3];  // dm a_j
#pragma unroll
      for (int r = 0; r < 3; ++r) sa[r] = m[r].d[q] * a[3 * j] + m[r + 3].d[q] * a[3 * j + 1] + m[r + 6].d[q] * a[3 * j + 2];
      val[j].d[q] = a[3 * j] * sa[0] + a[3 * j + 1] * sa[1] + a[3 * j + 2] * sa[2];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k == j || l[j] == l[k] || mergedPair(l, j < k ? j : k, j < k ? k : j)) continue;
        const T coef = (a[3 * k] * sa[0] + a[3 * k + 1] * sa[1] + a[3 * k + 2] * sa[2]) / (l[j] - l[k]);
#pragma unroll
        for (int r = 0; r < 3; ++r) vec[r + 3 * j].d[q] += coef * a[r + 3 * k];
      }
    }
  }
}

}  // namespace rflu
