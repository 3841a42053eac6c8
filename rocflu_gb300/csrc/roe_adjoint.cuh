// Hand-written reverse mode of the second-order Roe face flux.
//
// Forward: the Roe flux with the Harten-Hyman entropy fix of
// RFLU_ROE_ComputeFlux2_TCP (modflu/RFLU_ModRoeFlux.F90:2513-2867) on the
// reconstructed states L = (rl,ul,vl,wl,pl), R = (rr,ur,vr,wr,pr), with
// T = p/(rho*gc), H = cp*T + |u|^2/2 (gc = cp - cp/gamma).
// Reverse: given fbar = dJ/dF (5), accumulates dJ/dL and dJ/dR, i.e. the
// transposed flux Jacobian applied to fbar, in one forward sweep that keeps
// its intermediates in registers and one backward sweep.  Derivatives follow
// the branch the forward sweep takes (entropy fix, absolute values).
#pragma once
#include <cmath>

namespace rflu {

template <typename T>
__host__ __device__ inline T sgn1(T x) { return (x < T(0)) ? T(-1) : T(1); }

// T: double in the FP64 modes, float in the mixed mode (the arithmetic of
// each mode's flux); the numerics parameters arrive in double.
template <typename T>
__host__ __device__ inline void roe2Adjoint(double gD, double cpD, double epsD, double dissFactD, T nx, T ny, T nz,
                                            T nm, const T *L, const T *R, const T *fbar, T *Lb, T *Rb) {
  const T g = T(gD), cp = T(cpD), eps = T(epsD), dissFact = T(dissFactD);
  // ---------------- forward ----------------
  const T rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
  const T rr = R[0], ur = R[1], vr = R[2], wr = R[3], pr = R[4];
  const T gc = cp - cp / g;
  const T tl = pl / (rl * gc), tr = pr / (rr * gc);
  const T Hl = cp * tl + T(0.5) * (ul * ul + vl * vl + wl * wl);
  const T Hr = cp * tr + T(0.5) * (ur * ur + vr * vr + wr * wr);
  const T ql = ul * nx + vl * ny + wl * nz;
  const T qr = ur * nx + vr * ny + wr * nz;
  const T rh = sqrt(rl * rr);
  const T wt = rl / (rl + rh), w1 = T(1.0) - wt;
  const T uh = wt * ul + w1 * ur, vh = wt * vl + w1 * vr, wh = wt * wl + w1 * wr;
  const T Hh = wt * Hl + w1 * Hr;
  const T qh = uh * nx + vh * ny + wh * nz;
  const T sh = T(0.5) * (uh * uh + vh * vh + wh * wh);
  const T ah = sqrt((g - T(1.0)) * (Hh - sh));
  const T L1 = fabs(qh - ah), L2 = fabs(qh), L5 = fabs(qh + ah);
  const T efc = eps * L5;
  const bool k1 = L1 > efc, k2 = L2 > efc, k5 = L5 > efc;
  const T l1 = k1 ? L1 : (L1 * L1 + efc * efc) / (T(2.0) * efc);
  const T l2 = k2 ? L2 : (L2 * L2 + efc * efc) / (T(2.0) * efc);
  const T l5 = k5 ? L5 : (L5 * L5 + efc * efc) / (T(2.0) * efc);
  const T dr = rr - rl, du = ur - ul, de = vr - vl, dw = wr - wl, dp = pr - pl;
  const T dq = du * nx + de * ny + dw * nz;
  const T den = T(2.0) * ah * ah;
  const T dv1 = (dp - rh * ah * dq) / den;
  const T dv5 = (dp + rh * ah * dq) / den;
  const T dv2 = dr - dp / (ah * ah);
  const T t1 = l1 * dv1, t2 = l2 * dv2, t3 = l2 * rh, t5 = l5 * dv5;

  // ---------------- reverse ----------------
  const T A = T(0.5) * nm, B = T(0.5) * dissFact * nm;
  const T F1 = fbar[0], F2 = fbar[1], F3 = fbar[2], F4 = fbar[3], F5 = fbar[4];
  T rlb = 0, ulb = 0, vlb = 0, wlb = 0, plb = 0, Hlb = 0, qlb = 0;
  T rrb = 0, urb = 0, vrb = 0, wrb = 0, prb = 0, Hrb = 0, qrb = 0;
  // convective part, flx += fc
  qlb += A * (rl * F1 + rl * ul * F2 + rl * vl * F3 + rl * wl * F4 + rl * Hl * F5);
  rlb += A * (ql * F1 + ql * ul * F2 + ql * vl * F3 + ql * wl * F4 + ql * Hl * F5);
  ulb += A * ql * rl * F2;
  vlb += A * ql * rl * F3;
  wlb += A * ql * rl * F4;
  Hlb += A * ql * rl * F5;
  plb += A * (nx * F2 + ny * F3 + nz * F4);
  qrb += A * (rr * F1 + rr * ur * F2 + rr * vr * F3 + rr * wr * F4 + rr * Hr * F5);
  rrb += A * (qr * F1 + qr * ur * F2 + qr * vr * F3 + qr * wr * F4 + qr * Hr * F5);
  urb += A * qr * rr * F2;
  vrb += A * qr * rr * F3;
  wrb += A * qr * rr * F4;
  Hrb += A * qr * rr * F5;
  prb += A * (nx * F2 + ny * F3 + nz * F4);
  // dissipative part, flx -= fd
  const T D1 = -B * F1, D2 = -B * F2, D3 = -B * F3, D4 = -B * F4, D5 = -B * F5;
  T t1b = D1 + D2 * (uh - nx * ah) + D3 * (vh - ny * ah) + D4 * (wh - nz * ah) + D5 * (Hh - qh * ah);
  T t2b = D1 + D2 * uh + D3 * vh + D4 * wh + D5 * sh;
  T t3b = D2 * (du - nx * dq) + D3 * (de - ny * dq) + D4 * (dw - nz * dq) +
               D5 * (uh * du + vh * de + wh * dw - qh * dq);
  T t5b = D1 + D2 * (uh + nx * ah) + D3 * (vh + ny * ah) + D4 * (wh + nz * ah) + D5 * (Hh + qh * ah);
  const T t125 = t1 + t2 + t5;
  T uhb = D2 * t125 + D5 * t3 * du;
  T vhb = D3 * t125 + D5 * t3 * de;
  T whb = D4 * t125 + D5 * t3 * dw;
  T ahb = (t5 - t1) * (D2 * nx + D3 * ny + D4 * nz) + D5 * (t5 - t1) * qh;
  T Hhb = D5 * (t1 + t5);
  T qhb = D5 * (-t1 * ah - t3 * dq + t5 * ah);
  T shb = D5 * t2;
  T dub = D2 * t3 + D5 * t3 * uh;
  T deb = D3 * t3 + D5 * t3 * vh;
  T dwb = D4 * t3 + D5 * t3 * wh;
  T dqb = -t3 * (D2 * nx + D3 * ny + D4 * nz) - D5 * t3 * qh;
  // t1 = l1 dv1, t2 = l2 dv2, t3 = l2 rh, t5 = l5 dv5
  T l1b = t1b * dv1, l2b = t2b * dv2 + t3b * rh, l5b = t5b * dv5;
  T dv1b = t1b * l1, dv2b = t2b * l2, dv5b = t5b * l5;
  T rhb = t3b * l2;
  // dv1, dv5, dv2
  T dpb = (dv1b + dv5b) / den - dv2b / (ah * ah);
  rhb += (-dv1b + dv5b) * ah * dq / den;
  ahb += dv1b * (-rh * dq / den - T(2.0) * dv1 / ah) + dv5b * (rh * dq / den - T(2.0) * dv5 / ah) +
         dv2b * (T(2.0) * dp / (ah * ah * ah));
  dqb += (-dv1b + dv5b) * rh * ah / den;
  T drb = dv2b;
  dub += dqb * nx;
  deb += dqb * ny;
  dwb += dqb * nz;
  // entropy fix
  T L1b = 0, L2b = 0, L5b = 0, efcb = 0;
  if (k1) L1b += l1b; else { L1b += l1b * L1 / efc; efcb += l1b * (efc * efc - L1 * L1) / (T(2.0) * efc * efc); }
  if (k2) L2b += l2b; else { L2b += l2b * L2 / efc; efcb += l2b * (efc * efc - L2 * L2) / (T(2.0) * efc * efc); }
  if (k5) L5b += l5b; else { L5b += l5b * L5 / efc; efcb += l5b * (efc * efc - L5 * L5) / (T(2.0) * efc * efc); }
  L5b += efcb * eps;
  const T s1 = sgn1(qh - ah), s2 = sgn1(qh), s5 = sgn1(qh + ah);
  qhb += L1b * s1 + L2b * s2 + L5b * s5;
  ahb += -L1b * s1 + L5b * s5;
  // ah = sqrt((g-1)(Hh - sh))
  const T ah2b = ahb / (T(2.0) * ah);
  Hhb += ah2b * (g - T(1.0));
  shb -= ah2b * (g - T(1.0));
  uhb += shb * uh + qhb * nx;
  vhb += shb * vh + qhb * ny;
  whb += shb * wh + qhb * nz;
  // Roe averages
  const T wtb = uhb * (ul - ur) + vhb * (vl - vr) + whb * (wl - wr) + Hhb * (Hl - Hr);
  ulb += uhb * wt; urb += uhb * w1;
  vlb += vhb * wt; vrb += vhb * w1;
  wlb += whb * wt; wrb += whb * w1;
  Hlb += Hhb * wt; Hrb += Hhb * w1;
  const T s = rl + rh;
  rlb += wtb * rh / (s * s);
  rhb += -wtb * rl / (s * s);
  rlb += rhb * rr / (T(2.0) * rh);
  rrb += rhb * rl / (T(2.0) * rh);
  // differences
  rrb += drb; rlb -= drb;
  urb += dub; ulb -= dub;
  vrb += deb; vlb -= deb;
  wrb += dwb; wlb -= dwb;
  prb += dpb; plb -= dpb;
  // normal velocities
  ulb += qlb * nx; vlb += qlb * ny; wlb += qlb * nz;
  urb += qrb * nx; vrb += qrb * ny; wrb += qrb * nz;
  // total enthalpies: H = cp p/(rho gc) + |u|^2/2
  plb += Hlb * cp / (rl * gc);
  rlb -= Hlb * cp * tl / rl;
  ulb += Hlb * ul; vlb += Hlb * vl; wlb += Hlb * wl;
  prb += Hrb * cp / (rr * gc);
  rrb -= Hrb * cp * tr / rr;
  urb += Hrb * ur; vrb += Hrb * vr; wrb += Hrb * wr;
  Lb[0] = rlb; Lb[1] = ulb; Lb[2] = vlb; Lb[3] = wlb; Lb[4] = plb;
  Rb[0] = rrb; Rb[1] = urb; Rb[2] = vrb; Rb[3] = wrb; Rb[4] = prb;
}

}  // namespace rflu
