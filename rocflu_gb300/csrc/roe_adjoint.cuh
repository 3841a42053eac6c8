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

__host__ __device__ inline double sgn1(double x) { return (x < 0.0) ? -1.0 : 1.0; }

__host__ __device__ inline void roe2Adjoint(double g, double cp, double eps, double dissFact, double nx, double ny,
                                            double nz, double nm, const double *L, const double *R,
                                            const double *fbar, double *Lb, double *Rb) {
  // ---------------- forward ----------------
  const double rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
  const double rr = R[0], ur = R[1], vr = R[2], wr = R[3], pr = R[4];
  const double gc = cp - cp / g;
  const double tl = pl / (rl * gc), tr = pr / (rr * gc);
  const double Hl = cp * tl + 0.5 * (ul * ul + vl * vl + wl * wl);
  const double Hr = cp * tr + 0.5 * (ur * ur + vr * vr + wr * wr);
  const double ql = ul * nx + vl * ny + wl * nz;
  const double qr = ur * nx + vr * ny + wr * nz;
  const double rh = sqrt(rl * rr);
  const double wt = rl / (rl + rh), w1 = 1.0 - wt;
  const double uh = wt * ul + w1 * ur, vh = wt * vl + w1 * vr, wh = wt * wl + w1 * wr;
  const double Hh = wt * Hl + w1 * Hr;
  const double qh = uh * nx + vh * ny + wh * nz;
  const double sh = 0.5 * (uh * uh + vh * vh + wh * wh);
  const double ah = sqrt((g - 1.0) * (Hh - sh));
  const double L1 = fabs(qh - ah), L2 = fabs(qh), L5 = fabs(qh + ah);
  const double efc = eps * L5;
  const bool k1 = L1 > efc, k2 = L2 > efc, k5 = L5 > efc;
  const double l1 = k1 ? L1 : (L1 * L1 + efc * efc) / (2.0 * efc);
  const double l2 = k2 ? L2 : (L2 * L2 + efc * efc) / (2.0 * efc);
  const double l5 = k5 ? L5 : (L5 * L5 + efc * efc) / (2.0 * efc);
  const double dr = rr - rl, du = ur - ul, de = vr - vl, dw = wr - wl, dp = pr - pl;
  const double dq = du * nx + de * ny + dw * nz;
  const double den = 2.0 * ah * ah;
  const double dv1 = (dp - rh * ah * dq) / den;
  const double dv5 = (dp + rh * ah * dq) / den;
  const double dv2 = dr - dp / (ah * ah);
  const double t1 = l1 * dv1, t2 = l2 * dv2, t3 = l2 * rh, t5 = l5 * dv5;

  // ---------------- reverse ----------------
  const double A = 0.5 * nm, B = 0.5 * dissFact * nm;
  const double F1 = fbar[0], F2 = fbar[1], F3 = fbar[2], F4 = fbar[3], F5 = fbar[4];
  double rlb = 0, ulb = 0, vlb = 0, wlb = 0, plb = 0, Hlb = 0, qlb = 0;
  double rrb = 0, urb = 0, vrb = 0, wrb = 0, prb = 0, Hrb = 0, qrb = 0;
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
  const double D1 = -B * F1, D2 = -B * F2, D3 = -B * F3, D4 = -B * F4, D5 = -B * F5;
  double t1b = D1 + D2 * (uh - nx * ah) + D3 * (vh - ny * ah) + D4 * (wh - nz * ah) + D5 * (Hh - qh * ah);
  double t2b = D1 + D2 * uh + D3 * vh + D4 * wh + D5 * sh;
  double t3b = D2 * (du - nx * dq) + D3 * (de - ny * dq) + D4 * (dw - nz * dq) +
               D5 * (uh * du + vh * de + wh * dw - qh * dq);
  double t5b = D1 + D2 * (uh + nx * ah) + D3 * (vh + ny * ah) + D4 * (wh + nz * ah) + D5 * (Hh + qh * ah);
  const double t125 = t1 + t2 + t5;
  double uhb = D2 * t125 + D5 * t3 * du;
  double vhb = D3 * t125 + D5 * t3 * de;
  double whb = D4 * t125 + D5 * t3 * dw;
  double ahb = (t5 - t1) * (D2 * nx + D3 * ny + D4 * nz) + D5 * (t5 - t1) * qh;
  double Hhb = D5 * (t1 + t5);
  double qhb = D5 * (-t1 * ah - t3 * dq + t5 * ah);
  double shb = D5 * t2;
  double dub = D2 * t3 + D5 * t3 * uh;
  double deb = D3 * t3 + D5 * t3 * vh;
  double dwb = D4 * t3 + D5 * t3 * wh;
  double dqb = -t3 * (D2 * nx + D3 * ny + D4 * nz) - D5 * t3 * qh;
  // t1 = l1 dv1, t2 = l2 dv2, t3 = l2 rh, t5 = l5 dv5
  double l1b = t1b * dv1, l2b = t2b * dv2 + t3b * rh, l5b = t5b * dv5;
  double dv1b = t1b * l1, dv2b = t2b * l2, dv5b = t5b * l5;
  double rhb = t3b * l2;
  // dv1, dv5, dv2
  double dpb = (dv1b + dv5b) / den - dv2b / (ah * ah);
  rhb += (-dv1b + dv5b) * ah * dq / den;
  ahb += dv1b * (-rh * dq / den - 2.0 * dv1 / ah) + dv5b * (rh * dq / den - 2.0 * dv5 / ah) +
         dv2b * (2.0 * dp / (ah * ah * ah));
  dqb += (-dv1b + dv5b) * rh * ah / den;
  double drb = dv2b;
  dub += dqb * nx;
  deb += dqb * ny;
  dwb += dqb * nz;
  // entropy fix
  double L1b = 0, L2b = 0, L5b = 0, efcb = 0;
  if (k1) L1b += l1b; else { L1b += l1b * L1 / efc; efcb += l1b * (efc * efc - L1 * L1) / (2.0 * efc * efc); }
  if (k2) L2b += l2b; else { L2b += l2b * L2 / efc; efcb += l2b * (efc * efc - L2 * L2) / (2.0 * efc * efc); }
  if (k5) L5b += l5b; else { L5b += l5b * L5 / efc; efcb += l5b * (efc * efc - L5 * L5) / (2.0 * efc * efc); }
  L5b += efcb * eps;
  const double s1 = sgn1(qh - ah), s2 = sgn1(qh), s5 = sgn1(qh + ah);
  qhb += L1b * s1 + L2b * s2 + L5b * s5;
  ahb += -L1b * s1 + L5b * s5;
  // ah = sqrt((g-1)(Hh - sh))
  const double ah2b = ahb / (2.0 * ah);
  Hhb += ah2b * (g - 1.0);
  shb -= ah2b * (g - 1.0);
  uhb += shb * uh + qhb * nx;
  vhb += shb * vh + qhb * ny;
  whb += shb * wh + qhb * nz;
  // Roe averages
  const double wtb = uhb * (ul - ur) + vhb * (vl - vr) + whb * (wl - wr) + Hhb * (Hl - Hr);
  ulb += uhb * wt; urb += uhb * w1;
  vlb += vhb * wt; vrb += vhb * w1;
  wlb += whb * wt; wrb += whb * w1;
  Hlb += Hhb * wt; Hrb += Hhb * w1;
  const double s = rl + rh;
  rlb += wtb * rh / (s * s);
  rhb += -wtb * rl / (s * s);
  rlb += rhb * rr / (2.0 * rh);
  rrb += rhb * rl / (2.0 * rh);
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
