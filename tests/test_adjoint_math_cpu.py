"""The hand-written reverse sweep of the second-order Roe flux against the
transposed Jacobian obtained with forward-mode dual numbers on the same
point-wise flux code (both compiled for the host; no GPU needed)."""
import os
import subprocess

import numpy as np

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "rocflu_gb300", "csrc")

HARNESS = r"""
#define __host__
#define __device__
#include <cstdio>
#include <random>
#include "physics.cuh"
#include "dual.cuh"
#include "roe_adjoint.cuh"
using namespace rflu;
int main() {
  std::mt19937_64 rng(5);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  const double g = 1.4, cp = 3.5, eps = 0.05, diss = 1.0;
  double worst = 0.0;
  for (int trial = 0; trial < 2000; ++trial) {
    double L[5] = {1.0 + 0.3 * U(rng), 0.5 * U(rng), 0.5 * U(rng), 0.5 * U(rng), 1.0 + 0.3 * U(rng)};
    double R[5] = {1.0 + 0.3 * U(rng), 0.5 * U(rng), 0.5 * U(rng), 0.5 * U(rng), 1.0 + 0.3 * U(rng)};
    if (trial % 3 == 0) { L[1] = 1.5 + U(rng); R[1] = 1.5 + U(rng); }   /* supersonic-ish */
    if (trial % 5 == 0) { R[1] = L[1]; R[2] = L[2]; R[3] = L[3]; }     /* entropy-fix branches */
    double n[3] = {U(rng), U(rng), U(rng)};
    double m = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (double &x : n) x /= m;
    const double nm = 0.3 + 0.5 * (U(rng) + 1.0);
    double fbar[5];
    for (double &x : fbar) x = U(rng);
    double Lb[5], Rb[5];
    roe2Adjoint(g, cp, eps, diss, n[0], n[1], n[2], nm, L, R, fbar, Lb, Rb);
    typedef Dual<10> D;
    D a[5], b[5], f[5];
    for (int k = 0; k < 5; ++k) { a[k] = D::seed(L[k], k); b[k] = D::seed(R[k], 5 + k); }
    D G(g), CP(cp), gc = CP - CP / G;
    D tl = a[4] / (a[0] * gc), tr = b[4] / (b[0] * gc);
    D Hl = perfHo(CP, tl, a[1], a[2], a[3]), Hr = perfHo(CP, tr, b[1], b[2], b[3]);
    roeFlux(G, D(eps), D(diss), D(n[0]), D(n[1]), D(n[2]), D(nm), a[0], a[1], a[2], a[3], a[4], Hl, b[0], b[1], b[2],
            b[3], b[4], Hr, f);
    for (int j = 0; j < 10; ++j) {
      double s = 0.0;
      for (int k = 0; k < 5; ++k) s += fbar[k] * f[k].d[j];
      double h = (j < 5) ? Lb[j] : Rb[j - 5];
      double err = fabs(s - h) / (1.0 + fabs(s));
      if (err > worst) worst = err;
    }
  }
  printf("%.3e\n", worst);
  return 0;
}
"""


def test_roe_reverse_sweep_matches_dual_jacobian(tmp_path):
    src = tmp_path / "roe_adj.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "roe_adj"
    subprocess.run(["g++", "-O1", "-std=c++17", "-w", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    assert float(out) < 1e-12, out
