"""The configurations at their full sizes, through properties that do not
depend on the mesh size (the element-by-element parity with the oracle runs
on smaller meshes in test_gpu_parity.py):

* C3, 128^3 hexes (2,097,152 cells), shock-sphere, HLLC + BJ eigenframe
  limiter: the mixed path's density and pressure L1 error against the FP64
  path after 10 steps and after the configured 500 steps (target <= 1e-5),
  and bit-identical reruns (no atomics anywhere on the path);
* C2 mesh, 64^3 x 6 jittered tetrahedra (1,572,864 cells), HLLC +
  Venkatakrishnan, a p = 4 blast: a closed slip-wall box, so every step
  conserves the totals of mass and energy as long as no cell takes the
  reference's positivity floor (which sets the energy).  On this mesh the
  reference's limiters (face offsets of the wrong sign) let the p = 100
  blast reconstruct negative face pressures within a few steps, floor one
  cell at p = 10 in step 2, and give 2 non-finite cells in step 3 at p = 2,
  the CPU oracle and the device alike; p = 4 stays clean for 3 steps;
* C4, 32^3 x 6 jittered tetrahedra (196,608 cells), Roe + componentwise BJ
  and BJ with the eigen-frame velocity limiter: the tangent/adjoint
  dot-product identity;
* C5, 64^3 hexes (262,144 cells), HLLC + BJ (eigen-frame) blast: the
  time-unrolled adjoint's value and gradient do not depend on the
  checkpoint interval.
"""
import numpy as np
import pytest

from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu


def test_c3_mixed_accuracy_and_reruns(gpu_lib):
    c = cases.shock_sphere(128)
    probe = gpu.Region(c, "fp64")
    c.num.dt_imposed = probe.timestep(1.0)  # the imposed first step = the CFL step
    probe.close()
    r64, rm = gpu.Region(c, "fp64"), gpu.Region(c, "mixed")
    for r in (r64, rm):
        n, _, rc = r.step(10, 0.0)
        assert n == 10 and rc == 0
    cv64, dv64 = r64.download()
    cvm, dvm = rm.download()
    assert np.isfinite(cvm).all()
    assert np.abs(cvm[:, 0] - cv64[:, 0]).mean() <= 1e-5
    assert np.abs(dvm[:, 0] - dv64[:, 0]).mean() <= 1e-5
    # a rerun from the same state gives the same bits
    for r, ref in ((rm, cvm), (r64, cv64)):
        r.upload(c.cv0)
        r.step(10, 0.0)
        again, _ = r.download()
        np.testing.assert_array_equal(again, ref)


def test_c3_mixed_accuracy_after_500_steps(gpu_lib):
    """The configuration's full run: 500 steps of the mixed and the FP64
    path from the same initial state (CFL time step each step); the shock
    crosses the sphere on the way.  L1 of density and pressure against the
    FP64 path <= 1e-5, no invalid or floored cells in either."""
    c = cases.shock_sphere(128)
    probe = gpu.Region(c, "fp64")
    c.num.dt_imposed = probe.timestep(1.0)
    probe.close()
    out = {}
    for prec in ("fp64", "mixed"):
        r = gpu.Region(c, prec)
        n, t, rc = r.step(500, 0.0)
        st = r.status()
        assert n == 500 and rc == 0 and st["nanCells"] == 0 and st["posFixCells"] == 0, st
        out[prec] = r.download() + (t,)
        r.close()
    (cv64, dv64, t64), (cvm, dvm, tm) = out["fp64"], out["mixed"]
    assert abs(tm - t64) <= 1e-5 * t64  # the mixed time step is an FP32 sum
    assert np.abs(cvm[:, 0] - cv64[:, 0]).mean() <= 1e-5
    assert np.abs(dvm[:, 0] - dv64[:, 0]).mean() <= 1e-5


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_c2_tets_closed_box_conserves(gpu_lib, prec, tol):
    c = cases.blast_tets(64, p_in=4.0)
    vol = gpu.Setup(c).vol
    r = gpu.Region(c, prec)
    m0, e0 = (c.cv0[:, 0] * vol).sum(), (c.cv0[:, 4] * vol).sum()
    dt = r.timestep(1.0)
    r.run_fixed_dt(3, dt)
    cv, _ = r.download()
    st = r.status()
    assert st["nanCells"] == 0 and st["posFixCells"] == 0
    assert np.isfinite(cv).all()
    assert abs((cv[:, 0] * vol).sum() - m0) / m0 < tol
    assert abs((cv[:, 4] * vol).sum() - e0) / e0 < tol


@pytest.mark.parametrize("reconst", [cases.RECONST_BJ_COMP, cases.RECONST_BJ])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-11), ("mixed", 1e-5)])
def test_c4_dot_product(gpu_lib, prec, tol, reconst):
    """<lambda, J v> = <J^T lambda, v> to the mode's accumulation error,
    relative to the summed magnitudes of the products; componentwise BJ and
    BJ with the eigen-frame velocity limiter."""
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_ROE, reconst=reconst)
    c = cases.adjoint_tets(32, num=num)
    r = gpu.Region(c, prec)
    rng = np.random.default_rng(3)
    scale = np.abs(c.cv0).mean(axis=0)
    for _ in range(2):
        v = rng.standard_normal(c.cv0.shape) * scale
        lam = rng.standard_normal(c.cv0.shape)
        jv, jtl = r.jvp(c.cv0, v), r.vjp(c.cv0, lam)
        a, b = (lam * jv).sum(), (jtl * v).sum()
        mag = max(np.abs(lam * jv).sum(), np.abs(jtl * v).sum())
        assert abs(a - b) <= tol * mag, (a, b, mag)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_c5_unrolled_adjoint_checkpoint_invariance(gpu_lib, prec):
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ, cfl=0.4)
    c = cases.blast_hex(64, num=num, p_in=10.0, radius=0.15)
    r = gpu.Region(c, prec)
    dt = r.timestep(1.0)
    J1, g1, _ = r.unrolled_adjoint(c.cv0, 20, dt, 4, 1)
    J2, g2, _ = r.unrolled_adjoint(c.cv0, 20, dt, 20, 1)
    assert np.isfinite(g1).all()
    assert J1 == J2
    np.testing.assert_array_equal(g1, g2)
