"""Tangent (JVP) and discrete adjoint (VJP) of the second-order residual.

* dot-product test: <lambda, J v> = <J^T lambda, v> to round-off;
* FP64 central finite differences (eps = 1e-6) against the VJP;
* the boundary-pressure functional's gradient against finite differences.
"""
import numpy as np
import pytest

from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu

FLUXES = [(cases.DISCR_ROE, "roe"), (cases.DISCR_HLLC, "hllc"), (cases.DISCR_AUSM, "ausm")]


def _case(discr, reconst, n=4, patch_order=2):
    num = cases.Numerics(space_order=2, space_discr=discr, reconst=reconst)
    c = cases.adjoint_tets(n, num=num)
    for p in c.patches:
        p.order = patch_order
    return c


def _dirs(case, k, seed):
    rng = np.random.default_rng(seed)
    scale = np.abs(case.cv0).mean(axis=0)
    return [rng.standard_normal(case.cv0.shape) * scale for _ in range(k)]


@pytest.mark.parametrize("discr,name", FLUXES)
@pytest.mark.parametrize("reconst", [cases.RECONST_NONE, cases.RECONST_VENKAT, cases.RECONST_BJ_COMP])
@pytest.mark.parametrize("patch_order", [1, 2])
def test_dot_product(gpu_lib, discr, name, reconst, patch_order):
    c = _case(discr, reconst, patch_order=patch_order)
    r = gpu.Region(c, "fp64")
    rng = np.random.default_rng(7)
    for v in _dirs(c, 3, 1):
        lam = rng.standard_normal(c.cv0.shape)
        jv = r.jvp(c.cv0, v)
        jtl = r.vjp(c.cv0, lam)
        a, b = (lam * jv).sum(), (jtl * v).sum()
        assert abs(a - b) <= 1e-11 * max(abs(a), abs(b), 1e-30), (a, b)


def test_tangent_covers_eigen_frame_limiter(gpu_lib):
    """RECONST 10: the tangent differentiates through the Jacobi eigen-solve;
    checked against central differences."""
    c = _case(cases.DISCR_HLLC, cases.RECONST_BJ)
    r = gpu.Region(c, "fp64")
    v = _dirs(c, 1, 5)[0]
    eps = 1e-7
    jv = r.jvp(c.cv0, v)
    rp, _ = r.residual(c.cv0 + eps * v, with_grad=False)
    rm, _ = r.residual(c.cv0 - eps * v, with_grad=False)
    fd = (rp - rm) / (2 * eps)
    err = np.abs(fd - jv).max() / np.abs(jv).max()
    assert err < 1e-4, err


@pytest.mark.parametrize("discr,name", FLUXES)
def test_vjp_vs_central_differences(gpu_lib, discr, name):
    """64 random directions, eps = 1e-6 relative to the state's scale:
    <lambda, (R(U+eps v) - R(U-eps v)) / 2 eps> against <J^T lambda, v>."""
    c = _case(discr, cases.RECONST_VENKAT)
    r = gpu.Region(c, "fp64")
    lam = np.random.default_rng(11).standard_normal(c.cv0.shape)
    g = r.vjp(c.cv0, lam)
    eps = 1e-6
    errs = []
    for v in _dirs(c, 64, 3):
        rp, _ = r.residual(c.cv0 + eps * v, with_grad=False)
        rm, _ = r.residual(c.cv0 - eps * v, with_grad=False)
        fd = (lam * (rp - rm)).sum() / (2 * eps)
        ad = (g * v).sum()
        errs.append(abs(fd - ad) / max(abs(ad), 1e-30))
    errs = np.array(errs)
    # directions whose +-eps perturbation crosses a limiter/flux branch switch
    # are not differentiable there; all others agree to 1e-6
    assert np.median(errs) < 1e-7, errs
    assert (errs < 1e-6).mean() >= 0.9, errs


def test_patch_pressure_gradient(gpu_lib):
    c = _case(cases.DISCR_ROE, cases.RECONST_VENKAT)
    r = gpu.Region(c, "fp64")
    ip = 1  # x = 1 patch
    J, g = r.patch_pressure(c.cv0, ip)
    assert J > 0
    eps = 1e-6
    for v in _dirs(c, 8, 9):
        jp, _ = r.patch_pressure(c.cv0 + eps * v, ip, with_grad=False)
        jm, _ = r.patch_pressure(c.cv0 - eps * v, ip, with_grad=False)
        fd = (jp - jm) / (2 * eps)
        ad = (g * v).sum()
        assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-12, (fd, ad)


def test_adjoint_rejects_eigen_frame(gpu_lib):
    c2 = _case(cases.DISCR_ROE, cases.RECONST_BJ)
    for prec in ("fp64", "mixed"):
        with pytest.raises(gpu.RfluError):
            gpu.Region(c2, prec).vjp(c2.cv0, c2.cv0)


# Mixed precision: the adjoint and tangent kernels evaluate the flux,
# reconstruction and limiter Jacobians in FP32 (the mixed primal's
# arithmetic) and the cons -> prim Jacobian in FP64.


@pytest.mark.parametrize("discr,name", FLUXES)
@pytest.mark.parametrize("reconst", [cases.RECONST_NONE, cases.RECONST_VENKAT, cases.RECONST_BJ_COMP])
def test_mixed_dot_product(gpu_lib, discr, name, reconst):
    """<lambda, J v> = <J^T lambda, v> for the mixed tangent and adjoint, to
    FP32 accumulation: 1e-5 of the summed magnitudes of the products (the
    sums cancel, so a bound relative to the result would measure the
    cancellation, not the adjoint)."""
    c = _case(discr, reconst)
    r = gpu.Region(c, "mixed")
    rng = np.random.default_rng(7)
    for v in _dirs(c, 3, 1):
        lam = rng.standard_normal(c.cv0.shape)
        jv, jtl = r.jvp(c.cv0, v), r.vjp(c.cv0, lam)
        a, b = (lam * jv).sum(), (jtl * v).sum()
        scale = max(np.abs(lam * jv).sum(), np.abs(jtl * v).sum())
        assert abs(a - b) <= 1e-5 * scale, (a, b, scale)


@pytest.mark.parametrize("discr,name", FLUXES)
@pytest.mark.parametrize("reconst", [cases.RECONST_VENKAT, cases.RECONST_BJ_COMP])
def test_mixed_vjp_against_fp64(gpu_lib, discr, name, reconst):
    """The mixed VJP against the FP64 VJP and against FP64 central
    differences (eps = 1e-6) of the FP64 residual on 16 directions: the
    mixed Jacobian is the FP64 one to FP32 rounding (median relative
    disagreement below 1e-4)."""
    c = _case(discr, reconst)
    rm, r64 = gpu.Region(c, "mixed"), gpu.Region(c, "fp64")
    rng = np.random.default_rng(11)
    lam = rng.standard_normal(c.cv0.shape)
    gm, g64 = rm.vjp(c.cv0, lam), r64.vjp(c.cv0, lam)
    assert np.isfinite(gm).all()
    assert np.abs(gm - g64).max() <= 2e-3 * np.abs(g64).max()
    errs = []
    eps = 1e-6
    for v in _dirs(c, 16, 3):
        rp, _ = r64.residual(c.cv0 + eps * v, with_grad=False)
        rmn, _ = r64.residual(c.cv0 - eps * v, with_grad=False)
        fd = (lam * (rp - rmn)).sum() / (2 * eps)
        errs.append(abs(fd - (gm * v).sum()) / abs(fd))
    assert np.median(errs) < 1e-4, errs


def test_mixed_patch_pressure_gradient(gpu_lib):
    c = _case(cases.DISCR_HLLC, cases.RECONST_VENKAT)
    Jm, gm = gpu.Region(c, "mixed").patch_pressure(c.cv0, 1)
    J64, g64 = gpu.Region(c, "fp64").patch_pressure(c.cv0, 1)
    assert abs(Jm - J64) <= 1e-6 * abs(J64)
    assert np.abs(gm - g64).max() <= 1e-4 * np.abs(g64).max()


@pytest.mark.parametrize("reconst", [cases.RECONST_BJ_COMP, cases.RECONST_VENKAT])
def test_adjoint_finite_with_tiny_differences(gpu_lib, reconst):
    """A state whose neighbour differences are ~1e-200 (the far field ahead
    of a wave): the limiter's active branch has d2 ~ 1e-200 and, at a local
    extreme, dext = 0; the VJP and the functional's gradient stay finite."""
    c = _case(cases.DISCR_HLLC, reconst)
    rng = np.random.default_rng(4)
    cv = np.tile(c.cv0.mean(axis=0), (c.cv0.shape[0], 1))
    cv[:, 1:4] += 1e-200 * rng.standard_normal((cv.shape[0], 3))
    r = gpu.Region(c, "fp64")
    g = r.vjp(cv, rng.standard_normal(cv.shape))
    assert np.isfinite(g).all()
    _, gp = r.patch_pressure(cv, 1)
    assert np.isfinite(gp).all()
