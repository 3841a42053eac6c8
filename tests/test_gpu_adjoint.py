"""Tangent (JVP) and discrete adjoint (VJP) of the second-order residual.

* dot-product test: <lambda, J v> = <J^T lambda, v> to round-off, every
  limiter (none, Venkatakrishnan, componentwise BJ, BJ with the eigen-frame
  velocity limiter, the simple and XYZ WENO smoothing);
* FP64 central finite differences (eps = 1e-6) against the VJP: every
  direction along which no cell changes its limiter's active branch between
  U - eps v and U + eps v (rflu_gpu_limiter_branches) agrees to 1e-6; the
  others cross a kink of the limiter and are reported, not held to it;
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


WENO = [cases.RECONST_WENO_SIMPLE, cases.RECONST_WENO_XYZ]
ADJ_LIMITERS = [cases.RECONST_NONE, cases.RECONST_VENKAT, cases.RECONST_BJ_COMP, cases.RECONST_BJ] + WENO


def _cd(f, cv, v, eps, richardson):
    """Central difference of f along v; with richardson, extrapolated from
    eps and eps/2 so that the eps^2 term cancels.  The XYZ WENO weights
    1/(t^2 + 1e-15) vary on the scale of the gradient component t itself,
    and the smallest of the 5760 components of the 4^3-tet case is ~1e-5:
    a plain difference at eps = 1e-6 moves it by a tenth of itself (errors
    up to 2e-4); XYZ therefore takes eps = 1e-8 and the extrapolation."""
    d = (f(cv + eps * v) - f(cv - eps * v)) / (2 * eps)
    if not richardson:
        return d
    h = eps / 2
    return (4 * (f(cv + h * v) - f(cv - h * v)) / (2 * h) - d) / 3


def _switches(r, cv, v, eps):
    """Whether any cell's limiter branch differs between cv - eps v, cv and
    cv + eps v."""
    b0 = r.limiter_branches(cv)
    return not (np.array_equal(r.limiter_branches(cv + eps * v), b0) and
                np.array_equal(r.limiter_branches(cv - eps * v), b0))


@pytest.mark.parametrize("discr,name", FLUXES)
@pytest.mark.parametrize("reconst", ADJ_LIMITERS)
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
    """RECONST 10: the tangent differentiates through the eigen-frame of the
    strain rate (first-order perturbation of the Jacobi eigenpairs); checked
    against central differences."""
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
@pytest.mark.parametrize("reconst", [cases.RECONST_VENKAT, cases.RECONST_BJ_COMP, cases.RECONST_BJ] + WENO)
def test_vjp_vs_central_differences(gpu_lib, discr, name, reconst):
    """64 random directions, eps = 1e-6 relative to the state's scale:
    <lambda, (R(U+eps v) - R(U-eps v)) / 2 eps> against <J^T lambda, v>.
    Barth-Jespersen (both forms) and the WENO smoothing (whose simple
    limiter is its one branch): every direction that keeps all limiter
    branches agrees to 1e-6, and at least half of the directions keep them.
    Venkatakrishnan has no branch switch to blame: the reference's factor
    divides by (denominator + 1e-12), so it rises from 0 to 1 within
    |d2| ~ 1e-9, a region of curvature that eps = 1e-6 differences do not
    resolve where a face sits near it; there the median agrees to 1e-7 and
    90% of the directions to 1e-6."""
    c = _case(discr, reconst)
    r = gpu.Region(c, "fp64")
    lam = np.random.default_rng(11).standard_normal(c.cv0.shape)
    g = r.vjp(c.cv0, lam)
    eps = 1e-8 if reconst == cases.RECONST_WENO_XYZ else 1e-6
    errs, sw = [], []
    f = lambda cv: (lam * r.residual(cv, with_grad=False)[0]).sum()  # noqa: E731
    # XYZ: the round-off of the extrapolated difference at eps = 1e-8, a few
    # ulps of the summed |lambda R| over eps, is taken off the error
    ro = 0.0
    if reconst == cases.RECONST_WENO_XYZ:
        ro = 8 * np.finfo(float).eps * np.abs(lam * r.residual(c.cv0, with_grad=False)[0]).sum() / eps
    for v in _dirs(c, 64, 3):
        fd = _cd(f, c.cv0, v, eps, reconst == cases.RECONST_WENO_XYZ)
        ad = (g * v).sum()
        errs.append(max(abs(fd - ad) - ro, 0.0) / max(abs(ad), 1e-30))
        sw.append(_switches(r, c.cv0, v, eps))
    errs, sw = np.array(errs), np.array(sw)
    assert (~sw).sum() >= 32, sw.sum()
    if reconst == cases.RECONST_VENKAT:
        assert np.median(errs[~sw]) < 1e-7, errs
        assert (errs[~sw] < 1e-6).mean() >= 0.9, errs
    else:
        assert (errs[~sw] < 1e-6).all(), (errs[~sw].max(), np.flatnonzero(~sw & (errs >= 1e-6)))


@pytest.mark.parametrize("reconst", [cases.RECONST_VENKAT, cases.RECONST_BJ, cases.RECONST_WENO_XYZ])
def test_patch_pressure_gradient(gpu_lib, reconst):
    c = _case(cases.DISCR_ROE, reconst)
    r = gpu.Region(c, "fp64")
    ip = 1  # x = 1 patch
    J, g = r.patch_pressure(c.cv0, ip)
    assert J > 0
    eps = 1e-8 if reconst == cases.RECONST_WENO_XYZ else 1e-6
    f = lambda cv: r.patch_pressure(cv, ip, with_grad=False)[0]  # noqa: E731
    for v in _dirs(c, 8, 9):
        fd = _cd(f, c.cv0, v, eps, reconst == cases.RECONST_WENO_XYZ)
        ad = (g * v).sum()
        assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-12, (fd, ad)


@pytest.mark.parametrize("reconst", WENO)
def test_weno_tangent_vs_central_differences(gpu_lib, reconst):
    """RECONST 1, 2: the tangent through the WENO averages (weights
    differentiated) against central differences of the residual (XYZ:
    extrapolated, see _cd) along directions in which the simple limiter
    zeroes no gradient (it would make the residual non-differentiable)."""
    c = _case(cases.DISCR_HLLC, reconst)
    r = gpu.Region(c, "fp64")
    eps = 1e-8 if reconst == cases.RECONST_WENO_XYZ else 1e-6
    errs = []
    f = lambda cv: r.residual(cv, with_grad=False)[0]  # noqa: E731
    for v in _dirs(c, 4, 5):
        assert not _switches(r, c.cv0, v, eps)
        jv = r.jvp(c.cv0, v)
        fd = _cd(f, c.cv0, v, eps, reconst == cases.RECONST_WENO_XYZ)
        errs.append(np.abs(fd - jv).max() / np.abs(jv).max())
    assert max(errs) < 1e-6, errs


def test_weno_positivity_zeroing_has_no_derivative(gpu_lib):
    """A state scaled by 5e-4 + x^2 (density and pressure fall towards x = 0
    at fixed velocity and temperature; convex, so that a cell's gradient
    overshoots towards x = 0, and of one sign, which the WENO averages
    keep): the simple limiter zeroes density and pressure gradients near
    x = 0 (reported as branch -2).  The tangent and the adjoint stay each
    other's transpose, and differences along the directions that keep every
    branch agree with the adjoint."""
    c = _case(cases.DISCR_HLLC, cases.RECONST_WENO_XYZ)
    x = gpu.Setup(c).cofg
    ramp = 5e-4 + x[:, 0] ** 2
    cv = c.cv0 * ramp[:, None]
    r = gpu.Region(c, "fp64")
    b = r.limiter_branches(cv)
    assert (b[:, 0, 0] == -2).any() and set(np.unique(b[:, :, 0])) <= {-2, -1}
    rng = np.random.default_rng(2)
    lam = rng.standard_normal(cv.shape)
    g = r.vjp(cv, lam)
    eps = 1e-8
    f = lambda u: (lam * r.residual(u, with_grad=False)[0]).sum()  # noqa: E731
    kept = 0
    for v in _dirs(c, 8, 8):
        v = v * ramp[:, None]
        jv = r.jvp(cv, v)
        a, bb = (lam * jv).sum(), (g * v).sum()
        assert abs(a - bb) <= 1e-11 * max(abs(a), abs(bb)), (a, bb)
        if _switches(r, cv, v, eps):
            continue
        kept += 1
        fd = _cd(f, cv, v, eps, True)
        assert abs(fd - bb) <= 1e-6 * abs(bb), (fd, bb)
    assert kept >= 4


def _constrained(which, reconst, prec_case=None):
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=reconst, cfl=0.4, c_reconst=1)
    if which == "tets":
        c = cases.adjoint_tets(4, num=num)  # slip walls on y and z
        for p in c.patches:
            p.order = 2
        return c
    if which == "burning":
        # a burning injection wall: its constraint values follow the pressure
        # of the face's cell
        return cases.open_channel(6, num=num, inflow=cases.BC_INFLOW_VELTEMP)
    # inflow, outflow, farfield, a no-slip wall and a non-burning injection wall
    return cases.open_channel(6, num=num, inflow=cases.BC_INFLOW_VELTEMP, injection=0.0)


@pytest.mark.parametrize("which", ["tets", "channel", "burning"])
@pytest.mark.parametrize("reconst", [cases.RECONST_NONE, cases.RECONST_BJ, cases.RECONST_BJ_COMP, cases.RECONST_WENO_XYZ])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-11), ("mixed", 1e-5)])
def test_constrained_dot_product(gpu_lib, which, reconst, prec, tol):
    """CRECONSTC 1 (gradients constrained at the wall and injection faces):
    the tangent through the constrained fit (dual numbers over the plan's
    rows, the burning injection's values through the face cell's pressure)
    and the adjoint (the plan's rows transposed over the transposed stencil,
    the burning rows gathered by the face cell) are each other's
    transpose."""
    c = _constrained(which, reconst)
    r = gpu.Region(c, prec)
    rng = np.random.default_rng(7)
    for v in _dirs(c, 3, 1):
        lam = rng.standard_normal(c.cv0.shape)
        jv, jtl = r.jvp(c.cv0, v), r.vjp(c.cv0, lam)
        a, b = (lam * jv).sum(), (jtl * v).sum()
        if prec == "fp64":
            assert abs(a - b) <= tol * max(abs(a), abs(b)), (a, b)
        else:
            scale = max(np.abs(lam * jv).sum(), np.abs(jtl * v).sum())
            assert abs(a - b) <= tol * scale, (a, b, scale)


@pytest.mark.parametrize("which", ["tets", "channel", "burning"])
def test_constrained_vjp_vs_central_differences(gpu_lib, which):
    """FP64, componentwise BJ with CRECONSTC 1: the VJP against central
    differences of the residual (eps = 1e-6) on 32 directions; every
    direction that keeps all limiter branches agrees to 1e-6."""
    c = _constrained(which, cases.RECONST_BJ_COMP)
    r = gpu.Region(c, "fp64")
    lam = np.random.default_rng(11).standard_normal(c.cv0.shape)
    g = r.vjp(c.cv0, lam)
    eps = 1e-6
    errs, sw = [], []
    f = lambda cv: (lam * r.residual(cv, with_grad=False)[0]).sum()  # noqa: E731
    for v in _dirs(c, 32, 3):
        fd = _cd(f, c.cv0, v, eps, False)
        ad = (g * v).sum()
        errs.append(abs(fd - ad) / max(abs(ad), 1e-30))
        sw.append(_switches(r, c.cv0, v, eps))
    errs, sw = np.array(errs), np.array(sw)
    assert (~sw).sum() >= 8, sw.sum()
    assert (errs[~sw] < 1e-6).all(), (errs[~sw].max(), np.flatnonzero(~sw & (errs >= 1e-6)))


def test_constrained_burning_vjp_vs_central_differences_unlimited(gpu_lib):
    """FP64, no limiter, CRECONSTC 1 with a burning injection wall: the
    residual is smooth, so every one of 16 directions agrees with central
    differences (Richardson) to 1e-7, among them four that change only the
    energy, hence the pressure, of the cells on the burning wall (z-low)."""
    c = _constrained("burning", cases.RECONST_NONE)
    r = gpu.Region(c, "fp64")
    lam = np.random.default_rng(12).standard_normal(c.cv0.shape)
    g = r.vjp(c.cv0, lam)
    f = lambda cv: (lam * r.residual(cv, with_grad=False)[0]).sum()  # noqa: E731
    zc = c.xyz[c.c2v].mean(axis=1)[:, 2]
    wall = np.isclose(zc, zc.min())
    rng = np.random.default_rng(6)
    dirs = _dirs(c, 12, 5)
    for _ in range(4):
        v = np.zeros_like(c.cv0)
        v[wall, 4] = rng.standard_normal(wall.sum()) * np.abs(c.cv0[:, 4]).mean()
        dirs.append(v)
    for v in dirs:
        fd = _cd(f, c.cv0, v, 1e-5, True)
        ad = (g * v).sum()
        assert abs(fd - ad) <= 1e-7 * max(abs(ad), 1e-30), (fd, ad)


@pytest.mark.parametrize("which", ["channel", "burning"])
def test_constrained_mixed_vjp_against_fp64(gpu_lib, which):
    c = _constrained(which, cases.RECONST_WENO_XYZ)
    lam = np.random.default_rng(3).standard_normal(c.cv0.shape)
    gm, g64 = gpu.Region(c, "mixed").vjp(c.cv0, lam), gpu.Region(c, "fp64").vjp(c.cv0, lam)
    assert np.linalg.norm(gm - g64) <= 1e-4 * np.linalg.norm(g64)


def test_limiter_branches_record(gpu_lib):
    """rflu_gpu_limiter_branches: componentwise BJ reports per variable the
    active face (an index among the cell's faces) and the neighbour holding
    the active extreme; RECONST 10 reports its velocity axes with a side."""
    for reconst in (cases.RECONST_BJ_COMP, cases.RECONST_BJ):
        c = _case(cases.DISCR_ROE, reconst)
        r = gpu.Region(c, "fp64")
        b = r.limiter_branches(c.cv0)
        assert b.shape == (c.n_cells, 5, 2)
        assert (b[..., 0] >= -1).all() and (b[..., 1] >= -1).all() and (b[..., 1] < c.n_cells).all()
        assert (b[..., 0] >= 0).any()
        if reconst == cases.RECONST_BJ:
            sides = b[:, 1:4, 0][b[:, 1:4, 0] >= 0] % 4
            assert set(np.unique(sides)) <= {1, 2} and len(sides) > 0
        else:
            assert (b[:, :, 0] < 4).all()  # tetrahedra: 4 faces
    # the WENO smoothing limits nothing on this state (no zeroed gradient)
    c = _case(cases.DISCR_ROE, cases.RECONST_WENO_SIMPLE)
    b = gpu.Region(c, "fp64").limiter_branches(c.cv0)
    assert (b == -1).all()


# Mixed precision: the adjoint and tangent kernels evaluate the flux,
# reconstruction and limiter Jacobians in FP32 (the mixed primal's
# arithmetic) and the cons -> prim Jacobian in FP64.


@pytest.mark.parametrize("discr,name", FLUXES)
@pytest.mark.parametrize("reconst", ADJ_LIMITERS)
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
@pytest.mark.parametrize("reconst", [cases.RECONST_VENKAT, cases.RECONST_BJ_COMP, cases.RECONST_BJ] + WENO)
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


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_eigen_frame_one_dimensional_velocity(gpu_lib, prec):
    """RECONST 10 on a state whose velocity has an x component only (v = w
    = 0 exactly, u varying in all three directions): the strain rate then
    has an axis along which the velocity does not vary, and the limiter's
    factor on it is a ratio of two rounding residues.  Its derivative (of
    order 1 / rounding, 1e13 here) is held at zero in the tangent and the
    adjoint, so both stay bounded, stay each other's transpose, and follow
    central differences.  The held factor's value is itself a ratio of
    rounding residues, different in FP32 and FP64; it multiplies the idle
    axis's O(1) projection derivative, so the mixed mode's adjoint follows
    the FP64 one only to the share of those terms (2% here)."""
    c = _case(cases.DISCR_HLLC, cases.RECONST_BJ)
    x = gpu.Setup(c).cofg
    cv = c.cv0.copy()
    bg = np.sin(2 * np.pi * x[:, 0] + 0.3) * np.sin(2 * np.pi * x[:, 1] + 0.7) * np.sin(2 * np.pi * x[:, 2] + 1.1)
    cv[:, 0] *= 1 + 0.05 * bg
    cv[:, 1] = 0.2 * cv[:, 0] * (1 + 0.5 * np.roll(bg, 3))
    cv[:, 2:4] = 0.0
    r = gpu.Region(c, prec)
    ref = gpu.Region(c, "fp64")
    rng = np.random.default_rng(3)
    lam = rng.standard_normal(cv.shape)
    g = r.vjp(cv, lam)
    g64 = ref.vjp(cv, lam)
    assert np.abs(g64).max() < 1e3, np.abs(g64).max()
    if prec == "mixed":
        assert np.linalg.norm(g - g64) <= 5e-2 * np.linalg.norm(g64)
        return
    eps = 1e-7
    errs = []
    for v in _dirs(c, 8, 9):
        jv = r.jvp(cv, v)
        a, b = (lam * jv).sum(), (g * v).sum()
        assert abs(a - b) <= 1e-11 * max(abs(a), abs(b)), (a, b)
        rp, _ = r.residual(cv + eps * v, with_grad=False)
        rm, _ = r.residual(cv - eps * v, with_grad=False)
        fd = (rp - rm) / (2 * eps)
        errs.append(np.abs(fd - jv).max() / np.abs(fd).max())
    print("relative max-norm error of J v against central differences:", errs)
    assert np.median(errs) < 1e-2 and max(errs) < 0.2, errs
