"""Symmetry (mirror) patches on the device against the oracle through the C
ABI: FP64_EXACT bit for bit (gradients, residual, steps) on the reference's
symmetry gas-jump box and on a smooth 3-D state with one to three symmetry
planes (hexahedra and jittered tetrahedra, every flux and limiter, first
and second order); FP64 within 1e-10 and the mixed mode (its gather
gradient kernel with the reflected members) within L1(rho) 1e-5; the mixed
half box against the mixed doubled box (the mirror's known answer on the
device, the doubled box running the tiled kernels); the run to the golden's
end time equals the oracle's, and through it matches the reference's golden
as the oracle does; the tangent and the adjoint through the reflections
(dot products, central differences)."""
import json
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gas_jump_symmetry_np1.json")
FLUXES = [cases.DISCR_ROE, cases.DISCR_HLLC, cases.DISCR_AUSM]
LIMITERS = [cases.RECONST_NONE, cases.RECONST_WENO_SIMPLE, cases.RECONST_WENO_XYZ, cases.RECONST_BJ,
            cases.RECONST_VENKAT, cases.RECONST_BJ_COMP]


def _jump(reconst=cases.RECONST_WENO_XYZ):
    c = cases.gas_jump_symmetry()
    c.num.c_reconst = 0
    c.num.reconst = reconst
    return c


def _bit_exact(c, steps):
    setup = gpu.Setup(c)
    o = Oracle(c)
    o.set_state(c.cv0)
    r = gpu.Region(c, "fp64_exact", grid=setup)
    rhs_o, grad_o = o.residual()
    rhs_g, grad_g = r.residual(c.cv0)
    np.testing.assert_array_equal(grad_g, grad_o)
    np.testing.assert_array_equal(rhs_g, rhs_o)
    n_o, t_o = o.run(steps, 0.0)
    n_g, t_g, rc = r.step(steps, 0.0)
    assert rc == 0 and (n_g, t_g) == (n_o, t_o)
    np.testing.assert_array_equal(r.download()[0], o.state()[0])


@pytest.mark.parametrize("reconst", [cases.RECONST_WENO_XYZ, cases.RECONST_BJ, cases.RECONST_BJ_COMP])
def test_gas_jump_bit_exact(gpu_lib, reconst):
    _bit_exact(_jump(reconst), 20)


@pytest.mark.parametrize("discr", FLUXES)
@pytest.mark.parametrize("reconst", LIMITERS)
@pytest.mark.parametrize("tets", [False, True])
def test_mirror_box_bit_exact(gpu_lib, discr, reconst, tets):
    num = cases.Numerics(space_order=2, space_discr=discr, reconst=reconst, rk_scheme=cases.RK_WRAY3, cfl=0.4)
    _bit_exact(cases.mirror_box(4, axes=(0, 1, 2), num=num, tets=tets), 5)


@pytest.mark.parametrize("discr", FLUXES)
def test_mirror_box_first_order_bit_exact(gpu_lib, discr):
    num = cases.Numerics(space_order=1, space_discr=discr, reconst=cases.RECONST_NONE, rk_scheme=cases.RK_WRAY3,
                         cfl=0.4)
    _bit_exact(cases.mirror_box(4, axes=(0, 2), num=num), 5)


@pytest.mark.parametrize("which", ["jump", "mirror"])
def test_fp64_and_mixed(gpu_lib, which):
    if which == "jump":
        c = _jump()
    else:
        num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ,
                             rk_scheme=cases.RK_WRAY3, cfl=0.4)
        c = cases.mirror_box(6, axes=(0, 1, 2), num=num)
    setup = gpu.Setup(c)
    o = Oracle(c)
    o.set_state(c.cv0)
    o.run(20, 0.0)
    cv_o = o.state()[0]
    f = gpu.Region(c, "fp64", grid=setup)
    f.step(20, 0.0)
    assert np.abs(f.download()[0] - cv_o).max() <= 1e-10 * np.abs(cv_o).max()
    m = gpu.Region(c, "mixed", grid=setup)
    m.step(20, 0.0)
    assert np.abs(m.download()[0][:, 0] - cv_o[:, 0]).mean() <= 1e-5 * np.abs(cv_o[:, 0]).max()


def test_mixed_half_box_is_the_doubled_box(gpu_lib):
    """The mixed mode's untiled path with reflected members on the half box
    against its tiled path on the doubled box: equal to FP32 rounding."""
    n = 8
    out = []
    for doubled in (False, True):
        num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_WENO_XYZ,
                             rk_scheme=cases.RK_WRAY3, cfl=0.4)
        c = cases.mirror_box(n, axes=(0, 1), doubled=doubled, num=num)
        r = gpu.Region(c, "mixed")
        r.step(20, 0.0)
        out.append(r.download()[0])
    half, full = out
    i = np.arange(n)
    I, J, K = np.meshgrid(i, i, i, indexing="ij")
    hid = (I + n * J + n * n * K).ravel()
    fid = (I + 2 * n * J + 4 * n * n * K).ravel()
    err = np.abs(half[hid] - full[fid]).max(axis=0) / np.abs(full).max(axis=0)
    assert err.max() <= 1e-5, err


def test_golden_through_the_device(gpu_lib):
    with open(GOLDEN) as fh:
        golden = json.load(fh)
    G = np.stack([np.array(golden["gas"]["0"][n]) for n in ("q1", "q2", "q3", "q4", "q5")], axis=1)
    G = G.reshape(8, 8, 8, 5)  # z, y, x
    c = _jump()
    setup = gpu.Setup(c)
    r = gpu.Region(c, "fp64_exact", grid=setup)
    o = Oracle(c)
    n_o, t_o = o.run(100000, 0.0, c.end_time)
    n_g, t_g, rc = r.step(100000, 0.0, c.end_time)
    assert rc == 0 and n_g == n_o and t_g == t_o
    assert abs(t_g - golden["time"]) <= 1e-9 * golden["time"]
    cv = r.download()[0]
    np.testing.assert_array_equal(cv, o.state()[0])
    assert abs((cv[:, 0] * setup.vol).sum() - golden["totals"]["gas_rho"]) <= 1e-13 * golden["totals"]["gas_rho"]
    ix = np.floor(setup.cofg[:, 0] / 0.001).astype(int)
    prof = np.array([cv[ix == k].mean(axis=0) for k in range(8)])
    gm = G.mean(axis=(0, 1))
    assert np.abs(prof[:, 0] - gm[:, 0]).max() / np.abs(G[..., 0]).max() <= 3e-4


def _adj_case(reconst, discr=cases.DISCR_HLLC, tets=False, order=2):
    """The mirror box with three symmetry planes and a seeded 2% perturbation
    (exact symmetries of a state leave gradient components at rounding
    level, where the WENO weights are not resolvable by differences)."""
    num = cases.Numerics(space_order=order, space_discr=discr, reconst=reconst, rk_scheme=cases.RK_WRAY3, cfl=0.4)
    c = cases.mirror_box(4, axes=(0, 1, 2), num=num, tets=tets)
    c.cv0 = c.cv0 * (1 + 0.02 * np.random.default_rng(5).standard_normal(c.cv0.shape))
    return c


def _dirs(c, k, seed):
    rng = np.random.default_rng(seed)
    scale = np.abs(c.cv0).mean(axis=0)
    return [rng.standard_normal(c.cv0.shape) * scale for _ in range(k)]


@pytest.mark.parametrize("discr", [cases.DISCR_ROE, cases.DISCR_HLLC])
@pytest.mark.parametrize("reconst", LIMITERS)
@pytest.mark.parametrize("tets", [False, True])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_symmetry_dot_product(gpu_lib, discr, reconst, tets, prec):
    """The tangent and the adjoint with symmetry patches (reflected stencil
    members, the symmetry faces' fluxes against the cell's reflection and
    their limiter terms) are each other's transpose."""
    c = _adj_case(reconst, discr, tets)
    r = gpu.Region(c, prec)
    rng = np.random.default_rng(7)
    for v in _dirs(c, 3, 1):
        lam = rng.standard_normal(c.cv0.shape)
        jv, jtl = r.jvp(c.cv0, v), r.vjp(c.cv0, lam)
        a, b = (lam * jv).sum(), (jtl * v).sum()
        if prec == "fp64":
            assert abs(a - b) <= 1e-11 * max(abs(a), abs(b)), (a, b)
        else:
            tol = 5e-5 if reconst == cases.RECONST_VENKAT else 1e-5
            scale = max(np.abs(lam * jv).sum(), np.abs(jtl * v).sum())
            assert abs(a - b) <= tol * scale, (a, b, scale)


@pytest.mark.parametrize("discr", FLUXES)
def test_symmetry_first_order_dot_product(gpu_lib, discr):
    c = _adj_case(cases.RECONST_NONE, discr, order=1)
    r = gpu.Region(c, "fp64")
    lam = np.random.default_rng(2).standard_normal(c.cv0.shape)
    for v in _dirs(c, 2, 4):
        a, b = (lam * r.jvp(c.cv0, v)).sum(), (r.vjp(c.cv0, lam) * v).sum()
        assert abs(a - b) <= 1e-11 * max(abs(a), abs(b)), (a, b)


@pytest.mark.parametrize("reconst", [cases.RECONST_NONE, cases.RECONST_WENO_SIMPLE, cases.RECONST_WENO_XYZ,
                                     cases.RECONST_BJ_COMP, cases.RECONST_BJ])
def test_symmetry_vjp_vs_central_differences(gpu_lib, reconst):
    """FP64: the VJP against central differences of the residual along 16
    directions that keep every branch (WENO: eps = 1e-8 with Richardson
    extrapolation, less the difference's round-off), to 1e-6; the mixed VJP
    follows the FP64 one to FP32 rounding."""
    c = _adj_case(reconst, cases.DISCR_ROE)
    r = gpu.Region(c, "fp64")
    lam = np.random.default_rng(11).standard_normal(c.cv0.shape)
    g = r.vjp(c.cv0, lam)
    weno = reconst in (cases.RECONST_WENO_SIMPLE, cases.RECONST_WENO_XYZ)
    eps = 1e-8 if weno else 1e-6
    f = lambda cv: (lam * r.residual(cv, with_grad=False)[0]).sum()  # noqa: E731
    ro = 8 * np.finfo(float).eps * np.abs(lam * r.residual(c.cv0, with_grad=False)[0]).sum() / eps if weno else 0.0
    b0 = r.limiter_branches(c.cv0)
    kept = 0
    for v in _dirs(c, 16, 3):
        if not (np.array_equal(r.limiter_branches(c.cv0 + eps * v), b0) and
                np.array_equal(r.limiter_branches(c.cv0 - eps * v), b0)):
            continue
        kept += 1
        fd = (f(c.cv0 + eps * v) - f(c.cv0 - eps * v)) / (2 * eps)
        if weno:
            h = eps / 2
            fd = (4 * (f(c.cv0 + h * v) - f(c.cv0 - h * v)) / (2 * h) - fd) / 3
        ad = (g * v).sum()
        assert abs(fd - ad) <= 1e-6 * abs(ad) + ro, (fd, ad, ro)
    assert kept >= 2, kept
    gm = gpu.Region(c, "mixed").vjp(c.cv0, lam)
    assert np.linalg.norm(gm - g) <= 1e-3 * np.linalg.norm(g)
