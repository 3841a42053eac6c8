"""Known answers and the reference's own property checks, applied to the CPU
oracle (the restatement the GPU path is compared with bit for bit):

* Sod shock tube against the exact Riemann solution;
* LSQ gradients exact for linear fields (the reference's DEBUG check,
  modflu/RFLU_ModDifferentiationCells.F90:576-583);
* free-stream preservation: F(U,U) sums to zero over closed cells;
* mass and gas-energy conservation in a closed box to 1e-10
  (tests/rocpicl_tests/checks.py:365);
* frame invariance of the Barth-Jespersen limiter with eigen-frame velocity
  limiting (RECONST 10) under a rotated mesh, to 1e-7 of the field maximum
  (the limiter-frame regression, checks.py:305); the componentwise limiter
  (RECONST 100) is not frame invariant;
* the energy-slot behaviour of the PICL build on first-order outflow patches.
"""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, meshgen


def exact_riemann(x, t, left, right, gamma=1.4, x0=0.5):
    """Exact solution of the 1D Riemann problem (rho, u, p) (Toro, ch. 4)."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = math.sqrt(gamma * pl / rl), math.sqrt(gamma * pr / rr)

    def f(p, rk, pk, ck):
        if p > pk:
            a, b = 2 / ((gamma + 1) * rk), (gamma - 1) / (gamma + 1) * pk
            return (p - pk) * math.sqrt(a / (p + b))
        return 2 * ck / (gamma - 1) * ((p / pk) ** ((gamma - 1) / (2 * gamma)) - 1)

    lo, hi = 1e-8, 10 * max(pl, pr)
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if f(mid, rl, pl, cl) + f(mid, rr, pr, cr) + ur - ul > 0:
            hi = mid
        else:
            lo = mid
    ps = 0.5 * (lo + hi)
    us = 0.5 * (ul + ur) + 0.5 * (f(ps, rr, pr, cr) - f(ps, rl, pl, cl))
    out = np.zeros((len(x), 3))
    g = gamma
    for i, xi in enumerate(x):
        s = (xi - x0) / t
        if s < us:  # left of contact
            if ps > pl:
                sh = ul - cl * math.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                out[i] = (rl, ul, pl) if s < sh else (rl * ((ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1)), us, ps)
            else:
                csl = cl * (ps / pl) ** ((g - 1) / (2 * g))
                if s < ul - cl:
                    out[i] = (rl, ul, pl)
                elif s > us - csl:
                    out[i] = (rl * (ps / pl) ** (1 / g), us, ps)
                else:
                    u = 2 / (g + 1) * (cl + (g - 1) / 2 * ul + s)
                    c = 2 / (g + 1) * (cl + (g - 1) / 2 * (ul - s))
                    r = rl * (c / cl) ** (2 / (g - 1))
                    out[i] = (r, u, pl * (c / cl) ** (2 * g / (g - 1)))
        else:
            if ps > pr:
                sh = ur + cr * math.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                out[i] = (rr, ur, pr) if s > sh else (rr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1)), us, ps)
            else:
                csr = cr * (ps / pr) ** ((g - 1) / (2 * g))
                if s > ur + cr:
                    out[i] = (rr, ur, pr)
                elif s < us + csr:
                    out[i] = (rr * (ps / pr) ** (1 / g), us, ps)
                else:
                    u = 2 / (g + 1) * (-cr + (g - 1) / 2 * ur + s)
                    c = 2 / (g + 1) * (cr - (g - 1) / 2 * (ur - s))
                    out[i] = (rr * (c / cr) ** (2 / (g - 1)), u, pr * (c / cr) ** (2 * g / (g - 1)))
    return out


def test_sod_against_exact_solution():
    c = cases.sod(400, 1, 1)
    o = Oracle(c)
    n, t = o.run(100000, 0.0, 0.2)
    assert t == 0.2
    cv, dv = o.state()
    x = o.cells()[1][:, 0]
    ex = exact_riemann(x, 0.2, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1))
    l1_rho = np.abs(cv[:, 0] - ex[:, 0]).mean()
    l1_p = np.abs(dv[:, 0] - ex[:, 2]).mean()
    # first-order Roe at 400 cells smears the contact and shock over several cells
    assert l1_rho < 1.0e-2 and l1_p < 8e-3, (l1_rho, l1_p)
    # the star-state plateau (between rarefaction tail and contact)
    plateau = (x > 0.55) & (x < 0.62)
    assert np.abs(dv[plateau, 0] - 0.30313).max() < 2e-3


@pytest.mark.parametrize("make", [lambda: cases.shock_sphere(6), lambda: cases.blast_tets(4)])
def test_lsq_gradient_exact_for_linear_fields(make):
    c = make()
    c.num.reconst = cases.RECONST_NONE
    o = Oracle(c)
    _, cofg = o.cells()
    x, y, z = cofg.T
    rho = 1.0 + 0.1 * x - 0.2 * y + 0.05 * z
    u, v, w = 0.3 * x + 0.1, -0.2 * y + 0.05 * z, 0.1 * x + 0.2 * y
    p = 2.0 + 0.5 * x + 0.25 * y - 0.125 * z
    o.set_state(cases.conserved(rho, u, v, w, p, 1.4))
    _, grad = o.residual()
    expect = np.array([[0.1, -0.2, 0.05], [0.3, 0, 0], [0, -0.2, 0.05], [0.1, 0.2, 0], [0.5, 0.25, -0.125]])
    assert np.abs(grad - expect[None]).max() < 1e-9


@pytest.mark.parametrize("reconst", [cases.RECONST_WENO_SIMPLE, cases.RECONST_WENO_XYZ])
@pytest.mark.parametrize("make", [lambda: cases.shock_sphere(6), lambda: cases.blast_tets(4)])
def test_weno_keeps_linear_gradients(make, reconst):
    """WENO smoothing (RFLU_ModWENO.F90) averages the gradients of a cell and
    its stencil members with normalised weights; for a linear field all of
    them are the exact gradient, so the average is too, and the simple
    limiter leaves the positive density and pressure alone."""
    c = make()
    c.num.reconst = reconst
    o = Oracle(c)
    _, cofg = o.cells()
    x, y, z = cofg.T
    rho = 1.0 + 0.1 * x - 0.2 * y + 0.05 * z
    u, v, w = 0.3 * x + 0.1, -0.2 * y + 0.05 * z, 0.1 * x + 0.2 * y
    p = 2.0 + 0.5 * x + 0.25 * y - 0.125 * z
    o.set_state(cases.conserved(rho, u, v, w, p, 1.4))
    _, grad = o.residual()
    expect = np.array([[0.1, -0.2, 0.05], [0.3, 0, 0], [0, -0.2, 0.05], [0.1, 0.2, 0], [0.5, 0.25, -0.125]])
    assert np.abs(grad - expect[None]).max() < 1e-9


@pytest.mark.parametrize("reconst", [cases.RECONST_WENO_SIMPLE, cases.RECONST_WENO_XYZ])
def test_simple_limiter_zeroes_nonpositive_face_values(reconst):
    """RFLU_LimitGradCellsSimple (RFLU_ModLimiters.F90:1147-1300): a pressure
    p = x - 0.05 is positive at every cell centre of the 6^3 box but not at
    the x = 0 faces, so the first layer's pressure gradient is zeroed; the
    other layers and the (positive) density keep theirs."""
    c = cases.shock_sphere(6)
    c.num.reconst = reconst
    o = Oracle(c)
    _, cofg = o.cells()
    x = cofg[:, 0]
    one = np.ones_like(x)
    o.set_state(cases.conserved(1.0 + 0.1 * x, 0 * one, 0 * one, 0 * one, x - 0.05, 1.4))
    _, grad = o.residual()
    first = x < 1.0 / 6
    assert np.all(grad[first, 4] == 0.0)
    assert np.abs(grad[~first, 4] - np.array([1.0, 0, 0])).max() < 1e-9
    assert np.abs(grad[:, 0] - np.array([0.1, 0, 0])).max() < 1e-9


@pytest.mark.parametrize("discr", [cases.DISCR_ROE, cases.DISCR_HLLC, cases.DISCR_AUSM])
@pytest.mark.parametrize("order", [1, 2])
def test_free_stream_preserved(discr, order):
    num = cases.Numerics(space_order=order, space_discr=discr,
                         reconst=cases.RECONST_VENKAT if order == 2 else 0)
    c = cases.adjoint_tets(4, num=num)
    for p in c.patches:
        p.order = order
    one = np.ones(c.n_cells)
    c.cv0 = cases.conserved(one, 0.5 * one, 0 * one, 0 * one, one / 1.4, 1.4)
    o = Oracle(c)
    rhs, _ = o.residual()
    assert np.abs(rhs).max() < 1e-15 * 10


def test_conservation_closed_box():
    c = cases.blast_hex(6)
    o = Oracle(c)
    vol, _ = o.cells()
    m0, e0 = (c.cv0[:, 0] * vol).sum(), (c.cv0[:, 4] * vol).sum()
    o.run(10, 1.0)  # t > 1e-8: the CFL step from the start
    cv, _ = o.state()
    assert abs((cv[:, 0] * vol).sum() - m0) / m0 < 1e-10
    assert abs((cv[:, 4] * vol).sum() - e0) / e0 < 1e-10


def _rotated_pair(reconst, deg=3.7, n=6, steps=4):
    out = []
    for angle in (0.0, deg):
        num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=reconst)
        c = cases.blast_hex(n, num=num)
        a = math.radians(angle)
        ca, sa = math.cos(a), math.sin(a)
        xyz = c.xyz.copy()
        x, y = xyz[:, 0] - 0.5, xyz[:, 1] - 0.5
        xyz[:, 0], xyz[:, 1] = ca * x - sa * y + 0.5, sa * x + ca * y + 0.5
        c.xyz = xyz
        # blast centre off the mesh's symmetry points (no exact ties in the
        # limiter's minima), carried along with the rotation
        c0 = np.array([0.47 - 0.5, 0.52 - 0.5, 0.49])
        ctr = np.array([ca * c0[0] - sa * c0[1] + 0.5, sa * c0[0] + ca * c0[1] + 0.5, c0[2]])
        cen = meshgen.cell_centers({"xyz": xyz, "c2v": c.c2v}) - ctr
        r = np.sqrt((cen ** 2).sum(axis=1))
        p = 1.0 + 9.0 * np.exp(-(r / 0.15) ** 2)  # smooth blast: no cell sits on a jump
        one = np.ones(c.n_cells)
        c.cv0 = cases.conserved(one, 0 * one, 0 * one, 0 * one, p, 1.4)
        o = Oracle(c)
        o.run_fixed_dt(steps, 2e-3)
        cv, dv = o.state()
        u = cv[:, 1:4] / cv[:, :1]
        ur = u.copy()
        ur[:, 0], ur[:, 1] = ca * u[:, 0] + sa * u[:, 1], -sa * u[:, 0] + ca * u[:, 1]  # back to the unrotated frame
        out.append((cv[:, 0], dv[:, 0], ur))
    return out


def test_barth_jespersen_frame_invariance():
    (r0, p0, u0), (r1, p1, u1) = _rotated_pair(cases.RECONST_BJ)
    assert np.abs(r1 - r0).max() <= 1e-7 * np.abs(r0).max()
    assert np.abs(p1 - p0).max() <= 1e-7 * np.abs(p0).max()
    assert np.abs(u1 - u0).max() <= 1e-7 * np.abs(u0).max()


def test_componentwise_limiter_is_not_frame_invariant():
    (r0, p0, u0), (r1, p1, u1) = _rotated_pair(cases.RECONST_BJ_COMP)
    assert np.abs(u1 - u0).max() > 1e-7 * np.abs(u0).max()


def test_energy_slot_of_picl_build_on_first_order_outflow():
    """RFLU_ConvertCvPrim2Cons with PICL compiled in leaves p in cv(ENER)
    while the fluxes run; a first-order outflow patch of a second-order run
    reads it.  The PICL and non-PICL builds differ only in outflow cells."""
    res = {}
    for picl in (0, 1):
        c = cases.shock_sphere(6)
        c.num.picl_build = picl
        for p in c.patches:
            p.order = 1
        o = Oracle(c)
        res[picl], _ = o.residual()
    diff = np.abs(res[1] - res[0]).max(axis=1) > 0
    s = cases.shock_sphere(6)
    out_cells = set()
    o = Oracle(s)
    for ip in (0, 1):  # the two outflow patches
        out_cells |= set(o.patch(ip)[0].tolist())
    assert diff.any()
    assert set(np.nonzero(diff)[0].tolist()) <= out_cells


def test_gas_jump_closed_box_matches_reference_golden():
    """The oracle against the reference's own result (its test suite's
    tests/goldens/box/gas-jump/closed-creconst0/np2, extracted by
    tests/golden/make_gas_jump_closed.py): HLLC, second order, WENO-XYZ with
    the simple limiter, first-order slip walls, Wray RK3 from the imposed
    1e-9 steps to t = 1.05e-4 at CFL 0.4.  Every cell within 1e-10 of the
    field's maximum, the reference harness's tolerance (checks.py:18)."""
    from golden import gas_jump

    golden, layers, scales = gas_jump.load()
    c = cases.gas_jump_closed()
    o = Oracle(c)
    _, t = o.run(100000, 0.0, c.end_time)
    assert abs(t - golden["time"]) <= 1e-9 * golden["time"]
    cv, _ = o.state()
    ix = gas_jump.layer_of_cells(c)
    err = np.abs(cv - layers[ix]) / scales
    assert err.max() <= 1e-10, err.max(axis=0)


@pytest.mark.parametrize("mesh,discr,reconst,p_in", [
    ("hex", cases.DISCR_HLLC, cases.RECONST_BJ, None),
    ("hex", cases.DISCR_AUSM, cases.RECONST_VENKAT, None),
    ("hex", cases.DISCR_ROE, cases.RECONST_WENO_XYZ, None),
    ("tet", cases.DISCR_HLLC, cases.RECONST_BJ_COMP, 10.0),
    ("tet", cases.DISCR_HLLC, cases.RECONST_VENKAT, 100.0),  # NaN cells within a few steps
])
def test_oracle_results_independent_of_threads(mesh, discr, reconst, p_in):
    """The oracle's face loops run as per-cell gathers over each cell's faces
    in the reference's loop order, so one thread and several give the same
    bits: residual, gradients, states after whole steps (NaN cells included)
    and the event counters."""
    from oracle import oracle as orc

    num = cases.Numerics(space_order=2, space_discr=discr, reconst=reconst, cfl=0.4)
    if mesh == "hex":
        c = cases.shock_sphere(10, num=num)
    else:
        c = cases.blast_tets(6, num=num, p_in=p_in)
    c.num.dt_imposed = 1e-3
    out = []
    prev = orc.threads()
    try:
        for nt in (1, 4):
            orc.set_threads(nt)
            o = Oracle(c)
            rhs, grad = o.residual()
            done, t = o.run(6, 0.0)
            cv, dv = o.state()
            out.append((rhs, grad, t, cv, dv, o.counters()))
    finally:
        orc.set_threads(prev)
    a, b = out
    for x, y in zip(a, b):
        if isinstance(x, np.ndarray):
            np.testing.assert_array_equal(x, y)
        else:
            assert x == y


def test_oracle_stage_pieces_equal_whole_stage():
    """orc_rk_init, orc_cell_gradients, orc_convective_fluxes, orc_add_rhs
    (a zero source) and orc_rk_update give orc_rk_stage's state; a nonzero
    source changes the update by exactly -adtv * src in the first stage."""
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ, cfl=0.4)
    c = cases.shock_sphere(8, num=num)
    c.num.dt_imposed = 1e-3
    a, b = Oracle(c), Oracle(c)
    dt = a.timestep(1.0)
    for s in range(1, 4):
        a.rk_stage(s, dt)
        b.rk_init(s)
        b.cell_gradients()
        b.convective_fluxes()
        b.add_rhs(np.zeros_like(c.cv0))
        b.rk_update(s, dt)
        np.testing.assert_array_equal(a.state()[0], b.state()[0])
        np.testing.assert_array_equal(a.state()[1], b.state()[1])
    p, q = Oracle(c), Oracle(c)
    vol, _ = p.cells()
    src = np.outer(vol, [0.0, 0.0, 1.0, 0.0, 0.0])
    for o, add in ((p, False), (q, True)):
        o.rk_init(1)
        o.cell_gradients()
        o.convective_fluxes()
        if add:
            o.add_rhs(src)
        o.rk_update(1, dt)
    dmom = q.state()[0][:, 2] - p.state()[0][:, 2]
    np.testing.assert_allclose(dmom, -(8.0 / 15.0) * dt * np.ones_like(dmom), rtol=1e-9, atol=1e-15)


def test_periodic_gas_jump_against_reference_golden():
    """Translational periodic patches (BC_PERIODIC) as a periodic mesh: the
    reference's periodic gas-jump box (tests/goldens/box/gas-jump/periodic/
    np1, extracted by tests/golden/make_gas_jump_periodic.py) to t = 1.05e-4.
    The oracle conserves mass and energy to round-off and keeps the flow
    one-dimensional.  The reference's result is not one-dimensional: its
    virtual cells near the box's edges and corners (copies built per patch,
    modflu/RFLU_ModSymmetryPeriodic.F90:471-787, whose own stencils and raw
    gradients enter the WENO smoothing of the cells next to the patches)
    leave a y/z variation of 6.4e-5 of the density maximum in the golden.
    The oracle's x profile lies within that variation of the golden's y/z
    mean (6.6e-5 in density, 1e-5 in energy), not within the harness's 1e-10,
    which would need those virtual cells restated."""
    import json
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gas_jump_periodic_np1.json")
    with open(path) as f:
        golden = json.load(f)
    G = np.stack([np.array(golden["gas"]["0"][n]) for n in ("q1", "q2", "q3", "q4", "q5")], axis=1)
    G = G.reshape(8, 8, 8, 5)  # z, y, x
    c = cases.gas_jump_periodic()
    o = Oracle(c)
    vol, _ = o.cells()
    m0, e0 = (c.cv0[:, 0] * vol).sum(), (c.cv0[:, 4] * vol).sum()
    _, t = o.run(100000, 0.0, c.end_time)
    assert abs(t - golden["time"]) <= 1e-9 * golden["time"]
    cv, _ = o.state()
    assert abs((cv[:, 0] * vol).sum() - m0) <= 1e-13 * m0
    assert abs((cv[:, 4] * vol).sum() - e0) <= 1e-13 * e0
    assert abs((cv[:, 0] * vol).sum() - golden["totals"]["gas_rho"]) <= 1e-13 * m0
    ix = gas_jump_layer(c)
    prof = np.array([cv[ix == k].mean(axis=0) for k in range(8)])
    for k in range(8):
        assert np.abs(cv[ix == k] - prof[k]).max() <= 1e-9 * np.abs(prof).max()
    scale = np.abs(G[..., 0]).max()
    golden_spread = np.abs(G[..., 0] - G[..., 0].mean(axis=(0, 1))).max() / scale
    assert 5e-5 < golden_spread < 1e-4
    gm = G.mean(axis=(0, 1))
    assert np.abs(prof[:, 0] - gm[:, 0]).max() / scale <= 1.2 * golden_spread
    assert np.abs(prof[:, 4] - gm[:, 4]).max() / np.abs(G[..., 4]).max() <= 2e-5


def gas_jump_layer(case):
    from golden import gas_jump

    return gas_jump.layer_of_cells(case)
