"""GPU path (through the C ABI) against the CPU oracle on the same inputs.

fp64_exact: bit-exact (integer-for-integer, bit-for-bit) with the oracle.
fp64:       FMA contraction allowed; single residual within 1e-12 relative
            to the field maximum (the reference's regression tolerance is
            1e-10, tests/rocpicl_tests/checks.py:18).
mixed:      FP32 state/flux math; density L1 error vs the FP64 run <= 1e-5.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu

FLUXES = [(cases.DISCR_ROE, "roe"), (cases.DISCR_HLLC, "hllc"), (cases.DISCR_AUSM, "ausm")]
LIMITERS = [cases.RECONST_NONE, cases.RECONST_BJ, cases.RECONST_VENKAT, cases.RECONST_BJ_COMP,
            cases.RECONST_WENO_SIMPLE, cases.RECONST_WENO_XYZ]


def _perturbed(case, seed=3, amp=0.05):
    rng = np.random.default_rng(seed)
    cv = case.cv0.copy()
    cv *= 1.0 + amp * rng.standard_normal(cv.shape)
    cv[:, 1:4] += amp * rng.standard_normal((cv.shape[0], 3))
    return cv


def _rel(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return (np.abs(a - b) / scale).max()


def _hex_case(discr, reconst, order=2, patch_order=2, picl=1, n=6):
    num = cases.Numerics(space_order=order, space_discr=discr, reconst=reconst if order == 2 else 0, picl_build=picl,
                         cfl=0.4)
    c = cases.shock_sphere(n, num=num)
    for p in c.patches:
        p.order = min(patch_order, order)
    c.num.dt_imposed = 1e-4
    return c


@pytest.mark.parametrize("discr,name", FLUXES)
@pytest.mark.parametrize("reconst", LIMITERS)
def test_residual_bit_exact_hex(gpu_lib, discr, name, reconst):
    c = _hex_case(discr, reconst)
    cv = _perturbed(c)
    o = Oracle(c)
    o.set_state(cv)
    rhs_o, grad_o = o.residual()
    r = gpu.Region(c, "fp64_exact")
    rhs_g, grad_g = r.residual(cv)
    np.testing.assert_array_equal(grad_g, grad_o)
    np.testing.assert_array_equal(rhs_g, rhs_o)


@pytest.mark.parametrize("discr,name", FLUXES)
@pytest.mark.parametrize("reconst", [cases.RECONST_BJ, cases.RECONST_VENKAT, cases.RECONST_WENO_XYZ])
def test_residual_bit_exact_tets(gpu_lib, discr, name, reconst):
    num = cases.Numerics(space_order=2, space_discr=discr, reconst=reconst)
    c = cases.adjoint_tets(5, num=num)
    cv = c.cv0
    o = Oracle(c)
    o.set_state(cv)
    rhs_o, grad_o = o.residual()
    r = gpu.Region(c, "fp64_exact")
    rhs_g, grad_g = r.residual(cv)
    np.testing.assert_array_equal(grad_g, grad_o)
    np.testing.assert_array_equal(rhs_g, rhs_o)


@pytest.mark.parametrize("reconst", [cases.RECONST_WENO_SIMPLE, cases.RECONST_WENO_XYZ])
@pytest.mark.parametrize("prec", ["fp64_exact", "mixed"])
def test_simple_limiter_zeroes_nonpositive_face_values(gpu_lib, reconst, prec):
    """RFLU_LimitGradCellsSimple after the WENO smoothing: a pressure
    p = x - 0.05 (perturbed by 1%) is positive at every cell centre but not at
    the x = 0 faces, so the first layer's pressure gradients are zeroed; the
    residual and gradients follow the oracle bit for bit (FP64_EXACT), and
    the mixed path zeroes the same gradients."""
    c = _hex_case(cases.DISCR_HLLC, reconst)
    x = gpu.Setup(c).cofg[:, 0]
    one = np.ones_like(x)
    rng = np.random.default_rng(5)
    p = (x - 0.05) * (1 + 0.01 * rng.standard_normal(x.shape))
    cv = cases.conserved(1.0 + 0.1 * x, 0.1 * one, 0 * one, 0 * one, p, 1.4)
    o = Oracle(c)
    o.set_state(cv)
    rhs_o, grad_o = o.residual()
    first = x < 1.0 / 6
    assert np.all(grad_o[first, 4] == 0.0) and np.all(grad_o[~first, 4, 0] > 0.5)
    r = gpu.Region(c, prec)
    rhs_g, grad_g = r.residual(cv)
    if prec == "fp64_exact":
        np.testing.assert_array_equal(grad_g, grad_o)
        np.testing.assert_array_equal(rhs_g, rhs_o)
    else:
        np.testing.assert_array_equal(grad_g[:, 4] == 0.0, grad_o[:, 4] == 0.0)
        assert np.abs(grad_g - grad_o).max() <= 1e-4 * np.abs(grad_o).max()


@pytest.mark.parametrize("picl", [0, 1])
@pytest.mark.parametrize("patch_order", [1, 2])
def test_patch_orders_and_energy_slot(gpu_lib, picl, patch_order):
    """First-order outflow patches in a second-order run read cv as
    CellGradientsMP left it (energy slot = p in the PICL build)."""
    c = _hex_case(cases.DISCR_HLLC, cases.RECONST_BJ, patch_order=patch_order, picl=picl)
    cv = _perturbed(c)
    o = Oracle(c)
    o.set_state(cv)
    rhs_o, _ = o.residual()
    r = gpu.Region(c, "fp64_exact")
    rhs_g, _ = r.residual(cv)
    np.testing.assert_array_equal(rhs_g, rhs_o)


@pytest.mark.parametrize("discr,name", FLUXES)
def test_residual_first_order(gpu_lib, discr, name):
    c = _hex_case(discr, 0, order=1, patch_order=1)
    cv = _perturbed(c)
    o = Oracle(c)
    o.set_state(cv)
    rhs_o, _ = o.residual()
    rhs_g, _ = gpu.Region(c, "fp64_exact").residual(cv)
    np.testing.assert_array_equal(rhs_g, rhs_o)
    rhs_f, _ = gpu.Region(c, "fp64").residual(cv)
    assert _rel(rhs_f, rhs_o) < 1e-12


@pytest.mark.parametrize("discr,name", FLUXES)
def test_residual_fp64_fma_within_tolerance(gpu_lib, discr, name):
    c = _hex_case(discr, cases.RECONST_BJ)
    cv = _perturbed(c)
    o = Oracle(c)
    o.set_state(cv)
    rhs_o, grad_o = o.residual()
    rhs_g, grad_g = gpu.Region(c, "fp64").residual(cv)
    assert _rel(rhs_g, rhs_o) < 1e-10
    assert _rel(grad_g.reshape(-1, 15), grad_o.reshape(-1, 15)) < 1e-10


def test_drop_in_with_reference_setup_products(gpu_lib):
    """rflu_gpu_create fed with the oracle's own setup arrays (as the Fortran
    host would pass them) gives the same residual as with rflu_setup_build."""
    c = _hex_case(cases.DISCR_ROE, cases.RECONST_VENKAT)
    o = Oracle(c)
    f2c, f2v, fn, fc = o.faces()
    vol, cofg = o.cells()
    off, idx, moms = o.stencil()
    pb = [o.patch(i) for i in range(len(c.patches))]
    po = np.zeros(len(c.patches) + 1, np.int32)
    for i, p in enumerate(pb):
        po[i + 1] = po[i] + len(p[0])

    class G:
        pass

    g = G()
    g.f2c, g.fn, g.fc, g.vol, g.cofg = f2c + 1, fn, fc, vol, cofg
    g.bf2c = np.concatenate([p[0] for p in pb]) + 1
    g.bfn = np.concatenate([p[1] for p in pb])
    g.bfc = np.concatenate([p[2] for p in pb])
    g.patch_off, g.c2cs_off, g.c2cs, g.moms = po, off, idx + 1, moms
    cv = _perturbed(c)
    a, _ = gpu.Region(c, "fp64_exact", grid=g).residual(cv)
    b, _ = gpu.Region(c, "fp64_exact").residual(cv)
    o.set_state(cv)
    ref, _ = o.residual()
    np.testing.assert_array_equal(a, ref)
    np.testing.assert_array_equal(b, ref)


def test_timestep_bit_exact(gpu_lib):
    c = _hex_case(cases.DISCR_HLLC, cases.RECONST_BJ)
    cv = _perturbed(c)
    o = Oracle(c)
    o.set_state(cv)
    r = gpu.Region(c, "fp64_exact")
    r.upload(cv)
    for t in (0.0, 1.0):  # imposed first step, then the CFL step
        assert r.timestep(t) == o.timestep(t)


@pytest.mark.parametrize("nx,nyz", [(100, 2), (400, 4)])
def test_sod_full_run_bit_exact(gpu_lib, nx, nyz):
    """Sod tube to t = 0.2 (first-order Roe, Wray RK3, CFL 0.5), also at the
    full 400 x 4 x 4 size: every time step and stage on the device; final
    state identical to the oracle."""
    c = cases.sod(nx, nyz, nyz)
    c.num.dt_imposed = c.num.cfl * (1.0 / nx) / (6.0 * np.sqrt(1.4))
    o = Oracle(c)
    n_o, t_o = o.run(100000, 0.0, 0.2)
    r = gpu.Region(c, "fp64_exact")
    n_g, t_g, rc = r.step(100000, 0.0, 0.2)
    assert rc == 0
    assert n_g == n_o and t_g == t_o == 0.2
    cv_o, dv_o = o.state()
    cv_g, dv_g = r.download()
    np.testing.assert_array_equal(cv_g, cv_o)
    np.testing.assert_array_equal(dv_g, dv_o)


@pytest.mark.parametrize("discr,name", FLUXES)
def test_second_order_steps_bit_exact(gpu_lib, discr, name):
    c = _hex_case(discr, cases.RECONST_BJ)
    o = Oracle(c)
    n_o, t_o = o.run(5, 0.0)
    r = gpu.Region(c, "fp64_exact")
    n_g, t_g, rc = r.step(5, 0.0)
    assert n_g == n_o == 5 and t_g == t_o
    cv_o, _ = o.state()
    cv_g, _ = r.download()
    np.testing.assert_array_equal(cv_g, cv_o)


@pytest.mark.parametrize("mesh", ["hex", "tets"])
def test_mixed_timestep_entry_matches_step(gpu_lib, mesh):
    """The time-step entry (RFLU_MinimumTimeStep's place) and the time step
    that a mixed step takes from the same state are the same number."""
    c = cases.shock_sphere(24) if mesh == "hex" else cases.blast_tets(8)
    r = gpu.Region(c, "mixed")
    dt = r.timestep(1.0)
    n, t, rc = r.step(1, 1.0)
    assert rc == 0 and n == 1
    assert r.status()["dtMin"] == dt


def test_rk_stage_entry_matches_step(gpu_lib):
    c = _hex_case(cases.DISCR_AUSM, cases.RECONST_VENKAT)
    o = Oracle(c)
    r = gpu.Region(c, "fp64_exact")
    dt = 2.0e-4
    for s in (1, 2, 3):
        o.rk_stage(s, dt)
        r.rk_stage(s, dt)
    np.testing.assert_array_equal(r.download()[0], o.state()[0])


def test_mixed_precision_density_error(gpu_lib):
    """Mixed FP32/FP64 vs the FP64 device run on the shock-sphere set-up."""
    c = cases.shock_sphere(24)
    r64 = gpu.Region(c, "fp64")
    dt = r64.timestep(1.0)
    r64.run_fixed_dt(20, dt)
    rmx = gpu.Region(c, "mixed")
    rmx.run_fixed_dt(20, dt)
    a, dva = r64.download()
    b, dvb = rmx.download()
    l1 = np.abs(a[:, 0] - b[:, 0]).mean()
    assert l1 <= 1e-5, l1
    assert np.abs(dva[:, 0] - dvb[:, 0]).mean() / np.abs(dva[:, 0]).mean() < 1e-4


@pytest.mark.parametrize("layout", ["tiled", "untiled"])
@pytest.mark.parametrize("mesh", ["hex", "tets"])
@pytest.mark.parametrize("reconst", LIMITERS)
@pytest.mark.parametrize("discr,dname", FLUXES)
def test_mixed_matches_fp64_all_limiters(gpu_lib, mesh, reconst, discr, dname, layout):
    """The mixed path (tiled gradient kernel specialised per limiter, packed
    records; and the gather-based gradient kernels that meshes too irregular
    for the tile plan take, forced by RFLU_OPT_UNTILED) against the FP64
    device run, every limiter and flux, hexahedra and jittered tetrahedra:
    density L1 error <= 1e-5 (Venkatakrishnan 5e-5) after 10 Wray steps from
    the same state with the same dt."""
    num = cases.Numerics(space_order=2, space_discr=discr, reconst=reconst, cfl=0.4)
    # a blast every flux/limiter pair of the reference scheme carries stably
    # (unlimited second order only across a weak jump)
    p_in = 1.5 if reconst == cases.RECONST_NONE else 4.0
    if mesh == "hex":
        c = cases.blast_hex(16, num=num, p_in=p_in, radius=0.3)
    else:
        c = cases.blast_tets(8, num=num, p_in=p_in, radius=0.3)
    r64 = gpu.Region(c, "fp64")
    dt = r64.timestep(1.0)
    r64.run_fixed_dt(10, dt)
    rmx = gpu.Region(c, "mixed", options=gpu.OPT_UNTILED if layout == "untiled" else 0)
    rmx.run_fixed_dt(10, dt)
    a, _ = r64.download()
    b, _ = rmx.download()
    assert np.isfinite(a).all()
    assert np.isfinite(b).all()
    l1 = np.abs(a[:, 0] - b[:, 0]).mean()
    # Venkatakrishnan's limiter is a smooth function of near-zero neighbour
    # differences: in this blast FMA contraction alone moves the FP64 density
    # by ~1e-7 (L1), and FP32 rounding by ~2e-5 (measured 1.7e-5 to 2.3e-5
    # over the three fluxes, 2.1e-5 to 2.7e-5 with the per-member weights)
    tol = 5e-5 if reconst == cases.RECONST_VENKAT else 1e-5
    assert l1 <= tol, l1
    assert rmx.status()["nanCells"] == 0


def test_conservation_closed_box(gpu_lib):
    """Mass and gas energy in a slip-wall box stay constant to 1e-10 in the
    FP64 modes (tests/rocpicl_tests/checks.py:365).  The mixed mode rounds
    each cell's RK increment to FP32 before adding it to the FP64 state, so
    its drift is bounded by ~6e-8 of the summed |increments| per stage:
    1e-8 over these 30 stages (measured ~5e-10)."""
    c = cases.blast_hex(8)
    vol = gpu.Setup(c).vol
    for prec, tol in (("fp64", 1e-10), ("fp64_exact", 1e-10), ("mixed", 1e-8)):
        r = gpu.Region(c, prec)
        m0 = (c.cv0[:, 0] * vol).sum()
        e0 = (c.cv0[:, 4] * vol).sum()
        dt = r.timestep(1.0)
        r.run_fixed_dt(10, dt)
        cv, _ = r.download()
        assert abs((cv[:, 0] * vol).sum() - m0) / m0 < tol, prec
        assert abs((cv[:, 4] * vol).sum() - e0) / e0 < tol, prec


def test_positivity_fix_counted(gpu_lib):
    """Two gas halves flying apart at low pressure: the update drives the
    pressure negative, RFLU_CheckPositivity floors the energy, and the device
    counter and state follow the oracle."""
    c = cases.sod(20, 1, 1)
    c.num.rk_scheme = cases.RK_EULER
    x = np.arange(20) + 0.5
    u = np.where(x < 10, -3.0, 3.0)
    one = np.ones(20)
    c.cv0 = cases.conserved(one, u, 0 * one, 0 * one, 0.01 * one, 1.4)
    r = gpu.Region(c, "fp64_exact")
    o = Oracle(c)
    for _ in range(2):
        r.rk_stage(1, 0.002)
        o.rk_stage(1, 0.002)
    pf, neg, nan = o.counters()
    assert pf > 0
    assert r.status()["posFixCells"] == pf
    np.testing.assert_array_equal(r.download()[0], o.state()[0])


def test_nan_cells_reported_as_event(gpu_lib):
    """A NaN cell is reported by the validity check (rc = RFLU_EVENT_NAN and
    the first bad cell in reference numbering), never trapped on the device."""
    c = _hex_case(cases.DISCR_HLLC, cases.RECONST_BJ)
    cv = c.cv0.copy()
    cv[17, :] = np.nan
    r = gpu.Region(c, "fp64")
    r.upload(cv)
    rc = r.rk_stage(1, 1e-4)
    assert rc == gpu.EVENT_NAN
    st = r.status()
    assert st["nanCells"] > 0 and st["firstBadCell"] >= 1


@pytest.mark.parametrize("prec", ["fp64_exact", "mixed"])
def test_pinned_host_buffers_match_pageable(gpu_lib, prec):
    """Upload and download through pinned host buffers give the same bits
    as through pageable buffers."""
    torch = pytest.importorskip("torch")
    c = cases.shock_sphere(8)
    cv0 = _perturbed(c)
    a = gpu.Region(c, prec)
    a.upload(cv0)
    a.step(2, 0.0)
    cv_a, dv_a = a.download()
    pin_cv = torch.from_numpy(cv0.copy()).pin_memory()
    pin_dv = torch.empty((cv0.shape[0], 3), dtype=torch.float64).pin_memory()
    b = gpu.Region(c, prec)
    b.upload(pin_cv.numpy())
    b.step(2, 0.0)
    b.download(pin_cv.numpy(), pin_dv.numpy())
    np.testing.assert_array_equal(pin_cv.numpy(), cv_a)
    np.testing.assert_array_equal(pin_dv.numpy(), dv_a)


def test_mixed_conversions_match_hardware(gpu_lib):
    """The mixed update's integer-pipe float<->double conversions give the
    hardware conversions' bits on 2^26 generated values per seed (random
    doubles, the float exponent range with denormal and overflowing results,
    rounding ties, widened floats and float midpoints)."""
    for seed in (1, 2):
        assert gpu.check_conversions(1 << 26, seed) == 0


def test_mixed_newton_refinements_error_bound(gpu_lib):
    """The mixed update's FP64 1/rho and sound speed come from FP32 seeds
    (approximate division, rsqrtf) refined by one Newton-Raphson step; over
    2^24 values 2^e*m (|e| <= 100) per seed they stay within 2^-40 relative
    of IEEE FP64 division and sqrt (a seed error e becomes ~e^2 ~ 2^-44, plus
    the FP64 rounding of the step), far below the FP32 increments they
    multiply."""
    for seed in (1, 2):
        rr, rs = gpu.check_refinements(1 << 24, seed)
        assert 0.0 < rr <= 2.0 ** -40, rr
        assert 0.0 < rs <= 2.0 ** -40, rs


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_chunked_transfers_round_trip(gpu_lib, prec):
    """Meshes of 2^18 cells and more move cv and dv in chunks, each chunk's
    copy overlapped with the permutation kernel of the one before: an upload
    followed by a download returns the uploaded cv bit for bit, through
    pageable and through pinned buffers, with the same dv both ways and p
    the pressure of cv."""
    torch = pytest.importorskip("torch")
    c = cases.shock_sphere(64)
    assert c.cv0.shape[0] >= 1 << 18
    cv0 = _perturbed(c)
    r = gpu.Region(c, prec)
    r.upload(cv0)
    cv1, dv1 = r.download()
    np.testing.assert_array_equal(cv1, cv0)
    pin_in = torch.from_numpy(cv0.copy()).pin_memory()
    pin_cv = torch.empty(cv0.shape, dtype=torch.float64).pin_memory()
    pin_dv = torch.empty((cv0.shape[0], 3), dtype=torch.float64).pin_memory()
    r.upload(pin_in.numpy())
    r.download(pin_cv.numpy(), pin_dv.numpy())
    np.testing.assert_array_equal(pin_cv.numpy(), cv0)
    np.testing.assert_array_equal(pin_dv.numpy(), dv1)
    g = c.num.gamma
    p = (g - 1.0) * (cv0[:, 4] - 0.5 * (cv0[:, 1:4] ** 2).sum(axis=1) / cv0[:, 0])
    np.testing.assert_allclose(dv1[:, 0], p, rtol=1e-12)


@pytest.mark.parametrize("prec,tol", [("fp64_exact", 1e-10), ("fp64", 1e-10), ("mixed", 1e-5)])
def test_gas_jump_closed_box_matches_reference_golden(gpu_lib, prec, tol):
    """The device through the C ABI against the reference's own result of its
    closed gas-jump box (tests/golden/gas_jump_closed_creconst0_np2.json:
    HLLC, second order, WENO-XYZ + simple limiter, first-order slip walls,
    Wray RK3 from the imposed 1e-9 steps to t = 1.05e-4): the FP64 modes
    within the reference harness's 1e-10 of each field's maximum
    (tests/rocpicl_tests/checks.py:18), FP64_EXACT also bit for bit equal to
    the oracle, the mixed mode within 1e-5."""
    from golden import gas_jump

    golden, layers, scales = gas_jump.load()
    c = cases.gas_jump_closed()
    r = gpu.Region(c, prec)
    steps, t, rc = r.step(100000, 0.0, c.end_time)
    assert rc == 0 and abs(t - golden["time"]) <= 1e-9 * golden["time"]
    cv, _ = r.download()
    err = np.abs(cv - layers[gas_jump.layer_of_cells(c)]) / scales
    assert err.max() <= tol, err.max(axis=0)
    if prec == "fp64_exact":
        o = Oracle(c)
        n_o, _ = o.run(100000, 0.0, c.end_time)
        assert n_o == steps
        np.testing.assert_array_equal(cv, o.state()[0])


@pytest.mark.parametrize("prec", ["fp64_exact", "fp64", "mixed"])
def test_evaluations_leave_the_context_state_untouched(gpu_lib, prec):
    """The residual, tangent, adjoint, functional, unrolled-adjoint and
    kernel-timing calls evaluate other states in the context's scratch
    state: the context's cv, dv and status (time, counters) are the same bits
    before and after, and the next stage continues as if they had not run."""
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_ROE, reconst=cases.RECONST_BJ_COMP, cfl=0.4)
    c = cases.adjoint_tets(4, num=num)
    a, b = gpu.Region(c, prec), gpu.Region(c, prec)
    dt = a.timestep(1.0)
    for r in (a, b):
        r.rk_stage(1, dt)
    before = b.download(), b.status()
    cv = _perturbed(c, seed=9)
    b.residual(cv)
    b.vjp(cv, cv)
    b.jvp(cv, cv)
    b.patch_pressure(cv, 1)
    b.unrolled_adjoint(cv, 2, dt, 1, 1)
    b.kernel_times(1)
    after = b.download(), b.status()
    np.testing.assert_array_equal(after[0][0], before[0][0])
    np.testing.assert_array_equal(after[0][1], before[0][1])
    assert after[1] == before[1]
    for r in (a, b):
        r.rk_stage(2, dt)
        r.rk_stage(3, dt)
    np.testing.assert_array_equal(b.download()[0], a.download()[0])
