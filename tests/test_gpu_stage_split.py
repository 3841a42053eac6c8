"""One RK stage at the reference's subroutine granularity through the C ABI:
rflu_gpu_cell_gradients (CellGradientsMP), rflu_gpu_convective_fluxes
(ConvectiveFluxesMP), rflu_gpu_add_rhs (the SourceTermsMP / PICL_Runge slot
of libfloflu/RungeKuttaMP.F90:274-290) and rflu_gpu_rk_update (RKUpdateMP +
RFLU_SetVarsContWrapper + AfterUpdateMP).

* without a source the four calls leave the state rflu_gpu_rk_stage leaves,
  bit for bit, in every precision mode;
* with a source they follow the oracle's stage with the same source added to
  its rhs: bit for bit in FP64_EXACT (rhs and gradient read-outs included),
  within the mixed mode's tolerance otherwise;
* device buffers work as the host ones do, and calls out of order are
  refused with RFLU_ERR_STATE."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu

ERR_STATE = -4


def _case(reconst=cases.RECONST_BJ, discr=cases.DISCR_HLLC, n=8):
    num = cases.Numerics(space_order=2, space_discr=discr, reconst=reconst, cfl=0.4)
    c = cases.shock_sphere(n, num=num)
    c.num.dt_imposed = 1e-3
    return c


def _source(case, stage, vol, cofg):
    """A smooth source in rhs units (-vol * S), different per stage: a body
    force along y with its work, and a small mass and energy deposition."""
    x = cofg
    rho = case.cv0[:, 0]
    g = 0.5 * (1.0 + 0.2 * stage)
    S = np.zeros_like(case.cv0)
    S[:, 0] = 0.01 * np.sin(2 * np.pi * x[:, 0])
    S[:, 2] = rho * g
    S[:, 4] = 0.05 * np.cos(2 * np.pi * x[:, 1]) + case.cv0[:, 2] * g
    return -vol[:, None] * S


@pytest.mark.parametrize("reconst", [cases.RECONST_BJ, cases.RECONST_WENO_XYZ, cases.RECONST_VENKAT])
@pytest.mark.parametrize("prec", ["fp64_exact", "fp64", "mixed"])
def test_split_stage_equals_rk_stage(gpu_lib, prec, reconst):
    c = _case(reconst)
    a, b = gpu.Region(c, prec), gpu.Region(c, prec)
    dt = a.timestep(1.0)
    zero = np.zeros_like(c.cv0)
    for step in range(2):
        for s in range(1, a.n_stages + 1):
            assert a.rk_stage(s, dt) == 0
            gpu.CellGradientsMP(b)
            gpu.ConvectiveFluxesMP(b)
            if s == 2:
                b.add_rhs(zero)
            assert gpu.RKUpdateMP(b, 1, s, dt) == 0
            cva, dva = a.download()
            cvb, dvb = b.download()
            np.testing.assert_array_equal(cvb, cva)
            np.testing.assert_array_equal(dvb, dva)


@pytest.mark.parametrize("reconst", [cases.RECONST_BJ, cases.RECONST_WENO_XYZ])
def test_split_stage_with_source_matches_oracle(gpu_lib, reconst):
    c = _case(reconst)
    setup = gpu.Setup(c)
    o = Oracle(c)
    r = gpu.Region(c, "fp64_exact", grid=setup)
    dt = o.timestep(1.0)
    assert r.timestep(1.0) == dt
    for step in range(2):
        for s in range(1, o.n_stages() + 1):
            src = _source(c, s, setup.vol, setup.cofg)
            o.rk_init(s)
            o.cell_gradients()
            o.convective_fluxes()
            rhs_o = o.rhs()
            o.add_rhs(src)
            r.cell_gradients()
            np.testing.assert_array_equal(r.get_grad(), o.grad())
            r.convective_fluxes()
            np.testing.assert_array_equal(r.get_rhs(), rhs_o)
            r.add_rhs(src)
            np.testing.assert_array_equal(r.get_rhs(), o.rhs())
            o.rk_update(s, dt)
            assert r.rk_update(s, dt) == 0
            np.testing.assert_array_equal(r.download()[0], o.state()[0])
    cv_o, dv_o = o.state()
    cv_g, dv_g = r.download()
    np.testing.assert_array_equal(dv_g, dv_o)
    # the source changed the run: the y momentum picked up the body force
    ref = gpu.Region(c, "fp64_exact", grid=setup)
    ref.run_fixed_dt(2, dt)
    assert np.abs(ref.download()[0][:, 2] - cv_g[:, 2]).max() > 1e-6


def test_split_stage_with_source_mixed_and_device_buffers(gpu_lib):
    """The mixed mode with the same source against the FP64 oracle (density
    L1 <= 1e-5 after two steps), the source and the read-outs passed as
    device buffers; the host and device forms agree."""
    import torch

    c = _case()
    setup = gpu.Setup(c)
    o = Oracle(c)
    m = gpu.Region(c, "mixed", grid=setup)
    h = gpu.Region(c, "mixed", grid=setup)
    dt = o.timestep(1.0)
    for step in range(2):
        for s in range(1, o.n_stages() + 1):
            src = _source(c, s, setup.vol, setup.cofg)
            o.rk_init(s)
            o.cell_gradients()
            o.convective_fluxes()
            o.add_rhs(src)
            o.rk_update(s, dt)
            src_dev = torch.from_numpy(src).cuda()
            rhs_dev = torch.empty_like(src_dev)
            grad_dev = torch.empty((c.n_cells, 5, 3), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            for reg, dev in ((m, True), (h, False)):
                reg.cell_gradients()
                reg.convective_fluxes()
                reg.add_rhs(src_dev.data_ptr() if dev else src)
                if dev:
                    reg.get_rhs(rhs_dev.data_ptr())
                    reg.get_grad(grad_dev.data_ptr())
                else:
                    h_rhs = reg.get_rhs()
                    h_grad = reg.get_grad()
                assert reg.rk_update(s, dt) == 0
            np.testing.assert_array_equal(rhs_dev.cpu().numpy(), h_rhs)
            np.testing.assert_array_equal(grad_dev.cpu().numpy(), h_grad)
            np.testing.assert_array_equal(m.download()[0], h.download()[0])
    cv_o, _ = o.state()
    cv_m, _ = m.download()
    assert np.abs(cv_m[:, 0] - cv_o[:, 0]).mean() <= 1e-5


def test_split_stage_order_is_checked(gpu_lib):
    c = _case()
    r = gpu.Region(c, "fp64")
    dt = r.timestep(1.0)
    src = np.zeros_like(c.cv0)
    for call in (lambda: r.rk_update(1, dt), lambda: r.add_rhs(src), lambda: r.get_rhs(),
                 lambda: r.get_grad(), lambda: r.convective_fluxes()):
        with pytest.raises(gpu.RfluError) as e:
            call()
        assert e.value.code == ERR_STATE
    r.cell_gradients()
    r.convective_fluxes()
    assert r.rk_update(1, dt) == 0
    # the update ends the sequence; an upload or a whole stage ends it too
    with pytest.raises(gpu.RfluError) as e:
        r.add_rhs(src)
    assert e.value.code == ERR_STATE
    r.cell_gradients()
    r.upload(c.cv0)
    with pytest.raises(gpu.RfluError) as e:
        r.convective_fluxes()
    assert e.value.code == ERR_STATE
    # host memory passed as a device buffer is refused
    with pytest.raises(gpu.RfluError) as e:
        r.cell_gradients()
        r.convective_fluxes()
        r.add_rhs(src.ctypes.data)
    assert e.value.code == -1 and "device" in str(e.value)
