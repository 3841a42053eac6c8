"""Inflow (TOTANG, VELTEMP), farfield, injection and no-slip patches on the
device against the oracle, through the C ABI (rocflu/RFLU_CentralFirstPatch.
F90, RFLU_CentralSecondPatch.F90):

* FP64_EXACT equals the oracle bit for bit (residual, gradients, five RK
  steps) wherever no power of a face state enters: VELTEMP inflow, the
  supersonic TOTANG state (its powers are of patch constants, formed on the
  host), farfield, burning injection, walls.  The subsonic TOTANG state
  (p = p_tot (T/T_tot)^(g/(g-1))) and the non-burning injection wall's rind
  pressure take a power per face: CUDA's pow and the C library's may differ
  in the last bit, so those agree to 1e-13 relative;
* FP64 within 1e-10 and the mixed mode within L1(rho) 1e-5 after five steps;
* the tangent and adjoint through the new patches are each other's
  transpose (dot-product test) and the tangent follows central differences."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu

EXACT = [(cases.BC_INFLOW_VELTEMP, cases.BCOPT_SUBSONIC, 0.05), (cases.BC_INFLOW_VELTEMP, cases.BCOPT_SUPERSONIC, 0.05),
         (cases.BC_INFLOW_TOTANG, cases.BCOPT_SUPERSONIC, 0.05)]
POW = [(cases.BC_INFLOW_TOTANG, cases.BCOPT_SUBSONIC, 0.05), (cases.BC_INFLOW_TOTANG, cases.BCOPT_MIXED, 0.05),
       (cases.BC_INFLOW_VELTEMP, cases.BCOPT_SUBSONIC, 0.0)]


def _case(inflow, itype, inj, order, reconst=cases.RECONST_BJ, tets=False):
    num = cases.Numerics(space_order=2 if order == 2 else 1, space_discr=cases.DISCR_HLLC,
                         reconst=reconst if order == 2 else cases.RECONST_NONE, cfl=0.4)
    return cases.open_channel(6, num=num, inflow=inflow, inflow_type=itype, order=order, injection=inj, tets=tets)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("inflow,itype,inj", EXACT)
def test_patches_bit_exact(gpu_lib, inflow, itype, inj, order):
    c = _case(inflow, itype, inj, order)
    o = Oracle(c)
    r = gpu.Region(c, "fp64_exact")
    rhs_o, grad_o = o.residual()
    rhs_g, grad_g = r.residual(c.cv0)
    np.testing.assert_array_equal(rhs_g, rhs_o)
    np.testing.assert_array_equal(grad_g, grad_o)
    o.run(5, 0.0)
    r.step(5, 0.0)
    np.testing.assert_array_equal(r.download()[0], o.state()[0])


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("inflow,itype,inj", POW)
def test_patches_with_face_powers(gpu_lib, inflow, itype, inj, order):
    c = _case(inflow, itype, inj, order)
    o = Oracle(c)
    r = gpu.Region(c, "fp64_exact")
    rhs_o, _ = o.residual()
    rhs_g, _ = r.residual(c.cv0)
    assert np.abs(rhs_g - rhs_o).max() <= 1e-13 * np.abs(rhs_o).max()
    o.run(5, 0.0)
    r.step(5, 0.0)
    cv_o = o.state()[0]
    assert np.abs(r.download()[0] - cv_o).max() <= 1e-12 * np.abs(cv_o).max()


@pytest.mark.parametrize("tets", [False, True])
@pytest.mark.parametrize("inflow,itype,inj", EXACT[:1] + POW[:1])
def test_patches_fp64_and_mixed(gpu_lib, inflow, itype, inj, tets):
    c = _case(inflow, itype, inj, 2, tets=tets)
    o = Oracle(c)
    o.run(5, 0.0)
    cv_o = o.state()[0]
    f = gpu.Region(c, "fp64")
    f.step(5, 0.0)
    assert np.abs(f.download()[0] - cv_o).max() <= 1e-10 * np.abs(cv_o).max()
    m = gpu.Region(c, "mixed")
    m.step(5, 0.0)
    assert np.abs(m.download()[0][:, 0] - cv_o[:, 0]).mean() <= 1e-5


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("inflow,itype,inj", EXACT + POW)
def test_patch_adjoint_dot_product(gpu_lib, inflow, itype, inj, prec):
    c = _case(inflow, itype, inj, 2, reconst=cases.RECONST_VENKAT)
    r = gpu.Region(c, prec)
    rng = np.random.default_rng(5)
    scale = np.abs(c.cv0).mean(axis=0)
    for _ in range(2):
        v = rng.standard_normal(c.cv0.shape) * scale
        lam = rng.standard_normal(c.cv0.shape)
        jv, jtl = r.jvp(c.cv0, v), r.vjp(c.cv0, lam)
        a, b = (lam * jv).sum(), (jtl * v).sum()
        if prec == "fp64":
            assert abs(a - b) <= 1e-11 * max(abs(a), abs(b)), (a, b)
        else:  # FP32 accumulation: relative to the summed magnitudes of the products
            assert abs(a - b) <= 1e-5 * max(np.abs(lam * jv).sum(), np.abs(jtl * v).sum()), (a, b)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("inflow,itype,inj", EXACT + POW)
def test_patch_tangent_vs_central_differences(gpu_lib, inflow, itype, inj, order):
    """No limiter (RECONST 0), so the residual is smooth: J v against
    (R(U + eps v) - R(U - eps v)) / 2 eps, eps = 1e-7, FP64."""
    c = _case(inflow, itype, inj, order, reconst=cases.RECONST_NONE)
    r = gpu.Region(c, "fp64")
    v = np.random.default_rng(8).standard_normal(c.cv0.shape) * np.abs(c.cv0).mean(axis=0)
    eps = 1e-7
    jv = r.jvp(c.cv0, v)
    rp, _ = r.residual(c.cv0 + eps * v, with_grad=False)
    rm, _ = r.residual(c.cv0 - eps * v, with_grad=False)
    fd = (rp - rm) / (2 * eps)
    assert np.abs(fd - jv).max() <= 1e-6 * np.abs(jv).max()


def test_patch_data_checked(gpu_lib):
    c = _case(*EXACT[0], 2)
    c.patches[2].switches = (1, 0)  # the farfield vortex correction
    with pytest.raises(gpu.RfluError) as e:
        gpu.Region(c, "fp64")
    assert e.value.code == -3 and "CORR" in str(e.value)
    c = _case(*EXACT[0], 2)
    c.patches[0].switches = (7, 0)
    with pytest.raises(gpu.RfluError) as e:
        gpu.Region(c, "fp64")
    assert e.value.code == -1
