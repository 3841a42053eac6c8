"""The inflow, farfield, injection and no-slip patches of the oracle
(oracle/oracle.cpp: bcondInflowPerf, rindStateFarfieldPerf, injectionFlux,
after rocflu/RFLU_CentralFirstPatch.F90 and RFLU_CentralSecondPatch.F90)
against known answers:

* a uniform flow that every patch is consistent with (inflow at the flow's
  own total or static conditions, subsonic outflow at its pressure, farfield
  at its Mach number, pressure and temperature, a non-burning injection wall
  and a no-slip wall parallel to it) has a zero residual, first and second
  order;
* a burning injection patch adds exactly -m_inj times its area to the mass
  residual;
* the supersonic TOTANG state built from total conditions is the VELTEMP
  state of the same static conditions;
* a run through every patch stays finite and keeps the state near the
  uniform flow."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, gpu

INFLOWS = [(cases.BC_INFLOW_TOTANG, cases.BCOPT_SUBSONIC), (cases.BC_INFLOW_TOTANG, cases.BCOPT_SUPERSONIC),
           (cases.BC_INFLOW_TOTANG, cases.BCOPT_MIXED), (cases.BC_INFLOW_VELTEMP, cases.BCOPT_SUBSONIC),
           (cases.BC_INFLOW_VELTEMP, cases.BCOPT_SUPERSONIC)]


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("inflow,itype", INFLOWS)
def test_uniform_flow_is_steady(inflow, itype, order):
    c = cases.open_channel(6, inflow=inflow, inflow_type=itype, order=order, pert=0.0, injection=0.0)
    rhs, _ = Oracle(c).residual()
    scale = np.abs(c.cv0).max(axis=0)
    assert np.abs(rhs).max(axis=0).max() <= 1e-12 * scale.max(), np.abs(rhs).max(axis=0)


@pytest.mark.parametrize("order", [1, 2])
def test_injection_adds_its_mass_flux(order):
    minj = 0.05
    base = cases.open_channel(6, order=order, pert=0.0, injection=0.0)
    burn = cases.open_channel(6, order=order, pert=0.0, injection=minj)
    r0, _ = Oracle(base).residual()
    r1, _ = Oracle(burn).residual()
    area = 1.0 * 0.5  # the z-low face of [0,1] x [0,0.5]^2
    assert abs((r1[:, 0].sum() - r0[:, 0].sum()) - (-minj * area)) <= 1e-12


def test_supersonic_totang_is_the_veltemp_state():
    a = cases.open_channel(6, inflow=cases.BC_INFLOW_TOTANG, inflow_type=cases.BCOPT_SUPERSONIC)
    b = cases.open_channel(6, inflow=cases.BC_INFLOW_VELTEMP, inflow_type=cases.BCOPT_SUPERSONIC)
    ra, _ = Oracle(a).residual()
    rb, _ = Oracle(b).residual()
    assert np.abs(ra - rb).max() <= 1e-13 * np.abs(rb).max()


@pytest.mark.parametrize("inflow,itype", INFLOWS)
def test_run_through_every_patch(inflow, itype):
    c = cases.open_channel(6, inflow=inflow, inflow_type=itype, order=2)
    o = Oracle(c)
    o.run(20, 0.0)
    cv, dv = o.state()
    assert np.isfinite(cv).all() and np.isfinite(dv).all()
    assert np.abs(cv[:, 0] - 1.0).max() < 0.2


def test_patch_values_layout():
    """The values and switches reach the C ABI in BCDAT / BCSWI order."""
    c = cases.open_channel(4)
    vals, sw = gpu.patch_values(c)
    assert vals.shape == (6, gpu.BCDAT_N) and sw.shape == (6, gpu.BCSWI_N)
    assert vals[2, 0] == 0.3 and sw[0, 0] == cases.BCOPT_SUBSONIC
