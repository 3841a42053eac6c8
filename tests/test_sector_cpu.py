"""The eigen-frame Barth-Jespersen limiter (RECONST 10, the bench's
limiter) against the reference's own limiter-frame goldens
(tests/goldens/sector/limiter-frame/theta0-0 and theta0-3.7/np2: a
cylindrical gas jump in a 90-degree annulus sector, HLLC, Wray RK3, two z
layers, t = 4e-6), the runs' grids written by the reference's own mesh tool
(tests/golden/make_sector_limiter_frame.py).  The rotational periodic
planes and the z periodic pair run as symmetry patches and the NSCBC
outflow as an outflow of its TYPE (tests/golden/sector.py says why both
are exact here; the run checks the premises: the flow stays axisymmetric
and the outer ring keeps its initial state).

* the oracle reaches the golden's time in the same run and its cell values
  equal the golden's to 1e-10 of each field's largest magnitude (measured:
  2.5e-12 in density, 1.4e-11 in momentum, 4.3e-12 in energy, both runs);
* the pin tells the limiters apart: componentwise Barth-Jespersen (RECONST
  100) and the WENO smoothing (RECONST 2) end 8e-3 and 1.6e-2 from the
  golden in density, on the same grid and state."""
import os
import sys

import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden import sector  # noqa: E402


def _run(run, reconst=None):
    c, gold, r = sector.case(run, reconst)
    o = Oracle(c)
    vol, cen = o.cells()
    n, t = o.run(100000, 0.0, c.end_time)
    cv, _ = o.state()
    return c, gold, r, vol, cen, t, cv


@pytest.mark.parametrize("run", sector.RUNS)
def test_limiter_frame_against_reference_golden(run):
    c, gold, r, vol, cen, t, cv = _run(run)
    assert abs(t - sector.load()[run]["time"]) <= 1e-9 * t
    d = sector.sorted_distance(cv, gold)
    assert (d <= 1e-10).all(), d
    # premises of the patch substitution: no wave reached r_out (its ring
    # keeps the initial state but for the decayed tail of the second-order
    # stencils, 1.4e-10 of each field), the flow stays axisymmetric (every
    # ring's density, energy and radial momentum equal around it) and
    # z-invariant, and mass is conserved but for what of that tail the
    # outflow passes
    mom = np.abs(gold[:, 1:3]).max()
    outer = r > r.max() - 1e-9
    scale = np.array([np.abs(gold[:, 0]).max(), mom, mom, mom, np.abs(gold[:, 4]).max()])
    assert (np.abs(cv[outer] - c.cv0[outer]).max(axis=0) <= 1e-9 * scale).all()
    ring = np.round(r, 12)
    th = np.arctan2(cen[:, 1], cen[:, 0])
    mr = cv[:, 1] * np.cos(th) + cv[:, 2] * np.sin(th)
    for v in np.unique(ring):
        k = ring == v
        assert np.ptp(cv[k, 0]) <= 1e-12 * np.abs(gold[:, 0]).max()
        assert np.ptp(cv[k, 4]) <= 1e-12 * np.abs(gold[:, 4]).max()
        assert np.ptp(mr[k]) <= 1e-11 * mom
    assert np.abs(cv[:, 3]).max() <= 1e-12 * mom
    m0 = (c.cv0[:, 0] * vol).sum()
    assert abs((cv[:, 0] * vol).sum() - m0) <= 1e-11 * m0  # measured: 1.5e-12


@pytest.mark.parametrize("reconst,miss", [(cases.RECONST_BJ_COMP, 5e-3), (cases.RECONST_WENO_XYZ, 1e-2)])
def test_limiter_frame_golden_tells_limiters_apart(reconst, miss):
    _, gold, _, _, _, _, cv = _run("theta0-0", reconst)
    assert sector.sorted_distance(cv, gold)[0] >= miss
