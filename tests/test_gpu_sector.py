"""The reference's limiter-frame sector goldens on the device (the
eigen-frame Barth-Jespersen limiter, RECONST 10; grids of the reference's
own mesh tool; the rotational periodic and z periodic pairs as symmetry
patches and the NSCBC outflow as an outflow of its TYPE, exact for these
runs: tests/golden/sector.py): the run to the golden's end time through
the C ABI equals the oracle's bit for bit in FP64_EXACT, and so matches the
golden to 1e-10 of each field's largest magnitude; FP64 stays within 1e-10
of it and the mixed mode within L1(rho) 1e-5."""
import os
import sys

import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import gpu

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from golden import sector  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("run", sector.RUNS)
def test_limiter_frame_golden_through_the_device(gpu_lib, run):
    c, gold, _ = sector.case(run)
    o = Oracle(c)
    n_o, t_o = o.run(100000, 0.0, c.end_time)
    cv_o = o.state()[0]
    setup = gpu.Setup(c)
    r = gpu.Region(c, "fp64_exact", grid=setup)
    n_g, t_g, rc = r.step(100000, 0.0, c.end_time)
    assert rc == 0 and n_g == n_o and t_g == t_o
    cv = r.download()[0]
    np.testing.assert_array_equal(cv, cv_o)
    assert (sector.sorted_distance(cv, gold) <= 1e-10).all()
    scale = np.abs(cv_o).max(axis=0)
    scale[1:4] = np.abs(cv_o[:, 1:4]).max()
    r64 = gpu.Region(c, "fp64", grid=setup)
    n_6, t_6, rc = r64.step(100000, 0.0, c.end_time)
    assert rc == 0 and n_6 == n_o and abs(t_6 - t_o) <= 1e-12 * t_o
    assert (np.abs(r64.download()[0] - cv_o).max(axis=0) <= 1e-10 * scale).all()
    rm = gpu.Region(c, "mixed", grid=setup)
    n_m, t_m, rc = rm.step(100000, 0.0, c.end_time)
    assert rc == 0
    cvm = rm.download()[0]
    assert abs(t_m - t_o) <= 1e-6 * t_o
    assert np.abs(cvm[:, 0] - cv_o[:, 0]).mean() <= 1e-5 * scale[0]
