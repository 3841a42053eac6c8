"""rflu_gpu_residual_static: the residual computed in the library's fixed
static scratch, for callers that cannot allocate device memory per call,
against the allocating rflu_gpu_residual on two calls in a row.

Collected last (file name) so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu


def _case(discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ, n=6):
    num = cases.Numerics(space_order=2, space_discr=discr, reconst=reconst, cfl=0.4)
    c = cases.shock_sphere(n, num=num)
    c.num.dt_imposed = 1e-4
    return c


def _state(case, seed):
    rng = np.random.default_rng(seed)
    cv = case.cv0 * (1.0 + 0.05 * rng.standard_normal(case.cv0.shape))
    cv[:, 1:4] += 0.05 * rng.standard_normal((case.n_cells, 3))
    return cv


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64", "mixed"])
def test_residual_static_matches_allocating_entry(gpu_lib, precision):
    import torch

    c = _case()
    r = gpu.Region(c, precision)
    for call in range(2):
        cv = _state(c, seed=10 + call)
        ref, _ = r.residual(cv, with_grad=False)      # the allocating entry point
        cv_dev = torch.from_numpy(cv).cuda()
        rhs_dev = torch.full_like(cv_dev, float("nan"))
        torch.cuda.synchronize()
        r.residual_static(cv_dev.data_ptr(), rhs_dev.data_ptr())
        torch.cuda.synchronize()
        got = rhs_dev.cpu().numpy()
        # same kernels on the same inputs: identical in every precision mode
        np.testing.assert_array_equal(got, ref)
    # the context's own device state is untouched by the static call
    cv_ctx, _ = r.download()
    np.testing.assert_array_equal(cv_ctx, c.cv0)


def test_residual_static_rejects_oversized_mesh(gpu_lib):
    import torch

    c = _case(n=64)
    r = gpu.Region(c, "fp64")
    cv_dev = torch.from_numpy(c.cv0).cuda()
    rhs_dev = torch.empty_like(cv_dev)
    with pytest.raises(gpu.RfluError) as e:
        r.residual_static(cv_dev.data_ptr(), rhs_dev.data_ptr())
    assert e.value.code == -1 and "static scratch" in str(e.value)


def test_residual_static_rejects_host_pointers(gpu_lib):
    c = _case()
    r = gpu.Region(c, "fp64")
    cv = np.ascontiguousarray(c.cv0)
    rhs = np.empty_like(cv)
    with pytest.raises(gpu.RfluError) as e:
        r.residual_static(cv.ctypes.data, rhs.ctypes.data)
    assert "device" in str(e.value)
