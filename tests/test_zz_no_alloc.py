"""rflu_gpu_residual_static: the residual computed in the library's fixed
static scratch, for callers that cannot allocate device memory per call,
against the allocating rflu_gpu_residual on two calls in a row.

The scratch layout depends on the reconstruction: WENO smoothing (RECONST 1
and 2) carves a second gradient array for the unsmoothed gradients, first
order carves gradients it never writes, and the mixed mode packs its records
differently; every combination is compared with the allocating entry in all
three precision modes.

Collected last (file name) so that a run stopping at the first failure has
already run every other test."""
import numpy as np
import pytest

from rocflu_gb300 import cases, gpu

pytestmark = pytest.mark.gpu

# (space order, RECONST, create options): the BJ eigenframe limiter (tiled
# and gather-based gradient kernels in the mixed mode), WENO-XYZ and simple
# WENO smoothing (second gradient array), and first order (no gradients)
VARIANTS = [(2, cases.RECONST_BJ, 0), (2, cases.RECONST_BJ, gpu.OPT_UNTILED), (2, cases.RECONST_WENO_XYZ, 0),
            (2, cases.RECONST_WENO_SIMPLE, 0), (1, cases.RECONST_NONE, 0)]


def _case(discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ, n=6, order=2):
    num = cases.Numerics(space_order=order, space_discr=discr, reconst=reconst, cfl=0.4)
    c = cases.shock_sphere(n, num=num)
    for p in c.patches:
        p.order = min(p.order, order)
    c.num.dt_imposed = 1e-4
    return c


def _state(case, seed):
    rng = np.random.default_rng(seed)
    cv = case.cv0 * (1.0 + 0.05 * rng.standard_normal(case.cv0.shape))
    cv[:, 1:4] += 0.05 * rng.standard_normal((case.n_cells, 3))
    return cv


@pytest.mark.parametrize("order,reconst,options", VARIANTS)
@pytest.mark.parametrize("precision", ["fp64_exact", "fp64", "mixed"])
def test_residual_static_matches_allocating_entry(gpu_lib, precision, order, reconst, options):
    import torch

    c = _case(reconst=reconst, order=order)
    r = gpu.Region(c, precision, options=options)
    r.step(1, 0.0)  # a context state that differs from the inputs below
    cv_before, dv_before = r.download()
    status_before = r.status()
    for call in range(2):
        cv = _state(c, seed=10 + call)
        ref, _ = r.residual(cv, with_grad=False)      # the allocating entry point
        cv_dev = torch.from_numpy(cv).cuda()
        rhs_dev = torch.full_like(cv_dev, float("nan"))
        torch.cuda.synchronize()
        r.residual_static(cv_dev.data_ptr(), rhs_dev.data_ptr())
        got = rhs_dev.cpu().numpy()                   # complete on return
        # same kernels on the same inputs: identical in every precision mode
        np.testing.assert_array_equal(got, ref)
    # the context's own state and counters are untouched by the static call
    cv_after, dv_after = r.download()
    np.testing.assert_array_equal(cv_after, cv_before)
    np.testing.assert_array_equal(dv_after, dv_before)
    assert r.status() == status_before


@pytest.mark.parametrize("creconst", [0, 1])
@pytest.mark.parametrize("precision", ["fp64_exact", "mixed"])
def test_residual_static_open_patches_and_constrained(gpu_lib, precision, creconst):
    """Inflow, farfield, injection and no-slip patches (their per-patch
    constants) and the constrained-gradient plan of CRECONSTC 1: context
    data the static entry reads as the allocating one does."""
    import torch

    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ, cfl=0.4,
                         c_reconst=creconst)
    c = cases.open_channel(6, num=num, inflow=cases.BC_INFLOW_VELTEMP)
    r = gpu.Region(c, precision)
    cv = _state(c, seed=3)
    ref, _ = r.residual(cv, with_grad=False)
    cv_dev = torch.from_numpy(cv).cuda()
    rhs_dev = torch.full_like(cv_dev, float("nan"))
    torch.cuda.synchronize()
    r.residual_static(cv_dev.data_ptr(), rhs_dev.data_ptr())
    np.testing.assert_array_equal(rhs_dev.cpu().numpy(), ref)


@pytest.mark.parametrize("precision", ["fp64_exact", "mixed"])
def test_residual_static_symmetry_mesh(gpu_lib, precision):
    """Symmetry patches: the reflected stencil members (their reflections and
    offsets) and the patches' reflections are context data the static entry
    reads as the allocating one does."""
    import torch

    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_WENO_XYZ, cfl=0.4)
    c = cases.mirror_box(6, axes=(0, 1, 2), num=num)
    r = gpu.Region(c, precision)
    ref, _ = r.residual(c.cv0, with_grad=False)
    cv_dev = torch.from_numpy(np.ascontiguousarray(c.cv0)).cuda()
    rhs_dev = torch.full_like(cv_dev, float("nan"))
    torch.cuda.synchronize()
    r.residual_static(cv_dev.data_ptr(), rhs_dev.data_ptr())
    np.testing.assert_array_equal(rhs_dev.cpu().numpy(), ref)


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
    import torch

    c = _case()
    r = gpu.Region(c, "fp64")
    cv = np.ascontiguousarray(c.cv0)
    rhs = np.empty_like(cv)
    with pytest.raises(gpu.RfluError) as e:
        r.residual_static(cv.ctypes.data, rhs.ctypes.data)
    assert "device" in str(e.value)
    # pinned host memory is refused as well (a kernel could reach it, slowly)
    pinned = torch.from_numpy(cv).pin_memory()
    with pytest.raises(gpu.RfluError) as e:
        r.residual_static(pinned.data_ptr(), pinned.data_ptr())
    assert "device" in str(e.value)
