"""The adjoint inside torch.autograd (rocflu_gb300.autograd) and the
time-unrolled, checkpointed adjoint (rflu_gpu_unrolled_adjoint).

* torch.autograd.gradcheck of a scalar reduction of the residual along a few
  seeded directions: reverse mode (adjoint kernels) and forward mode (tangent
  kernels) against FP64 central differences;
* forward/reverse dot-product test through torch's own forward-mode AD;
* the unrolled adjoint: gradient independent of the checkpoint interval, and
  against central differences of the unrolled functional.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from rocflu_gb300 import autograd, cases, gpu  # noqa: E402

pytestmark = pytest.mark.gpu


def _tets(reconst=cases.RECONST_VENKAT, discr=cases.DISCR_ROE, n=4):
    num = cases.Numerics(space_order=2, space_discr=discr, reconst=reconst)
    return cases.adjoint_tets(n, num=num)


def _dirs(cv0, k, seed):
    rng = np.random.default_rng(seed)
    scale = np.abs(cv0).mean(axis=0)
    return np.stack([rng.standard_normal(cv0.shape) * scale for _ in range(k)])


@pytest.mark.parametrize("reconst", [cases.RECONST_NONE, cases.RECONST_VENKAT, cases.RECONST_BJ_COMP,
                                     cases.RECONST_WENO_XYZ])
def test_gradcheck_residual(gpu_lib, reconst):
    c = _tets(reconst)
    r = gpu.Region(c, "fp64")
    cv0 = torch.from_numpy(c.cv0)
    D = torch.from_numpy(_dirs(c.cv0, 4, 11))
    w = torch.from_numpy(np.random.default_rng(3).standard_normal(c.cv0.shape))

    def f(theta):
        cv = cv0 + torch.einsum("k,kij->ij", theta, D)
        return (autograd.residual(cv, r) * w).sum()

    theta = torch.zeros(4, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(f, (theta,), eps=1e-6, atol=1e-6, rtol=1e-5, check_forward_ad=True,
                                    check_backward_ad=True, check_undefined_grad=False, check_batched_grad=False)


def test_autograd_dot_product(gpu_lib):
    """<w, J v> by forward mode equals <J^T w, v> by reverse mode."""
    import torch.autograd.forward_ad as fwAD

    c = _tets()
    r = gpu.Region(c, "fp64")
    cv = torch.from_numpy(c.cv0.copy())
    v = torch.from_numpy(_dirs(c.cv0, 1, 4)[0])
    w = torch.from_numpy(np.random.default_rng(9).standard_normal(c.cv0.shape))
    with fwAD.dual_level():
        out = autograd.residual(fwAD.make_dual(cv, v), r)
        jv = fwAD.unpack_dual(out).tangent
    x = cv.clone().requires_grad_(True)
    (jtw,) = torch.autograd.grad((autograd.residual(x, r) * w).sum(), x)
    a, b = float((w * jv).sum()), float((jtw * v).sum())
    assert abs(a - b) <= 1e-11 * max(abs(a), abs(b)), (a, b)


def test_patch_pressure_through_autograd(gpu_lib):
    c = _tets()
    r = gpu.Region(c, "fp64")
    x = torch.from_numpy(c.cv0.copy()).requires_grad_(True)
    J = autograd.patch_pressure(x, r, 1)
    (g,) = torch.autograd.grad(J, x)
    v = _dirs(c.cv0, 1, 6)[0]
    eps = 1e-6
    jp, _ = r.patch_pressure(c.cv0 + eps * v, 1, with_grad=False)
    jm, _ = r.patch_pressure(c.cv0 - eps * v, 1, with_grad=False)
    fd = (jp - jm) / (2 * eps)
    ad = float((g.numpy() * v).sum())
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def _blast(n=8):
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_VENKAT, cfl=0.4)
    return cases.blast_hex(n, num=num, p_in=10.0, radius=0.15)


def _smooth_background(case):
    """The blast with a smooth 2% variation on density, energy and x-momentum,
    so that no region is exactly uniform.  On an exactly uniform state the
    limiters sit on their d2 = 0 branch, where the discrete scheme (the
    reference's) is not differentiable: one-sided differences there differ
    from the adjoint by an amount that does not shrink with eps."""
    x = gpu.Setup(case).cofg
    bg = np.sin(2 * np.pi * x[:, 0] + 0.3) * np.sin(2 * np.pi * x[:, 1] + 0.7) * np.sin(2 * np.pi * x[:, 2] + 1.1)
    cv = case.cv0.copy()
    cv[:, 0] *= 1 + 0.02 * bg
    cv[:, 4] *= 1 + 0.02 * np.roll(bg, 7)
    cv[:, 1] += 0.01 * bg
    return cv


def _density_blobs(case, k, seed):
    """Smooth seeded density perturbations (Gaussian blobs) at fixed u, p."""
    rng = np.random.default_rng(seed)
    reg = gpu.Setup(case)
    xc = reg.cofg
    out = []
    for _ in range(k):
        c0 = rng.uniform(0.25, 0.75, 3)
        w = np.exp(-((xc - c0) ** 2).sum(axis=1) / (2 * 0.1 ** 2))
        d = np.zeros_like(case.cv0)
        d[:, 0] = w * rng.choice([-1.0, 1.0])
        out.append(d)
    return out


def test_unrolled_adjoint_checkpoint_interval_invariant(gpu_lib):
    c = _blast()
    r = gpu.Region(c, "fp64")
    dt = r.timestep(1.0)
    J1, g1, s1 = r.unrolled_adjoint(c.cv0, 12, dt, 1, 1)
    J5, g5, s5 = r.unrolled_adjoint(c.cv0, 12, dt, 5, 1)
    J12, g12, _ = r.unrolled_adjoint(c.cv0, 12, dt, 12, 1)
    Jf, _, _ = r.unrolled_adjoint(c.cv0, 12, dt, 5, 1, with_grad=False)
    assert J1 == J5 == J12 == Jf
    np.testing.assert_array_equal(g1, g5)
    np.testing.assert_array_equal(g1, g12)
    assert s1["checkpoints"] == 12 and s5["checkpoints"] == 3


@pytest.mark.parametrize("reconst", [cases.RECONST_VENKAT, cases.RECONST_BJ_COMP, cases.RECONST_WENO_XYZ])
def test_unrolled_adjoint_finite_differences(gpu_lib, reconst):
    """dJ/drho0 along smooth density perturbations against FP64 central
    differences (eps = 1e-6) of the unrolled functional, 20 Wray steps with
    a checkpoint every 5 (measured agreement 3e-7 to 1.4e-6)."""
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=reconst, cfl=0.4)
    c = cases.blast_hex(8, num=num, p_in=10.0, radius=0.15)
    cv0 = _smooth_background(c)
    r = gpu.Region(c, "fp64")
    r.upload(cv0)
    dt = r.timestep(1.0)
    n, every = 20, 5
    J, g, _ = r.unrolled_adjoint(cv0, n, dt, every, 1)
    assert J > 0
    eps = 1e-6
    fd, ad = [], []
    for d in _density_blobs(c, 4, 21):
        jp, _, _ = r.unrolled_adjoint(cv0 + eps * d, n, dt, every, 1, with_grad=False)
        jm, _, _ = r.unrolled_adjoint(cv0 - eps * d, n, dt, every, 1, with_grad=False)
        fd.append((jp - jm) / (2 * eps))
        ad.append(float((g * d).sum()))
    fd, ad = np.array(fd), np.array(ad)
    # relative to the gradient's scale over the directions: a direction with
    # a small derivative is dominated by the differences' round-off (~1e-12)
    assert (np.abs(fd - ad) <= 1e-5 * np.abs(ad).max()).all(), (fd, ad)


def test_unrolled_adjoint_rejections(gpu_lib):
    """A zero checkpoint interval is an argument error."""
    c = _blast()
    with pytest.raises(gpu.RfluError):
        gpu.Region(c, "fp64").unrolled_adjoint(c.cv0, 2, 1e-3, 0, 1)


def test_unrolled_adjoint_mixed_against_fp64(gpu_lib):
    """The mixed primal sweeps and mixed stage VJPs give the FP64 unrolled
    gradient to FP32 accuracy on the smooth-background blast, and the
    checkpoint interval still does not change it."""
    num = cases.Numerics(space_order=2, space_discr=cases.DISCR_HLLC, reconst=cases.RECONST_BJ_COMP, cfl=0.4)
    c = cases.blast_hex(8, num=num, p_in=10.0, radius=0.15)
    cv0 = _smooth_background(c)
    r64, rm = gpu.Region(c, "fp64"), gpu.Region(c, "mixed")
    r64.upload(cv0)
    dt = r64.timestep(1.0)
    J64, g64, _ = r64.unrolled_adjoint(cv0, 20, dt, 5, 1)
    Jm, gm, _ = rm.unrolled_adjoint(cv0, 20, dt, 5, 1)
    Jm4, gm4, _ = rm.unrolled_adjoint(cv0, 20, dt, 4, 1)
    assert abs(Jm - J64) <= 1e-6 * abs(J64)
    assert np.abs(gm - g64).max() <= 1e-3 * np.abs(g64).max()
    assert Jm4 == Jm
    np.testing.assert_array_equal(gm4, gm)
