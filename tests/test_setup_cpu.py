"""Host set-up (rflu_setup_build) against the oracle's restatement of
RFLU_BuildFaceList / RFLU_BuildGeometry / RFLU_BuildC2CStencil /
RFLU_ComputeWtsC2C: integer arrays and FP64 values must be identical."""
import re

import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, gpu


def _compare(case):
    o = Oracle(case)
    s = gpu.Setup(case)
    f2c, f2v, fn, fc = o.faces()
    vol, cofg = o.cells()
    np.testing.assert_array_equal(f2c + 1, s.f2c)
    np.testing.assert_array_equal(fn, s.fn)
    np.testing.assert_array_equal(fc, s.fc)
    np.testing.assert_array_equal(vol, s.vol)
    np.testing.assert_array_equal(cofg, s.cofg)
    pb = [o.patch(i) for i in range(len(case.patches))]
    np.testing.assert_array_equal(np.concatenate([p[0] for p in pb]) + 1, s.bf2c)
    np.testing.assert_array_equal(np.concatenate([p[1] for p in pb]), s.bfn)
    np.testing.assert_array_equal(np.concatenate([p[2] for p in pb]), s.bfc)
    off, idx, moms = o.stencil()
    np.testing.assert_array_equal(off, s.c2cs_off)
    np.testing.assert_array_equal(idx + 1, s.c2cs)
    if case.num.space_order > 1:
        np.testing.assert_array_equal(moms, s.moms)
    return o, s


def test_setup_sod_first_order():
    o, s = _compare(cases.sod(40, 4, 4))
    assert s.n_faces == 39 * 16 + 40 * 3 * 4 * 2
    assert len(s.c2cs) == 0


def test_setup_hex_second_order():
    o, s = _compare(cases.shock_sphere(6))
    sizes = np.diff(s.c2cs_off)
    assert sizes.max() == 26 and sizes.min() == 7   # interior / corner cells


def test_setup_jittered_tets_truncated_stencils():
    o, s = _compare(cases.blast_tets(5))
    sizes = np.diff(s.c2cs_off)
    assert sizes.max() == 40                          # truncated by shared-vertex rank


def test_setup_tiny_meshes():
    for nx, ny, nz in ((1, 1, 3), (2, 2, 2), (3, 1, 1)):
        c = cases.sod(nx, ny, nz)
        _compare(c)


def test_face_orientation_and_closure():
    """Face normals point from f2c(1) to f2c(2); every closed cell has a zero
    area-vector sum (interior faces +-, patch faces +)."""
    c = cases.blast_tets(4)
    s = gpu.Setup(c)
    acc = np.zeros((s.n_cells, 3))
    a = s.fn[:, :3] * s.fn[:, 3:4]
    np.add.at(acc, s.f2c[:, 0] - 1, a)
    np.add.at(acc, s.f2c[:, 1] - 1, -a)
    np.add.at(acc, s.bf2c - 1, s.bfn[:, :3] * s.bfn[:, 3:4])
    assert np.abs(acc).max() < 1e-15
    d = s.cofg[s.f2c[:, 1] - 1] - s.cofg[s.f2c[:, 0] - 1]
    assert (np.einsum("ij,ij->i", d, s.fn[:, :3]) > 0).all()
    assert abs(s.vol.sum() - 1.0) < 1e-12


def test_library_exports_every_header_symbol():
    """librflu_gpu.so loads without a GPU and exports each entry point that
    include/rflu_gpu.h declares."""
    import os
    import subprocess

    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "rflu_gpu.h")).read()
    declared = set(re.findall(r"\b(rflu_(?:gpu|setup)_\w+)\s*\(", hdr))
    L = gpu.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", gpu.library_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (rflu_\w+)", out))
    assert declared, "no declarations parsed"
    assert declared <= exported, declared - exported
    for name in declared:
        assert hasattr(L, name)


def test_setup_periodic_mesh_matches_oracle():
    """Translational periodic patch pairs: rflu_setup_build identifies the
    pairs' vertices as the oracle does and gives the same faces (across-period
    faces after the others), geometry in each cell's own frame, the faces'
    centroids in their second cells' frames (fc2), stencils on the
    identified mesh, moments with the members' nearest images, and those
    images' translations (c2csShift), bit for bit; the periodic patches keep
    no boundary faces."""
    c = cases.gas_jump_periodic()
    s = gpu.Setup(c)
    o = Oracle(c)
    f2c, _, fn, fc = o.faces()
    np.testing.assert_array_equal(s.f2c - 1, f2c)
    np.testing.assert_array_equal(s.fn, fn)
    np.testing.assert_array_equal(s.fc, fc)
    vol, cofg = o.cells()
    np.testing.assert_array_equal(s.vol, vol)
    np.testing.assert_array_equal(s.cofg, cofg)
    off, idx, moms = o.stencil()
    np.testing.assert_array_equal(s.c2cs_off, off)
    np.testing.assert_array_equal(s.c2cs - 1, idx)
    np.testing.assert_array_equal(s.moms, moms)
    fc2, sh = o.periodic()
    np.testing.assert_array_equal(s.fc2, fc2)
    px = cofg[idx] - np.repeat(cofg, np.diff(off), axis=0)
    np.testing.assert_array_equal(px + s.c2cs_shift, px + sh)
    assert (np.abs(s.c2cs_shift).max(axis=1) > 0).sum() > 0
    assert (s.patch_off == 0).all() and len(s.bf2c) == 0
    # a non-periodic mesh exports neither
    s2 = gpu.Setup(cases.gas_jump_closed())
    assert s2.fc2 is None and s2.c2cs_shift is None
