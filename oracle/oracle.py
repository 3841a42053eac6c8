"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this module, as the checker and as the timed CPU restatement.  It builds
oracle/_build/liboracle.so with the committed Makefile on first use.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class MeshDesc(C.Structure):
    _fields_ = [("nVert", C.c_int), ("nCells", C.c_int), ("nVertPerCell", C.c_int),
                ("xyz", C.POINTER(C.c_double)), ("c2v", C.POINTER(C.c_int)),
                ("nPatches", C.c_int), ("patchFaceOff", C.POINTER(C.c_int)),
                ("bf2v", C.POINTER(C.c_int)), ("patchBcType", C.POINTER(C.c_int)),
                ("patchOutflowType", C.POINTER(C.c_int)), ("patchPout", C.POINTER(C.c_double)),
                ("patchOrder", C.POINTER(C.c_int)), ("patchRelated", C.POINTER(C.c_int)),
                ("patchVals", C.POINTER(C.c_double)), ("patchSwitches", C.POINTER(C.c_int))]


class NumDesc(C.Structure):
    _fields_ = [("spaceOrder", C.c_int), ("spaceDiscr", C.c_int), ("reconst", C.c_int),
                ("rkScheme", C.c_int), ("piclBuild", C.c_int),
                ("cp", C.c_double), ("gamma", C.c_double), ("cfl", C.c_double),
                ("epsEntr", C.c_double), ("dissFact", C.c_double),
                ("dtImposed", C.c_double), ("dtMinLimit", C.c_double),
                ("cReconstCells", C.c_int), ("cReconstCellsWeight", C.c_double)]


def build():
    """Compile oracle.cpp as the committed Makefile does (-O2
    -ffp-contract=off -fopenmp); g++ is called directly so make is not
    required."""
    out = os.path.join(_HERE, "_build")
    os.makedirs(out, exist_ok=True)
    tmp = os.path.join(out, "liboracle.so.tmp")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-std=c++17", "-shared", "-o", tmp,
                    os.path.join(_HERE, "oracle.cpp")], check=True)
    os.replace(tmp, os.path.join(out, "liboracle.so"))


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        src = os.path.join(_HERE, "oracle.cpp")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(MeshDesc), C.POINTER(NumDesc)]
        L.orc_destroy.argtypes = [P]
        for n in ("orc_nfaces", "orc_stencil_nnz", "orc_nstages"):
            getattr(L, n).restype = C.c_int
            getattr(L, n).argtypes = [P]
        L.orc_patch_nfaces.restype = C.c_int
        L.orc_patch_nfaces.argtypes = [P, C.c_int]
        L.orc_timestep.restype = C.c_double
        L.orc_timestep.argtypes = [P, C.c_double]
        L.orc_rk_stage.argtypes = [P, C.c_int, C.c_double]
        L.orc_run.restype = C.c_int
        L.orc_run.argtypes = [P, C.c_int, C.POINTER(C.c_double), C.c_double]
        L.orc_run_fixed_dt.argtypes = [P, C.c_int, C.c_double]
        # every handle and array crosses as a full 64-bit pointer
        DP, IP, LLP = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_longlong)
        L.orc_get_faces.argtypes = [P, IP, IP, DP, DP]
        L.orc_get_cells.argtypes = [P, DP, DP]
        L.orc_get_patch.argtypes = [P, C.c_int, IP, DP, DP]
        L.orc_get_stencil.argtypes = [P, IP, IP, DP]
        L.orc_get_bface_stencil.argtypes = [P, IP, IP]
        L.orc_get_periodic.argtypes = [P, DP, DP]
        L.orc_get_periodic.restype = None
        L.orc_n_reflections.argtypes = [P]
        L.orc_n_reflections.restype = C.c_int
        L.orc_get_symmetry.argtypes = [P, IP, DP, DP]
        L.orc_get_symmetry.restype = None
        L.orc_set_state.argtypes = [P, DP]
        L.orc_get_state.argtypes = [P, DP, DP]
        L.orc_get_rhs.argtypes = [P, DP]
        L.orc_get_grad.argtypes = [P, DP]
        L.orc_residual.argtypes = [P, DP, DP]
        L.orc_counters.argtypes = [P, LLP, LLP, LLP]
        L.orc_rk_init.argtypes = [P, C.c_int]
        L.orc_cell_gradients.argtypes = [P]
        L.orc_convective_fluxes.argtypes = [P]
        L.orc_add_rhs.argtypes = [P, DP]
        L.orc_rk_update.argtypes = [P, C.c_int, C.c_double]
        for name in ("orc_rk_init", "orc_cell_gradients", "orc_convective_fluxes", "orc_add_rhs", "orc_rk_update"):
            getattr(L, name).restype = None
        L.orc_set_dt_imposed.argtypes = [P, C.c_double]
        L.orc_set_dt_imposed.restype = None
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = None
        L.orc_threads.argtypes = []
        L.orc_threads.restype = C.c_int
        for name in ("orc_get_faces", "orc_get_cells", "orc_get_patch", "orc_get_stencil", "orc_get_bface_stencil",
                     "orc_set_state",
                     "orc_get_state", "orc_get_rhs", "orc_get_grad", "orc_residual", "orc_counters",
                     "orc_rk_stage", "orc_run_fixed_dt", "orc_destroy"):
            getattr(L, name).restype = None
        _LIB = L
    return _LIB


def set_threads(n):
    """Threads of the oracle's OpenMP loops in this process (results do not
    depend on it)."""
    lib().orc_set_threads(int(n))


def threads():
    return lib().orc_threads()


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _mesh_arrays(case):
    xyz = np.ascontiguousarray(case.xyz, dtype=np.float64)
    c2v = np.ascontiguousarray(case.c2v, dtype=np.int32)
    off = np.zeros(len(case.patches) + 1, dtype=np.int32)
    for i, p in enumerate(case.patches):
        off[i + 1] = off[i] + len(p.bf2v)
    bf2v = np.ascontiguousarray(np.concatenate([p.bf2v for p in case.patches]).astype(np.int32))
    bct = np.array([p.bc_type for p in case.patches], dtype=np.int32)
    oft = np.array([p.outflow_type for p in case.patches], dtype=np.int32)
    pout = np.array([p.p_out for p in case.patches], dtype=np.float64)
    order = np.array([p.order for p in case.patches], dtype=np.int32)
    rel = np.array([getattr(p, "related", -1) for p in case.patches], dtype=np.int32)
    np_ = max(len(case.patches), 1)
    vals = np.zeros((np_, 8), dtype=np.float64)
    sw = np.zeros((np_, 2), dtype=np.int32)
    for i, p in enumerate(case.patches):
        v, w = tuple(getattr(p, "vals", ()) or ()), tuple(getattr(p, "switches", ()) or ())
        vals[i, :len(v)] = v
        sw[i, :len(w)] = w
    return xyz, c2v, off, bf2v, bct, oft, pout, order, rel, vals, sw


def num_desc(num):
    return NumDesc(num.space_order, num.space_discr, num.reconst, num.rk_scheme, num.picl_build,
                   num.cp, num.gamma, num.cfl, num.eps_entr, num.diss_fact, num.dt_imposed, num.dt_min_limit,
                   int(getattr(num, "c_reconst", 0)), float(getattr(num, "c_reconst_weight", 1.0)))


class Oracle:
    """The reference path on the CPU, one region, reference cell numbering.
    State arrays are returned as (nCells, 5) views of cv(5,nCells)."""

    def __init__(self, case):
        self.case = case
        self._keep = _mesh_arrays(case)
        xyz, c2v, off, bf2v, bct, oft, pout, order, rel, vals, sw = self._keep
        md = MeshDesc(xyz.shape[0], c2v.shape[0], c2v.shape[1], _ptr(xyz, C.c_double), _ptr(c2v, C.c_int),
                      len(case.patches), _ptr(off, C.c_int), _ptr(bf2v, C.c_int), _ptr(bct, C.c_int),
                      _ptr(oft, C.c_int), _ptr(pout, C.c_double), _ptr(order, C.c_int),
                      _ptr(rel, C.c_int) if (rel >= 0).any() else None, _ptr(vals, C.c_double),
                      _ptr(sw, C.c_int))
        self.nd = num_desc(case.num)
        self.h = lib().orc_create(C.byref(md), C.byref(self.nd))
        self.n_cells = c2v.shape[0]
        self.n_faces = lib().orc_nfaces(self.h)
        if case.cv0 is not None:
            self.set_state(case.cv0)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    # setup products
    def faces(self):
        nf = self.n_faces
        f2c = np.zeros((nf, 2), np.int32)
        f2v = np.zeros((nf, 4), np.int32)
        fn = np.zeros((nf, 4))
        fc = np.zeros((nf, 3))
        lib().orc_get_faces(self.h, _ptr(f2c, C.c_int), _ptr(f2v, C.c_int), _ptr(fn, C.c_double), _ptr(fc, C.c_double))
        return f2c, f2v, fn, fc

    def cells(self):
        vol = np.zeros(self.n_cells)
        cofg = np.zeros((self.n_cells, 3))
        lib().orc_get_cells(self.h, _ptr(vol, C.c_double), _ptr(cofg, C.c_double))
        return vol, cofg

    def patch(self, ip):
        n = lib().orc_patch_nfaces(self.h, ip)
        bf2c = np.zeros(n, np.int32)
        fn = np.zeros((n, 4))
        fc = np.zeros((n, 3))
        lib().orc_get_patch(self.h, ip, _ptr(bf2c, C.c_int), _ptr(fn, C.c_double), _ptr(fc, C.c_double))
        return bf2c, fn, fc

    def periodic(self):
        """(fc2 (nFaces, 3), stShift (nnz, 3)): face centroids in the second
        cell's frame and the translation of each stencil member's image."""
        nnz = lib().orc_stencil_nnz(self.h)
        fc2 = np.zeros((self.n_faces, 3))
        sh = np.zeros((max(nnz, 1), 3))
        lib().orc_get_periodic(self.h, _ptr(fc2, C.c_double), _ptr(sh, C.c_double))
        return fc2, sh[:nnz]

    def symmetry(self):
        """(stXf (nnz,), stShift (nnz, 3), Q (nXf, 3, 3)): per stencil member
        the reflection it is seen through (-1: none), the offset of its
        reflected centroid from its own, and the velocity reflections."""
        nnz = lib().orc_stencil_nnz(self.h)
        nx = lib().orc_n_reflections(self.h)
        xf = np.zeros(max(nnz, 1), np.int32)
        sh = np.zeros((max(nnz, 1), 3))
        q = np.zeros((max(nx, 1), 3, 3))
        lib().orc_get_symmetry(self.h, _ptr(xf, C.c_int), _ptr(sh, C.c_double), _ptr(q, C.c_double))
        return xf[:nnz], sh[:nnz], q[:nx]

    def stencil(self):
        off = np.zeros(self.n_cells + 1, np.int32)
        nnz = lib().orc_stencil_nnz(self.h)
        idx = np.zeros(max(nnz, 1), np.int32)
        moms = np.zeros((self.n_cells, 10))
        lib().orc_get_stencil(self.h, _ptr(off, C.c_int), _ptr(idx, C.c_int), _ptr(moms, C.c_double))
        return off, idx[:nnz], moms

    def bface_stencil(self):
        """CRECONSTC 1's boundary-face stencil: (off, faces), 0-based boundary
        face indices, patch after patch, nearest first."""
        off = np.zeros(self.n_cells + 1, np.int32)
        lib().orc_get_bface_stencil(self.h, _ptr(off, C.c_int), None)
        faces = np.zeros(max(int(off[-1]), 1), np.int32)
        lib().orc_get_bface_stencil(self.h, _ptr(off, C.c_int), _ptr(faces, C.c_int))
        return off, faces[:int(off[-1])]

    # state
    def set_state(self, cv):
        cv = np.ascontiguousarray(cv, dtype=np.float64)
        lib().orc_set_state(self.h, _ptr(cv, C.c_double))

    def state(self):
        cv = np.zeros((self.n_cells, 5))
        dv = np.zeros((self.n_cells, 3))
        lib().orc_get_state(self.h, _ptr(cv, C.c_double), _ptr(dv, C.c_double))
        return cv, dv

    def residual(self):
        rhs = np.zeros((self.n_cells, 5))
        grad = np.zeros((self.n_cells, 5, 3))
        lib().orc_residual(self.h, _ptr(rhs, C.c_double), _ptr(grad, C.c_double))
        return rhs, grad

    def timestep(self, t):
        return lib().orc_timestep(self.h, t)

    def rk_stage(self, istage, dt):
        lib().orc_rk_stage(self.h, istage, dt)

    def run(self, n_steps, t=0.0, end_time=0.0):
        tt = C.c_double(t)
        done = lib().orc_run(self.h, n_steps, C.byref(tt), end_time)
        return done, tt.value

    # one stage in the pieces of RungeKuttaMP's stage body
    def rk_init(self, istage):
        lib().orc_rk_init(self.h, istage)

    def cell_gradients(self):
        lib().orc_cell_gradients(self.h)

    def convective_fluxes(self):
        lib().orc_convective_fluxes(self.h)

    def add_rhs(self, src):
        s = np.ascontiguousarray(src, dtype=np.float64)
        lib().orc_add_rhs(self.h, _ptr(s, C.c_double))

    def rk_update(self, istage, dt):
        lib().orc_rk_update(self.h, istage, dt)

    def rhs(self):
        r = np.zeros((self.n_cells, 5))
        lib().orc_get_rhs(self.h, _ptr(r, C.c_double))
        return r

    def grad(self):
        g = np.zeros((self.n_cells, 5, 3))
        lib().orc_get_grad(self.h, _ptr(g, C.c_double))
        return g

    def n_stages(self):
        return lib().orc_nstages(self.h)

    def set_dt_imposed(self, dt):
        """TIMESTEP, the imposed first time step (the numerics are copied at
        creation)."""
        lib().orc_set_dt_imposed(self.h, dt)

    def run_fixed_dt(self, n_steps, dt):
        lib().orc_run_fixed_dt(self.h, n_steps, dt)

    def counters(self):
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
        lib().orc_counters(self.h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value
