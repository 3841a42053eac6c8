"""The reference's file formats on the host side of the drop-in: grids in the
CENTAUR ASCII format the solver reads (GRIDSRC 0) and the fluid dumps it
restarts from and the test harness compares.

* CENTAUR ASCII grid (`.hyb.asc`), as RFLU_ReadGridCENTAURASCII reads it
  (utilities/part/RFLU_ModCENTAUR.F90:776-1315): an A80 title; the vertex
  count (I16); the x, then y, then z coordinates of every vertex, five per
  line (E16.9 or E24.16, told apart by the first line's width); a block of
  vertex flags (10I16 per line, read and discarded); then for tetrahedra,
  hexahedra, prisms and pyramids in turn a count (I16), one block per local
  vertex (10I16 per line, 1-based vertex ids) and a block of flags; the patch
  count (I16) and, if > 0, three blocks of the patch table bInfo(3, nPatches)
  (boundary type, last boundary triangle, last boundary quad of each patch,
  cumulative: RFLU_ModCENTAUR.F90:484-499), the patch names (A80 each), the
  boundary triangle count and three vertex blocks, the boundary quad count
  and four vertex blocks.
* Fluid dump (`restart_data/fluid_SSSSSSSS_RRRRR.dat`), as
  RFLU_WriteRestartData writes it (modflu/RFLU_ModRestartData.F90:146-230):
  an unformatted stream file (no record markers): 'RFLUDUMP', version 5
  (int32), step (int64), time (float64), global region, cells, nCv, form
  (1 pure, 2 volume-weighted), PICL flag (int32 each); nCv arrays of the
  cells' conserved variables (float64, cell order of the region); then the
  count of NSCBC patches with stored face states (int32) and, per patch, its
  global id and face count (int32) and nCv arrays over its faces.  Written
  to `<name>.tmp` and renamed (RFLU_FinishRestartFile).
"""
import os
import struct

import numpy as np

FLUID_DUMP_HEADER = struct.Struct("<8siqd5i")
FLUID_DUMP_VERSION = 5
FORM_PURE, FORM_VOLUME_WEIGHTED = 1, 2
CELL_BLOCKS = (("tet2v", 4), ("hex2v", 8), ("pri2v", 6), ("pyr2v", 5))


# ---------------------------------------------------------------------------
# fluid dumps
# ---------------------------------------------------------------------------
def fluid_dump_name(out_dir, step, region):
    """restart_data/fluid_<step:08d>_<region:05d>.dat under out_dir
    (FluidDumpName, RFLU_ModRestartData.F90)."""
    return os.path.join(out_dir, "restart_data", "fluid_%08d_%05d.dat" % (step, region))


def write_fluid_dump(path, cv, step, time, region=1, form=FORM_PURE, nscbc=None):
    """cv: (nCells, nCv) conserved variables in the region's cell order.
    nscbc: {global patch id: (nFaces, nCv) face states} of NSCBC patches."""
    cv = np.asarray(cv, dtype="<f8")
    n, ncv = cv.shape
    nscbc = nscbc or {}
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(FLUID_DUMP_HEADER.pack(b"RFLUDUMP", FLUID_DUMP_VERSION, int(step), float(time), int(region), n, ncv,
                                       int(form), 0))
        for k in range(ncv):
            f.write(np.ascontiguousarray(cv[:, k]).tobytes())
        f.write(struct.pack("<i", len(nscbc)))
        for patch in sorted(nscbc):
            fs = np.asarray(nscbc[patch], dtype="<f8")
            f.write(struct.pack("<2i", int(patch), fs.shape[0]))
            for k in range(ncv):
                f.write(np.ascontiguousarray(fs[:, k]).tobytes())
    os.replace(tmp, path)


def read_fluid_dump(path):
    """dict: step, time, region, form, cv (nCells, nCv), nscbc {patch: (nFaces,
    nCv)}.  Dumps with PICL data (withPicl = 1) are rejected: the particle
    coupling is not part of this path."""
    with open(path, "rb") as f:
        data = f.read()
    magic, version, step, time, region, n, ncv, form, with_picl = FLUID_DUMP_HEADER.unpack_from(data, 0)
    if magic != b"RFLUDUMP" or version != FLUID_DUMP_VERSION:
        raise ValueError("%s: not a version %d fluid dump" % (path, FLUID_DUMP_VERSION))
    if with_picl:
        raise ValueError("%s: a dump with particle data (not on this path)" % path)
    pos = FLUID_DUMP_HEADER.size
    cv = np.frombuffer(data, "<f8", n * ncv, pos).reshape(ncv, n).T.copy()
    pos += 8 * n * ncv
    (npatch,) = struct.unpack_from("<i", data, pos)
    pos += 4
    nscbc = {}
    for _ in range(npatch):
        patch, nf = struct.unpack_from("<2i", data, pos)
        pos += 8
        nscbc[patch] = np.frombuffer(data, "<f8", nf * ncv, pos).reshape(ncv, nf).T.copy()
        pos += 8 * nf * ncv
    if pos != len(data):
        raise ValueError("%s: %d trailing bytes" % (path, len(data) - pos))
    return {"step": step, "time": time, "region": region, "form": form, "cv": cv, "nscbc": nscbc}


# ---------------------------------------------------------------------------
# CENTAUR ASCII grids
# ---------------------------------------------------------------------------
def _fortran_real(tok):
    return float(tok.replace("D", "E").replace("d", "e"))


class _Lines:
    def __init__(self, path):
        with open(path) as f:
            self.lines = f.read().splitlines()
        self.i = 0

    def line(self):
        s = self.lines[self.i]
        self.i += 1
        return s

    def fixed(self, count, width, per_line, conv):
        """count values in fixed-width fields, per_line to a line (Fortran
        list-directed by format: a short last line holds the rest)."""
        out = []
        while len(out) < count:
            s = self.line()
            m = min(per_line, count - len(out))
            for k in range(m):
                out.append(conv(s[k * width:(k + 1) * width]))
        return out


def read_centaur_ascii(path):
    """dict: title, xyz (nVert, 3), tet2v/hex2v/pri2v/pyr2v (n, nv) 0-based,
    patches [{bc_type, name, tris (n, 3), quads (n, 4)}] (0-based vertices)."""
    L = _Lines(path)
    title = L.line()[:80]
    (nvert,) = L.fixed(1, 16, 1, int)
    first = L.lines[L.i]
    per = min(5, nvert)
    width = len(first.rstrip()) // per if per else 16
    if width not in (16, 24) or len(first.rstrip()) != per * width:
        raise ValueError("%s: coordinates must be 5 values per line, 16 or 24 characters each" % path)
    xyz = np.empty((nvert, 3))
    for k in range(3):
        xyz[:, k] = L.fixed(nvert, width, 5, _fortran_real)
    L.fixed(nvert, 16, 10, int)  # vertex flags
    out = {"title": title.rstrip(), "xyz": xyz}
    for name, nv in CELL_BLOCKS:
        (n,) = L.fixed(1, 16, 1, int)
        a = np.empty((n, nv), dtype=np.int32)
        if n > 0:
            for k in range(nv):
                a[:, k] = L.fixed(n, 16, 10, int)
            L.fixed(n, 16, 10, int)  # cell flags
        out[name] = a - 1
    (npatch,) = L.fixed(1, 16, 1, int)
    patches = []
    if npatch > 0:
        binfo = np.array([L.fixed(npatch, 16, 10, int) for _ in range(3)], dtype=np.int64)
        names = [L.line()[:80].rstrip() for _ in range(npatch)]
        (ntri,) = L.fixed(1, 16, 1, int)
        tris = np.empty((ntri, 3), dtype=np.int32)
        for k in range(3):
            if ntri:
                tris[:, k] = L.fixed(ntri, 16, 10, int)
        (nquad,) = L.fixed(1, 16, 1, int)
        quads = np.empty((nquad, 4), dtype=np.int32)
        for k in range(4):
            if nquad:
                quads[:, k] = L.fixed(nquad, 16, 10, int)
        t0 = q0 = 0
        for p in range(npatch):
            t1, q1 = binfo[1, p], binfo[2, p]
            patches.append({"bc_type": int(binfo[0, p]), "name": names[p], "tris": tris[t0:t1] - 1,
                            "quads": quads[q0:q1] - 1})
            t0, q0 = t1, q1
    out["patches"] = patches
    return out


def write_centaur_ascii(path, xyz, cells, patches, title="", wide=True):
    """The inverse of read_centaur_ascii: cells {"tet2v"|"hex2v"|"pri2v"|
    "pyr2v": (n, nv) 0-based}, patches [{bc_type, name, tris, quads}].
    wide: E24.16 coordinates (else E16.9)."""
    def ints(f, vals):
        vals = list(vals)
        for k in range(0, len(vals), 10):
            f.write("".join("%16d" % v for v in vals[k:k + 10]) + "\n")

    def reals(f, vals):
        fmt = "%24.16E" if wide else "%16.9E"
        vals = list(vals)
        for k in range(0, len(vals), 5):
            f.write("".join(fmt % v for v in vals[k:k + 5]) + "\n")

    xyz = np.asarray(xyz, float)
    with open(path, "w") as f:
        f.write("%-80s\n" % title[:80])
        ints(f, [xyz.shape[0]])
        for k in range(3):
            reals(f, xyz[:, k])
        ints(f, [0] * xyz.shape[0])
        for name, nv in CELL_BLOCKS:
            a = np.asarray(cells.get(name, np.zeros((0, nv), np.int32)))
            ints(f, [a.shape[0]])
            if a.shape[0]:
                for k in range(nv):
                    ints(f, a[:, k] + 1)
                ints(f, [0] * a.shape[0])
        ints(f, [len(patches)])
        if patches:
            nt = np.cumsum([len(p["tris"]) for p in patches])
            nq = np.cumsum([len(p["quads"]) for p in patches])
            ints(f, [p["bc_type"] for p in patches])
            ints(f, nt)
            ints(f, nq)
            for p in patches:
                f.write("%-80s\n" % p["name"][:80])
            tris = np.concatenate([np.asarray(p["tris"], np.int64).reshape(-1, 3) for p in patches])
            quads = np.concatenate([np.asarray(p["quads"], np.int64).reshape(-1, 4) for p in patches])
            ints(f, [len(tris)])
            for k in range(3):
                if len(tris):
                    ints(f, tris[:, k] + 1)
            ints(f, [len(quads)])
            for k in range(4):
                if len(quads):
                    ints(f, quads[:, k] + 1)


def case_from_centaur(grid, kinds, num, cv0=None, name="centaur"):
    """A Case of this package from a read_centaur_ascii grid: one cell type
    (all tetrahedra or all hexahedra: the set-up takes one vertex count per
    mesh), patch p's boundary conditions from kinds[p] (the .bc file's
    sections, e.g. {"bc_type": cases.BC_SLIPWALL, "order": 1})."""
    from . import cases

    blocks = [(k, grid[k]) for k, _ in CELL_BLOCKS if len(grid[k])]
    if len(blocks) != 1 or blocks[0][0] not in ("tet2v", "hex2v"):
        raise ValueError("the set-up takes meshes of one cell type, tetrahedra or hexahedra")
    c2v = np.ascontiguousarray(blocks[0][1], dtype=np.int32)
    patches = []
    for p, k in zip(grid["patches"], kinds):
        if len(p["tris"]) and len(p["quads"]):
            raise ValueError("patch %s mixes triangles and quadrilaterals" % p["name"])
        bf2v = np.full((len(p["tris"]) + len(p["quads"]), 4), -1, dtype=np.int32)  # triangles: -1 fourth
        if len(p["tris"]):
            bf2v[:, :3] = p["tris"]
        else:
            bf2v[:, :] = p["quads"]
        patches.append(cases.Patch(bf2v=bf2v, name=p["name"], **k))
    return cases.Case(name, np.ascontiguousarray(grid["xyz"]), c2v, patches, num, cv0)


# ---------------------------------------------------------------------------
# input deck (.inp) and boundary-condition file (.bc)
# ---------------------------------------------------------------------------
def read_deck(text):
    """Sections of a deck in the reference's syntax (libfloflu/ReadSection):
    a line '# NAME' opens a section, a line '#' closes it, each line in
    between is 'KEY value' with '!' starting a comment.  Returns
    {NAME: {KEY: value string}}; sections of the same name accumulate in a
    list under 'NAME*' (the .bc file repeats BC sections)."""
    out, name, cur = {}, None, None
    for raw in text.splitlines():
        line = raw.split("!", 1)[0].rstrip()
        s = line.strip()
        if not s:
            continue
        if s.startswith("#"):
            tag = s[1:].strip().split()
            if name is not None:
                out.setdefault(name + "*", []).append(cur)
                out.setdefault(name, cur)
                name = cur = None
            if tag and tag[0] != "END":
                name, cur = tag[0].upper(), {}
            continue
        if cur is not None:
            tok = s.split()
            cur[tok[0].upper()] = " ".join(tok[1:])
    if name is not None:
        out.setdefault(name + "*", []).append(cur)
        out.setdefault(name, cur)
    return out


def apply_overrides(deck, overrides):
    """overrides {"SECTION/KEY": value} (the reference test harness's form)."""
    for k, v in overrides.items():
        sec, key = k.split("/")
        deck.setdefault(sec, {})[key] = str(v)
    return deck


def numerics_from_deck(deck):
    """(cases.Numerics, end time, boundary-face order) from a deck's NUMERICS,
    TIMESTEP and REFERENCE sections, with the reference's defaults where a
    key is absent (libflu/RFLU_InitInputValues.F90:181-200: DISCR 1, ORDER 1,
    RECONST 2, CFL 3, DISSFACT 1, no constrained gradients, ORDERBF 1); keys
    without a default here must be present.  Settings off this path (viscous
    model, constrained gradients, AUSM+up, steady flow) raise ValueError."""
    from . import cases

    num = deck.get("NUMERICS", {})
    ts = deck.get("TIMESTEP", {})
    ref = deck.get("REFERENCE", {})
    flow = deck.get("FLOWMODEL", {})

    def val(sec, key, default=None, conv=float):
        if key in sec:
            return conv(float(sec[key]))
        if default is None:
            raise ValueError("deck: %s is required" % key)
        return default

    if val(flow, "MODEL", 0, int) != 0:
        raise ValueError("deck: only the Euler model (MODEL 0) is on this path")
    if val(ts, "FLOWTYPE", 1, int) != 1:
        raise ValueError("deck: only unsteady flow (FLOWTYPE 1) is on this path")
    creconst = val(num, "CRECONSTC", 0, int)
    if creconst not in (0, 1):
        raise ValueError("deck: CRECONSTC must be 0 or 1")
    discr = val(num, "DISCR", 1, int)
    if discr not in (1, 3, 4):
        raise ValueError("deck: DISCR must be 1 (Roe), 3 (HLLC) or 4 (AUSM+)")
    n = cases.Numerics(space_order=val(num, "ORDER", 1, int), space_discr=discr, reconst=val(num, "RECONST", 2, int),
                       rk_scheme=val(ts, "RKSCHEME", None, int), cfl=val(num, "CFL", 3.0),
                       cp=val(ref, "CP"), gamma=val(ref, "GAMMA"), eps_entr=val(num, "ENTROPY", 0.05),
                       diss_fact=val(num, "DISSFACT", 1.0), dt_imposed=val(ts, "TIMESTEP"),
                       dt_min_limit=val(ts, "DTMINLIMIT"), c_reconst=creconst,
                       c_reconst_weight=abs(val(num, "CRECONSTCW", 1.0)))
    return n, val(ts, "MAXTIME"), val(num, "ORDERBF", 1, int)


def patch_kinds_from_bc(bc_deck, n_patches, order_default=1):
    """Boundary conditions per patch from a .bc file's sections (read_deck of
    its text), as modflu/RFLU_ModReadBcInputFile.F90 reads them: BC_SLIPW;
    BC_OUTFLOW (TYPE 0 supersonic, 1 subsonic at PRESS, 2 mixed);
    BC_NOSLIP / BC_NOSLIP_HFLUX and BC_NOSLIP_TEMP; BC_FARF (MACH, ATTACK and
    SLIP in degrees, PRESS, TEMP, CORR); BC_INFLOW / BC_INFLOW_TOTANG (TYPE,
    FIXED, PTOT, TTOT, BETAH and BETAV in degrees, MACH unless subsonic);
    BC_INFLOW_VELTEMP (TYPE, VELX, VELY, VELZ, TEMP, PRESS unless subsonic);
    BC_INJECT (MFRATE, TEMP); BC_SYMMETRY; BC_PERIODIC with RELPATCH lo hi
    (translational: ANGLE 0); each over PATCH lo hi (1-based), ORDER 2 or the
    boundary-face order.  Angles are converted with the reference's
    global%deg2rad (libflu/RFLU_InitGlobal.F90:331-333).  Other conditions
    raise ValueError."""
    import math

    from . import cases

    deg2rad = 1.0 / (180.0 / (4.0 * math.atan(1.0)))

    def f(s, key, default=None):
        if key in s:
            return float(s[key])
        if default is None:
            raise ValueError("bc: %s is required" % key)
        return default

    def kind_of(sec, s):
        if sec == "BC_SLIPW":
            return {"bc_type": cases.BC_SLIPWALL}
        if sec == "BC_OUTFLOW":
            return {"bc_type": cases.BC_OUTFLOW, "outflow_type": int(f(s, "TYPE", 0)), "p_out": f(s, "PRESS", 0.0)}
        if sec in ("BC_NOSLIP", "BC_NOSLIP_HFLUX"):
            return {"bc_type": cases.BC_NOSLIPWALL_HFLUX}
        if sec == "BC_NOSLIP_TEMP":
            return {"bc_type": cases.BC_NOSLIPWALL_TEMP}
        if sec == "BC_FARF":
            return {"bc_type": cases.BC_FARFIELD, "switches": (int(f(s, "CORR", 0)), 0),
                    "vals": (f(s, "MACH"), f(s, "ATTACK") * deg2rad, f(s, "SLIP") * deg2rad, f(s, "PRESS"),
                             f(s, "TEMP"))}
        if sec in ("BC_INFLOW", "BC_INFLOW_TOTANG"):
            t = int(f(s, "TYPE"))
            mach = f(s, "MACH") if t != cases.BCOPT_SUBSONIC else 0.0
            return {"bc_type": cases.BC_INFLOW_TOTANG, "switches": (t, int(f(s, "FIXED", 0))),
                    "vals": (f(s, "PTOT"), f(s, "TTOT"), f(s, "BETAH") * deg2rad, f(s, "BETAV") * deg2rad, mach)}
        if sec == "BC_INFLOW_VELTEMP":
            t = int(f(s, "TYPE"))
            press = f(s, "PRESS") if t != cases.BCOPT_SUBSONIC else 0.0
            return {"bc_type": cases.BC_INFLOW_VELTEMP, "switches": (t, 0),
                    "vals": (f(s, "VELX"), f(s, "VELY"), f(s, "VELZ"), f(s, "TEMP"), press)}
        if sec == "BC_INJECT":
            return {"bc_type": cases.BC_INJECTION, "vals": (f(s, "MFRATE"), f(s, "TEMP"))}
        if sec == "BC_SYMMETRY":
            return {"bc_type": cases.BC_SYMMETRY}
        if sec == "BC_PERIODIC":
            if f(s, "ANGLE", 0.0) != 0.0:
                raise ValueError("bc: rotational periodic patches are not on this path")
            return {"bc_type": cases.BC_PERIODIC}
        return None

    known = ("BC_SLIPW", "BC_OUTFLOW", "BC_NOSLIP", "BC_NOSLIP_HFLUX", "BC_NOSLIP_TEMP", "BC_FARF", "BC_INFLOW",
             "BC_INFLOW_TOTANG", "BC_INFLOW_VELTEMP", "BC_INJECT", "BC_SYMMETRY", "BC_PERIODIC")
    kinds = [None] * n_patches
    for sec in known:
        for s in bc_deck.get(sec + "*", []):
            lo, hi = (int(float(v)) for v in s["PATCH"].split()[:2])
            k = kind_of(sec, s)
            # (a symmetry face is an interior face to its virtual cell: the
            # device takes the interior order there whatever the patch's)
            k["order"] = 2 if int(float(s.get("ORDER", order_default))) == 2 else 1
            rel = None
            if sec == "BC_PERIODIC":
                if "RELPATCH" not in s:
                    raise ValueError("bc: BC_PERIODIC needs RELPATCH")
                rel = int(float(s["RELPATCH"].split()[0]))
            for p in range(lo, hi + 1):
                kinds[p - 1] = dict(k, related=(rel + p - lo - 1)) if rel is not None else k
    others = [k for k in bc_deck if k.startswith("BC_") and not k.endswith("*") and k not in known]
    if others or any(k is None for k in kinds):
        raise ValueError("bc: conditions not on this path (%s)" % ", ".join(others))
    return kinds
