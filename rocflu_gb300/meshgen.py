"""Synthetic unstructured meshes in Rocflu's cell conventions.

Cells use the reference's local vertex order (modflu/RFLU_ModGrid.F90:92-96):
hexahedra have vertices 1-4 counter-clockwise on the low-z face and 5-8 above
them; tetrahedra are oriented so that local face (1,2,3) points away from
vertex 4.  Boundary faces are found as faces owned by a single cell and take
that cell's local vertex order, so their normals point out of the domain, as
the CENTAUR grids read by RFLU_ReadGridCENTAUR (utilities/part/
RFLU_ModCENTAUR.F90:776-1315) do.

A mesh is a dict with
  xyz    (nVert, 3) float64
  c2v    (nCells, 4 or 8) int32, 0-based
  patches: list of dicts {name, bf2v (n, 4) int32 with -1 in slot 3 for triangles}
Patches are ordered x-low, x-high, y-low, y-high, z-low, z-high.
"""
import numpy as np

# Local faces, 1-based as in the reference (RFLU_ModGrid.F90:92-96).
F2V_TET = np.array([[1, 2, 3], [2, 4, 3], [1, 3, 4], [1, 4, 2]]) - 1
F2V_HEX = np.array([[1, 4, 3, 2], [1, 2, 6, 5], [2, 3, 7, 6], [3, 4, 8, 7], [1, 5, 8, 4], [5, 6, 7, 8]]) - 1

PATCH_NAMES = ("xlow", "xhigh", "ylow", "yhigh", "zlow", "zhigh")


def _grid_vertices(nx, ny, nz, lo, hi):
    xs = np.linspace(lo[0], hi[0], nx + 1)
    ys = np.linspace(lo[1], hi[1], ny + 1)
    zs = np.linspace(lo[2], hi[2], nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    xyz = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    ijk = np.stack(np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij"), axis=-1)
    ijk = ijk.reshape(-1, 3)[:, ::-1]  # (i, j, k)
    return xyz, ijk


def _hex_c2v(nx, ny, nz):
    def vid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    c2v = np.stack([vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k),
                    vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1), vid(i, j + 1, k + 1)], axis=1)
    return c2v.astype(np.int64)


def _boundary_patches(c2v, ijk, dims):
    """Faces owned by one cell, grouped by the box side they lie on, in order
    of discovery (cell loop x local-face loop)."""
    nvc = c2v.shape[1]
    f2v = F2V_TET if nvc == 4 else F2V_HEX
    nfl, fvs = f2v.shape
    nc = c2v.shape[0]
    fv = c2v[:, f2v]                      # (nc, nfl, fvs)
    fv = fv.reshape(nc * nfl, fvs)
    key = np.sort(fv, axis=1)
    order = np.lexsort(key.T[::-1])
    ks = key[order]
    same_next = np.all(ks[1:] == ks[:-1], axis=1)
    dup = np.zeros(len(ks), dtype=bool)
    dup[1:] |= same_next
    dup[:-1] |= same_next
    single = np.sort(order[~dup])         # face slots (cell*nfl + lf) in discovery order
    bfv = fv[single]
    patches = []
    for side in range(6):
        axis, at_hi = side // 2, side % 2
        target = dims[axis] if at_hi else 0
        on = np.all(ijk[bfv][:, :, axis] == target, axis=1)
        faces = bfv[on]
        bf2v = np.full((len(faces), 4), -1, dtype=np.int32)
        bf2v[:, :fvs] = faces
        patches.append({"name": PATCH_NAMES[side], "bf2v": bf2v})
    return patches


def hex_box(nx, ny, nz, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """Hexahedral box of nx*ny*nz cells, cells numbered i-fastest."""
    xyz, ijk = _grid_vertices(nx, ny, nz, lo, hi)
    c2v = _hex_c2v(nx, ny, nz)
    patches = _boundary_patches(c2v, ijk, (nx, ny, nz))
    return {"xyz": np.ascontiguousarray(xyz), "c2v": c2v.astype(np.int32), "patches": patches}


# Kuhn (Freudenthal) split of the unit cube along the diagonal from local
# vertex 1 (0,0,0) to vertex 7 (1,1,1): one tetrahedron per ordering of the
# three axis steps.  The split is the same in every hex, so faces conform.
_CUBE = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])


def _kuhn_tets():
    tets = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        p = np.zeros(3, dtype=int)
        pts = [p.copy()]
        for ax in perm:
            p[ax] += 1
            pts.append(p.copy())
        ids = [int(np.where((_CUBE == q).all(axis=1))[0][0]) for q in pts]
        tets.append(ids)
    return np.array(tets)


KUHN_TETS = _kuhn_tets()


def tet_box(n, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), jitter=0.2, seed=0):
    """n^3 hexahedra, each split into 6 tetrahedra (Kuhn split); interior
    vertices moved by a seeded uniform jitter of +-jitter*h per coordinate
    (numpy PCG64 with the given seed).  Cell order: hex order (i fastest),
    6 tetrahedra per hex in KUHN_TETS order."""
    xyz, ijk = _grid_vertices(n, n, n, lo, hi)
    h = (np.asarray(hi, float) - np.asarray(lo, float)) / n
    if jitter:
        rng = np.random.Generator(np.random.PCG64(seed))
        d = rng.uniform(-jitter, jitter, size=xyz.shape) * h
        interior = np.all((ijk > 0) & (ijk < n), axis=1)
        xyz = xyz + d * interior[:, None]
    hexes = _hex_c2v(n, n, n)
    c2v = hexes[:, KUHN_TETS].reshape(-1, 4)
    # orient: det[v2-v1, v3-v1, v4-v1] < 0 so that face (1,2,3) points away from vertex 4
    p = xyz[c2v]
    det = np.einsum("ij,ij->i", np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])
    if np.any(det == 0):
        raise ValueError("degenerate tetrahedron in tet_box")
    flip = det > 0
    c2v[flip, 1], c2v[flip, 2] = c2v[flip, 2].copy(), c2v[flip, 1].copy()
    patches = _boundary_patches(c2v, ijk, (n, n, n))
    return {"xyz": np.ascontiguousarray(xyz), "c2v": c2v.astype(np.int32), "patches": patches}


def cell_centers(mesh):
    """Vertex-average cell centres (RFLU_ComputeApproxCentroids)."""
    return mesh["xyz"][mesh["c2v"]].mean(axis=1)
