// Host set-up of one region: face list, geometry, C2C stencils and stencil
// moments, reproducing the numbering and the FP64 values that
// RFLU_InitFlowSolver (rocflu/RFLU_InitFlowSolver.F90:496-931) leaves in
// t_grid.  Built with -ffp-contract=off so that every value matches the
// reference's no-FMA evaluation bit for bit.
//
// Face list: the reference hashes each cell face in the cell loop and numbers
// faces by first insertion (RFLU_BuildFaceList, modflu/RFLU_ModFaceList.F90:
// 784-1585; RFLU_HashFace, modflu/RFLU_ModHashTable.F90:618-734).  Here every
// (cell, local face) slot gets a vertex key, slots are bucketed by smallest
// vertex and sorted, and a matched pair's face id is the rank of its lower
// slot -- the same order, built without a hash table and in parallel.
#include "constr.h"
#include <algorithm>
#include <map>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "../../include/rflu_gpu.h"
#include "errors.h"

namespace {

// Local faces (modflu/RFLU_ModGrid.F90:92-96), 0-based.
const int kTetFace[4][3] = {{0, 1, 2}, {1, 3, 2}, {0, 2, 3}, {0, 3, 1}};
const int kHexFace[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};

struct SlotKey {
  int k1, k2;    // 2nd and 3rd smallest vertex (bucket = smallest)
  int64_t slot;  // cell*nLocalFaces + localFace, or -(1+boundary face index)
};

// Face vector and centroid of a triangle or quadrilateral, the formulas of
// FaceVectorTria/Quad (libfloflu/FaceVector.F90) and FaceCentroidTria/Quad
// (libfloflu/FaceCentroid.F90).
void faceGeom(const double *xyz, const int *v, int nv, double *vec, double *cen) {
  const double *a = xyz + 3 * (size_t)v[0], *b = xyz + 3 * (size_t)v[1], *c = xyz + 3 * (size_t)v[2];
  if (nv == 3) {
    double e1x = a[0] - b[0], e1y = a[1] - b[1], e1z = a[2] - b[2];
    double e2x = a[0] - c[0], e2y = a[1] - c[1], e2z = a[2] - c[2];
    vec[0] = 0.5 * (e1y * e2z - e2y * e1z);
    vec[1] = -0.5 * (e1x * e2z - e2x * e1z);
    vec[2] = 0.5 * (e1x * e2y - e2x * e1y);
    const double third = 1.0 / 3.0;
    for (int d = 0; d < 3; ++d) cen[d] = third * (a[d] + b[d] + c[d]);
  } else {
    const double *q = xyz + 3 * (size_t)v[3];
    double dax = c[0] - a[0], day = c[1] - a[1], daz = c[2] - a[2];
    double dbx = b[0] - q[0], dby = b[1] - q[1], dbz = b[2] - q[2];
    vec[0] = 0.5 * (daz * dby - day * dbz);
    vec[1] = 0.5 * (dax * dbz - daz * dbx);
    vec[2] = 0.5 * (day * dbx - dax * dby);
    for (int d = 0; d < 3; ++d) cen[d] = 0.25 * (a[d] + b[d] + c[d] + q[d]);
  }
}

// Unstable quicksort of (fraction, cell) pairs by fraction.  Equal
// fractions keep the order this particular partition scheme produces, which
// decides which equally-shared neighbours survive the 40-member cap; it is
// the partition of QuickSortRFREALInteger (modfloflu/ModSortSearch.F90:
// 990-1091), which the stencil must reproduce exactly.
void sortFractions(double *a, int *b, int n) {
  if (n <= 0) return;
  int lo[50], hi[50], top = 0;
  lo[0] = 0;
  hi[0] = n - 1;
  top = 1;
  while (top > 0) {
    --top;
    int l = lo[top], r = hi[top];
    while (l < r) {
      int i = l, j = r;
      const double pivot = a[(l + r + 2) / 2 - 1];
      for (;;) {
        while (a[i] < pivot) ++i;
        while (pivot < a[j]) --j;
        if (i > j) break;
        std::swap(a[i], a[j]);
        std::swap(b[i], b[j]);
        ++i;
        --j;
        if (i > j) break;
      }
      if (j - l >= r - i) {
        if (l < j) { lo[top] = l; hi[top] = j; ++top; }
        l = i;
      } else {
        if (i < r) { lo[top] = i; hi[top] = r; ++top; }
        r = j;
      }
    }
  }
}

// Singular-value ratio test of RFLU_InvertMatrixSVD (libflu/
// RFLU_InvertMatrixSVD.F90) on the n x n normal matrix g = A^T A of a
// column-scaled matrix A (n <= 4): its eigenvalues (cyclic Jacobi) are the
// squared singular values; returns how many count as zero.
int normalSingularCount(double g[4][4], int n) {
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = 0; q < n; ++q) (p == q ? tot : off) += g[p][q] * g[p][q];
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        if (g[p][q] == 0.0) continue;
        double th = (g[q][q] - g[p][p]) / (2.0 * g[p][q]);
        double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double gkp = g[k][p], gkq = g[k][q];
          g[k][p] = c * gkp - s * gkq;
          g[k][q] = s * gkp + c * gkq;
        }
        for (int k = 0; k < n; ++k) {
          double gpk = g[p][k], gqk = g[q][k];
          g[p][k] = c * gpk - s * gqk;
          g[q][k] = s * gpk + c * gqk;
        }
      }
  }
  double sv[4];
  for (int p = 0; p < n; ++p) sv[p] = std::sqrt(std::max(g[p][p], 0.0));
  std::sort(sv, sv + n, [](double x, double y) { return x > y; });
  int count = (sv[0] > 100.0 * 2.220446049250313e-16) ? 0 : 1;
  for (int i = 1; i < n; ++i)
    if (!(sv[i] > 0.01 * sv[i - 1])) { count += n - i; break; }
  return count;
}

// The same for a rows x 4 stencil matrix A (row-major).
int singularCount(const std::vector<double> &A, int rows) {
  double g[4][4] = {};
  for (int p = 0; p < 4; ++p)
    for (int q = p; q < 4; ++q) {
      double s = 0.0;
      for (int r = 0; r < rows; ++r) s += A[r * 4 + p] * A[r * 4 + q];
      g[p][q] = g[q][p] = s;
    }
  return normalSingularCount(g, 4);
}

}  // namespace

namespace rflu {

namespace {
// FloatEqual (modfloflu/ModTools.F90:129-148)
bool floatEqual(double a, double b, double tol) { return std::fabs(a - b) <= (1.0 + 0.5 * std::fabs(a + b)) * tol; }

bool isWallOrInjection(int t) { return t == 70 || t == 71 || t == 60 || t == 90; }

// RFLU_GetConstrType for a TCPERF gas and the variables (rho, u, v, w, p):
// whether boundary face b of a patch of type t constrains variable k.
bool dirichlet(int t, double minj, const double *n, int k) {
  if (k == 0) return t == 90 && minj > 0.0;
  if (k == 4) return false;
  if (t == 70 || t == 71) return true;
  if (t == 60 || t == 90) return floatEqual(std::fabs(n[k - 1]), 1.0, 1.0e-6);
  return false;
}
}  // namespace

int planConstrained(const ConstrInput &in, ConstrPlan &P, int *bad, bool withWeights) {
  const int nc = in.nCells;
  const int maxTemp = 18, maxMembs = 9;
  // per wall/injection patch: each cell's face on it (the last one when a
  // cell has several: RFLU_AddBFaces keys its sorted copy of bf2c face by
  // face, so equal cells end up with the last face's key)
  std::vector<std::vector<int>> faceOf(in.nPatches);
  for (int ip = 0; ip < in.nPatches; ++ip) {
    if (!isWallOrInjection(in.patchType[ip]) || in.patchFaceOff[ip + 1] == in.patchFaceOff[ip]) continue;
    faceOf[ip].assign(nc, -1);
    for (int b = in.patchFaceOff[ip]; b < in.patchFaceOff[ip + 1]; ++b) faceOf[ip][in.bf2c[b]] = b;
  }
  P.bfOff.assign(nc + 1, 0);
  P.bfIdx.clear();
  std::vector<int> found;
  std::vector<double> dist;
  std::vector<int> key;
  for (int ic = 0; ic < nc; ++ic) {
    found.clear();
    bool full = false;
    for (int m = -1; m < in.stOff[ic + 1] - in.stOff[ic] && !full; ++m) {
      const int cell = (m < 0) ? ic : in.stIdx[in.stOff[ic] + m];
      for (int ip = 0; ip < in.nPatches; ++ip) {
        if (faceOf[ip].empty()) continue;
        const int b = faceOf[ip][cell];
        if (b < 0) continue;
        if ((int)found.size() >= maxTemp) {
          full = true;
          break;
        }
        found.push_back(b);
      }
    }
    const int n = (int)found.size();
    dist.resize(n);
    key.resize(n);
    const double *x = &in.cofg[3 * (size_t)ic];
    for (int k = 0; k < n; ++k) {
      const double *f = &in.bfc[3 * (size_t)found[k]];
      const double dx = f[0] - x[0], dy = f[1] - x[1], dz = f[2] - x[2];
      dist[k] = dx * dx + dy * dy + dz * dz;
      key[k] = k;
    }
    sortFractions(dist.data(), key.data(), n);
    for (int k = 0; k < std::min(n, maxMembs); ++k) P.bfIdx.push_back(found[key[k]]);
    P.bfOff[ic + 1] = (int)P.bfIdx.size();
  }
  if (!withWeights) return 0;
  // patch of each boundary face
  std::vector<int> patchOf(in.patchFaceOff[in.nPatches]);
  for (int ip = 0; ip < in.nPatches; ++ip)
    for (int b = in.patchFaceOff[ip]; b < in.patchFaceOff[ip + 1]; ++b) patchOf[b] = ip;
  P.cells.clear(); P.nCon.clear(); P.rowOff.clear(); P.w.clear(); P.rowFace.clear();
  std::vector<double> A;
  std::vector<double> term;
  std::vector<int> rowB;
  for (int ic = 0; ic < nc; ++ic) {
    if (P.bfOff[ic + 1] == P.bfOff[ic]) continue;
    const double *x = &in.cofg[3 * (size_t)ic];
    P.cells.push_back(ic);
    P.rowOff.push_back((int)P.rowFace.size());
    for (int k = 0; k < 5; ++k) {
      rowB.clear();
      for (int e = P.bfOff[ic]; e < P.bfOff[ic + 1]; ++e) {
        const int b = P.bfIdx[e], ip = patchOf[b];
        if (dirichlet(in.patchType[ip], in.patchMinj[ip], &in.bfn[4 * (size_t)b], k)) rowB.push_back(b);
      }
      P.nCon.push_back((int)rowB.size());
      if (rowB.empty()) continue;
      const int nm = in.stOff[ic + 1] - in.stOff[ic], nr = nm + (int)rowB.size();
      A.assign(3 * (size_t)nr, 0.0);
      term.assign(nr, 0.0);
      for (int r = 0; r < nr; ++r) {
        const double *y = (r < nm) ? &in.cofg[3 * (size_t)in.stIdx[in.stOff[ic] + r]] : &in.bfc[3 * (size_t)rowB[r - nm]];
        const double dx = y[0] - x[0], dy = y[1] - x[1], dz = y[2] - x[2];
        const double t = ((r < nm) ? 1.0 : in.cwt) / std::sqrt(dx * dx + dy * dy + dz * dz);
        term[r] = t;
        A[3 * r] = t * dx; A[3 * r + 1] = t * dy; A[3 * r + 2] = t * dz;
      }
      // pinv(A) = (A^T A)^-1 A^T, the inverse by cofactors
      double m00 = 0, m01 = 0, m02 = 0, m11 = 0, m12 = 0, m22 = 0;
      for (int r = 0; r < nr; ++r) {
        const double a0 = A[3 * r], a1 = A[3 * r + 1], a2 = A[3 * r + 2];
        m00 = m00 + a0 * a0; m01 = m01 + a0 * a1; m02 = m02 + a0 * a2;
        m11 = m11 + a1 * a1; m12 = m12 + a1 * a2; m22 = m22 + a2 * a2;
      }
      const double c00 = m11 * m22 - m12 * m12, c01 = m02 * m12 - m01 * m22, c02 = m01 * m12 - m02 * m11;
      const double c11 = m00 * m22 - m02 * m02, c12 = m01 * m02 - m00 * m12, c22 = m00 * m11 - m01 * m01;
      const double det = m00 * c00 + m01 * c01 + m02 * c02;
      // the singular-value test of RFLU_InvertMatrixSVD on the matrix with
      // its columns scaled by their largest magnitude, as the reference
      // scales it before the decomposition
      {
        double cm[3] = {0.0, 0.0, 0.0};
        for (int r = 0; r < nr; ++r)
          for (int c = 0; c < 3; ++c) cm[c] = std::max(cm[c], std::fabs(A[3 * r + c]));
        double g[4][4] = {};
        const double m[3][3] = {{m00, m01, m02}, {m01, m11, m12}, {m02, m12, m22}};
        for (int p = 0; p < 3; ++p)
          for (int q = 0; q < 3; ++q) g[p][q] = m[p][q] / (cm[p] * cm[q]);
        if (normalSingularCount(g, 3) != 0 || !(det != 0.0)) {
          if (bad) *bad = ic;
          return -1;
        }
      }
      const double id = 1.0 / det;
      const double i00 = id * c00, i01 = id * c01, i02 = id * c02, i11 = id * c11, i12 = id * c12, i22 = id * c22;
      for (int r = 0; r < nr; ++r) {
        const double a0 = A[3 * r], a1 = A[3 * r + 1], a2 = A[3 * r + 2];
        const double p0 = i00 * a0 + i01 * a1 + i02 * a2;
        const double p1 = i01 * a0 + i11 * a1 + i12 * a2;
        const double p2 = i02 * a0 + i12 * a1 + i22 * a2;
        P.w.push_back(term[r] * p0);
        P.w.push_back(term[r] * p1);
        P.w.push_back(term[r] * p2);
        P.rowFace.push_back(r < nm ? -1 : rowB[r - nm]);
      }
    }
  }
  P.rowOff.push_back((int)P.rowFace.size());
  return 0;
}

}  // namespace rflu

struct rflu_setup {
  int nCells = 0, nFaces = 0, nPatches = 0;
  std::vector<int> f2c;
  std::vector<double> fn, fc, vol, cofg;
  std::vector<int> patchFaceOff, bf2c;
  std::vector<double> bfn, bfc;
  std::vector<int> c2csOff, c2csMembs;
  std::vector<double> xyzMoms;
  std::vector<double> fc2, c2csShift;  // periodic and symmetry meshes only
  std::vector<int> c2csXf;             // symmetry meshes only
  std::vector<double> xfQ;
};

extern "C" int rflu_setup_build(const rflu_mesh_desc *m, int spaceOrder, rflu_setup **out) {
  if (!m || !out || !m->xyz || !m->c2v || m->nCells <= 0 || (m->nVertPerCell != 4 && m->nVertPerCell != 8))
    return rflu::fail(RFLU_ERR_ARG, "rflu_setup_build: bad mesh description (pure tet or hex meshes only)");
  rflu_setup *S = new (std::nothrow) rflu_setup();
  if (!S) return rflu::fail(RFLU_ERR_ARG, "rflu_setup_build: out of host memory");
  const int nc = m->nCells, nvc = m->nVertPerCell, nv = m->nVert;
  const int nfl = (nvc == 4) ? 4 : 6, fvs = (nvc == 4) ? 3 : 4;
  auto vert = [&](int ic, int k) { return m->c2v[(size_t)nvc * ic + k] - 1; };
  auto localFace = [&](int lf, int k) { return (nvc == 4) ? kTetFace[lf][k] : kHexFace[lf][k]; };
  S->nCells = nc;

  // ---- translational periodic patch pairs ------------------------------------
  // The reference builds virtual cells beyond each periodic patch (modflu/
  // RFLU_ModSymmetryPeriodic.F90:471-787); here, as in the CPU restatement,
  // the two patches' vertices are identified (their coordinates differ by
  // one translation per pair, the mean difference of the two vertex sets,
  // matched within 1e-7 of the box's extent): faces and stencils are built
  // on the identified vertex ids (vid), geometry on each cell's own
  // vertices, and a face or stencil member across a period carries the
  // translation between the two cells' frames.
  std::vector<int> rep;
  std::vector<std::array<double, 3>> perShift;
  std::vector<char> periodicPatch(std::max(m->nPatches, 1), 0);
  if (m->patchBcType && m->patchRelated && m->patchFaceOff) {
    for (int ip = 0; ip < m->nPatches; ++ip) periodicPatch[ip] = (m->patchBcType[ip] == 110);
    bool any = false;
    for (int ip = 0; ip < m->nPatches; ++ip) any = any || periodicPatch[ip];
    if (any) {
      rep.resize(nv);
      std::iota(rep.begin(), rep.end(), 0);
      auto find = [&](int v) {
        while (rep[v] != v) { rep[v] = rep[rep[v]]; v = rep[v]; }
        return v;
      };
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      for (int v = 0; v < nv; ++v)
        for (int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], m->xyz[3 * (size_t)v + d]); hi[d] = std::max(hi[d], m->xyz[3 * (size_t)v + d]); }
      const double tol = 1e-7 * std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
      auto patchVerts = [&](int ip) {
        std::vector<int> v;
        for (int b = m->patchFaceOff[ip]; b < m->patchFaceOff[ip + 1]; ++b)
          for (int k = 0; k < 4; ++k)
            if (m->bf2v[4 * (size_t)b + k] > 0) v.push_back(m->bf2v[4 * (size_t)b + k] - 1);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        return v;
      };
      for (int ip = 0; ip < m->nPatches; ++ip) {
        const int iq = m->patchRelated[ip];
        if (!periodicPatch[ip] || iq <= ip) continue;
        if (iq >= m->nPatches || m->patchBcType[iq] != 110 || m->patchRelated[iq] != ip) {
          delete S;
          return rflu::fail(RFLU_ERR_ARG, "rflu_setup_build: periodic patches must relate to each other in pairs");
        }
        const std::vector<int> vp = patchVerts(ip), vq = patchVerts(iq);
        if (vp.size() != vq.size() || vp.empty()) {
          delete S;
          return rflu::fail(RFLU_ERR_ARG, "rflu_setup_build: periodic patches do not match");
        }
        std::array<double, 3> T;
        for (int d = 0; d < 3; ++d) {
          double sp = 0.0, sq = 0.0;
          for (int v : vp) sp += m->xyz[3 * (size_t)v + d];
          for (int v : vq) sq += m->xyz[3 * (size_t)v + d];
          T[d] = (sq - sp) / (double)vp.size();
        }
        perShift.push_back(T);
        std::map<std::array<long long, 3>, int> grid;
        for (int w : vq) {
          std::array<long long, 3> k;
          for (int d = 0; d < 3; ++d) k[d] = std::llround(m->xyz[3 * (size_t)w + d] / tol);
          grid[k] = w;
        }
        for (int v : vp) {
          int w = -1;
          std::array<long long, 3> k0;
          for (int d = 0; d < 3; ++d) k0[d] = std::llround((m->xyz[3 * (size_t)v + d] + T[d]) / tol);
          for (int a = -1; a <= 1 && w < 0; ++a)
            for (int b = -1; b <= 1 && w < 0; ++b)
              for (int e = -1; e <= 1 && w < 0; ++e) {
                auto it = grid.find({k0[0] + a, k0[1] + b, k0[2] + e});
                if (it != grid.end()) w = it->second;
              }
          if (w < 0) {
            delete S;
            return rflu::fail(RFLU_ERR_ARG, "rflu_setup_build: a periodic vertex has no image on its related patch");
          }
          const int rv = find(v), rw = find(w);
          if (rv != rw) rep[std::max(rv, rw)] = std::min(rv, rw);
        }
      }
      for (int v = 0; v < nv; ++v) rep[v] = find(v);
    }
  }
  const bool periodic = !rep.empty();
  auto vid = [&](int ic, int k) { const int v = vert(ic, k); return periodic ? rep[v] : v; };
  // offset of stencil member j from cell i for the image of j nearest to i
  // (the virtual cell standing for j in the reference), and its translation
  // symmetry patches: the cells near them also seen reflected across them
  // (images, stencil ids nc + k): real cell, reflection, centroid, vertices
  std::vector<int> imgCell, imgXf, imgC2v;
  std::vector<double> imgPos;
  std::vector<std::array<double, 9>> xfQ;
  int nvExt = nv;
  auto memberOffset = [&](const double *cg, int i, int j, double &dx, double &dy, double &dz, double *sh) {
    if (j >= nc) {
      // the image's cell's offset plus the image's translation from its
      // cell, summed in that order (as the kernels add c2csShift)
      const double *x = &imgPos[3 * (size_t)(j - nc)], *x0 = &cg[3 * (size_t)imgCell[j - nc]];
      dx = (x0[0] - cg[3 * (size_t)i]) + (x[0] - x0[0]);
      dy = (x0[1] - cg[3 * (size_t)i + 1]) + (x[1] - x0[1]);
      dz = (x0[2] - cg[3 * (size_t)i + 2]) + (x[2] - x0[2]);
      if (sh) for (int d = 0; d < 3; ++d) sh[d] = x[d] - x0[d];
      return;
    }
    dx = cg[3 * (size_t)j] - cg[3 * (size_t)i];
    dy = cg[3 * (size_t)j + 1] - cg[3 * (size_t)i + 1];
    dz = cg[3 * (size_t)j + 2] - cg[3 * (size_t)i + 2];
    if (sh) sh[0] = sh[1] = sh[2] = 0.0;
    if (perShift.empty()) return;
    double best = dx * dx + dy * dy + dz * dz, bx = dx, by = dy, bz = dz, s0 = 0.0, s1 = 0.0, s2 = 0.0;
    const int np = (int)perShift.size();
    int combos = 1;
    for (int p = 0; p < np; ++p) combos *= 3;
    for (int mm = 1; mm < combos; ++mm) {
      double sx = 0.0, sy = 0.0, sz = 0.0;
      int r = mm;
      for (int p = 0; p < np; ++p, r /= 3) {
        const double f = (double)(r % 3 == 2 ? -1 : r % 3);
        sx += f * perShift[p][0];
        sy += f * perShift[p][1];
        sz += f * perShift[p][2];
      }
      const double ex = dx + sx, ey = dy + sy, ez = dz + sz;
      const double d2 = ex * ex + ey * ey + ez * ez;
      if (d2 < best) { best = d2; bx = ex; by = ey; bz = ez; s0 = sx; s1 = sy; s2 = sz; }
    }
    dx = bx; dy = by; dz = bz;
    if (sh) { sh[0] = s0; sh[1] = s1; sh[2] = s2; }
  };

  // ---- slot keys, bucketed by smallest vertex (counting sort) -------------
  const int64_t nSlots = (int64_t)nc * nfl;
  // the boundary faces that stay boundary faces: those of periodic patches
  // become interior faces of the identified mesh
  std::vector<int> keep;
  std::vector<int> patchOffKept(m->nPatches + 1, 0);
  for (int ip = 0; ip < m->nPatches; ++ip) {
    if (!(periodic && periodicPatch[ip]))
      for (int b = m->patchFaceOff[ip]; b < m->patchFaceOff[ip + 1]; ++b) keep.push_back(b);
    patchOffKept[ip + 1] = (int)keep.size();
  }
  const int nb = (int)keep.size();
  std::vector<int> bucketOff(nv + 1, 0);
  std::vector<int> smallest(nSlots + nb);
  std::vector<SlotKey> keys(nSlots + nb);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < nSlots; ++s) {
    int ic = (int)(s / nfl), lf = (int)(s % nfl), fv[4];
    for (int k = 0; k < fvs; ++k) fv[k] = vid(ic, localFace(lf, k));
    std::sort(fv, fv + fvs);
    smallest[s] = fv[0];
    keys[s] = {fv[1], fv[2], s};
  }
  for (int b = 0; b < nb; ++b) {
    const int *bv = m->bf2v + 4 * (size_t)keep[b];
    int n = (bv[3] <= 0) ? 3 : 4, fv[4];
    for (int k = 0; k < n; ++k) fv[k] = periodic ? rep[bv[k] - 1] : bv[k] - 1;
    std::sort(fv, fv + n);
    smallest[nSlots + b] = fv[0];
    keys[nSlots + b] = {fv[1], fv[2], -(int64_t)(b + 1)};
  }
  for (int64_t s = 0; s < nSlots + nb; ++s) bucketOff[smallest[s] + 1]++;
  for (int v = 0; v < nv; ++v) bucketOff[v + 1] += bucketOff[v];
  std::vector<SlotKey> sorted(nSlots + nb);
  {
    std::vector<int> fill(bucketOff.begin(), bucketOff.end() - 1);
    for (int64_t s = 0; s < nSlots + nb; ++s) sorted[fill[smallest[s]]++] = keys[s];
  }
  keys.clear();
  keys.shrink_to_fit();
#pragma omp parallel for schedule(dynamic, 1024)
  for (int v = 0; v < nv; ++v)
    std::sort(sorted.begin() + bucketOff[v], sorted.begin() + bucketOff[v + 1], [](const SlotKey &a, const SlotKey &b) {
      if (a.k1 != b.k1) return a.k1 < b.k1;
      if (a.k2 != b.k2) return a.k2 < b.k2;
      return a.slot > b.slot;  // boundary entries (negative) after cell slots
    });

  // ---- pair matching: interior faces, boundary owners -----------------------
  std::vector<int64_t> lowSlot;       // per interior face: lower slot
  std::vector<int> highCell;
  std::vector<int> bOwner(nb, -1);
  std::vector<char> bad(1, 0);
  lowSlot.reserve(nSlots / 2 + 1);
  for (int v = 0; v < nv; ++v) {
    // a group of equal keys never spans two buckets
    size_t i = bucketOff[v], n = bucketOff[v + 1];
    while (i < n) {
      size_t j = i + 1;
      while (j < n && sorted[j].k1 == sorted[i].k1 && sorted[j].k2 == sorted[i].k2) ++j;
      // group [i,j): cell slots in descending order, then boundary entries
      int nCellSlots = 0;
      for (size_t k = i; k < j; ++k) nCellSlots += (sorted[k].slot >= 0);
      if (nCellSlots == 2) {
        int64_t a = sorted[i].slot, b = sorted[i + 1].slot;  // a > b
        lowSlot.push_back(b);
        highCell.push_back((int)(a / nfl));
        if (j - i > 2) bad[0] = 1;  // a boundary face on an interior face
      } else if (nCellSlots == 1) {
        for (size_t k = i + 1; k < j; ++k) bOwner[-sorted[k].slot - 1] = (int)(sorted[i].slot / nfl);
      } else {
        bad[0] = 1;
      }
      i = j;
    }
  }
  sorted.clear();
  sorted.shrink_to_fit();
  if (bad[0]) { delete S; return rflu::fail(RFLU_ERR_ARG, "rflu_setup_build: non-conforming mesh"); }
  for (int b = 0; b < nb; ++b)
    if (bOwner[b] < 0) { delete S; return rflu::fail(RFLU_ERR_ARG, "rflu_setup_build: boundary face without a cell"); }

  // faces in first-insertion order = ascending lower slot
  const int nf = (int)lowSlot.size();
  std::vector<int> order(nf);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int a, int b) { return lowSlot[a] < lowSlot[b]; });
  if (periodic) {
    // faces across a period (the reference's actual-virtual faces) follow
    // the others, both in first-insertion order: across when the second
    // cell holds the face's first vertex under another vertex id
    auto across = [&](int o) {
      const int64_t sl = lowSlot[o];
      const int ic = (int)(sl / nfl), lf = (int)(sl % nfl), c2 = highCell[o];
      const int a = vert(ic, localFace(lf, 0));
      for (int k = 0; k < nvc; ++k)
        if (vert(c2, k) == a) return false;
      return true;
    };
    std::stable_partition(order.begin(), order.end(), [&](int o) { return !across(o); });
  }
  S->nFaces = nf;
  S->f2c.resize(2 * (size_t)nf);
  std::vector<int> f2v(4 * (size_t)nf, -1);
  for (int f = 0; f < nf; ++f) {
    int64_t s = lowSlot[order[f]];
    int ic = (int)(s / nfl), lf = (int)(s % nfl);
    S->f2c[2 * (size_t)f] = ic;
    S->f2c[2 * (size_t)f + 1] = highCell[order[f]];
    for (int k = 0; k < fvs; ++k) f2v[4 * (size_t)f + k] = vert(ic, localFace(lf, k));
  }

  // ---- geometry (RFLU_BuildGeometry) ----------------------------------------
  const double *xyz = m->xyz;
  std::vector<double> app(3 * (size_t)nc);
  const double w = (nvc == 4) ? 0.25 : 0.125;
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic)
    for (int d = 0; d < 3; ++d) {
      double s = xyz[3 * (size_t)vert(ic, 0) + d];
      for (int k = 1; k < nvc; ++k) s = s + xyz[3 * (size_t)vert(ic, k) + d];
      app[3 * (size_t)ic + d] = w * s;
    }
  S->fn.resize(4 * (size_t)nf);
  S->fc.resize(3 * (size_t)nf);
  std::vector<double> fvec(3 * (size_t)nf);
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    int nvf = (f2v[4 * (size_t)f + 3] < 0) ? 3 : 4;
    double *v = &fvec[3 * (size_t)f], *cen = &S->fc[3 * (size_t)f];
    faceGeom(xyz, &f2v[4 * (size_t)f], nvf, v, cen);
    double mag = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double inv = 1.0 / mag;
    double *n = &S->fn[4 * (size_t)f];
    n[0] = v[0] * inv; n[1] = v[1] * inv; n[2] = v[2] * inv; n[3] = mag;
  }
  S->nPatches = m->nPatches;
  S->patchFaceOff = patchOffKept;
  // each face's centroid in its second cell's frame: the translation between
  // the two cells' own coordinates of the face's first vertex (zero unless
  // across a period)
  if (periodic) {
    S->fc2.assign(S->fc.begin(), S->fc.end());
    for (int f = 0; f < nf; ++f) {
      const int c1 = S->f2c[2 * (size_t)f], c2 = S->f2c[2 * (size_t)f + 1], a = f2v[4 * (size_t)f];
      double sh[3] = {0.0, 0.0, 0.0};
      for (int k = 0; k < nvc; ++k) {
        if (vert(c1, k) != a) continue;
        for (int k2 = 0; k2 < nvc; ++k2)
          if (vid(c2, k2) == vid(c1, k)) {
            const int b = vert(c2, k2);
            if (b != a)
              for (int d = 0; d < 3; ++d) sh[d] = xyz[3 * (size_t)b + d] - xyz[3 * (size_t)a + d];
          }
      }
      if (sh[0] != 0.0 || sh[1] != 0.0 || sh[2] != 0.0)
        for (int d = 0; d < 3; ++d) S->fc2[3 * (size_t)f + d] = S->fc[3 * (size_t)f + d] + sh[d];
    }
  }
  S->bf2c.resize(nb);
  S->bfn.resize(4 * (size_t)nb);
  S->bfc.resize(3 * (size_t)nb);
  std::vector<double> bvec(3 * (size_t)nb);
  for (int b = 0; b < nb; ++b) {
    int v[4];
    const int *bv = m->bf2v + 4 * (size_t)keep[b];
    int nvf = (bv[3] <= 0) ? 3 : 4;
    for (int k = 0; k < nvf; ++k) v[k] = bv[k] - 1;
    double *vv = &bvec[3 * (size_t)b], *cen = &S->bfc[3 * (size_t)b];
    faceGeom(xyz, v, nvf, vv, cen);
    double mag = std::sqrt(vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
    double inv = 1.0 / mag;
    double *n = &S->bfn[4 * (size_t)b];
    n[0] = vv[0] * inv; n[1] = vv[1] * inv; n[2] = vv[2] * inv; n[3] = mag;
    S->bf2c[b] = bOwner[b];
  }
  // Volume and centroid sums need the reference's face order per cell: the
  // interior faces in face order, then the patch faces.  Gather them per cell.
  std::vector<int> cfOff(nc + 1, 0);
  for (int f = 0; f < nf; ++f) { cfOff[S->f2c[2 * (size_t)f] + 1]++; cfOff[S->f2c[2 * (size_t)f + 1] + 1]++; }
  for (int b = 0; b < nb; ++b) cfOff[bOwner[b] + 1]++;
  for (int ic = 0; ic < nc; ++ic) cfOff[ic + 1] += cfOff[ic];
  std::vector<int> cfEnt(cfOff[nc]);
  {
    std::vector<int> fill(cfOff.begin(), cfOff.end() - 1);
    for (int f = 0; f < nf; ++f) {
      cfEnt[fill[S->f2c[2 * (size_t)f]]++] = 2 * f;
      cfEnt[fill[S->f2c[2 * (size_t)f + 1]]++] = 2 * f + 1;
    }
    for (int b = 0; b < nb; ++b) cfEnt[fill[bOwner[b]]++] = 2 * nf + b;
  }
  S->vol.assign(nc, 0.0);
  S->cofg.assign(3 * (size_t)nc, 0.0);
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    double vol = 0.0, cg[3] = {0.0, 0.0, 0.0};
    const double *a = &app[3 * (size_t)ic];
    for (int e = cfOff[ic]; e < cfOff[ic + 1]; ++e) {
      int code = cfEnt[e];
      const double *vv, *cen;
      bool minus = false;
      if (code < 2 * nf) {
        vv = &fvec[3 * (size_t)(code >> 1)];
        minus = code & 1;
        cen = (minus && periodic) ? &S->fc2[3 * (size_t)(code >> 1)] : &S->fc[3 * (size_t)(code >> 1)];
      } else {
        vv = &bvec[3 * (size_t)(code - 2 * nf)];
        cen = &S->bfc[3 * (size_t)(code - 2 * nf)];
      }
      double t = (cen[0] - a[0]) * vv[0] + (cen[1] - a[1]) * vv[1] + (cen[2] - a[2]) * vv[2];
      vol = minus ? vol - t : vol + t;
      t = cen[0] * vv[0] + cen[1] * vv[1] + cen[2] * vv[2];
      for (int d = 0; d < 3; ++d) cg[d] = minus ? cg[d] - t * cen[d] : cg[d] + t * cen[d];
    }
    vol = (1.0 / 3.0) * vol;
    double t = 1.0 / (4.0 * vol);
    S->vol[ic] = vol;
    for (int d = 0; d < 3; ++d) S->cofg[3 * (size_t)ic + d] = t * cg[d];
  }

  // ---- symmetry (mirror) patches -----------------------------------------------
  // The reference adds the cells near each symmetry patch as virtual cells
  // reflected across it, and reflected copies of earlier patches' virtual
  // cells near it (the corner images) (modflu/RFLU_ModSymmetryPeriodic.F90:
  // 148-335, 471-787); their state and gradients are the actual cells',
  // reflected (modflu/RFLU_ModRelatedPatches.F90:268-435).  Here each
  // symmetry patch must be planar and two patches parallel or
  // perpendicular; the cells within three vertex layers of a patch are seen
  // reflected across every set of such patches without two parallel ones,
  // and an image's vertices off its reflecting planes get new ids, so that
  // the stencils below grow across the planes as over virtual cells.
  bool symmetry = false;
  for (int ip = 0; ip < m->nPatches && m->patchBcType; ++ip)
    symmetry = symmetry || (m->patchBcType[ip] == RFLU_BC_SYMMETRY && patchOffKept[ip + 1] > patchOffKept[ip]);
  if (symmetry && periodic) {
    delete S;
    return rflu::fail(RFLU_ERR_UNSUPPORTED, "rflu_setup_build: symmetry and periodic patches in one mesh");
  }
  if (symmetry && spaceOrder > 1) {
    struct Plane { double n[3], p0[3]; std::vector<int> verts; };
    std::vector<Plane> planes;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int v = 0; v < nv; ++v)
      for (int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], xyz[3 * (size_t)v + d]); hi[d] = std::max(hi[d], xyz[3 * (size_t)v + d]); }
    const double tol = 1e-7 * std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
    for (int ip = 0; ip < m->nPatches; ++ip) {
      if (m->patchBcType[ip] != RFLU_BC_SYMMETRY || patchOffKept[ip + 1] == patchOffKept[ip]) continue;
      Plane P;
      const int b0 = patchOffKept[ip];
      for (int d = 0; d < 3; ++d) { P.n[d] = S->bfn[4 * (size_t)b0 + d]; P.p0[d] = S->bfc[3 * (size_t)b0 + d]; }
      for (int b = b0; b < patchOffKept[ip + 1]; ++b) {
        const double cosA = S->bfn[4 * (size_t)b] * P.n[0] + S->bfn[4 * (size_t)b + 1] * P.n[1] + S->bfn[4 * (size_t)b + 2] * P.n[2];
        for (int k = 0; k < 4; ++k) {
          const int v = m->bf2v[4 * (size_t)keep[b] + k] - 1;
          if (v < 0) continue;
          const double h = (xyz[3 * (size_t)v] - P.p0[0]) * P.n[0] + (xyz[3 * (size_t)v + 1] - P.p0[1]) * P.n[1] +
                           (xyz[3 * (size_t)v + 2] - P.p0[2]) * P.n[2];
          if (std::fabs(h) > tol || cosA < 1.0 - 1e-10) {
            delete S;
            return rflu::fail(RFLU_ERR_UNSUPPORTED, "rflu_setup_build: a symmetry patch is not planar");
          }
          P.verts.push_back(v);
        }
      }
      planes.push_back(std::move(P));
    }
    const int np = (int)planes.size();
    if (np > 30) { delete S; return rflu::fail(RFLU_ERR_UNSUPPORTED, "rflu_setup_build: more than 30 symmetry patches"); }
    std::vector<int> parallel(np, 0);
    for (int a = 0; a < np; ++a)
      for (int q = 0; q < np; ++q) {
        if (q == a) continue;
        const double d = std::fabs(planes[a].n[0] * planes[q].n[0] + planes[a].n[1] * planes[q].n[1] + planes[a].n[2] * planes[q].n[2]);
        if (d > 1.0 - 1e-10) parallel[a] |= 1 << q;
        else if (d > 1e-10) {
          delete S;
          return rflu::fail(RFLU_ERR_UNSUPPORTED, "rflu_setup_build: two symmetry patches neither parallel nor perpendicular");
        }
      }
    std::vector<int> vmask(nv, 0), nearMask(nc, 0);
    std::vector<int> v2cOff0(nv + 1, 0);
    for (int ic = 0; ic < nc; ++ic)
      for (int k = 0; k < nvc; ++k) v2cOff0[vert(ic, k) + 1]++;
    for (int v = 0; v < nv; ++v) v2cOff0[v + 1] += v2cOff0[v];
    std::vector<int> v2c0(v2cOff0[nv]);
    {
      std::vector<int> fill(v2cOff0.begin(), v2cOff0.end() - 1);
      for (int ic = 0; ic < nc; ++ic)
        for (int k = 0; k < nvc; ++k) v2c0[fill[vert(ic, k)]++] = ic;
    }
    const int kLayers = 3;
    for (int a = 0; a < np; ++a) {
      std::vector<char> vIn(nv, 0), cIn(nc, 0);
      std::vector<int> front;
      for (int v : planes[a].verts) {
        vmask[v] |= 1 << a;
        if (!vIn[v]) { vIn[v] = 1; front.push_back(v); }
      }
      for (int layer = 0; layer < kLayers; ++layer) {
        std::vector<int> next;
        for (int v : front)
          for (int e = v2cOff0[v]; e < v2cOff0[v + 1]; ++e) {
            const int ic = v2c0[e];
            if (cIn[ic]) continue;
            cIn[ic] = 1;
            nearMask[ic] |= 1 << a;
            for (int k = 0; k < nvc; ++k) {
              const int w = vert(ic, k);
              if (!vIn[w]) { vIn[w] = 1; next.push_back(w); }
            }
          }
        front.swap(next);
      }
    }
    struct Img { int top, set, cell; };
    std::vector<Img> imgs;
    for (int ic = 0; ic < nc; ++ic) {
      const int mk = nearMask[ic];
      for (int Sm = mk; Sm > 0; Sm = (Sm - 1) & mk) {
        bool ok = true;
        for (int a = 0; a < np && ok; ++a)
          if ((Sm >> a & 1) && (Sm & parallel[a])) ok = false;
        if (!ok) continue;
        int top = 0;
        while ((Sm >> (top + 1)) != 0) ++top;
        imgs.push_back({top, Sm, ic});
      }
    }
    std::sort(imgs.begin(), imgs.end(), [](const Img &x, const Img &y) {
      if (x.top != y.top) return x.top < y.top;
      if (x.set != y.set) return x.set < y.set;
      return x.cell < y.cell;
    });
    // reflections Q_S = Q_a1 Q_a2 ... in plane order (RFLU_RELP_TransformMatrix's I - 2 n n^T)
    std::map<int, int> xfOf;
    auto xfIndex = [&](int Sm) {
      auto it = xfOf.find(Sm);
      if (it != xfOf.end()) return it->second;
      std::array<double, 9> Q{};
      bool first = true;
      for (int a = 0; a < np; ++a) {
        if (!(Sm >> a & 1)) continue;
        const double nx = planes[a].n[0], ny = planes[a].n[1], nz = planes[a].n[2];
        const double Qa[9] = {1.0 - 2.0 * nx * nx, -2.0 * nx * ny, -2.0 * nx * nz,
                              -2.0 * nx * ny, 1.0 - 2.0 * ny * ny, -2.0 * ny * nz,
                              -2.0 * nx * nz, -2.0 * ny * nz, 1.0 - 2.0 * nz * nz};
        if (first) {
          for (int k = 0; k < 9; ++k) Q[k] = Qa[k];
          first = false;
          continue;
        }
        std::array<double, 9> P;
        for (int r = 0; r < 3; ++r)
          for (int col = 0; col < 3; ++col) {
            double t = Q[3 * r] * Qa[col];
            t = t + Q[3 * r + 1] * Qa[3 + col];
            t = t + Q[3 * r + 2] * Qa[6 + col];
            P[3 * r + col] = t;
          }
        Q = P;
      }
      const int idx = (int)xfQ.size();
      xfQ.push_back(Q);
      xfOf[Sm] = idx;
      return idx;
    };
    for (int a = 0; a < np; ++a) xfIndex(1 << a);
    std::map<std::pair<int, int>, int> vext;
    for (const Img &im : imgs) {
      imgCell.push_back(im.cell);
      imgXf.push_back(xfIndex(im.set));
      double x[3] = {S->cofg[3 * (size_t)im.cell], S->cofg[3 * (size_t)im.cell + 1], S->cofg[3 * (size_t)im.cell + 2]};
      for (int a = 0; a < np; ++a) {
        if (!(im.set >> a & 1)) continue;
        const double *n = planes[a].n, *p0 = planes[a].p0;
        const double h = (x[0] - p0[0]) * n[0] + (x[1] - p0[1]) * n[1] + (x[2] - p0[2]) * n[2];
        for (int d = 0; d < 3; ++d) x[d] = x[d] - 2.0 * h * n[d];
      }
      for (int d = 0; d < 3; ++d) imgPos.push_back(x[d]);
      for (int k = 0; k < nvc; ++k) {
        const int v = vert(im.cell, k);
        const int Sv = im.set & ~vmask[v];
        if (Sv == 0) {
          imgC2v.push_back(v);
          continue;
        }
        auto it = vext.find({v, Sv});
        if (it == vext.end()) it = vext.emplace(std::make_pair(v, Sv), nvExt++).first;
        imgC2v.push_back(it->second);
      }
    }
  }

  // ---- C2C stencils and moments (ORDER > 1) ---------------------------------
  S->c2csOff.assign(nc + 1, 0);
  if (spaceOrder > 1) {
    const int minSize = 4, maxSize = 40, maxLayers = 6;
    // the cells and the symmetry images (ids nc + k) with their vertices
    const int ne = nc + (int)imgCell.size();
    auto cellVert = [&](int e, int k) { return e < nc ? vid(e, k) : imgC2v[(size_t)nvc * (e - nc) + k]; };
    std::vector<int> v2cOff(nvExt + 1, 0);
    for (int ic = 0; ic < ne; ++ic)
      for (int k = 0; k < nvc; ++k) v2cOff[cellVert(ic, k) + 1]++;
    for (int v = 0; v < nvExt; ++v) v2cOff[v + 1] += v2cOff[v];
    std::vector<int> v2c(v2cOff[nvExt]);
    {
      std::vector<int> fill(v2cOff.begin(), v2cOff.end() - 1);
      for (int ic = 0; ic < ne; ++ic)
        for (int k = 0; k < nvc; ++k) v2c[fill[cellVert(ic, k)]++] = ic;
    }
    std::vector<std::vector<int>> memb(nc);
    const double invNv = 1.0 / (double)nvc;
    const double *cg = S->cofg.data();
#pragma omp parallel
    {
      std::vector<int> cand, sv(nvc), sv2(nvc), help;
      std::vector<double> frac, A;
#pragma omp for schedule(dynamic, 256)
      for (int ic = 0; ic < nc; ++ic) {
        cand.clear();
        for (int k = 0; k < nvc; ++k) {
          int v = vid(ic, k);
          cand.insert(cand.end(), v2c.begin() + v2cOff[v], v2c.begin() + v2cOff[v + 1]);
        }
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        cand.erase(std::lower_bound(cand.begin(), cand.end(), ic));
        const int nCand = (int)cand.size();
        for (int k = 0; k < nvc; ++k) sv[k] = vid(ic, k);
        std::sort(sv.begin(), sv.end());
        frac.resize(nCand);
        for (int i = 0; i < nCand; ++i) {
          for (int k = 0; k < nvc; ++k) sv2[k] = cellVert(cand[i], k);
          std::sort(sv2.begin(), sv2.end());
          int shared = 0;
          for (int a = 0, b = 0; a < nvc && b < nvc;) {
            if (sv[a] == sv2[b]) { ++shared; ++a; ++b; }
            else if (sv[a] < sv2[b]) ++a;
            else ++b;
          }
          frac[i] = shared * invNv;
        }
        sortFractions(frac.data(), cand.data(), nCand);
        std::vector<int> st;
        for (int i = nCand - 1; i >= std::max(nCand - maxSize, 0); --i) st.push_back(cand[i]);
        std::sort(st.begin(), st.end());
        int layerBeg = 0, layerEnd = (int)st.size();
        for (int layer = 2; layer <= maxLayers; ++layer) {
          int degr = (int)st.size(), sCount = 0;
          if (degr >= minSize) {
            A.assign(4 * (size_t)degr, 0.0);
            for (int r = 0; r < degr; ++r) {
              int j = st[r];
              double dx, dy, dz;
              memberOffset(cg, ic, j, dx, dy, dz, nullptr);
              double t = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
              A[4 * r] = t; A[4 * r + 1] = t * dx; A[4 * r + 2] = t * dy; A[4 * r + 3] = t * dz;
            }
            for (int col = 0; col < 4; ++col) {
              double mx = 0.0;
              for (int r = 0; r < degr; ++r) mx = std::max(mx, std::fabs(A[4 * r + col]));
              for (int r = 0; r < degr; ++r) A[4 * r + col] /= mx;
            }
            sCount = singularCount(A, degr);
          }
          if (sCount == 0 && degr >= minSize) break;
          // one more vertex-neighbour layer (RFLU_AddCellLayer,
          // modflu/RFLU_ModStencilsUtils.F90:696-949)
          std::vector<int> have(st);
          std::sort(have.begin(), have.end());
          help.clear();
          bool full = false;
          for (int i = layerBeg; i < layerEnd && !full; ++i)
            for (int k = 0; k < nvc && !full; ++k) {
              int v = cellVert(st[i], k);
              for (int e = v2cOff[v]; e < v2cOff[v + 1]; ++e) {
                int c2 = v2c[e];
                if (c2 == ic || std::binary_search(have.begin(), have.end(), c2)) continue;
                auto it = std::lower_bound(help.begin(), help.end(), c2);
                if (it != help.end() && *it == c2) continue;
                if ((int)help.size() >= maxSize) { full = true; break; }
                help.insert(it, c2);
              }
            }
          layerBeg = layerEnd;
          for (int h : help)
            if ((int)st.size() < maxSize) st.push_back(h);
          layerEnd = (int)st.size();
        }
        memb[ic].swap(st);
      }
    }
    for (int ic = 0; ic < nc; ++ic) S->c2csOff[ic + 1] = S->c2csOff[ic] + (int)memb[ic].size();
    S->c2csMembs.resize(S->c2csOff[nc]);
    for (int ic = 0; ic < nc; ++ic)
      for (size_t k = 0; k < memb[ic].size(); ++k) {
        const int j = memb[ic][k];
        S->c2csMembs[S->c2csOff[ic] + k] = (j < nc ? j : imgCell[j - nc]) + 1;
      }
    if (!imgCell.empty()) {
      S->c2csXf.assign(S->c2csOff[nc], -1);
      for (int ic = 0; ic < nc; ++ic)
        for (size_t k = 0; k < memb[ic].size(); ++k)
          if (memb[ic][k] >= nc) S->c2csXf[S->c2csOff[ic] + k] = imgXf[memb[ic][k] - nc];
      for (const auto &Q : xfQ) S->xfQ.insert(S->xfQ.end(), Q.begin(), Q.end());
    }
    // stencil moments: RFLU_ComputeStencilMoments3D1 (modflu/RFLU_ModWeights.F90:1770-1915)
    S->xyzMoms.assign(10 * (size_t)nc, 0.0);
    const bool shifts = periodic || !imgCell.empty();
    if (shifts) S->c2csShift.assign(3 * (size_t)S->c2csOff[nc], 0.0);
#pragma omp parallel for schedule(static)
    for (int ic = 0; ic < nc; ++ic) {
      double mm[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int e = S->c2csOff[ic]; e < S->c2csOff[ic + 1]; ++e) {
        int j = memb[ic][e - S->c2csOff[ic]];
        double dx, dy, dz;
        memberOffset(cg, ic, j, dx, dy, dz, shifts ? &S->c2csShift[3 * (size_t)e] : nullptr);
        double wt = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
        dx = wt * dx; dy = wt * dy; dz = wt * dz;
        mm[0] = mm[0] + dx * dx; mm[1] = mm[1] + dx * dy; mm[2] = mm[2] + dy * dy;
        mm[3] = mm[3] + dx * dz; mm[4] = mm[4] + dy * dz; mm[5] = mm[5] + dz * dz;
        mm[6] = mm[6] + wt * dx; mm[7] = mm[7] + wt * dy; mm[8] = mm[8] + wt * dz; mm[9] = mm[9] + wt * wt;
      }
      double *r = &S->xyzMoms[10 * (size_t)ic];
      r[0] = std::sqrt(mm[0]);
      double i11 = 1.0 / r[0];
      r[1] = i11 * mm[1];
      r[2] = std::sqrt(mm[2] - r[1] * r[1]);
      double i22 = 1.0 / r[2];
      r[3] = i11 * mm[3];
      r[4] = i22 * (mm[4] - r[1] * r[3]);
      r[5] = std::sqrt(mm[5] - (r[3] * r[3] + r[4] * r[4]));
      double i33 = 1.0 / r[5];
      r[6] = i11 * mm[6];
      r[7] = i22 * (mm[7] - r[1] * r[6]);
      r[8] = i33 * (mm[8] - (r[3] * r[6] + r[4] * r[7]));
      r[9] = std::sqrt(mm[9] - (r[6] * r[6] + r[7] * r[7] + r[8] * r[8]));
    }
  }
  // 1-based ids in the exported arrays, as the Fortran host holds them
  for (auto &x : S->f2c) x += 1;
  for (auto &x : S->bf2c) x += 1;
  *out = S;
  return RFLU_OK;
}

extern "C" int rflu_setup_grid(rflu_setup *S, rflu_grid_desc *g) {
  if (!S || !g) return rflu::fail(RFLU_ERR_ARG, "rflu_setup_grid: null argument");
  g->nCells = S->nCells;
  g->nFaces = S->nFaces;
  g->f2c = S->f2c.data();
  g->fn = S->fn.data();
  g->fc = S->fc.data();
  g->vol = S->vol.data();
  g->cofg = S->cofg.data();
  g->nPatches = S->nPatches;
  g->patchFaceOff = S->patchFaceOff.data();
  g->bf2c = S->bf2c.data();
  g->bfn = S->bfn.data();
  g->bfc = S->bfc.data();
  g->c2csOff = S->c2csOff.data();
  g->c2csMembs = S->c2csMembs.empty() ? nullptr : S->c2csMembs.data();
  g->xyzMoms = S->xyzMoms.empty() ? nullptr : S->xyzMoms.data();
  g->fc2 = S->fc2.empty() ? nullptr : S->fc2.data();
  g->c2csShift = S->c2csShift.empty() ? nullptr : S->c2csShift.data();
  g->c2csXf = S->c2csXf.empty() ? nullptr : S->c2csXf.data();
  g->nXf = (int)(S->xfQ.size() / 9);
  g->xfQ = S->xfQ.empty() ? nullptr : S->xfQ.data();
  return RFLU_OK;
}

extern "C" int rflu_setup_destroy(rflu_setup *S) {
  delete S;
  return RFLU_OK;
}

extern "C" int rflu_setup_bface_stencil(const rflu_grid_desc *g, int *off, int *faces) {
  if (!g || !off || !g->cofg || !g->c2csOff || (!g->c2csMembs && g->c2csOff[g->nCells] > 0) || !g->patchFaceOff ||
      (g->nPatches > 0 && (!g->patchBcType || !g->bf2c || !g->bfc)))
    return rflu::fail(RFLU_ERR_ARG, "rflu_setup_bface_stencil: incomplete grid description");
  const int nc = g->nCells, nb = g->patchFaceOff[g->nPatches];
  std::vector<int> stIdx(g->c2csOff[nc]), bf2c(nb);
  for (int e = 0; e < g->c2csOff[nc]; ++e) stIdx[e] = g->c2csMembs[e] - 1;
  for (int b = 0; b < nb; ++b) bf2c[b] = g->bf2c[b] - 1;
  std::vector<double> minj(std::max(g->nPatches, 1), 0.0);
  rflu::ConstrInput in{nc, g->cofg, g->c2csOff, stIdx.data(), g->nPatches, g->patchFaceOff, g->patchBcType,
                       minj.data(), bf2c.data(), g->bfn, g->bfc, 1.0};
  rflu::ConstrPlan plan;
  rflu::planConstrained(in, plan, nullptr, false);
  std::memcpy(off, plan.bfOff.data(), sizeof(int) * (nc + 1));
  if (faces && !plan.bfIdx.empty()) std::memcpy(faces, plan.bfIdx.data(), sizeof(int) * plan.bfIdx.size());
  return RFLU_OK;
}
