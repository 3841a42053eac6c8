/*
 * CPU oracle: FP64 restatement of the RocfluMP explicit residual-and-update
 * path (thierrydaoud/Rocflu).  TEST INFRASTRUCTURE ONLY -- see oracle.h.
 *
 * Build: g++ -O2 -ffp-contract=off -fopenmp -fPIC -shared (oracle/Makefile).
 * The reference release flags are -O / -O2 -ffp-contract=off
 * (CMakeLists.txt:44, machines/dane.sh:6): no fused multiply-add,
 * left-to-right evaluation.
 *
 * Threads: the reference's face loops scatter into both cells of a face
 * (rhs(:,c1) += F, rhs(:,c2) -= F and the limiters' running min/max).  Each
 * cell sees its faces in face order there, interior faces first and then
 * the patches in order, so the same sums and min/max taken per cell over its
 * faces in that order (the cfOff/cfEnt lists below) give the same bits, NaN
 * propagation included, and every cell can be done by its own thread.  Face
 * values (fluxes, spectral radii) are formed once per face first.  Built
 * without OpenMP the pragmas are ignored and every loop runs in order.
 */
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <array>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* ------------------------------------------------------------------------ */
/* Perfect-gas relations, libfloflu/MixtPerf_*.F90                           */
/* ------------------------------------------------------------------------ */
inline double MixtPerf_R_CpG(double cp, double g) { return cp - cp / g; }         /* MixtPerf_R.F90:78 */
inline double MixtPerf_R_M(double m) { return 8314.3 / m; }                       /* MixtPerf_R.F90:93 */
inline double MixtPerf_M_R(double r) { return 8314.3 / r; }                       /* MixtPerf_M.F90:78 */
inline double MixtPerf_G_CpR(double cp, double r) { return cp / (cp - r); }       /* MixtPerf_G.F90:78 */
inline double MixtPerf_P_DEoGVm2(double d, double eo, double g, double vm2) {    /* MixtPerf_P.F90:78 */
  return (g - 1.0) * d * (eo - 0.5 * vm2);
}
inline double MixtPerf_T_DPR(double d, double p, double r) { return p / (d * r); } /* MixtPerf_T.F90:124 */
inline double MixtPerf_C_GRT(double g, double r, double t) { return std::sqrt(g * r * t); } /* MixtPerf_C.F90:125 */
inline double MixtPerf_C_DGP(double d, double g, double p) { return std::sqrt(g * p / d); } /* MixtPerf_C.F90:95 */
inline double MixtPerf_C_GHoVm2(double g, double ho, double vm2) {                 /* MixtPerf_C.F90:110 */
  return std::sqrt((g - 1.0) * (ho - 0.5 * vm2));
}
inline double MixtPerf_Eo_DGPUVW(double d, double g, double p, double u, double v, double w) { /* MixtPerf_E.F90:79 */
  return p / (d * (g - 1.0)) + 0.5 * (u * u + v * v + w * w);
}
inline double MixtPerf_Ho_CpTUVW(double cp, double t, double u, double v, double w) { /* MixtPerf_H.F90:78 */
  return cp * t + 0.5 * (u * u + v * v + w * w);
}
/* modflu/RFLU_ModEntropyFixes.F90:95-106 */
inline double EntropyFixHartenHyman(double l, double d) {
  if (l > d) return l;
  return (l * l + d * d) / (2.0 * d);
}
/* Fortran MIN/MAX for two reals as gfortran emits them for finite inputs. */
inline double fmin2(double a, double b) { return (b < a) ? b : a; }
inline double fmax2(double a, double b) { return (b > a) ? b : a; }

/* ------------------------------------------------------------------------ */
/* modfloflu/ModSortSearch.F90:990-1091 QuickSortRFREALInteger (Wirth).      */
/* The tie order of this unstable sort decides which equal-fraction          */
/* neighbours survive stencil truncation, so it is restated step by step.    */
/* a, b are 1-based views of length n.                                       */
/* ------------------------------------------------------------------------ */
void QuickSortRFREALInteger(double *a1, int *b1, int n) {
  double *a = a1 - 1;
  int *b = b1 - 1;
  int stackl[50], stackr[50];
  int s = 1;
  stackl[0] = 1;
  stackr[0] = n;
  int l, r, i, j, k;
  double x, w;
  int v;
L10:
  l = stackl[s - 1];
  r = stackr[s - 1];
  s = s - 1;
L20:
  i = l;
  j = r;
  k = (l + r) / 2;
  x = a[k];
  for (;;) {
    while (a[i] < x) i = i + 1;
    while (x < a[j]) j = j - 1;
    if (i <= j) {
      w = a[i]; a[i] = a[j]; a[j] = w;
      v = b[i]; b[i] = b[j]; b[j] = v;
      i = i + 1;
      j = j - 1;
      if (i > j) break;
    } else {
      break;
    }
  }
  if (j - l >= r - i) {
    if (l < j) { s = s + 1; stackl[s - 1] = l; stackr[s - 1] = j; }
    l = i;
  } else {
    if (i < r) { s = s + 1; stackl[s - 1] = i; stackr[s - 1] = r; }
    r = j;
  }
  if (l < r) goto L20;
  if (s != 0) goto L10;
}

/* Singular values (descending) of a nRows x nCols matrix by one-sided Jacobi.
 * Stands in for LAPACK dgesdd inside RFLU_InvertMatrixSVD
 * (libflu/RFLU_InvertMatrixSVD.F90); only the singular values are used by the
 * stencil builder, through the ratio test below. */
void singularValues(int nRows, int nCols, std::vector<double> a /* col-major */, double *s) {
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < nCols - 1; ++p)
      for (int q = p + 1; q < nCols; ++q) {
        double alpha = 0, beta = 0, gamma = 0;
        for (int i = 0; i < nRows; ++i) {
          double ap = a[i + p * nRows], aq = a[i + q * nRows];
          alpha += ap * ap; beta += aq * aq; gamma += ap * aq;
        }
        if (gamma == 0.0) continue;
        double c = std::fabs(gamma) / std::sqrt(alpha * beta);
        off = std::max(off, c);
        if (c < 1e-15) continue;
        double zeta = (beta - alpha) / (2.0 * gamma);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        double cs = 1.0 / std::sqrt(1.0 + t * t), sn = cs * t;
        for (int i = 0; i < nRows; ++i) {
          double ap = a[i + p * nRows], aq = a[i + q * nRows];
          a[i + p * nRows] = cs * ap - sn * aq;
          a[i + q * nRows] = sn * ap + cs * aq;
        }
      }
    if (off < 1e-15) break;
  }
  for (int p = 0; p < nCols; ++p) {
    double n2 = 0;
    for (int i = 0; i < nRows; ++i) n2 += a[i + p * nRows] * a[i + p * nRows];
    s[p] = std::sqrt(n2);
  }
  std::sort(s, s + nCols, [](double x, double y) { return x > y; });
}

/* sCount of RFLU_InvertMatrixSVD (libflu/RFLU_InvertMatrixSVD.F90): number of
 * singular values treated as zero (first below 100*eps, later ones below 1e-2
 * of their predecessor, everything after the first drop). */
int svdSingularCount(int nRows, int nCols, const std::vector<double> &a) {
  double s[4];
  singularValues(nRows, nCols, a, s);
  int sCount = 0;
  if (!(s[0] > 100.0 * 2.220446049250313e-16)) sCount = 1;
  for (int i = 1; i < nCols; ++i) {
    if (!(s[i] > 0.01 * s[i - 1])) {
      sCount += nCols - i;
      break;
    }
  }
  return sCount;
}

struct Patch {
  int bcType, outflowType, order, related = -1;
  double pOut;
  double vals[ORC_BCDAT_N] = {0, 0, 0, 0, 0, 0, 0, 0}; /* pPatch%mixt%vals(:,0), BCDAT order */
  int sw[ORC_BCSWI_N] = {0, 0};                         /* pPatch%mixt%switches, BCSWI order */
  int n;
  std::vector<int> bf2v, bf2c;
  std::vector<double> fn, fc;
};

} // namespace

struct orc_ctx {
  /* mesh */
  int nVert, nCells, nvc;
  std::vector<double> xyz;
  /* c2vGeo: the cells' own vertex ids (their coordinates); c2v: the same
     after the vertices of translational periodic patch pairs are identified
     (topology: faces, stencils) */
  std::vector<int> c2v, c2vGeo;
  std::vector<std::array<double, 3>> perShift;  /* translation of each periodic pair */
  int nFaces;
  std::vector<int> f2c, f2v;
  /* fc2: face centroid in the frame of the face's second cell (fc translated
     for a periodic face, else fc) */
  std::vector<double> fn, fc, fc2, vol, cofg;
  std::vector<Patch> patches;
  /* symmetry (mirror) patches: the cells near them are also seen reflected
     across them, as images with ids nCells + k in the stencils (stIdx):
     the image's real cell, its reflection (an index into xfQ, the velocity
     reflections, 9 values row-major), its centroid and its vertices (ids
     past nVert for vertices off the reflecting planes); patchXf: each
     symmetry patch's own reflection (-1 for the other patches) */
  std::vector<int> imgCell, imgXf, imgC2v, patchXf;
  std::vector<double> imgPos;
  std::vector<std::array<double, 9>> xfQ;
  int nVertExt = 0;
  std::vector<int> stOff, stIdx;
  std::vector<double> moms;
  /* CRECONSTC 1: the boundary-face stencil (global boundary face index) */
  std::vector<int> bfOff, bfIdx;
  std::vector<double> epsq;     /* unused cache slot kept empty: Venkat recomputes vol**(1/3) per face */
  /* numerics */
  orc_num_desc num;
  int nrkSteps;
  double ark[5], grk[5];
  double refCp, refGamma, gvMol, gvCp;
  /* cell -> face entries in the order the reference's face loops reach a
     cell: its interior faces by face id (entry 2*f + side, side 1 when the
     cell is the face's second cell f2c(2)), then its boundary faces patch
     by patch (entry -(1 + b), b numbering the boundary faces of all patches
     in order, bPatch/bFace giving the patch and the index in it) */
  std::vector<int> cfOff, cfEnt, bPatch, bFace;
  /* state */
  std::vector<double> cv, dv, cvOld, rhs, rhsSum, diss, grad, lim;
  std::vector<double> flux;     /* 5 per interior face, then 5 per boundary face */
  long long posFixCount = 0, negPCount = 0, nanCount = 0;
  double dtCells;
};

namespace {

/* ------------------------------------------------------------------------ */
/* Translational periodic patch pairs (BC_PERIODIC, RELPATCH).  The reference */
/* copies cells near the related patch as virtual cells beyond each periodic  */
/* patch (modflu/RFLU_ModSymmetryPeriodic.F90:148-335, 471-787) and copies    */
/* the actual cells' state and gradients into them every stage               */
/* (libfloflu/RungeKuttaMP.F90:225-236, 448-459).  Here the two patches'      */
/* vertices are identified instead: their faces pair up as interior faces of */
/* a periodic mesh, every cell keeps its own vertex coordinates for its       */
/* geometry, and each face across the period and each stencil member seen    */
/* across it carries the translation between the two cells' frames.  A cell's */
/* gradient, fluxes and residual then see the neighbours its virtual cells   */
/* stand for; what differs is the order of the sums (the reference numbers    */
/* actual-virtual faces after the actual ones; so do periodic faces here) and */
/* the virtual cells' own raw gradients, which enter the WENO smoothing of    */
/* the cells next to the patch: for a flow that varies along the period only, */
/* as in the reference's periodic gas-jump golden, those equal their actual   */
/* cells' because every stencil stays symmetric along the period.            */
/* ------------------------------------------------------------------------ */
int findRep(std::vector<int> &rep, int v) {
  while (rep[v] != v) {
    rep[v] = rep[rep[v]];
    v = rep[v];
  }
  return v;
}

void identifyPeriodicVertices(orc_ctx *c) {
  std::vector<int> rep(c->nVert);
  for (int v = 0; v < c->nVert; ++v) rep[v] = v;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int v = 0; v < c->nVert; ++v)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], c->xyz[3 * v + d]);
      hi[d] = std::max(hi[d], c->xyz[3 * v + d]);
    }
  const double tol = 1e-7 * std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  auto verts = [&](const Patch &p) {
    std::vector<int> v;
    for (int i = 0; i < p.n; ++i)
      for (int k = 0; k < 4; ++k)
        if (p.bf2v[4 * i + k] >= 0) v.push_back(p.bf2v[4 * i + k]);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    return v;
  };
  for (int ip = 0; ip < (int)c->patches.size(); ++ip) {
    const Patch &P = c->patches[ip];
    if (P.bcType != ORC_BC_PERIODIC || P.related <= ip) continue;
    const Patch &Q = c->patches[P.related];
    const std::vector<int> vp = verts(P), vq = verts(Q);
    if (vp.size() != vq.size() || vp.empty()) {
      std::fprintf(stderr, "oracle: periodic patches %d and %d do not match\n", ip, P.related);
      std::abort();
    }
    std::array<double, 3> T;
    for (int d = 0; d < 3; ++d) {
      double sp = 0.0, sq = 0.0;
      for (int v : vp) sp += c->xyz[3 * v + d];
      for (int v : vq) sq += c->xyz[3 * v + d];
      T[d] = (sq - sp) / (double)vp.size();
    }
    c->perShift.push_back(T);
    std::map<std::array<long long, 3>, int> grid;
    for (int w : vq) {
      std::array<long long, 3> k;
      for (int d = 0; d < 3; ++d) k[d] = std::llround(c->xyz[3 * w + d] / tol);
      grid[k] = w;
    }
    for (int v : vp) {
      int w = -1;
      std::array<long long, 3> k0;
      for (int d = 0; d < 3; ++d) k0[d] = std::llround((c->xyz[3 * v + d] + T[d]) / tol);
      for (int a = -1; a <= 1 && w < 0; ++a)
        for (int b = -1; b <= 1 && w < 0; ++b)
          for (int e = -1; e <= 1 && w < 0; ++e) {
            auto it = grid.find({k0[0] + a, k0[1] + b, k0[2] + e});
            if (it != grid.end()) w = it->second;
          }
      if (w < 0) {
        std::fprintf(stderr, "oracle: periodic vertex %d has no image on patch %d\n", v, P.related);
        std::abort();
      }
      const int rv = findRep(rep, v), rw = findRep(rep, w);
      if (rv != rw) rep[std::max(rv, rw)] = std::min(rv, rw);
    }
  }
  for (size_t k = 0; k < c->c2v.size(); ++k) c->c2v[k] = findRep(rep, c->c2vGeo[k]);
  /* the periodic patches' faces are interior faces now */
  for (Patch &p : c->patches)
    if (p.bcType == ORC_BC_PERIODIC) p.n = 0;
}

/* Offset of stencil member j from cell i, cofg(j) - cofg(i), for the image
 * of j nearest to i when the mesh is periodic (the virtual cell standing for
 * j in the reference).  A symmetry image's offset is its cell's offset plus
 * the image's translation from its cell, (cofg(cell) - cofg(i)) + (image -
 * cofg(cell)), summed in that order like a periodic image's. */
void memberOffset(const orc_ctx *c, int i, int j, double &dx, double &dy, double &dz) {
  if (j >= c->nCells) {
    const double *x = &c->imgPos[3 * (size_t)(j - c->nCells)], *x0 = &c->cofg[3 * c->imgCell[j - c->nCells]];
    dx = (x0[0] - c->cofg[3 * i]) + (x[0] - x0[0]);
    dy = (x0[1] - c->cofg[3 * i + 1]) + (x[1] - x0[1]);
    dz = (x0[2] - c->cofg[3 * i + 2]) + (x[2] - x0[2]);
    return;
  }
  const double *xj = &c->cofg[3 * j];
  dx = xj[0] - c->cofg[3 * i];
  dy = xj[1] - c->cofg[3 * i + 1];
  dz = xj[2] - c->cofg[3 * i + 2];
  if (c->perShift.empty()) return;
  double best = dx * dx + dy * dy + dz * dz, bx = dx, by = dy, bz = dz;
  const int np = (int)c->perShift.size();
  int combos = 1;
  for (int p = 0; p < np; ++p) combos *= 3;
  for (int m = 1; m < combos; ++m) {
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int r = m;
    for (int p = 0; p < np; ++p, r /= 3) {
      const double f = (double)(r % 3 == 2 ? -1 : r % 3);
      sx += f * c->perShift[p][0];
      sy += f * c->perShift[p][1];
      sz += f * c->perShift[p][2];
    }
    const double ex = dx + sx, ey = dy + sy, ez = dz + sz;
    const double d2 = ex * ex + ey * ey + ez * ez;
    if (d2 < best) { best = d2; bx = ex; by = ey; bz = ez; }
  }
  dx = bx; dy = by; dz = bz;
}

/* ------------------------------------------------------------------------ */
/* Symmetry (mirror) patches (BC_SYMMETRY).  The reference copies the cells  */
/* near each symmetry patch as virtual cells reflected across it (and copies */
/* of earlier patches' virtual cells near it, which makes the corner images) */
/* (modflu/RFLU_ModSymmetryPeriodic.F90:148-335, 471-787), sets their state  */
/* from the actual cells with the momentum reflected (modflu/               */
/* RFLU_ModRelatedPatches.F90:268-353) and, after the gradients, their       */
/* gradients transformed (:380-435: Q g for density and pressure, Q G Q^T   */
/* for the velocity gradient).  A face on the patch is an interior face to   */
/* its virtual cell: the limiters see the reflected cell as a neighbour, the */
/* time step counts the face as interior, and the flux is the interior flux  */
/* against the reflected state.  Here each patch must be planar, two patches */
/* parallel or perpendicular; the images are the cells within three vertex  */
/* layers of a patch, reflected across every set of such patches without   */
/* two parallel ones, and their vertices off the reflecting planes get new  */
/* ids, so that the stencils grow across the planes as over virtual cells.  */
/* An image's state and gradients are its cell's, reflected; the reference's */
/* virtual cells compute raw gradients of their own from their (truncated)   */
/* stencils, which only the WENO smoothing of the cells next to the patch   */
/* reads (libfloflu/RungeKuttaMP.F90:225-236); the images here carry the     */
/* reflected raw gradients instead.                                          */
/* ------------------------------------------------------------------------ */
const int kSymLayers = 3;

/* y = Q x for a row-major Q, summed in index order */
inline void reflect3(const double *Q, const double *x, double *y) {
  for (int a = 0; a < 3; ++a) {
    double s = Q[3 * a] * x[0];
    s = s + Q[3 * a + 1] * x[1];
    s = s + Q[3 * a + 2] * x[2];
    y[a] = s;
  }
}

void buildSymmetryImages(orc_ctx *c) {
  const int nc = c->nCells, nvc = c->nvc;
  struct Plane { int patch; double n[3], p0[3]; };
  std::vector<Plane> planes;
  c->patchXf.assign(c->patches.size(), -1);
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int v = 0; v < c->nVert; ++v)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], c->xyz[3 * v + d]);
      hi[d] = std::max(hi[d], c->xyz[3 * v + d]);
    }
  const double tol = 1e-7 * std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  for (int ip = 0; ip < (int)c->patches.size(); ++ip) {
    const Patch &p = c->patches[ip];
    if (p.bcType != ORC_BC_SYMMETRY || p.n == 0) continue;
    Plane P;
    P.patch = ip;
    for (int d = 0; d < 3; ++d) { P.n[d] = p.fn[d]; P.p0[d] = p.fc[d]; }
    for (int i = 0; i < p.n; ++i) {
      const double cosA = p.fn[4 * i] * P.n[0] + p.fn[4 * i + 1] * P.n[1] + p.fn[4 * i + 2] * P.n[2];
      for (int k = 0; k < 4; ++k) {
        const int v = p.bf2v[4 * i + k];
        if (v < 0) continue;
        const double h = (c->xyz[3 * v] - P.p0[0]) * P.n[0] + (c->xyz[3 * v + 1] - P.p0[1]) * P.n[1] +
                         (c->xyz[3 * v + 2] - P.p0[2]) * P.n[2];
        if (std::fabs(h) > tol || cosA < 1.0 - 1e-10) {
          std::fprintf(stderr, "oracle: symmetry patch %d is not planar\n", ip);
          std::abort();
        }
      }
    }
    planes.push_back(P);
  }
  const int np = (int)planes.size();
  if (np == 0) return;
  if (np > 30) { std::fprintf(stderr, "oracle: more than 30 symmetry patches\n"); std::abort(); }
  std::vector<int> parallel(np, 0);  /* bit q of parallel[a]: planes a and q are parallel */
  for (int a = 0; a < np; ++a)
    for (int q = 0; q < np; ++q) {
      if (q == a) continue;
      const double d = std::fabs(planes[a].n[0] * planes[q].n[0] + planes[a].n[1] * planes[q].n[1] +
                                 planes[a].n[2] * planes[q].n[2]);
      if (d > 1.0 - 1e-10) parallel[a] |= 1 << q;
      else if (d > 1e-10) {
        std::fprintf(stderr, "oracle: symmetry patches %d and %d are neither parallel nor perpendicular\n",
                     planes[a].patch, planes[q].patch);
        std::abort();
      }
    }
  /* vertices on each plane (its patch's vertices), cells near it */
  std::vector<int> vmask(c->nVert, 0), nearMask(nc, 0);
  std::vector<int> v2cOff(c->nVert + 1, 0), v2c;
  for (int ic = 0; ic < nc; ++ic)
    for (int k = 0; k < nvc; ++k) v2cOff[c->c2v[nvc * ic + k] + 1]++;
  for (int v = 0; v < c->nVert; ++v) v2cOff[v + 1] += v2cOff[v];
  v2c.resize(v2cOff[c->nVert]);
  {
    std::vector<int> fill(v2cOff.begin(), v2cOff.end() - 1);
    for (int ic = 0; ic < nc; ++ic)
      for (int k = 0; k < nvc; ++k) v2c[fill[c->c2v[nvc * ic + k]]++] = ic;
  }
  for (int a = 0; a < np; ++a) {
    const Patch &p = c->patches[planes[a].patch];
    std::vector<char> vIn(c->nVert, 0), cIn(nc, 0);
    std::vector<int> front;
    for (int i = 0; i < p.n; ++i)
      for (int k = 0; k < 4; ++k) {
        const int v = p.bf2v[4 * i + k];
        if (v < 0) continue;
        vmask[v] |= 1 << a;
        if (!vIn[v]) { vIn[v] = 1; front.push_back(v); }
      }
    for (int layer = 0; layer < kSymLayers; ++layer) {
      std::vector<int> next;
      for (int v : front)
        for (int e = v2cOff[v]; e < v2cOff[v + 1]; ++e) {
          const int ic = v2c[e];
          if (cIn[ic]) continue;
          cIn[ic] = 1;
          nearMask[ic] |= 1 << a;
          for (int k = 0; k < nvc; ++k) {
            const int w = c->c2v[nvc * ic + k];
            if (!vIn[w]) { vIn[w] = 1; next.push_back(w); }
          }
        }
      front.swap(next);
    }
  }
  /* images: (cell, plane set) in the order of the set's highest plane, the
     set, then the cell (the reference adds virtual cells patch by patch) */
  struct Img { int top, set, cell; };
  std::vector<Img> imgs;
  for (int ic = 0; ic < nc; ++ic) {
    const int m = nearMask[ic];
    for (int S = m; S > 0; S = (S - 1) & m) {
      bool ok = true;
      for (int a = 0; a < np && ok; ++a)
        if ((S >> a & 1) && (S & parallel[a])) ok = false;
      if (!ok) continue;
      int top = 0;
      while ((S >> (top + 1)) != 0) ++top;
      imgs.push_back({top, S, ic});
    }
  }
  std::sort(imgs.begin(), imgs.end(), [](const Img &x, const Img &y) {
    if (x.top != y.top) return x.top < y.top;
    if (x.set != y.set) return x.set < y.set;
    return x.cell < y.cell;
  });
  /* reflections: one per plane set, Q_S = Q_a1 Q_a2 ... in plane order */
  std::map<int, int> xfOf;
  auto planeQ = [&](int a, double *Q) {
    const double nx = planes[a].n[0], ny = planes[a].n[1], nz = planes[a].n[2];
    Q[0] = 1.0 - 2.0 * nx * nx; Q[1] = -2.0 * nx * ny;      Q[2] = -2.0 * nx * nz;
    Q[3] = Q[1];                Q[4] = 1.0 - 2.0 * ny * ny; Q[5] = -2.0 * ny * nz;
    Q[6] = Q[2];                Q[7] = Q[5];                Q[8] = 1.0 - 2.0 * nz * nz;
  };
  auto xfIndex = [&](int S) {
    auto it = xfOf.find(S);
    if (it != xfOf.end()) return it->second;
    std::array<double, 9> Q;
    bool first = true;
    for (int a = 0; a < np; ++a) {
      if (!(S >> a & 1)) continue;
      double Qa[9];
      planeQ(a, Qa);
      if (first) {
        for (int k = 0; k < 9; ++k) Q[k] = Qa[k];
        first = false;
      } else {
        std::array<double, 9> P;
        for (int r = 0; r < 3; ++r)
          for (int col = 0; col < 3; ++col) {
            double s = Q[3 * r] * Qa[col];
            s = s + Q[3 * r + 1] * Qa[3 + col];
            s = s + Q[3 * r + 2] * Qa[6 + col];
            P[3 * r + col] = s;
          }
        Q = P;
      }
    }
    const int idx = (int)c->xfQ.size();
    c->xfQ.push_back(Q);
    xfOf[S] = idx;
    return idx;
  };
  for (int a = 0; a < np; ++a) c->patchXf[planes[a].patch] = xfIndex(1 << a);
  std::map<std::pair<int, int>, int> vext;
  int nextV = c->nVert;
  for (const Img &im : imgs) {
    c->imgCell.push_back(im.cell);
    c->imgXf.push_back(xfIndex(im.set));
    double x[3] = {c->cofg[3 * im.cell], c->cofg[3 * im.cell + 1], c->cofg[3 * im.cell + 2]};
    for (int a = 0; a < np; ++a) {
      if (!(im.set >> a & 1)) continue;
      const double *n = planes[a].n, *p0 = planes[a].p0;
      const double h = (x[0] - p0[0]) * n[0] + (x[1] - p0[1]) * n[1] + (x[2] - p0[2]) * n[2];
      for (int d = 0; d < 3; ++d) x[d] = x[d] - 2.0 * h * n[d];
    }
    for (int d = 0; d < 3; ++d) c->imgPos.push_back(x[d]);
    for (int k = 0; k < nvc; ++k) {
      const int v = c->c2v[nvc * im.cell + k];
      const int S = im.set & ~vmask[v];
      if (S == 0) {
        c->imgC2v.push_back(v);
        continue;
      }
      auto it = vext.find({v, S});
      if (it == vext.end()) it = vext.emplace(std::make_pair(v, S), nextV++).first;
      c->imgC2v.push_back(it->second);
    }
  }
  c->nVertExt = nextV;
}

/* A stencil member's primitive state (rho, u, v, w, p) and raw gradient:
 * its cell's, reflected for an image. */
inline void memberVar(const orc_ctx *c, const std::vector<double> &var, int j, double *out) {
  if (j < c->nCells) {
    for (int k = 0; k < 5; ++k) out[k] = var[5 * (size_t)j + k];
    return;
  }
  const int cell = c->imgCell[j - c->nCells];
  const double *v = &var[5 * (size_t)cell];
  out[0] = v[0];
  reflect3(c->xfQ[c->imgXf[j - c->nCells]].data(), v + 1, out + 1);
  out[4] = v[4];
}
inline void transformGrad(const double *Q, const double *g, double *o) {
  reflect3(Q, g, o);
  reflect3(Q, g + 12, o + 12);
  /* velocity gradient G[a][c] = g[3 (1 + a) + c]: Q (G Q^T) */
  double T[9];
  for (int b = 0; b < 3; ++b)
    for (int col = 0; col < 3; ++col) {
      double s = g[3 * (1 + b)] * Q[3 * col];
      s = s + g[3 * (1 + b) + 1] * Q[3 * col + 1];
      s = s + g[3 * (1 + b) + 2] * Q[3 * col + 2];
      T[3 * b + col] = s;
    }
  for (int a = 0; a < 3; ++a)
    for (int col = 0; col < 3; ++col) {
      double s = Q[3 * a] * T[col];
      s = s + Q[3 * a + 1] * T[3 + col];
      s = s + Q[3 * a + 2] * T[6 + col];
      o[3 * (1 + a) + col] = s;
    }
}
inline void memberGrad(const orc_ctx *c, const std::vector<double> &grad, int j, double *out) {
  if (j < c->nCells) {
    for (int k = 0; k < 15; ++k) out[k] = grad[15 * (size_t)j + k];
    return;
  }
  transformGrad(c->xfQ[c->imgXf[j - c->nCells]].data(), &grad[15 * (size_t)c->imgCell[j - c->nCells]], out);
}
/* the symmetry patch of a boundary face entry (code < 0) of a cell's face
   list, else -1 */
inline int symmetryPatchOf(const orc_ctx *c, int code) {
  if (code >= 0 || c->patchXf.empty()) return -1;
  const int ip = c->bPatch[-code - 1];
  return c->patchXf[ip] >= 0 ? ip : -1;
}
/* The centroid the limiters' second face loop takes for a face entry of a
   cell: an interior face's (in the cell's frame), a symmetry patch face's
   (an interior face to the cell's reflection), else none. */
inline const double *limiterFaceCentroid(const orc_ctx *c, int code) {
  if (code >= 0) {
    const int f = code >> 1;
    return (code & 1) ? &c->fc2[3 * f] : &c->fc[3 * f];
  }
  const int ip = symmetryPatchOf(c, code);
  if (ip < 0) return nullptr;
  return &c->patches[ip].fc[3 * c->bFace[-code - 1]];
}
/* the cell's own state reflected across symmetry patch ip (its virtual
   neighbour across a face of the patch) */
inline void mirrorVar(const orc_ctx *c, const std::vector<double> &var, int ic, int ip, double *out) {
  const double *v = &var[5 * (size_t)ic];
  out[0] = v[0];
  reflect3(c->xfQ[c->patchXf[ip]].data(), v + 1, out + 1);
  out[4] = v[4];
}

/* ------------------------------------------------------------------------ */
/* Face list: RFLU_BuildFaceList (modflu/RFLU_ModFaceList.F90:784-1585) with  */
/* the hash table of RFLU_HashFace (modflu/RFLU_ModHashTable.F90:618-734):    */
/* faces numbered by first insertion in the cell loop x local-face loop,      */
/* f2c(1) = inserting cell, f2c(2) = second cell, f2v from the inserting      */
/* cell's local face; boundary faces (one cell) leave the interior list.      */
/* Local face tables f2vTet/f2vHex: modflu/RFLU_ModGrid.F90:92-96.            */
/* ------------------------------------------------------------------------ */
const int f2vTet[4][3] = {{1, 2, 3}, {2, 4, 3}, {1, 3, 4}, {1, 4, 2}};
const int f2vHex[6][4] = {{1, 4, 3, 2}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 4, 8, 7}, {1, 5, 8, 4}, {5, 6, 7, 8}};

void buildFaceList(orc_ctx *c) {
  struct Rec { int c1, c2, ifl; };
  std::map<std::array<int, 3>, int> table;
  std::vector<Rec> rec;
  const int nfl = (c->nvc == 4) ? 4 : 6;
  const int fvs = (c->nvc == 4) ? 3 : 4;
  for (int icg = 0; icg < c->nCells; ++icg) {
    for (int ifl = 0; ifl < nfl; ++ifl) {
      int fv[4];
      for (int k = 0; k < fvs; ++k)
        fv[k] = c->c2v[c->nvc * icg + ((fvs == 3) ? f2vTet[ifl][k] : f2vHex[ifl][k]) - 1];
      std::sort(fv, fv + fvs);
      std::array<int, 3> key = {fv[0], fv[1], fv[2]};
      auto it = table.find(key);
      if (it == table.end()) {
        table.emplace(key, (int)rec.size());
        rec.push_back({icg, -1, ifl});
      } else {
        rec[it->second].c2 = icg;
      }
    }
  }
  /* interior (AA) faces keep the first-insertion order; faces across a
     period (the reference's actual-virtual faces) follow them in the same
     order.  f2v: the first cell's own vertex ids (geometry) */
  c->f2c.clear(); c->f2v.clear();
  for (int pass = 0; pass < 2; ++pass)
    for (const Rec &r : rec) {
      if (r.c2 < 0) continue;
      int fvGeo[4] = {-1, -1, -1, -1};
      for (int k = 0; k < fvs; ++k)
        fvGeo[k] = c->c2vGeo[c->nvc * r.c1 + ((fvs == 3) ? f2vTet[r.ifl][k] : f2vHex[r.ifl][k]) - 1];
      /* across a period: the second cell holds the face's first vertex
         under another vertex id */
      bool across = true;
      for (int k = 0; k < c->nvc; ++k)
        if (c->c2vGeo[c->nvc * r.c2 + k] == fvGeo[0]) across = false;
      if (across != (pass == 1)) continue;
      c->f2c.push_back(r.c1);
      c->f2c.push_back(r.c2);
      for (int k = 0; k < 4; ++k) c->f2v.push_back(fvGeo[k]);
    }
  c->nFaces = (int)c->f2c.size() / 2;
  /* boundary faces: RFLU_UnHashBFace gives the owning cell */
  for (Patch &p : c->patches) {
    p.bf2c.assign(p.n, -1);
    for (int i = 0; i < p.n; ++i) {
      int fv[4];
      int n = (p.bf2v[4 * i + 3] < 0) ? 3 : 4;
      for (int k = 0; k < n; ++k) fv[k] = p.bf2v[4 * i + k];
      std::sort(fv, fv + n);
      auto it = table.find({fv[0], fv[1], fv[2]});
      if (it == table.end() || rec[it->second].c2 >= 0) {
        std::fprintf(stderr, "oracle: boundary face %d not found as a single-cell face\n", i);
        std::abort();
      }
      p.bf2c[i] = rec[it->second].c1;
    }
  }
}

/* The per-cell face lists of orc_ctx (cfOff, cfEnt) from f2c and bf2c. */
void buildCellFaces(orc_ctx *c) {
  const int nc = c->nCells;
  c->bPatch.clear();
  c->bFace.clear();
  for (int ip = 0; ip < (int)c->patches.size(); ++ip)
    for (int i = 0; i < c->patches[ip].n; ++i) {
      c->bPatch.push_back(ip);
      c->bFace.push_back(i);
    }
  const int nb = (int)c->bPatch.size();
  std::vector<int> cnt(nc + 1, 0);
  for (int f = 0; f < c->nFaces; ++f) { cnt[c->f2c[2 * f] + 1]++; cnt[c->f2c[2 * f + 1] + 1]++; }
  for (int b = 0; b < nb; ++b) cnt[c->patches[c->bPatch[b]].bf2c[c->bFace[b]] + 1]++;
  c->cfOff.assign(nc + 1, 0);
  for (int ic = 0; ic < nc; ++ic) c->cfOff[ic + 1] = c->cfOff[ic] + cnt[ic + 1];
  c->cfEnt.assign(c->cfOff[nc], 0);
  std::vector<int> fill(c->cfOff.begin(), c->cfOff.end() - 1);
  for (int f = 0; f < c->nFaces; ++f) {
    c->cfEnt[fill[c->f2c[2 * f]]++] = 2 * f;
    c->cfEnt[fill[c->f2c[2 * f + 1]]++] = 2 * f + 1;
  }
  for (int b = 0; b < nb; ++b) c->cfEnt[fill[c->patches[c->bPatch[b]].bf2c[c->bFace[b]]]++] = -(1 + b);
  c->flux.assign(5 * ((size_t)c->nFaces + nb), 0.0);
}

/* FaceVectorTria / FaceVectorQuad (libfloflu/FaceVector.F90),
 * FaceCentroidTria / FaceCentroidQuad (libfloflu/FaceCentroid.F90). */
void faceVectorCentroid(const double *xyz, const int *v, int nv, double &fx, double &fy, double &fz,
                        double &cx, double &cy, double &cz) {
  const double *p1 = xyz + 3 * v[0], *p2 = xyz + 3 * v[1], *p3 = xyz + 3 * v[2];
  if (nv == 3) {
    double dxa = p1[0] - p2[0], dya = p1[1] - p2[1], dza = p1[2] - p2[2];
    double dxb = p1[0] - p3[0], dyb = p1[1] - p3[1], dzb = p1[2] - p3[2];
    fx = 0.5 * (dya * dzb - dyb * dza);
    fy = -0.5 * (dxa * dzb - dxb * dza);
    fz = 0.5 * (dxa * dyb - dxb * dya);
    const double thrd = 1.0 / 3.0;
    cx = thrd * (p1[0] + p2[0] + p3[0]);
    cy = thrd * (p1[1] + p2[1] + p3[1]);
    cz = thrd * (p1[2] + p2[2] + p3[2]);
  } else {
    const double *p4 = xyz + 3 * v[3];
    double dxa = p3[0] - p1[0], dya = p3[1] - p1[1], dza = p3[2] - p1[2];
    double dxb = p2[0] - p4[0], dyb = p2[1] - p4[1], dzb = p2[2] - p4[2];
    fx = 0.5 * (dza * dyb - dya * dzb);
    fy = 0.5 * (dxa * dzb - dza * dxb);
    fz = 0.5 * (dya * dxb - dxa * dyb);
    cx = 0.25 * (p1[0] + p2[0] + p3[0] + p4[0]);
    cy = 0.25 * (p1[1] + p2[1] + p3[1] + p4[1]);
    cz = 0.25 * (p1[2] + p2[2] + p3[2] + p4[2]);
  }
}

/* RFLU_BuildGeometry (modflu/RFLU_ModGeometry.F90:307-700) with approximate
 * centroids from RFLU_ComputeApproxCentroids (:1277-1497). */
void buildGeometry(orc_ctx *c) {
  const int nc = c->nCells;
  std::vector<double> app(3 * nc);
  for (int ic = 0; ic < nc; ++ic) {
    const int *v = &c->c2vGeo[c->nvc * ic];
    for (int d = 0; d < 3; ++d) {
      double s = c->xyz[3 * v[0] + d];
      for (int k = 1; k < c->nvc; ++k) s = s + c->xyz[3 * v[k] + d];
      app[3 * ic + d] = ((c->nvc == 4) ? (1.0 / 4.0) : (1.0 / 8.0)) * s;
    }
  }
  c->vol.assign(nc, 0.0);
  c->cofg.assign(3 * nc, 0.0);
  c->fn.assign(4 * c->nFaces, 0.0);
  c->fc.assign(3 * c->nFaces, 0.0);
  c->fc2.assign(3 * c->nFaces, 0.0);
  auto accum = [&](int cell, double sgn, double fx, double fy, double fz, double cx, double cy, double cz) {
    double term = (cx - app[3 * cell]) * fx + (cy - app[3 * cell + 1]) * fy + (cz - app[3 * cell + 2]) * fz;
    if (sgn > 0) c->vol[cell] = c->vol[cell] + term; else c->vol[cell] = c->vol[cell] - term;
    term = cx * fx + cy * fy + cz * fz;
    if (sgn > 0) {
      c->cofg[3 * cell] = c->cofg[3 * cell] + term * cx;
      c->cofg[3 * cell + 1] = c->cofg[3 * cell + 1] + term * cy;
      c->cofg[3 * cell + 2] = c->cofg[3 * cell + 2] + term * cz;
    } else {
      c->cofg[3 * cell] = c->cofg[3 * cell] - term * cx;
      c->cofg[3 * cell + 1] = c->cofg[3 * cell + 1] - term * cy;
      c->cofg[3 * cell + 2] = c->cofg[3 * cell + 2] - term * cz;
    }
  };
  auto store = [](double *fn, double *fc, double fx, double fy, double fz, double cx, double cy, double cz) {
    double m = std::sqrt(fx * fx + fy * fy + fz * fz);
    double term = 1.0 / m;
    fn[0] = fx * term; fn[1] = fy * term; fn[2] = fz * term; fn[3] = m;
    fc[0] = cx; fc[1] = cy; fc[2] = cz;
  };
  for (int f = 0; f < c->nFaces; ++f) {
    int nv = (c->f2v[4 * f + 3] < 0) ? 3 : 4;
    double fx, fy, fz, cx, cy, cz;
    faceVectorCentroid(c->xyz.data(), &c->f2v[4 * f], nv, fx, fy, fz, cx, cy, cz);
    store(&c->fn[4 * f], &c->fc[3 * f], fx, fy, fz, cx, cy, cz);
    accum(c->f2c[2 * f], 1.0, fx, fy, fz, cx, cy, cz);
    /* the second cell's frame: the translation between the two cells' own
       coordinates of the face's first vertex (zero unless across a period) */
    const int c1 = c->f2c[2 * f], c2 = c->f2c[2 * f + 1], a = c->f2v[4 * f];
    double s[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < c->nvc; ++k) {
      if (c->c2vGeo[c->nvc * c1 + k] != a) continue;
      for (int k2 = 0; k2 < c->nvc; ++k2)
        if (c->c2v[c->nvc * c2 + k2] == c->c2v[c->nvc * c1 + k]) {
          const int b = c->c2vGeo[c->nvc * c2 + k2];
          if (b != a)
            for (int d = 0; d < 3; ++d) s[d] = c->xyz[3 * b + d] - c->xyz[3 * a + d];
        }
    }
    double *f2 = &c->fc2[3 * f];
    if (s[0] == 0.0 && s[1] == 0.0 && s[2] == 0.0) {
      f2[0] = cx; f2[1] = cy; f2[2] = cz;
    } else {
      f2[0] = cx + s[0]; f2[1] = cy + s[1]; f2[2] = cz + s[2];
    }
    accum(c2, -1.0, fx, fy, fz, f2[0], f2[1], f2[2]);
  }
  for (Patch &p : c->patches) {
    p.fn.assign(4 * p.n, 0.0);
    p.fc.assign(3 * p.n, 0.0);
    for (int i = 0; i < p.n; ++i) {
      int nv = (p.bf2v[4 * i + 3] < 0) ? 3 : 4;
      double fx, fy, fz, cx, cy, cz;
      faceVectorCentroid(c->xyz.data(), &p.bf2v[4 * i], nv, fx, fy, fz, cx, cy, cz);
      store(&p.fn[4 * i], &p.fc[3 * i], fx, fy, fz, cx, cy, cz);
      accum(p.bf2c[i], 1.0, fx, fy, fz, cx, cy, cz);
    }
  }
  const double THRD = 1.0 / 3.0;
  for (int ic = 0; ic < nc; ++ic) {
    c->vol[ic] = THRD * c->vol[ic];
    double term = 1.0 / (4.0 * c->vol[ic]);
    c->cofg[3 * ic] = term * c->cofg[3 * ic];
    c->cofg[3 * ic + 1] = term * c->cofg[3 * ic + 1];
    c->cofg[3 * ic + 2] = term * c->cofg[3 * ic + 2];
  }
}

/* ------------------------------------------------------------------------ */
/* C2C stencils: RFLU_BuildC2CStencil (modflu/RFLU_ModStencilsCells.F90:    */
/* 750-1206), RFLU_BuildC2CStencilBasic (:1207-1440), RFLU_AddCellLayer      */
/* (modflu/RFLU_ModStencilsUtils.F90:696-949), sizes from                    */
/* RFLU_SetInfoC2CStencil (:2816-2932): nLayersMax 6, min 4, max 40 in 3D.   */
/* v2c lists hold cells in increasing order (RFLU_BuildVert2CellList).       */
/* ------------------------------------------------------------------------ */
void buildStencils(orc_ctx *c) {
  const int nc = c->nCells, nvc = c->nvc;
  const int stencilSizeMin = 4, stencilSizeMax = 40, nLayersMax = 6;
  /* the cells and the symmetry images (ids nc + k) with their vertices */
  const int ne = nc + (int)c->imgCell.size(), nve = std::max(c->nVert, c->nVertExt);
  auto cellVert = [&](int e, int k) { return e < nc ? c->c2v[nvc * e + k] : c->imgC2v[nvc * (size_t)(e - nc) + k]; };
  std::vector<int> v2cOff(nve + 1, 0), v2c;
  for (int ic = 0; ic < ne; ++ic)
    for (int k = 0; k < nvc; ++k) v2cOff[cellVert(ic, k) + 1]++;
  for (int v = 0; v < nve; ++v) v2cOff[v + 1] += v2cOff[v];
  v2c.resize(v2cOff[nve]);
  {
    std::vector<int> fill(v2cOff.begin(), v2cOff.end() - 1);
    for (int ic = 0; ic < ne; ++ic)
      for (int k = 0; k < nvc; ++k) v2c[fill[cellVert(ic, k)]++] = ic;
  }
  const double iNVert = 1.0 / (double)nvc;
  c->stOff.assign(nc + 1, 0);
  c->stIdx.clear();
  std::vector<int> c2cs(stencilSizeMax), layerBeg(nLayersMax + 1), layerEnd(nLayersMax + 1);
  std::vector<int> tmp;
  std::vector<double> frac;
  for (int icg = 0; icg < nc; ++icg) {
    /* --- RFLU_BuildC2CStencilBasic --- */
    tmp.clear();
    for (int k = 0; k < nvc; ++k) {
      int v = c->c2v[nvc * icg + k];
      for (int j = v2cOff[v]; j < v2cOff[v + 1]; ++j) tmp.push_back(v2c[j]);
    }
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    tmp.erase(std::find(tmp.begin(), tmp.end(), icg));
    int nCells2 = (int)tmp.size();
    int vT[8];
    for (int k = 0; k < nvc; ++k) vT[k] = c->c2v[nvc * icg + k];
    std::sort(vT, vT + nvc);
    frac.resize(nCells2);
    for (int i = 0; i < nCells2; ++i) {
      int vT2[8];
      for (int k = 0; k < nvc; ++k) vT2[k] = cellVert(tmp[i], k);
      std::sort(vT2, vT2 + nvc);
      int nCommon = 0, a = 0, b = 0;
      while (a < nvc && b < nvc) {
        if (vT[a] == vT2[b]) { nCommon++; a++; b++; }
        else if (vT[a] < vT2[b]) a++;
        else b++;
      }
      frac[i] = nCommon * iNVert;
    }
    if (nCells2 > 0) QuickSortRFREALInteger(frac.data(), tmp.data(), nCells2);
    int degr = 0;
    for (int icl2 = nCells2; icl2 >= std::max(nCells2 - stencilSizeMax + 1, 1); --icl2) c2cs[degr++] = tmp[icl2 - 1];
    std::sort(c2cs.begin(), c2cs.begin() + degr);
    layerBeg[1] = 1;
    layerEnd[1] = degr;
    int nLayers = 1;
    for (int iLayer = 2; iLayer <= nLayersMax; ++iLayer) {
      int sCount = 0;
      if (degr >= stencilSizeMin) {
        std::vector<double> a(degr * 4);
        for (int isl = 0; isl < degr; ++isl) {
          int j = c2cs[isl];
          double dx, dy, dz;
          memberOffset(c, icg, j, dx, dy, dz);
          double term = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
          a[isl] = term; a[isl + degr] = term * dx; a[isl + 2 * degr] = term * dy; a[isl + 3 * degr] = term * dz;
        }
        for (int col = 0; col < 4; ++col) {
          double m = -1.79769313486231571e308;
          for (int r = 0; r < degr; ++r) m = std::max(m, std::fabs(a[r + col * degr]));
          for (int r = 0; r < degr; ++r) a[r + col * degr] = a[r + col * degr] / m;
        }
        sCount = svdSingularCount(degr, 4, a);
      }
      if (sCount != 0 || degr < stencilSizeMin) {
        /* --- RFLU_AddCellLayer --- */
        int beg = layerBeg[iLayer - 1], end = layerEnd[iLayer - 1];
        std::vector<int> sorted(c2cs.begin(), c2cs.begin() + degr);
        std::sort(sorted.begin(), sorted.end());
        std::vector<int> help;
        bool stop = false;
        for (int isl = beg; isl <= end && !stop; ++isl) {
          int m = c2cs[isl - 1];
          for (int k = 0; k < nvc && !stop; ++k) {
            int v = cellVert(m, k);
            for (int j = v2cOff[v]; j < v2cOff[v + 1]; ++j) {
              int icg2 = v2c[j];
              if (icg2 == icg) continue;
              if (std::binary_search(sorted.begin(), sorted.end(), icg2)) continue;
              if (std::binary_search(help.begin(), help.end(), icg2)) continue;
              if ((int)help.size() < stencilSizeMax) {
                help.push_back(icg2);
                std::sort(help.begin(), help.end());
              } else { stop = true; break; }
            }
          }
        }
        for (int h : help) if (degr < stencilSizeMax) c2cs[degr++] = h;
        nLayers++;
        layerBeg[iLayer] = layerEnd[iLayer - 1] + 1;
        layerEnd[iLayer] = degr;
      } else {
        break;
      }
    }
    (void)nLayers;
    for (int i = 0; i < degr; ++i) c->stIdx.push_back(c2cs[i]);
    c->stOff[icg + 1] = (int)c->stIdx.size();
  }
}

/* RFLU_ComputeWtsC2C + RFLU_ComputeStencilMoments3D1
 * (modflu/RFLU_ModWeights.F90:1025-1183, 1770-1915). moms[10*ic + k] in the
 * order r11,r12,r22,r13,r23,r33,r14,r24,r34,r44 (XYZ_MOM_11..XYZ_MOM_44). */
void buildMoments(orc_ctx *c) {
  c->moms.assign(10 * c->nCells, 0.0);
  for (int icg = 0; icg < c->nCells; ++icg) {
    double *x = &c->moms[10 * icg];
    for (int k = 0; k < 10; ++k) x[k] = 0.0;
    for (int s = c->stOff[icg]; s < c->stOff[icg + 1]; ++s) {
      int j = c->stIdx[s];
      double dx, dy, dz;
      memberOffset(c, icg, j, dx, dy, dz);
      double wt = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
      dx = wt * dx; dy = wt * dy; dz = wt * dz;
      x[0] = x[0] + dx * dx; x[1] = x[1] + dx * dy; x[2] = x[2] + dy * dy;
      x[3] = x[3] + dx * dz; x[4] = x[4] + dy * dz; x[5] = x[5] + dz * dz;
      x[6] = x[6] + wt * dx; x[7] = x[7] + wt * dy; x[8] = x[8] + wt * dz; x[9] = x[9] + wt * wt;
    }
    double r11 = std::sqrt(x[0]);
    double ir11 = 1.0 / r11;
    double r12 = ir11 * x[1];
    double r22 = std::sqrt(x[2] - r12 * r12);
    double ir22 = 1.0 / r22;
    double r13 = ir11 * x[3];
    double r23 = ir22 * (x[4] - r12 * r13);
    double r33 = std::sqrt(x[5] - (r13 * r13 + r23 * r23));
    double ir33 = 1.0 / r33;
    double r14 = ir11 * x[6];
    double r24 = ir22 * (x[7] - r12 * r14);
    double r34 = ir33 * (x[8] - (r13 * r14 + r23 * r24));
    double r44 = std::sqrt(x[9] - (r14 * r14 + r24 * r24 + r34 * r34));
    x[0] = r11; x[1] = r12; x[2] = r22; x[3] = r13; x[4] = r23; x[5] = r33;
    x[6] = r14; x[7] = r24; x[8] = r34; x[9] = r44;
  }
}

/* ------------------------------------------------------------------------ */
/* Dependent variables: RFLU_SetDependentVars TCPERF branch                  */
/* (libflu/RFLU_SetDependentVars.F90:234-289) with gv from RFLU_SetGasVars   */
/* (libflu/RFLU_SetGasVars.F90:173-178): R -> M = 8314.3/R -> R round trip.  */
/* ------------------------------------------------------------------------ */
void setDependentVars(orc_ctx *c, int ic) {
  double gc = MixtPerf_R_M(c->gvMol);
  double g = MixtPerf_G_CpR(c->gvCp, gc);
  const double *cv = &c->cv[5 * ic];
  double r = cv[0];
  double ir = 1.0 / r;
  double Eo = ir * cv[4];
  double Vm2 = ir * ir * (cv[1] * cv[1] + cv[2] * cv[2] + cv[3] * cv[3]);
  double p = MixtPerf_P_DEoGVm2(r, Eo, g, Vm2);
  double t = MixtPerf_T_DPR(r, p, gc);
  c->dv[3 * ic] = p;
  c->dv[3 * ic + 1] = t;
  c->dv[3 * ic + 2] = MixtPerf_C_GRT(g, gc, t);
}

/* ------------------------------------------------------------------------ */
/* Gradients: RFLU_ComputeGradCellsFast_3D                                   */
/* (modflu/RFLU_ModDifferentiationCells.F90:931-1178).                       */
/* var = cv in DUVWP state (rho,u,v,w,p).                                    */
/* ------------------------------------------------------------------------ */
void computeGradCells(orc_ctx *c, const std::vector<double> &var, std::vector<double> &grad) {
#pragma omp parallel for schedule(static)
  for (int icg = 0; icg < c->nCells; ++icg) {
    const double *m = &c->moms[10 * icg];
    double r11 = m[0], r12 = m[1], r22 = m[2], r13 = m[3], r23 = m[4], r33 = m[5];
    double c11 = 1.0 / r11, c22 = 1.0 / r22, c33 = 1.0 / r33;
    double c12 = -c11 * r12;
    double c13 = -(c11 * r13 + c12 * c22 * r23);
    double c23 = -c22 * r23;
    double c1111 = c11 * c11, c2222 = c22 * c22, c3333 = c33 * c33;
    double *g = &grad[15 * icg];
    for (int k = 0; k < 15; ++k) g[k] = 0.0;
    for (int s = c->stOff[icg]; s < c->stOff[icg + 1]; ++s) {
      int j = c->stIdx[s];
      double dx, dy, dz;
      memberOffset(c, icg, j, dx, dy, dz);
      double term = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
      dx = term * dx; dy = term * dy; dz = term * dz;
      double term1 = c1111 * (dx);
      double term2 = c2222 * (dy + c12 * dx);
      double term3 = c3333 * (dz + c23 * dy + c13 * dx);
      double wtx = term * (term1 + c12 * term2 + c13 * term3);
      double wty = term * (term2 + c23 * term3);
      double wtz = term * (term3);
      double vj[5];
      memberVar(c, var, j, vj);
      for (int iv = 0; iv < 5; ++iv) {
        double dVar = vj[iv] - var[5 * icg + iv];
        g[3 * iv] = g[3 * iv] + wtx * dVar;
        g[3 * iv + 1] = g[3 * iv + 1] + wty * dVar;
        g[3 * iv + 2] = g[3 * iv + 2] + wtz * dVar;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Limiters: modflu/RFLU_ModLimiters.F90                                      */
/* ------------------------------------------------------------------------ */
/* The neighbour extremes of the limiters' first face loop: per face,
 * vmin(c1) = min(vmin(c1), var(c2)), vmin(c2) = min(vmin(c2), var(c1)) and
 * the same for vmax, here per cell over its interior faces in face order. */
void neighbourExtremes(orc_ctx *c, const std::vector<double> &var, std::vector<double> &vmin,
                       std::vector<double> &vmax, bool skipVel) {
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < c->nCells; ++ic) {
    for (int e = c->cfOff[ic]; e < c->cfOff[ic + 1]; ++e) {
      const int code = c->cfEnt[e];
      double vother[5];
      if (code < 0) {
        /* a face on a symmetry patch: the neighbour is the reflected cell */
        const int ip = symmetryPatchOf(c, code);
        if (ip < 0) continue;
        mirrorVar(c, var, ic, ip, vother);
      } else {
        const int other = c->f2c[(code & ~1) + 1 - (code & 1)];
        for (int iv = 0; iv < 5; ++iv) vother[iv] = var[5 * other + iv];
      }
      for (int iv = 0; iv < 5; ++iv) {
        if (skipVel && iv >= 1 && iv <= 3) continue;
        double vo = vother[iv];
        vmin[5 * ic + iv] = fmin2(vmin[5 * ic + iv], vo);
        vmax[5 * ic + iv] = fmax2(vmax[5 * ic + iv], vo);
      }
    }
  }
}

/* RFLU_ComputeLimiterBarthJesp (:132-322); skipVel excludes vars 2..4.  The
 * second face loop's two sides (c1 with dx1 = cofg(c1) - fc, c2 with dx2)
 * per cell over its interior faces in face order. */
void limiterBarthJesp(orc_ctx *c, const std::vector<double> &var, const std::vector<double> &grad,
                      std::vector<double> &lim, bool skipVel) {
  const int nc = c->nCells;
  std::vector<double> vmin(var), vmax(var);
  for (int k = 0; k < 5 * nc; ++k) lim[k] = 1.0;
  neighbourExtremes(c, var, vmin, vmax, skipVel);
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    for (int e = c->cfOff[ic]; e < c->cfOff[ic + 1]; ++e) {
      const int code = c->cfEnt[e];
      const double *fcs = limiterFaceCentroid(c, code);
      if (!fcs) continue;
      double xc = fcs[0], yc = fcs[1], zc = fcs[2];
      double dx1 = c->cofg[3 * ic] - xc, dy1 = c->cofg[3 * ic + 1] - yc, dz1 = c->cofg[3 * ic + 2] - zc;
      for (int iv = 0; iv < 5; ++iv) {
        if (skipVel && iv >= 1 && iv <= 3) continue;
        double v1 = var[5 * ic + iv];
        double d1min1 = vmin[5 * ic + iv] - v1, d1max1 = vmax[5 * ic + iv] - v1;
        const double *g1 = &grad[15 * ic + 3 * iv];
        double d21 = g1[0] * dx1 + g1[1] * dy1 + g1[2] * dz1;
        double term;
        if (d21 > 0.0) { term = fmin2(1.0, d1max1 / d21); lim[5 * ic + iv] = fmin2(term, lim[5 * ic + iv]); }
        else if (d21 < 0.0) { term = fmin2(1.0, d1min1 / d21); lim[5 * ic + iv] = fmin2(term, lim[5 * ic + iv]); }
      }
    }
  }
}

/* RFLU_ComputeLimiterVenkat (:353-587). */
void limiterVenkat(orc_ctx *c, const std::vector<double> &var, const std::vector<double> &grad,
                   std::vector<double> &lim) {
  const int nc = c->nCells;
  const double THRD = 1.0 / 3.0, TINY = 1.0e-12, K = 1.0;
  std::vector<double> vmin(var), vmax(var);
  for (int k = 0; k < 5 * nc; ++k) lim[k] = 1.0;
  neighbourExtremes(c, var, vmin, vmax, false);
  auto venk = [&](double dmm, double d2, double epsq) {
    double numer = (dmm * dmm + epsq) * d2 + 2 * d2 * d2 * dmm;
    double denom = d2 * (dmm * dmm + 2 * d2 * d2 + dmm * d2 + epsq);
    return numer / (denom + TINY);
  };
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    for (int e = c->cfOff[ic]; e < c->cfOff[ic + 1]; ++e) {
      const int code = c->cfEnt[e];
      const double *fcs = limiterFaceCentroid(c, code);
      if (!fcs) continue;
      double xc = fcs[0], yc = fcs[1], zc = fcs[2];
      double dx1 = c->cofg[3 * ic] - xc, dy1 = c->cofg[3 * ic + 1] - yc, dz1 = c->cofg[3 * ic + 2] - zc;
      double ds1 = std::pow(c->vol[ic], THRD);
      double epsq1 = (K * ds1) * (K * ds1) * (K * ds1);
      for (int iv = 0; iv < 5; ++iv) {
        double v1 = var[5 * ic + iv];
        double d1min1 = vmin[5 * ic + iv] - v1, d1max1 = vmax[5 * ic + iv] - v1;
        const double *g1 = &grad[15 * ic + 3 * iv];
        double d21 = g1[0] * dx1 + g1[1] * dy1 + g1[2] * dz1;
        if (d21 > 0.0) lim[5 * ic + iv] = fmin2(venk(d1max1, d21, epsq1), lim[5 * ic + iv]);
        else if (d21 < 0.0) lim[5 * ic + iv] = fmin2(venk(d1min1, d21, epsq1), lim[5 * ic + iv]);
      }
    }
  }
}

/* RFLU_SymmetricEigen3 (:791-912): cyclic Jacobi on a symmetric 3x3,
 * ascending eigenvalues, eigenvectors as columns.  m and vec column-major. */
void symmetricEigen3(const double m[9], double vec[9], double val[3]) {
  const int MAX_SWEEPS = 50;
  const double EIG_TOL = 1.0e-24;
  double r[9];
  for (int k = 0; k < 9; ++k) r[k] = m[k];
#define R(i, j) r[((i)-1) + 3 * ((j)-1)]
#define V(i, j) vec[((i)-1) + 3 * ((j)-1)]
  for (int k = 0; k < 9; ++k) vec[k] = 0.0;
  for (int i = 1; i <= 3; ++i) V(i, i) = 1.0;
  double total = 0.0;
  for (int k = 0; k < 9; ++k) total = total + r[k] * r[k];
  for (int sweep = 1; sweep <= MAX_SWEEPS; ++sweep) {
    double offDiag = R(1, 2) * R(1, 2) + R(1, 3) * R(1, 3) + R(2, 3) * R(2, 3);
    if (offDiag <= EIG_TOL * total) break;
    for (int ip = 1; ip <= 2; ++ip)
      for (int iq = ip + 1; iq <= 3; ++iq) {
        if (R(ip, iq) != 0.0) {
          double theta = (R(iq, iq) - R(ip, ip)) / (2.0 * R(ip, iq));
          double tangent;
          if (std::fabs(theta) > 1.0e150) tangent = 0.5 / theta;
          else tangent = std::copysign(1.0, theta) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
          double cosine = 1.0 / std::sqrt(tangent * tangent + 1.0);
          double sine = tangent * cosine;
          int ir = 6 - ip - iq;
          double arp = R(ir, ip), arq = R(ir, iq);
          R(ip, ip) = R(ip, ip) - tangent * R(ip, iq);
          R(iq, iq) = R(iq, iq) + tangent * R(ip, iq);
          R(ip, iq) = 0.0;
          R(iq, ip) = 0.0;
          R(ir, ip) = cosine * arp - sine * arq;
          R(ip, ir) = R(ir, ip);
          R(ir, iq) = sine * arp + cosine * arq;
          R(iq, ir) = R(ir, iq);
          for (int i = 1; i <= 3; ++i) {
            double vp = V(i, ip), vq = V(i, iq);
            V(i, ip) = cosine * vp - sine * vq;
            V(i, iq) = sine * vp + cosine * vq;
          }
        }
      }
  }
  for (int i = 1; i <= 3; ++i) val[i - 1] = R(i, i);
  for (int i = 1; i <= 2; ++i) {
    int iMin = i;
    for (int k = i + 1; k <= 3; ++k) if (val[k - 1] < val[iMin - 1]) iMin = k;
    if (iMin != i) {
      std::swap(val[i - 1], val[iMin - 1]);
      for (int k = 1; k <= 3; ++k) std::swap(V(k, i), V(k, iMin));
    }
  }
#undef R
#undef V
}

/* WENO smoothing of the cell gradients (modflu/RFLU_ModWENO.F90), 3-D
   stencils: every gradient becomes an average over the cell and its stencil
   members (the cell first, then the members in stencil order), weighted by
   an inverse squared magnitude + 1e-15, from the unsmoothed gradients of
   all cells.
   xyz = true:  RFLU_WENOGradCellsXYZFast_3D (:1366-1572, RECONST 2): each
                direction by its own component, sum of w*g over sum of w;
   xyz = false: RFLU_WENOGradCells_3D (:298-452, RECONST 1): one weight per
                cell from |gx|+|gy|+|gz|, normalised weights applied. */
void wenoGradCells(orc_ctx *c, std::vector<double> &grad, bool xyz) {
  const int nc = c->nCells;
  std::vector<double> out(grad.size());
#pragma omp parallel for schedule(static)
  for (int icg = 0; icg < nc; ++icg) {
    const int sb = c->stOff[icg], se = c->stOff[icg + 1];
    /* the members' raw gradients (reflected for symmetry images) */
    std::vector<double> mg(15 * (size_t)(se - sb));
    for (int s = sb; s < se; ++s) memberGrad(c, grad, c->stIdx[s], &mg[15 * (size_t)(s - sb)]);
    for (int iv = 0; iv < 5; ++iv) {
      const double *g0 = &grad[15 * icg + 3 * iv];
      double *o = &out[15 * icg + 3 * iv];
      if (xyz) {
        for (int d = 0; d < 3; ++d) {
          double term = g0[d];
          double sum = 1.0 / (term * term + 1.0e-15);
          double gl = sum * term;
          for (int s = sb; s < se; ++s) {
            term = mg[15 * (size_t)(s - sb) + 3 * iv + d];
            double w = 1.0 / (term * term + 1.0e-15);
            sum = sum + w;
            gl = gl + w * term;
          }
          o[d] = gl / sum;
        }
      } else {
        double term = std::fabs(g0[0]) + std::fabs(g0[1]) + std::fabs(g0[2]);
        const double w0 = 1.0 / (term * term + 1.0e-15);
        double sum = w0;
        for (int s = sb; s < se; ++s) {
          const double *gj = &mg[15 * (size_t)(s - sb) + 3 * iv];
          term = std::fabs(gj[0]) + std::fabs(gj[1]) + std::fabs(gj[2]);
          sum = sum + 1.0 / (term * term + 1.0e-15);
        }
        term = w0 / sum;
        o[0] = term * g0[0];
        o[1] = term * g0[1];
        o[2] = term * g0[2];
        for (int s = sb; s < se; ++s) {
          const double *gj = &mg[15 * (size_t)(s - sb) + 3 * iv];
          double t = std::fabs(gj[0]) + std::fabs(gj[1]) + std::fabs(gj[2]);
          term = (1.0 / (t * t + 1.0e-15)) / sum;
          o[0] = o[0] + term * gj[0];
          o[1] = o[1] + term * gj[1];
          o[2] = o[2] + term * gj[2];
        }
      }
    }
  }
  grad.swap(out);
}

/* RFLU_LimitGradCellsSimple (:1147-1300): the gradient of a positive
   variable (density and pressure, libflu/RFLU_SetVarInfo.F90:140-144) is
   zeroed when its reconstruction at a face of the cell,
   ((var + gx*dx) + gy*dy) + gz*dz with d = fc - cofg, is <= 0.  The
   reference's face loop stops at the first such face; whether any face
   does is independent of the order, so each cell's faces are visited
   (interior, then the patches) and its gradients zeroed afterwards. */
void limitGradCellsSimple(orc_ctx *c, const std::vector<double> &var, std::vector<double> &grad) {
  const int nc = c->nCells;
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    bool zero[5] = {false, false, false, false, false};
    for (int e = c->cfOff[ic]; e < c->cfOff[ic + 1]; ++e) {
      const int code = c->cfEnt[e];
      const double *fcp;
      if (code >= 0) {
        fcp = (code & 1) ? &c->fc2[3 * (code >> 1)] : &c->fc[3 * (code >> 1)];
      } else {
        const int b = -code - 1;
        fcp = &c->patches[c->bPatch[b]].fc[3 * c->bFace[b]];
      }
      const double dx = fcp[0] - c->cofg[3 * ic], dy = fcp[1] - c->cofg[3 * ic + 1], dz = fcp[2] - c->cofg[3 * ic + 2];
      for (int iv = 0; iv < 5; iv += 4) {
        const double *g = &grad[15 * ic + 3 * iv];
        const double varf = var[5 * ic + iv] + g[0] * dx + g[1] * dy + g[2] * dz;
        if (varf <= 0.0) zero[iv] = true;
      }
    }
    for (int iv = 0; iv < 5; ++iv)
      if (zero[iv]) grad[15 * ic + 3 * iv] = grad[15 * ic + 3 * iv + 1] = grad[15 * ic + 3 * iv + 2] = 0.0;
  }
}

/* RFLU_LimitGradVelocityBarthJesp (:588-790). gradVel(iComp,dir) = grad(dir, 2+iComp). */
void limitGradVelocityBarthJesp(orc_ctx *c, const std::vector<double> &var, std::vector<double> &grad,
                                std::vector<double> &lim) {
  const int nc = c->nCells;
  const double EQUAL_EIG_TOL = 1.0e-3;
  std::vector<double> axes(9 * nc), eig(3 * nc), alpha(3 * nc, 1.0), dmin(3 * nc, 0.0), dmax(3 * nc, 0.0);
  auto gv = [&](int ic, int i, int j) -> double & { return grad[15 * ic + 3 * (1 + (i - 1)) + (j - 1)]; };
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    double S[9];
    for (int i = 1; i <= 3; ++i)
      for (int j = 1; j <= 3; ++j) S[(i - 1) + 3 * (j - 1)] = 0.5 * (gv(ic, i, j) + gv(ic, j, i));
    symmetricEigen3(S, &axes[9 * ic], &eig[3 * ic]);
  }
  /* both face loops per cell (icl) over its interior faces in face order */
#pragma omp parallel for schedule(static)
  for (int icl = 0; icl < nc; ++icl) {
    for (int e = c->cfOff[icl]; e < c->cfOff[icl + 1]; ++e) {
      const int code = c->cfEnt[e];
      double du[3];
      int side = 0;
      if (code < 0) {
        /* a symmetry patch face: the reflected cell as the second cell */
        const int ip = symmetryPatchOf(c, code);
        if (ip < 0) continue;
        double vm[5];
        mirrorVar(c, var, icl, ip, vm);
        for (int k = 0; k < 3; ++k) du[k] = vm[1 + k] - var[5 * icl + 1 + k];
      } else {
        const int f = code >> 1;
        side = code & 1;
        int cc[2] = {c->f2c[2 * f], c->f2c[2 * f + 1]};
        for (int k = 0; k < 3; ++k) du[k] = var[5 * cc[1] + 1 + k] - var[5 * cc[0] + 1 + k];
      }
      for (int j = 0; j < 3; ++j) {
        const double *a = &axes[9 * icl + 3 * j];
        double proj = 0.0;
        proj = proj + a[0] * du[0]; proj = proj + a[1] * du[1]; proj = proj + a[2] * du[2];
        if (side == 1) proj = -proj;
        dmin[3 * icl + j] = fmin2(dmin[3 * icl + j], proj);
        dmax[3 * icl + j] = fmax2(dmax[3 * icl + j], proj);
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int icl = 0; icl < nc; ++icl) {
    for (int e = c->cfOff[icl]; e < c->cfOff[icl + 1]; ++e) {
      const int code = c->cfEnt[e];
      const double *fcs = limiterFaceCentroid(c, code);
      if (!fcs) continue;
      double off[3];
      for (int k = 0; k < 3; ++k) off[k] = c->cofg[3 * icl + k] - fcs[k];
      double shift[3];
      for (int i = 1; i <= 3; ++i) {
        double s = 0.0;
        for (int k = 1; k <= 3; ++k) s = s + gv(icl, i, k) * off[k - 1];
        shift[i - 1] = s;
      }
      for (int j = 0; j < 3; ++j) {
        const double *a = &axes[9 * icl + 3 * j];
        double proj = 0.0;
        proj = proj + a[0] * shift[0]; proj = proj + a[1] * shift[1]; proj = proj + a[2] * shift[2];
        if (proj > 0.0) alpha[3 * icl + j] = fmin2(alpha[3 * icl + j], dmax[3 * icl + j] / proj);
        else if (proj < 0.0) alpha[3 * icl + j] = fmin2(alpha[3 * icl + j], dmin[3 * icl + j] / proj);
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    double *e = &eig[3 * ic], *al = &alpha[3 * ic];
    double mx = std::fabs(e[0]);
    mx = fmax2(mx, std::fabs(e[1])); mx = fmax2(mx, std::fabs(e[2]));
    double eigScale = EQUAL_EIG_TOL * mx;
    bool eq12 = (e[1] - e[0] <= eigScale), eq23 = (e[2] - e[1] <= eigScale);
    if (eq12 && eq23) {
      double m = fmin2(fmin2(al[0], al[1]), al[2]);
      al[0] = al[1] = al[2] = m;
    } else if (eq12) {
      double m = fmin2(al[0], al[1]); al[0] = al[1] = m;
    } else if (eq23) {
      double m = fmin2(al[1], al[2]); al[1] = al[2] = m;
    }
  }
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    const double *A = &axes[9 * ic];
    double G[3][3], Rm[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) G[i][j] = gv(ic, i + 1, j + 1);
    /* rotated = MATMUL(TRANSPOSE(axes), gradVel) */
    for (int j = 0; j < 3; ++j)
      for (int col = 0; col < 3; ++col) {
        double s = 0.0;
        for (int i = 0; i < 3; ++i) s = s + A[i + 3 * j] * G[i][col];
        Rm[j][col] = s;
      }
    for (int j = 0; j < 3; ++j)
      for (int col = 0; col < 3; ++col) Rm[j][col] = alpha[3 * ic + j] * Rm[j][col];
    /* gradVel = MATMUL(axes, rotated) */
    for (int i = 0; i < 3; ++i)
      for (int col = 0; col < 3; ++col) {
        double s = 0.0;
        for (int j = 0; j < 3; ++j) s = s + A[i + 3 * j] * Rm[j][col];
        gv(ic, i + 1, col + 1) = s;
      }
    lim[5 * ic + 1] = lim[5 * ic + 2] = lim[5 * ic + 3] = 1.0;
  }
}

/* ------------------------------------------------------------------------ */
/* CellGradientsMP (libfloflu/CellGradientsMP.F90:160-295).  Works on c->cv  */
/* in place, as the reference does (cons -> prim -> cons round trip).        */
/* ------------------------------------------------------------------------ */
/* ------------------------------------------------------------------------ */
/* Constrained gradients (CRECONSTC 1).                                      */
/* The boundary-face stencil: RFLU_AddBFaces (modflu/RFLU_ModStencilsUtils.  */
/* F90:134-298) visits the cell and its stencil members in stencil order and */
/* for each the wall and injection patches in order, taking the cell's face  */
/* on the patch (the patch's face list keyed through a sorted copy of bf2c:  */
/* for a cell with several faces on one patch the last one), at most 18;    */
/* RFLU_SortBFaces (:1501-1585) orders them by squared distance to the      */
/* centroid with QuickSortRFREALInteger; RFLU_BuildC2CStencil keeps 9       */
/* (RFLU_SetInfoC2CStencil, modflu/RFLU_ModStencilsCells.F90:2816-2909).   */
/* ------------------------------------------------------------------------ */
bool wallOrInjection(int t) {
  return t == ORC_BC_NOSLIPWALL_HFLUX || t == ORC_BC_NOSLIPWALL_TEMP || t == ORC_BC_SLIPWALL || t == ORC_BC_INJECTION;
}

void buildBFaceStencil(orc_ctx *c) {
  const int nc = c->nCells, np = (int)c->patches.size();
  std::vector<int> off(np + 1, 0);
  for (int ip = 0; ip < np; ++ip) off[ip + 1] = off[ip] + c->patches[ip].n;
  std::vector<std::vector<int>> last(np);
  for (int ip = 0; ip < np; ++ip) {
    const Patch &p = c->patches[ip];
    if (!wallOrInjection(p.bcType) || p.n == 0) continue;
    last[ip].assign(nc, -1);
    for (int ifl = 0; ifl < p.n; ++ifl) last[ip][p.bf2c[ifl]] = ifl;
  }
  c->bfOff.assign(nc + 1, 0);
  c->bfIdx.clear();
  for (int icg = 0; icg < nc; ++icg) {
    int memb[18][2];
    int n = 0;
    bool done = false;
    for (int isl = 0; isl <= c->stOff[icg + 1] - c->stOff[icg] && !done; ++isl) {
      const int isg = (isl == 0) ? icg : c->stIdx[c->stOff[icg] + isl - 1];
      if (isg >= nc) continue;  /* symmetry images: no constrained faces here (refused with walls) */
      for (int ip = 0; ip < np && !done; ++ip) {
        if (last[ip].empty() || last[ip][isg] < 0) continue;
        if (n < 18) {
          memb[n][0] = ip;
          memb[n][1] = last[ip][isg];
          ++n;
        } else {
          done = true;
        }
      }
    }
    std::vector<double> dist(n);
    std::vector<int> key(n);
    const double *x = &c->cofg[3 * icg];
    for (int isl = 0; isl < n; ++isl) {
      const double *f = &c->patches[memb[isl][0]].fc[3 * memb[isl][1]];
      key[isl] = isl;
      dist[isl] = (f[0] - x[0]) * (f[0] - x[0]) + (f[1] - x[1]) * (f[1] - x[1]) + (f[2] - x[2]) * (f[2] - x[2]);
    }
    if (n > 0) QuickSortRFREALInteger(dist.data(), key.data(), n);
    for (int isl = 0; isl < std::min(n, 9); ++isl) c->bfIdx.push_back(off[memb[key[isl]][0]] + memb[key[isl]][1]);
    c->bfOff[icg + 1] = (int)c->bfIdx.size();
  }
}

/* FloatEqual (modfloflu/ModTools.F90:129-148). */
bool floatEqual(double a, double b, double tol) { return std::fabs(a - b) <= (1.0 + 0.5 * std::fabs(a + b)) * tol; }

/* RFLU_GetConstrType (modflu/RFLU_ModConstraintUtils.F90:122-334), TCPERF,
 * the primitive variables (rho, u, v, w, p). */
bool constrDirichlet(const Patch &p, int ifl, int iv) {
  const double *n = &p.fn[4 * ifl];
  switch (iv) {
  case 0: return p.bcType == ORC_BC_INJECTION && p.vals[0] > 0.0;
  case 1: case 2: case 3:
    if (p.bcType == ORC_BC_NOSLIPWALL_HFLUX || p.bcType == ORC_BC_NOSLIPWALL_TEMP) return true;
    if (p.bcType == ORC_BC_SLIPWALL || p.bcType == ORC_BC_INJECTION)
      return floatEqual(std::fabs(n[iv - 1]), 1.0, 1.0e-6);
    return false;
  default: return false;
  }
}

/* RFLU_GetConstrValue (:366-745), TCPERF, static grid (fs = fsu = 0). */
double constrValue(const orc_ctx *c, const Patch &p, int ifl, int iv) {
  if (p.bcType != ORC_BC_INJECTION) return 0.0;
  const double *n = &p.fn[4 * ifl];
  const double minj = p.vals[0];
  if (!(minj > 0.0)) return 0.0 * n[iv - 1]; /* fsu*nx */
  /* RFLU_SetRindStateInjectPerf from the face cell's pressure */
  const double pl = c->dv[3 * p.bf2c[ifl]];
  const double rGas = MixtPerf_R_M(c->gvMol);
  const double rl = pl / (rGas * p.vals[1]);
  if (iv == 0) return rl;
  const double ql = -minj / rl + 0.0;
  return ql * n[iv - 1];
}

/* RFLU_ComputeGradCellsConstr (modflu/RFLU_ModDifferentiationCells.F90:
 * 1180-1563), 3-D: for each cell with boundary-face members and each
 * variable some of them constrain, the least-squares fit to the stencil
 * differences (rows d/|d|) and to the constraint values (rows cwt d/|d|
 * from the centroid to the face centroid), gx = gx + term*aInv(1,row)*dVar
 * row by row.  aInv: the pseudo-inverse of the row matrix; the reference
 * takes it from LAPACK dgesdd (after scaling the columns), here from the
 * normal equations, (A^T A)^-1 A^T with the inverse by cofactors: the same
 * matrix for the full-rank systems the reference accepts, to rounding. */
void constrainedGradCells(orc_ctx *c, const std::vector<double> &var, std::vector<double> &grad) {
  const int nc = c->nCells, np = (int)c->patches.size();
  std::vector<int> patchOf, faceOf;
  for (int ip = 0; ip < np; ++ip)
    for (int ifl = 0; ifl < c->patches[ip].n; ++ifl) { patchOf.push_back(ip); faceOf.push_back(ifl); }
  const double cwt = c->num.cReconstCellsWeight;
#pragma omp parallel for schedule(dynamic, 64)
  for (int icg = 0; icg < nc; ++icg) {
    if (c->bfOff[icg + 1] == c->bfOff[icg]) continue;
    const double *x = &c->cofg[3 * icg];
    const int nm = c->stOff[icg + 1] - c->stOff[icg];
    for (int iv = 0; iv < 5; ++iv) {
      std::vector<int> rowB;
      for (int e = c->bfOff[icg]; e < c->bfOff[icg + 1]; ++e) {
        const int b = c->bfIdx[e];
        if (constrDirichlet(c->patches[patchOf[b]], faceOf[b], iv)) rowB.push_back(b);
      }
      if (rowB.empty()) continue;
      const int nr = nm + (int)rowB.size();
      std::vector<double> a(3 * (size_t)nr), term(nr), dVar(nr);
      for (int r = 0; r < nr; ++r) {
        double dx, dy, dz, t;
        if (r < nm) {
          const int j = c->stIdx[c->stOff[icg] + r];
          dx = c->cofg[3 * j] - x[0]; dy = c->cofg[3 * j + 1] - x[1]; dz = c->cofg[3 * j + 2] - x[2];
          t = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
          dVar[r] = var[5 * j + iv] - var[5 * icg + iv];
        } else {
          const Patch &p = c->patches[patchOf[rowB[r - nm]]];
          const int ifl = faceOf[rowB[r - nm]];
          dx = p.fc[3 * ifl] - x[0]; dy = p.fc[3 * ifl + 1] - x[1]; dz = p.fc[3 * ifl + 2] - x[2];
          t = cwt / std::sqrt(dx * dx + dy * dy + dz * dz);
          dVar[r] = constrValue(c, p, ifl, iv) - var[5 * icg + iv];
        }
        term[r] = t;
        a[3 * r] = t * dx; a[3 * r + 1] = t * dy; a[3 * r + 2] = t * dz;
      }
      double m00 = 0, m01 = 0, m02 = 0, m11 = 0, m12 = 0, m22 = 0;
      for (int r = 0; r < nr; ++r) {
        m00 = m00 + a[3 * r] * a[3 * r]; m01 = m01 + a[3 * r] * a[3 * r + 1]; m02 = m02 + a[3 * r] * a[3 * r + 2];
        m11 = m11 + a[3 * r + 1] * a[3 * r + 1]; m12 = m12 + a[3 * r + 1] * a[3 * r + 2];
        m22 = m22 + a[3 * r + 2] * a[3 * r + 2];
      }
      const double c00 = m11 * m22 - m12 * m12, c01 = m02 * m12 - m01 * m22, c02 = m01 * m12 - m02 * m11;
      const double c11 = m00 * m22 - m02 * m02, c12 = m01 * m02 - m00 * m12, c22 = m00 * m11 - m01 * m01;
      const double id = 1.0 / (m00 * c00 + m01 * c01 + m02 * c02);
      const double i00 = id * c00, i01 = id * c01, i02 = id * c02, i11 = id * c11, i12 = id * c12, i22 = id * c22;
      double gx = 0.0, gy = 0.0, gz = 0.0;
      for (int r = 0; r < nr; ++r) {
        const double a0 = a[3 * r], a1 = a[3 * r + 1], a2 = a[3 * r + 2];
        const double w0 = term[r] * (i00 * a0 + i01 * a1 + i02 * a2);
        const double w1 = term[r] * (i01 * a0 + i11 * a1 + i12 * a2);
        const double w2 = term[r] * (i02 * a0 + i12 * a1 + i22 * a2);
        gx = gx + w0 * dVar[r];
        gy = gy + w1 * dVar[r];
        gz = gz + w2 * dVar[r];
      }
      double *g = &grad[15 * icg + 3 * iv];
      g[0] = gx; g[1] = gy; g[2] = gz;
    }
  }
}

void cellGradients(orc_ctx *c) {
  if (c->num.spaceOrder <= 1) return;
  const int nc = c->nCells;
  /* RFLU_ConvertCvCons2Prim, DUVWP (modflu/RFLU_ModConvertCv.F90:124-397) */
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    double *cv = &c->cv[5 * ic];
    double ir = 1.0 / cv[0];
    cv[1] = ir * cv[1];
    cv[2] = ir * cv[2];
    cv[3] = ir * cv[3];
    cv[4] = c->dv[3 * ic];
  }
  computeGradCells(c, c->cv, c->grad);
  if (c->num.cReconstCells == 1) constrainedGradCells(c, c->cv, c->grad);
  switch (c->num.reconst) {
  case 0: break;
  case 1:
  case 2:
    wenoGradCells(c, c->grad, c->num.reconst == 2);
    limitGradCellsSimple(c, c->cv, c->grad);
    break;
  case 10:
    limiterBarthJesp(c, c->cv, c->grad, c->lim, true);
    limitGradVelocityBarthJesp(c, c->cv, c->grad, c->lim);
    break;
  case 100: limiterBarthJesp(c, c->cv, c->grad, c->lim, false); break;
  case 11: limiterVenkat(c, c->cv, c->grad, c->lim); break;
  default: std::fprintf(stderr, "oracle: RECONST %d not supported\n", c->num.reconst); std::abort();
  }
  if (c->num.reconst == 10 || c->num.reconst == 100 || c->num.reconst == 11) {
    /* RFLU_LimitGradCells (RFLU_ModLimiters.F90:1061-1146) */
#pragma omp parallel for schedule(static)
    for (int ic = 0; ic < nc; ++ic)
      for (int iv = 0; iv < 5; ++iv) {
        double l = c->lim[5 * ic + iv];
        double *g = &c->grad[15 * ic + 3 * iv];
        g[0] = l * g[0]; g[1] = l * g[1]; g[2] = l * g[2];
      }
  }
  /* RFLU_ConvertCvPrim2Cons (RFLU_ModConvertCv.F90:545-575) */
  double gc = MixtPerf_R_M(c->gvMol), g = MixtPerf_G_CpR(c->gvCp, gc);
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    double *cv = &c->cv[5 * ic];
    double r = cv[0], u = cv[1], v = cv[2], w = cv[3], p = c->dv[3 * ic];
    /* cv(ENER) = r*Eo(r,g,p,u,v,w) on the primitive velocities */
    cv[1] = r * u;
    cv[2] = r * v;
    cv[3] = r * w;
    /* With PICL compiled in and not used, the energy slot keeps p (:567-571). */
    if (!c->num.piclBuild) cv[4] = r * MixtPerf_Eo_DGPUVW(r, g, p, u, v, w);
  }
}

/* ------------------------------------------------------------------------ */
/* Interior face fluxes                                                      */
/* ------------------------------------------------------------------------ */
struct FaceState { double r, u, v, w, p; };

/* 2nd-order reconstruction common to the *_ComputeFlux2_TCP routines:
 * primitive from cv (ul = mom*irl), p from dv, plus grad . (fc - cofg). */
FaceState reconstruct(orc_ctx *c, int ic, double xc, double yc, double zc) {
  const double *cv = &c->cv[5 * ic];
  FaceState s;
  s.r = cv[0];
  double ir = 1.0 / s.r;
  s.u = cv[1] * ir; s.v = cv[2] * ir; s.w = cv[3] * ir;
  s.p = c->dv[3 * ic];
  double dx = xc - c->cofg[3 * ic], dy = yc - c->cofg[3 * ic + 1], dz = zc - c->cofg[3 * ic + 2];
  const double *g = &c->grad[15 * ic];
  s.r = s.r + g[0] * dx + g[1] * dy + g[2] * dz;
  s.u = s.u + g[3] * dx + g[4] * dy + g[5] * dz;
  s.v = s.v + g[6] * dx + g[7] * dy + g[8] * dz;
  s.w = s.w + g[9] * dx + g[10] * dy + g[11] * dz;
  s.p = s.p + g[12] * dx + g[13] * dy + g[14] * dz;
  return s;
}

/* Roe flux with the Harten-Hyman entropy fix: RFLU_ROE_ComputeFlux1_TCP
 * (modflu/RFLU_ModRoeFlux.F90:1683-1942) and ..._Flux2_TCP (:2513-2867).
 * Returns flx = flxConv - flxDiss. */
void roeFlux(orc_ctx *c, double nx, double ny, double nz, double nm, double fs, double rl, double ul, double vl,
             double wl, double pl, double Hl, double rr, double ur, double vr, double wr, double pr, double Hr,
             double flx[5]) {
  const double g = c->refGamma, epsentr = c->num.epsEntr, dissFact = c->num.dissFact;
  double ql = ul * nx + vl * ny + wl * nz - fs;
  double qr = ur * nx + vr * ny + wr * nz - fs;
  double rh = std::sqrt(rl * rr);
  double wt = rl / (rl + rh);
  double uh = wt * ul + (1.0 - wt) * ur;
  double vh = wt * vl + (1.0 - wt) * vr;
  double wh = wt * wl + (1.0 - wt) * wr;
  double Hh = wt * Hl + (1.0 - wt) * Hr;
  double qh = uh * nx + vh * ny + wh * nz - fs;
  double sh = 0.5 * (uh * uh + vh * vh + wh * wh);
  double ah = MixtPerf_C_GHoVm2(g, Hh, 2.0 * sh);
  double l1 = std::fabs(qh - ah), l2 = std::fabs(qh), l5 = std::fabs(qh + ah);
  double efc = epsentr * l5;
  l1 = EntropyFixHartenHyman(l1, efc);
  l2 = EntropyFixHartenHyman(l2, efc);
  l5 = EntropyFixHartenHyman(l5, efc);
  double dr = rr - rl, du = ur - ul, de = vr - vl, dw = wr - wl, dp = pr - pl;
  double dq = du * nx + de * ny + dw * nz;
  double dv1 = (dp - rh * ah * dq) / (2.0 * ah * ah);
  double dv5 = (dp + rh * ah * dq) / (2.0 * ah * ah);
  double dv2 = dr - dp / (ah * ah);
  double t1 = l1 * dv1, t2 = l2 * dv2, t3 = l2 * rh, t5 = l5 * dv5;
  double fc1 = 0.5 * (ql * rl + qr * rr) * nm;
  double fc2 = 0.5 * (ql * rl * ul + pl * nx + qr * rr * ur + pr * nx) * nm;
  double fc3 = 0.5 * (ql * rl * vl + pl * ny + qr * rr * vr + pr * ny) * nm;
  double fc4 = 0.5 * (ql * rl * wl + pl * nz + qr * rr * wr + pr * nz) * nm;
  double fc5 = 0.5 * (ql * rl * Hl + pl * fs + qr * rr * Hr + pr * fs) * nm;
  double fd1 = 0.5 * dissFact * (t1 + t2 + t5) * nm;
  double fd2 = 0.5 * dissFact * (t1 * (uh - nx * ah) + t2 * uh + t3 * (du - nx * dq) + t5 * (uh + nx * ah)) * nm;
  double fd3 = 0.5 * dissFact * (t1 * (vh - ny * ah) + t2 * vh + t3 * (de - ny * dq) + t5 * (vh + ny * ah)) * nm;
  double fd4 = 0.5 * dissFact * (t1 * (wh - nz * ah) + t2 * wh + t3 * (dw - nz * dq) + t5 * (wh + nz * ah)) * nm;
  double fd5 = 0.5 * dissFact *
               (t1 * (Hh - qh * ah) + t2 * sh + t3 * (uh * du + vh * de + wh * dw - qh * dq) + t5 * (Hh + qh * ah)) * nm;
  flx[0] = fc1 - fd1; flx[1] = fc2 - fd2; flx[2] = fc3 - fd3; flx[3] = fc4 - fd4; flx[4] = fc5 - fd5;
}

/* HLLC: RFLU_HLLC_ComputeFlux1_TCP (modflu/RFLU_ModHLLCFlux.F90:926-1194) and
 * ..._Flux2_TCP (:2131-2434).  el, al, Hl as computed by the caller. */
void hllcFlux(orc_ctx *c, double nx, double ny, double nz, double nm, double fs, double rl, double ul, double vl,
              double wl, double pl, double el, double al, double Hl, double rr, double ur, double vr, double wr,
              double pr, double er, double ar, double Hr, double flx[5]) {
  const double g = c->refGamma;
  double ql = ul * nx + vl * ny + wl * nz - fs;
  double qr = ur * nx + vr * ny + wr * nz - fs;
  double wt1 = std::sqrt(rr / rl);
  double wt2 = 1.0 / (1.0 + wt1);
  double us = wt2 * (ul + wt1 * ur);
  double vs = wt2 * (vl + wt1 * vr);
  double ws = wt2 * (wl + wt1 * wr);
  double qs = wt2 * (ql + wt1 * qr);
  double Hs = wt2 * (Hl + wt1 * Hr);
  double Vms = us * us + vs * vs + ws * ws;
  double as = MixtPerf_C_GHoVm2(g, Hs, Vms);
  double sl = fmin2(ql - al, qs - as);
  double sr = fmax2(qr + ar, qs + as);
  if (sl > 0.0) {
    flx[0] = ql * rl * nm;
    flx[1] = (ql * rl * ul + pl * nx) * nm;
    flx[2] = (ql * rl * vl + pl * ny) * nm;
    flx[3] = (ql * rl * wl + pl * nz) * nm;
    flx[4] = (ql * (rl * el + pl) + pl * fs) * nm;
  } else if (sr < 0.0) {
    flx[0] = qr * rr * nm;
    flx[1] = (qr * rr * ur + pr * nx) * nm;
    flx[2] = (qr * rr * vr + pr * ny) * nm;
    flx[3] = (qr * rr * wr + pr * nz) * nm;
    flx[4] = (qr * (rr * er + pr) + pr * fs) * nm;
  } else {
    double sm = (rr * qr * (sr - qr) - rl * ql * (sl - ql) - pr + pl) / (rr * (sr - qr) - rl * (sl - ql));
    double ps = pl + rl * (ql - sl) * (ql - sm);
    double rs, rus, rvs, rws, res;
    if (sm > 0.0) {
      double term = 1.0 / (sl - sm);
      rs = term * (sl - ql) * rl;
      rus = term * ((sl - ql) * rl * ul + (ps - pl) * nx);
      rvs = term * ((sl - ql) * rl * vl + (ps - pl) * ny);
      rws = term * ((sl - ql) * rl * wl + (ps - pl) * nz);
      res = term * ((sl - ql) * rl * el + (ps * sm - pl * ql));
    } else {
      double term = 1.0 / (sr - sm);
      rs = term * (sr - qr) * rr;
      rus = term * ((sr - qr) * rr * ur + (ps - pr) * nx);
      rvs = term * ((sr - qr) * rr * vr + (ps - pr) * ny);
      rws = term * ((sr - qr) * rr * wr + (ps - pr) * nz);
      res = term * ((sr - qr) * rr * er + (ps * sm - pr * qr));
    }
    flx[0] = sm * rs * nm;
    flx[1] = (sm * rus + ps * nx) * nm;
    flx[2] = (sm * rvs + ps * ny) * nm;
    flx[3] = (sm * rws + ps * nz) * nm;
    flx[4] = (sm * (res + ps) - ps * fs) * nm;
  }
}

/* AUSM+: RFLU_AUSM_FluxFunction (modflu/RFLU_ModAUSMFlux.F90:282-416). */
void ausmFlux(double nx, double ny, double nz, double nm, double fs, double rl, double ul, double vl, double wl,
              double pl, double Hl, double al, double rr, double ur, double vr, double wr, double pr, double Hr,
              double ar, double flx[5]) {
  double ql = ul * nx + vl * ny + wl * nz - fs;
  double qr = ur * nx + vr * ny + wr * nz - fs;
  double af = 0.5 * (al + ar);
  double ml = ql / af, mla = std::fabs(ml);
  double mr = qr / af, mra = std::fabs(mr);
  double mlp, wtl, mrm, wtr;
  if (mla <= 1.0) {
    mlp = 0.25 * (ml + 1.0) * (ml + 1.0) + 0.125 * (ml * ml - 1.0) * (ml * ml - 1.0);
    wtl = 0.25 * (ml + 1.0) * (ml + 1.0) * (2.0 - ml) + 0.1875 * ml * (ml * ml - 1.0) * (ml * ml - 1.0);
  } else {
    mlp = 0.5 * (ml + mla);
    wtl = 0.5 * (1.0 + ml / mla);
  }
  if (mra <= 1.0) {
    mrm = -0.25 * (mr - 1.0) * (mr - 1.0) - 0.125 * (mr * mr - 1.0) * (mr * mr - 1.0);
    wtr = 0.25 * (mr - 1.0) * (mr - 1.0) * (2.0 + mr) - 0.1875 * mr * (mr * mr - 1.0) * (mr * mr - 1.0);
  } else {
    mrm = 0.5 * (mr - mra);
    wtr = 0.5 * (1.0 - mr / mra);
  }
  double mf = mlp + mrm, mfa = std::fabs(mf);
  double mfp = 0.5 * (mf + mfa), mfm = 0.5 * (mf - mfa);
  double pf = wtl * pl + wtr * pr;
  flx[0] = (af * (mfp * rl + mfm * rr)) * nm;
  flx[1] = (af * (mfp * rl * ul + mfm * rr * ur) + pf * nx) * nm;
  flx[2] = (af * (mfp * rl * vl + mfm * rr * vr) + pf * ny) * nm;
  flx[3] = (af * (mfp * rl * wl + mfm * rr * wr) + pf * nz) * nm;
  flx[4] = (af * (mfp * rl * Hl + mfm * rr * Hr) + pf * fs) * nm;
}

/* The interior flux of a face from its two sides: first order the cells'
 * conserved (cl, cr) and dependent (dl, dr) variables, second order the
 * reconstructed states L, Rr and the cells' densities (cl[0], cr[0]). */
void sidesFlux(orc_ctx *c, double nx, double ny, double nz, double nm, const double *cl, const double *dl,
               const double *cr, const double *dr, const FaceState &L, const FaceState &Rr, double flx[5]) {
  const double fs = 0.0;
  const double cp = c->refCp, g = c->refGamma;
  const int disc = c->num.spaceDiscr;
  if (c->num.spaceOrder == 1) {
    double rl = cl[0], irl = 1.0 / rl, ul = cl[1] * irl, vl = cl[2] * irl, wl = cl[3] * irl;
    double rr = cr[0], irr = 1.0 / rr, ur = cr[1] * irr, vr = cr[2] * irr, wr = cr[3] * irr;
    double pl = dl[0], pr = dr[0];
    if (disc == 1) {
      double tl = dl[1], tr = dr[1];
      double Hl = MixtPerf_Ho_CpTUVW(cp, tl, ul, vl, wl), Hr = MixtPerf_Ho_CpTUVW(cp, tr, ur, vr, wr);
      roeFlux(c, nx, ny, nz, nm, fs, rl, ul, vl, wl, pl, Hl, rr, ur, vr, wr, pr, Hr, flx);
    } else if (disc == 3) {
      double el = cl[4] * irl, er = cr[4] * irr;
      double al = dl[2], ar = dr[2];
      double Hl = el + irl * pl, Hr = er + irr * pr;
      hllcFlux(c, nx, ny, nz, nm, fs, rl, ul, vl, wl, pl, el, al, Hl, rr, ur, vr, wr, pr, er, ar, Hr, flx);
    } else {
      /* RFLU_AUSM_ComputeFlux1 (RFLU_ModAUSMFlux.F90:550-1027) */
      double al = dl[2], ar = dr[2];
      double Hl = cl[4] * irl + pl / rl, Hr = cr[4] * irr + pr / rr;
      ausmFlux(nx, ny, nz, nm, fs, rl, ul, vl, wl, pl, Hl, al, rr, ur, vr, wr, pr, Hr, ar, flx);
    }
    return;
  }
  if (disc == 1) {
    double gc = MixtPerf_R_CpG(cp, g);
    double tl = MixtPerf_T_DPR(L.r, L.p, gc), Hl = MixtPerf_Ho_CpTUVW(cp, tl, L.u, L.v, L.w);
    double tr = MixtPerf_T_DPR(Rr.r, Rr.p, gc), Hr = MixtPerf_Ho_CpTUVW(cp, tr, Rr.u, Rr.v, Rr.w);
    roeFlux(c, nx, ny, nz, nm, fs, L.r, L.u, L.v, L.w, L.p, Hl, Rr.r, Rr.u, Rr.v, Rr.w, Rr.p, Hr, flx);
  } else if (disc == 3) {
    double irl = 1.0 / cl[0], irr = 1.0 / cr[0];
    double el = MixtPerf_Eo_DGPUVW(L.r, g, L.p, L.u, L.v, L.w), al = MixtPerf_C_DGP(L.r, g, L.p);
    double er = MixtPerf_Eo_DGPUVW(Rr.r, g, Rr.p, Rr.u, Rr.v, Rr.w), ar = MixtPerf_C_DGP(Rr.r, g, Rr.p);
    /* Hl = el + irl*pl with irl the inverse of the cell (unreconstructed) density */
    double Hl = el + irl * L.p, Hr = er + irr * Rr.p;
    hllcFlux(c, nx, ny, nz, nm, fs, L.r, L.u, L.v, L.w, L.p, el, al, Hl, Rr.r, Rr.u, Rr.v, Rr.w, Rr.p, er, ar, Hr,
             flx);
  } else {
    double gc = MixtPerf_R_CpG(cp, g);
    double tl = MixtPerf_T_DPR(L.r, L.p, gc), al = MixtPerf_C_GRT(g, gc, tl);
    double Hl = MixtPerf_Ho_CpTUVW(cp, tl, L.u, L.v, L.w);
    double tr = MixtPerf_T_DPR(Rr.r, Rr.p, gc), ar = MixtPerf_C_GRT(g, gc, tr);
    double Hr = MixtPerf_Ho_CpTUVW(cp, tr, Rr.u, Rr.v, Rr.w);
    ausmFlux(nx, ny, nz, nm, fs, L.r, L.u, L.v, L.w, L.p, Hl, al, Rr.r, Rr.u, Rr.v, Rr.w, Rr.p, Hr, ar, flx);
  }
}

void interiorFlux(orc_ctx *c, int f, double flx[5]) {
  const int c1 = c->f2c[2 * f], c2 = c->f2c[2 * f + 1];
  const double nx = c->fn[4 * f], ny = c->fn[4 * f + 1], nz = c->fn[4 * f + 2], nm = c->fn[4 * f + 3];
  FaceState L{}, Rr{};
  if (c->num.spaceOrder > 1) {
    L = reconstruct(c, c1, c->fc[3 * f], c->fc[3 * f + 1], c->fc[3 * f + 2]);
    Rr = reconstruct(c, c2, c->fc2[3 * f], c->fc2[3 * f + 1], c->fc2[3 * f + 2]);
  }
  sidesFlux(c, nx, ny, nz, nm, &c->cv[5 * c1], &c->dv[3 * c1], &c->cv[5 * c2], &c->dv[3 * c2], L, Rr, flx);
}

/* A face of a symmetry patch: the interior flux between the cell and its
 * reflection across the patch (the reference's virtual cell: momentum
 * reflected, modflu/RFLU_ModRelatedPatches.F90:268-353); second order the
 * reconstructed face state against its own reflection (the virtual cell's
 * reflected gradient reconstructs it at the face). */
void symmetryFlux(orc_ctx *c, const Patch &p, int ip, int i, double flx[5]) {
  const int c1 = p.bf2c[i];
  const double *Q = c->xfQ[c->patchXf[ip]].data();
  const double *cl = &c->cv[5 * c1];
  double cr[5];
  cr[0] = cl[0];
  reflect3(Q, cl + 1, cr + 1);
  cr[4] = cl[4];
  FaceState L{}, Rr{};
  if (c->num.spaceOrder > 1) {
    L = reconstruct(c, c1, p.fc[3 * i], p.fc[3 * i + 1], p.fc[3 * i + 2]);
    const double ul[3] = {L.u, L.v, L.w};
    double ur[3];
    reflect3(Q, ul, ur);
    Rr = {L.r, ur[0], ur[1], ur[2], L.p};
  }
  sidesFlux(c, p.fn[4 * i], p.fn[4 * i + 1], p.fn[4 * i + 2], p.fn[4 * i + 3], cl, &c->dv[3 * c1], cr,
            &c->dv[3 * c1], L, Rr, flx);
}

/* BcondOutflowPerf (libfloflu/BcondOutflowPerf.F90:88-159). */
void bcondOutflowPerf(int bcOpt, double pout, double sxn, double syn, double szn, double cpgas, double mol,
                      double rho, double rhou, double rhov, double rhow, double rhoe, double press, double &rhob,
                      double &rhoub, double &rhovb, double &rhowb, double &rhoeb) {
  double rgas = MixtPerf_R_M(mol);
  double gamma = MixtPerf_G_CpR(cpgas, rgas);
  double u = rhou / rho, v = rhov / rho, w = rhow / rho;
  double csound = MixtPerf_C_DGP(rho, gamma, press);
  double mach = std::sqrt(u * u + v * v + w * w) / csound;
  if (mach < 1.0 && (bcOpt == 1 || bcOpt == 2)) {
    double rrhoc = 1.0 / (rho * csound);
    double deltp = press - pout;
    rhob = rho - deltp / (csound * csound);
    double ub = u + sxn * deltp * rrhoc;
    double vb = v + syn * deltp * rrhoc;
    double wb = w + szn * deltp * rrhoc;
    double vnd = ub * sxn + vb * syn + wb * szn;
    if (vnd < 0.0) {
      ub = std::copysign(1.0, u) * fmax2(std::fabs(ub), std::fabs(u));
      vb = std::copysign(1.0, v) * fmax2(std::fabs(vb), std::fabs(v));
      wb = std::copysign(1.0, w) * fmax2(std::fabs(wb), std::fabs(w));
    }
    rhoub = rhob * ub; rhovb = rhob * vb; rhowb = rhob * wb;
    rhoeb = rhob * MixtPerf_Eo_DGPUVW(rhob, gamma, pout, ub, vb, wb);
  } else {
    rhob = rho; rhoub = rhou; rhovb = rhov; rhowb = rhow; rhoeb = rhoe;
  }
}

/* BcondInflowPerf (libfloflu/BcondInflowPerf.F90), TCPERF gas.  A subsonic
 * patch whose face sees |ql| >= al leaves the outputs unset in the
 * reference; they are NaN here. */
void bcondInflowPerf(int bcOptType, int bcOptFixed, double ptot, double ttot, double betah, double betav,
                     double mach, double sxn, double syn, double szn, double cpgas, double mm, double rl, double rul,
                     double rvl, double rwl, double &rr, double &rur, double &rvr, double &rwr, double &rer,
                     double &pr) {
  const double rgas = MixtPerf_R_M(mm);
  const double g = MixtPerf_G_CpR(cpgas, rgas);
  auto supersonic = [&]() {
    pr = ptot / std::pow(1.0 + 0.5 * (g - 1.0) * mach * mach, g / (g - 1.0)); /* MixtPerf_P_GMaPo */
    double tr = ttot / (1.0 + 0.5 * (g - 1.0) * mach * mach);                 /* MixtPerf_T_GMaTo */
    rr = pr / (rgas * tr);                                                    /* MixtPerf_D_PRT */
    double ar = std::sqrt(g * rgas * tr);                                     /* MixtPerf_C_GRT */
    double ur = mach * ar * std::cos(betah) * std::cos(betav);
    double vr = mach * ar * std::sin(betah);
    double wr = mach * ar * std::cos(betah) * std::sin(betav);
    rer = rr * MixtPerf_Eo_DGPUVW(rr, g, pr, ur, vr, wr);
    rur = rr * ur;
    rvr = rr * vr;
    rwr = rr * wr;
  };
  if (bcOptType == 1 || bcOptType == 2) { /* BCOPT_SUBSONIC, BCOPT_MIXED */
    double gm1 = g - 1.0;
    double ul = rul / rl, vl = rvl / rl, wl = rwl / rl;
    double a02 = g * rgas * ttot;                                             /* MixtPerf_C2_GRT */
    double al = std::sqrt(a02 - 0.5 * (g - 1.0) * (ul * ul + vl * vl + wl * wl)); /* MixtPerf_C_Co2GUVW */
    double ql = ul * sxn + vl * syn + wl * szn;
    if (std::fabs(ql) < al) {
      double sl = std::sqrt(ul * ul + vl * vl + wl * wl);
      double eta;
      if (bcOptFixed == 0) /* BCOPT_FIXED_NO */
        eta = (sl > 1.0e-6) ? ql / sl : -1.0;
      else
        eta = -1.0;
      double Rm = al - 0.5 * gm1 * ql;
      double disc = 0.5 * gm1 * (eta * eta) * (a02 / (Rm * Rm) * (1.0 + 0.5 * gm1 * (eta * eta)) - 1.0);
      double ar, tr, sr;
      if (disc < 0.0) {
        ar = std::sqrt(a02);
        tr = ttot;
        pr = ptot;
        sr = 0.0;
      } else {
        ar = Rm / (1.0 + 0.5 * gm1 * eta * eta) * (1.0 + std::sqrt(disc));
        tr = ar * ar / (g * rgas);                                           /* MixtPerf_T_CGR */
        pr = ptot * std::pow(tr / ttot, g / (g - 1.0));                      /* MixtPerf_P_GPoTTo */
        double c2 = ar * ar;                                                 /* MixtPerf_Vm_C2Co2G */
        sr = (a02 > c2) ? std::sqrt(2.0 / (g - 1.0) * (a02 - c2)) : 0.0;
      }
      rr = pr / (rgas * tr);
      double ur = sr * std::cos(betah) * std::cos(betav);
      double vr = sr * std::sin(betah);
      double wr = sr * std::cos(betah) * std::sin(betav);
      rer = rr * (pr / (rr * (g - 1.0)) + 0.5 * sr * sr);                   /* MixtPerf_Eo_DGPVm */
      rur = rr * ur;
      rvr = rr * vr;
      rwr = rr * wr;
    } else if (bcOptType == 2) {
      supersonic();
    } else {
      rr = rur = rvr = rwr = rer = pr = std::nan("");
    }
  } else {
    supersonic();
  }
}

/* RFLU_SetRindStateFarfieldPerf, corrFlag false
 * (modflu/RFLU_ModRindStates.F90:248-420). */
void rindStateFarfieldPerf(double cpGas, double mmGas, double nx, double ny, double nz, double machInf, double pInf,
                           double tInf, double alphaInf, double betaInf, double rl, double rul, double rvl,
                           double rwl, double rel, double &rr, double &rur, double &rvr, double &rwr, double &rer,
                           double &pr) {
  double rGas = MixtPerf_R_M(mmGas);
  double gGas = MixtPerf_G_CpR(cpGas, rGas);
  double ul = rul / rl, vl = rvl / rl, wl = rwl / rl;
  double ql = ul * nx + vl * ny + wl * nz;
  double el = rel / rl;
  double sl2 = ul * ul + vl * vl + wl * wl;
  double pl = MixtPerf_P_DEoGVm2(rl, el, gGas, sl2);
  double ri = pInf / (rGas * tInf); /* MixtPerf_D_PRT */
  double pi = pInf;
  double qi = machInf * MixtPerf_C_GRT(gGas, rGas, tInf);
  double ui = qi * std::cos(alphaInf) * std::cos(betaInf);
  double vi = qi * std::sin(alphaInf) * std::cos(betaInf);
  double wi = qi * std::sin(betaInf);
  if (machInf < 1.0) {
    double al = MixtPerf_C_DGP(rl, gGas, pl);
    double pb, rb, ub, vb, wb;
    if (ql < 0.0) {
      pb = 0.5 * (pi + pl - rl * al * ((ui - ul) * nx + (vi - vl) * ny + (wi - wl) * nz));
      rb = ri - (pi - pb) / (al * al);
      ub = ui - nx * (pi - pb) / (rl * al);
      vb = vi - ny * (pi - pb) / (rl * al);
      wb = wi - nz * (pi - pb) / (rl * al);
    } else {
      pb = pi;
      rb = rl - (pl - pi) / (al * al);
      ub = ul + nx * (pl - pi) / (rl * al);
      vb = vl + ny * (pl - pi) / (rl * al);
      wb = wl + nz * (pl - pi) / (rl * al);
    }
    rr = rb;
    rur = rb * ub;
    rvr = rb * vb;
    rwr = rb * wb;
    rer = rb * MixtPerf_Eo_DGPUVW(rb, gGas, pb, ub, vb, wb);
    pr = pb;
  } else if (ql < 0.0) {
    rr = ri;
    rur = ri * ui;
    rvr = ri * vi;
    rwr = ri * wi;
    rer = ri * (pi / (ri * (gGas - 1.0)) + 0.5 * qi * qi); /* MixtPerf_Eo_DGPVm */
    pr = pi;
  } else {
    rr = rl; rur = rul; rvr = rvl; rwr = rwl; rer = rel; pr = pl;
  }
}

/* RFLU_SetRindStateSlipWallPerf, fs = 0 (modflu/RFLU_ModRindStates.F90:
 * 535-584): returns the modified pl. */
double rindStateSlipWallPerf(double cpGas, double mmGas, double nx, double ny, double nz, double rl, double rul,
                             double rvl, double rwl, double pl) {
  double rGas = MixtPerf_R_M(mmGas);
  double gGas = MixtPerf_G_CpR(cpGas, rGas);
  double irl = 1.0 / rl;
  double ul = irl * rul, vl = irl * rvl, wl = irl * rwl;
  double ql = ul * nx + vl * ny + wl * nz - 0.0;
  double al = MixtPerf_C_DGP(rl, gGas, pl);
  if (ql < 0.0) {
    double term = 1.0 + 0.5 * (gGas - 1.0) * ql / al;
    return pl * std::pow(term, 2.0 * gGas / (gGas - 1.0));
  }
  double term = (gGas + 1.0) / 4.0;
  return pl + term * rl * ql * (ql + std::sqrt(al * al + term * term * ql * ql) / term);
}

/* The central boundary flux of the inflow/outflow/farfield cases
 * (rocflu/RFLU_CentralFirstPatch.F90:281-287), fs = 0. */
void centralBoundaryFlux(double nx, double ny, double nz, double nm, double rl, double rul, double rvl, double rwl,
                         double rel, double pl, double rr, double rur, double rvr, double rwr, double rer, double pr,
                         double flx[5]) {
  const double fs = 0.0;
  double ql = (rul * nx + rvl * ny + rwl * nz) / rl - fs;
  double qr = (rur * nx + rvr * ny + rwr * nz) / rr - fs;
  flx[0] = 0.5 * (ql * rl + qr * rr) * nm;
  flx[1] = 0.5 * (ql * rul + pl * nx + qr * rur + pr * nx) * nm;
  flx[2] = 0.5 * (ql * rvl + pl * ny + qr * rvr + pr * ny) * nm;
  flx[3] = 0.5 * (ql * rwl + pl * nz + qr * rwr + pr * nz) * nm;
  flx[4] = 0.5 * (ql * (rel + pl) + pl * fs + qr * (rer + pr) + pr * fs) * nm;
}

/* Injection (RFLU_CentralFirstPatch.F90:1043-1127 and
 * RFLU_CentralSecondPatch.F90:1229-1343 with RFLU_SetRindStateInjectPerf,
 * RFLU_ModRindStates.F90:459-501), fs = fsu = 0. */
void injectionFlux(const orc_ctx *c, const Patch &p, double nx, double ny, double nz, double nm, double rl,
                   double rul, double rvl, double rwl, double pl, double flx[5]);

/* The inflow, farfield and injection cases of the two patch routines, from
 * the interior state (rl, rul, rvl, rwl, rel, pl): cv and dv at first
 * order, the reconstructed face state at second. */
void remainingPatchFlux(const orc_ctx *c, const Patch &p, double nx, double ny, double nz, double nm, double rl,
                        double rul, double rvl, double rwl, double rel, double pl, double flx[5]);

/* Patch flux of one boundary face: RFLU_CentralFirstPatch
 * (rocflu/RFLU_CentralFirstPatch.F90:222-1146) and RFLU_CentralSecondPatch
 * (rocflu/RFLU_CentralSecondPatch.F90:233-1360): inflow (TOTANG, VELTEMP),
 * outflow, slip and no-slip walls, farfield (no vortex correction) and
 * injection, TCPERF gas, static grid. */
void patchFlux(orc_ctx *c, const Patch &p, int i, double flx[5]) {
  if (p.bcType == ORC_BC_SYMMETRY) {
    symmetryFlux(c, p, (int)(&p - c->patches.data()), i, flx);
    return;
  }
  const int c1 = p.bf2c[i];
  const double nx = p.fn[4 * i], ny = p.fn[4 * i + 1], nz = p.fn[4 * i + 2], nm = p.fn[4 * i + 3];
  const double fs = 0.0;
  const double *cv = &c->cv[5 * c1];
  flx[0] = 0.0;
  const bool wall = p.bcType == ORC_BC_SLIPWALL || p.bcType == ORC_BC_NOSLIPWALL_HFLUX ||
                    p.bcType == ORC_BC_NOSLIPWALL_TEMP;
  if (p.order == 1) {
    double rl = cv[0], rul = cv[1], rvl = cv[2], rwl = cv[3], rel = cv[4], pl = c->dv[3 * c1];
    if (wall) {
      flx[1] = pl * nx * nm; flx[2] = pl * ny * nm; flx[3] = pl * nz * nm; flx[4] = pl * fs * nm;
      return;
    }
    if (p.bcType != ORC_BC_OUTFLOW) {
      remainingPatchFlux(c, p, nx, ny, nz, nm, rl, rul, rvl, rwl, rel, pl, flx);
      return;
    }
    double pr = (p.outflowType != 0) ? p.pOut : pl;
    double rr, rur, rvr, rwr, rer;
    bcondOutflowPerf(p.outflowType, pr, nx, ny, nz, c->gvCp, c->gvMol, rl, rul, rvl, rwl, rel, pl, rr, rur, rvr,
                     rwr, rer);
    double ql = (rul * nx + rvl * ny + rwl * nz) / rl - fs;
    double qr = (rur * nx + rvr * ny + rwr * nz) / rr - fs;
    flx[0] = 0.5 * (ql * rl + qr * rr) * nm;
    flx[1] = 0.5 * (ql * rul + pl * nx + qr * rur + pr * nx) * nm;
    flx[2] = 0.5 * (ql * rvl + pl * ny + qr * rvr + pr * ny) * nm;
    flx[3] = 0.5 * (ql * rwl + pl * nz + qr * rwr + pr * nz) * nm;
    flx[4] = 0.5 * (ql * (rel + pl) + pl * fs + qr * (rer + pr) + pr * fs) * nm;
    return;
  }
  const double xc = p.fc[3 * i], yc = p.fc[3 * i + 1], zc = p.fc[3 * i + 2];
  FaceState L = reconstruct(c, c1, xc, yc, zc);
  double rl = L.r, ul = L.u, vl = L.v, wl = L.w, pl = L.p;
  double rul = rl * ul, rvl = rl * vl, rwl = rl * wl;
  if (wall) {
    flx[1] = pl * nx * nm; flx[2] = pl * ny * nm; flx[3] = pl * nz * nm; flx[4] = pl * fs * nm;
    return;
  }
  if (p.bcType == ORC_BC_INJECTION) {
    injectionFlux(c, p, nx, ny, nz, nm, rl, rul, rvl, rwl, pl, flx);
    return;
  }
  double pr = (p.outflowType != 0) ? p.pOut : pl;
  double rgas = MixtPerf_R_M(c->gvMol), g = MixtPerf_G_CpR(c->gvCp, rgas);
  double rel = rl * MixtPerf_Eo_DGPUVW(rl, g, pl, ul, vl, wl);
  if (p.bcType != ORC_BC_OUTFLOW) {
    remainingPatchFlux(c, p, nx, ny, nz, nm, rl, rul, rvl, rwl, rel, pl, flx);
    return;
  }
  double rr, rur, rvr, rwr, rer;
  bcondOutflowPerf(p.outflowType, pr, nx, ny, nz, c->gvCp, c->gvMol, rl, rul, rvl, rwl, rel, pl, rr, rur, rvr, rwr,
                   rer);
  double ql = (rul * nx + rvl * ny + rwl * nz) / rl - fs;
  double qr = (rur * nx + rvr * ny + rwr * nz) / rr - fs;
  flx[0] = 0.5 * (ql * rl + qr * rr) * nm;
  flx[1] = 0.5 * (ql * rul + pl * nx + qr * rur + pr * nx) * nm;
  flx[2] = 0.5 * (ql * rvl + pl * ny + qr * rvr + pr * ny) * nm;
  flx[3] = 0.5 * (ql * rwl + pl * nz + qr * rwr + pr * nz) * nm;
  flx[4] = 0.5 * (ql * (rel + pl) + pl * fs + qr * (rer + pr) + pr * fs) * nm;
}

void injectionFlux(const orc_ctx *c, const Patch &p, double nx, double ny, double nz, double nm, double rl,
                   double rul, double rvl, double rwl, double pl, double flx[5]) {
  const double fs = 0.0;
  const double minj = p.vals[0]; /* BCDAT_INJECT_MFRATE */
  if (minj > 0.0) {
    const double tinj = p.vals[1]; /* BCDAT_INJECT_TEMP */
    double rGas = MixtPerf_R_M(c->gvMol);
    double rb = pl / (rGas * tinj); /* MixtPerf_D_PRT */
    double qb = -minj / rb + fs;
    double ub = qb * nx, vb = qb * ny, wb = qb * nz;
    double hb = MixtPerf_Ho_CpTUVW(c->gvCp, tinj, ub, vb, wb);
    flx[0] = -minj * nm;
    flx[1] = (-minj * ub + pl * nx) * nm;
    flx[2] = (-minj * vb + pl * ny) * nm;
    flx[3] = (-minj * wb + pl * nz) * nm;
    flx[4] = (-minj * hb + pl * fs) * nm;
  } else {
    double pw = rindStateSlipWallPerf(c->gvCp, c->gvMol, nx, ny, nz, rl, rul, rvl, rwl, pl);
    flx[0] = 0.0;
    flx[1] = pw * nx * nm;
    flx[2] = pw * ny * nm;
    flx[3] = pw * nz * nm;
    flx[4] = pw * fs * nm;
  }
}

void remainingPatchFlux(const orc_ctx *c, const Patch &p, double nx, double ny, double nz, double nm, double rl,
                        double rul, double rvl, double rwl, double rel, double pl, double flx[5]) {
  if (p.bcType == ORC_BC_INJECTION) {
    injectionFlux(c, p, nx, ny, nz, nm, rl, rul, rvl, rwl, pl, flx);
    return;
  }
  double rr, rur, rvr, rwr, rer, pr;
  const double *v = p.vals;
  if (p.bcType == ORC_BC_FARFIELD) {
    rindStateFarfieldPerf(c->gvCp, c->gvMol, nx, ny, nz, v[0], v[3], v[4], v[1], v[2], rl, rul, rvl, rwl, rel, rr,
                          rur, rvr, rwr, rer, pr);
  } else if (p.bcType == ORC_BC_INFLOW_TOTANG) {
    const double mach = (p.sw[0] != 1) ? v[4] : 0.0; /* BCDAT_INFLOW_MACH unless subsonic */
    bcondInflowPerf(p.sw[0], p.sw[1], v[0], v[1], v[2], v[3], mach, nx, ny, nz, c->gvCp, c->gvMol, rl, rul, rvl,
                    rwl, rr, rur, rvr, rwr, rer, pr);
  } else { /* ORC_BC_INFLOW_VELTEMP (RFLU_CentralFirstPatch.F90:375-570) */
    const double ur = v[0], vr = v[1], wr = v[2], tr = v[3];
    double rgas = MixtPerf_R_M(c->gvMol);
    double g = MixtPerf_G_CpR(c->gvCp, rgas);
    if (p.sw[0] != 1) {
      pr = v[4];
      rr = pr / (rgas * tr); /* MixtPerf_D_PRT */
    } else {
      rr = rl;
      pr = rr * rgas * tr; /* MixtPerf_P_DRT */
    }
    rer = rr * MixtPerf_Eo_DGPUVW(rr, g, pr, ur, vr, wr);
    rur = rr * ur;
    rvr = rr * vr;
    rwr = rr * wr;
  }
  centralBoundaryFlux(nx, ny, nz, nm, rl, rul, rvl, rwl, rel, pl, rr, rur, rvr, rwr, rer, pr, flx);
}

/* ConvectiveFluxes (libfloflu/ConvectiveFluxes.F90:120-175): rhs = -diss,
 * interior face loop with the +/- scatter (rhs(c1) += F, rhs(c2) -= F), then
 * the patch loop (slip walls leave rhs(DENS)).  The face fluxes are formed
 * first; each cell then adds its faces' contributions in the loops' order. */
void convectiveFluxes(orc_ctx *c) {
  const int nc = c->nCells, nf = c->nFaces, nb = (int)c->bPatch.size();
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) interiorFlux(c, f, &c->flux[5 * (size_t)f]);
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nb; ++b)
    patchFlux(c, c->patches[c->bPatch[b]], c->bFace[b], &c->flux[5 * ((size_t)nf + b)]);
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    double *rhs = &c->rhs[5 * ic];
    for (int k = 0; k < 5; ++k) rhs[k] = -c->diss[5 * ic + k];
    for (int e = c->cfOff[ic]; e < c->cfOff[ic + 1]; ++e) {
      const int code = c->cfEnt[e];
      if (code >= 0) {
        const double *flx = &c->flux[5 * (size_t)(code >> 1)];
        if (code & 1)
          for (int k = 0; k < 5; ++k) rhs[k] = rhs[k] - flx[k];
        else
          for (int k = 0; k < 5; ++k) rhs[k] = rhs[k] + flx[k];
      } else {
        const int b = -code - 1;
        const double *flx = &c->flux[5 * ((size_t)nf + b)];
        const int bt = c->patches[c->bPatch[b]].bcType;
        const int k0 = (bt == ORC_BC_SLIPWALL || bt == ORC_BC_NOSLIPWALL_HFLUX || bt == ORC_BC_NOSLIPWALL_TEMP) ? 1 : 0;
        for (int k = k0; k < 5; ++k) rhs[k] = rhs[k] + flx[k];
      }
    }
  }
}

/* RkInitGeneric (libfloflu/RkInitGeneric.F90:120-170). */
void rkInit(orc_ctx *c, int iStage) {
  const int n = 5 * c->nCells;
  if (c->num.rkScheme == 1 && iStage != 1) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k) c->diss[k] = 0.0;
  } else {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k) { c->cvOld[k] = c->cv[k]; c->diss[k] = 0.0; }
  }
}

/* RkUpdateGeneric, static grid (libfloflu/RkUpdateGeneric.F90:257-322). */
void rkUpdate(orc_ctx *c, int iStage, double dtMin) {
  const double fac = c->ark[iStage - 1] * dtMin;
  const double grk = c->grk[iStage - 1];
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < c->nCells; ++ic) {
    double adtv = fac / c->vol[ic];
    for (int iv = 0; iv < 5; ++iv) {
      int k = 5 * ic + iv;
      switch (c->num.rkScheme) {
      case 1:
        if (iStage == 1) { c->cv[k] = c->cvOld[k] - adtv * c->rhs[k]; c->rhsSum[k] = c->rhs[k]; }
        else if (iStage == c->nrkSteps) c->cv[k] = c->cvOld[k] - adtv * (c->rhs[k] + c->rhsSum[k]);
        else { c->cv[k] = c->cvOld[k] - adtv * c->rhs[k]; c->rhsSum[k] = c->rhsSum[k] + grk * c->rhs[k]; }
        break;
      case 2:
        if (iStage == 1) { c->cv[k] = c->cvOld[k] - adtv * c->rhs[k]; c->rhsSum[k] = c->rhs[k]; }
        else if (iStage == 2) {
          c->cv[k] = c->cvOld[k] - adtv * (c->rhs[k] - grk * c->rhsSum[k]);
          c->rhsSum[k] = c->rhs[k];
        } else c->cv[k] = c->cvOld[k] - adtv * (c->rhs[k] - grk * c->rhsSum[k]);
        break;
      default: c->cv[k] = c->cvOld[k] - adtv * c->rhs[k];
      }
    }
  }
}

/* AfterUpdateMP (libfloflu/AfterUpdateMP.F90:134-136): RFLU_CheckValidity
 * (libflu/RFLU_CheckValidity.F90:165-214), RFLU_EnforceBounds
 * (libflu/RFLU_EnforceBounds.F90:165-230), RFLU_CheckPositivity
 * (libflu/RFLU_CheckPositivity.F90:173-193). */
void afterUpdate(orc_ctx *c) {
  const int nc = c->nCells;
  long long nNan = 0, nNegP = 0, nPosFix = 0;
#pragma omp parallel for schedule(static) reduction(+ : nNan)
  for (int ic = 0; ic < nc; ++ic) {
    const double *cv = &c->cv[5 * ic];
    double rho = cv[0], rrho = 1.0 / rho;
    double u = rrho * cv[1], v = rrho * cv[2], w = rrho * cv[3];
    double p = c->dv[3 * ic], t = c->dv[3 * ic + 1];
    if (std::isnan(rho) || std::isnan(u) || std::isnan(v) || std::isnan(w) || std::isnan(p) || std::isnan(t))
      nNan++;
  }
  const double pTol = 1.0e-12;
  double rgas = MixtPerf_R_M(c->gvMol), gamma = MixtPerf_G_CpR(c->gvCp, rgas);
#pragma omp parallel for schedule(static) reduction(+ : nNegP)
  for (int ic = 0; ic < nc; ++ic) {
    double *cv = &c->cv[5 * ic];
    double r = cv[0], ir = 1.0 / r;
    double u = ir * cv[1], v = ir * cv[2], w = ir * cv[3];
    double Eo = ir * cv[4];
    double Vm2 = u * u + v * v + w * w;
    double p = MixtPerf_P_DEoGVm2(r, Eo, gamma, Vm2);
    if (p <= 0.0 && std::fabs(p) <= pTol) {
      nNegP++;
      p = pTol;
      cv[4] = r * MixtPerf_Eo_DGPUVW(r, gamma, p, u, v, w);
    }
  }
#pragma omp parallel for schedule(static) reduction(+ : nPosFix)
  for (int ic = 0; ic < nc; ++ic) {
    double *cv = &c->cv[5 * ic];
    double rho = cv[0], rrho = 1.0 / rho;
    double u = rrho * cv[1], v = rrho * cv[2], w = rrho * cv[3];
    double Vm2 = u * u + v * v + w * w;
    double p = c->dv[3 * ic];
    if (p <= 0.0) {
      nPosFix++;
      double Eo = 1.0e4 + 0.5 * Vm2;
      cv[4] = rho * Eo;
      setDependentVars(c, ic);
    }
  }
  c->nanCount += nNan;
  c->negPCount += nNegP;
  c->posFixCount += nPosFix;
}

/* RKUpdateMP, RFLU_SetVarsContWrapper, AfterUpdateMP (RungeKuttaMP.F90:328-372). */
void updateStage(orc_ctx *c, int iStage, double dtMin) {
  rkUpdate(c, iStage, dtMin);
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < c->nCells; ++ic) setDependentVars(c, ic);
  afterUpdate(c);
}

void rkStage(orc_ctx *c, int iStage, double dtMin) {
  rkInit(c, iStage);
  cellGradients(c);
  convectiveFluxes(c);
  updateStage(c, iStage, dtMin);
}

/* RFLU_TimeStepInviscid (rocflu/RFLU_TimeStepInviscid.F90:120-333) and
 * RFLU_MinimumTimeStep (rocflu/RFLU_MinimumTimeStep.F90:100-245), one region. */
double timeStep(orc_ctx *c, double currentTime) {
  const int nc = c->nCells, nf = c->nFaces;
  std::vector<double> dt(nc, 0.0), srad(nf);
  /* the interior faces' spectral radius, added to both cells (c1, then c2
     in the reference's loop), then each patch face's to its cell */
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    int c1 = c->f2c[2 * f], c2 = c->f2c[2 * f + 1];
    double nx = c->fn[4 * f], ny = c->fn[4 * f + 1], nz = c->fn[4 * f + 2], nm = c->fn[4 * f + 3];
    double fsu = 0.0;
    double ir1 = 1.0 / c->cv[5 * c1], ir2 = 1.0 / c->cv[5 * c2];
    double u1 = c->cv[5 * c1 + 1] * ir1, v1 = c->cv[5 * c1 + 2] * ir1, w1 = c->cv[5 * c1 + 3] * ir1;
    double a1 = c->dv[3 * c1 + 2];
    double u2 = c->cv[5 * c2 + 1] * ir2, v2 = c->cv[5 * c2 + 2] * ir2, w2 = c->cv[5 * c2 + 3] * ir2;
    double a2 = c->dv[3 * c2 + 2];
    double vc = 0.5 * ((u1 + u2) * nx + (v1 + v2) * ny + (w1 + w2) * nz);
    double as = 0.5 * (a1 + a2);
    srad[f] = (std::fabs(vc - fsu) + as) * nm;
  }
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < nc; ++ic) {
    for (int e = c->cfOff[ic]; e < c->cfOff[ic + 1]; ++e) {
      const int code = c->cfEnt[e];
      if (code >= 0) {
        dt[ic] = dt[ic] + srad[code >> 1];
        continue;
      }
      const int b = -code - 1;
      const Patch &p = c->patches[c->bPatch[b]];
      const int i = c->bFace[b], c1 = ic;
      double nx = p.fn[4 * i], ny = p.fn[4 * i + 1], nz = p.fn[4 * i + 2], nm = p.fn[4 * i + 3];
      double fsu = 0.0;
      double ir1 = 1.0 / c->cv[5 * c1];
      double u1 = c->cv[5 * c1 + 1] * ir1, v1 = c->cv[5 * c1 + 2] * ir1, w1 = c->cv[5 * c1 + 3] * ir1;
      double a1 = c->dv[3 * c1 + 2];
      if (p.bcType == ORC_BC_SYMMETRY) {
        /* an interior face to the cell's reflection (momentum reflected) */
        double m2[3];
        reflect3(c->xfQ[c->patchXf[c->bPatch[b]]].data(), &c->cv[5 * c1 + 1], m2);
        double u2 = m2[0] * ir1, v2 = m2[1] * ir1, w2 = m2[2] * ir1;
        double vc = 0.5 * ((u1 + u2) * nx + (v1 + v2) * ny + (w1 + w2) * nz);
        double as = 0.5 * (a1 + a1);
        dt[c1] = dt[c1] + (std::fabs(vc - fsu) + as) * nm;
        continue;
      }
      double vc = u1 * nx + v1 * ny + w1 * nz;
      dt[c1] = dt[c1] + (std::fabs(vc - fsu) + a1) * nm;
    }
    dt[ic] = c->vol[ic] / dt[ic];
  }
  double dtMin = 1.79769313486231571e308;
  for (int ic = 0; ic < nc; ++ic) dtMin = fmin2(dtMin, dt[ic]);
  /* RFLU_MinimumTimeStep */
  double cfl = c->num.cfl;
  if (c->num.rkScheme == 1) cfl = fmin2(cfl, 3.0);
  else if (c->num.rkScheme == 2) cfl = fmin2(cfl, 2.0);
  else cfl = fmin2(cfl, 1.0);
  dtMin = cfl * dtMin;
  double wtI = 0.0, wtC = 0.0;
  if (currentTime <= 1.0e-8) wtI = 1.0; else wtC = 1.0;
  dtMin = wtI / c->num.dtImposed + wtC / dtMin;
  dtMin = 1.0 / dtMin;
  if (dtMin <= 0.0) dtMin = 6.0e-12;
  dtMin = fmax2(dtMin, c->num.dtMinLimit);
  return dtMin;
}

} // namespace

extern "C" {

orc_ctx *orc_create(const orc_mesh_desc *m, const orc_num_desc *num) {
  orc_ctx *c = new orc_ctx();
  c->nVert = m->nVert;
  c->nCells = m->nCells;
  c->nvc = m->nVertPerCell;
  c->xyz.assign(m->xyz, m->xyz + 3 * m->nVert);
  c->c2v.assign(m->c2v, m->c2v + c->nvc * m->nCells);
  for (int ip = 0; ip < m->nPatches; ++ip) {
    Patch p;
    p.bcType = m->patchBcType[ip];
    p.outflowType = m->patchOutflowType[ip];
    p.pOut = m->patchPout[ip];
    p.order = m->patchOrder[ip];
    p.related = m->patchRelated ? m->patchRelated[ip] : -1;
    if (m->patchVals)
      for (int k = 0; k < ORC_BCDAT_N; ++k) p.vals[k] = m->patchVals[ORC_BCDAT_N * ip + k];
    if (m->patchSwitches)
      for (int k = 0; k < ORC_BCSWI_N; ++k) p.sw[k] = m->patchSwitches[ORC_BCSWI_N * ip + k];
    int b = m->patchFaceOff[ip], e = m->patchFaceOff[ip + 1];
    p.n = e - b;
    p.bf2v.assign(m->bf2v + 4 * b, m->bf2v + 4 * e);
    c->patches.push_back(p);
  }
  c->num = *num;
  c->c2vGeo = c->c2v;
  bool periodic = false;
  for (const Patch &p : c->patches) periodic = periodic || p.bcType == ORC_BC_PERIODIC;
  if (periodic) identifyPeriodicVertices(c);
  buildFaceList(c);
  buildCellFaces(c);
  buildGeometry(c);
  c->nVertExt = c->nVert;
  bool symmetry = false;
  for (const Patch &p : c->patches) symmetry = symmetry || (p.bcType == ORC_BC_SYMMETRY && p.n > 0);
  if (symmetry && periodic) {
    std::fprintf(stderr, "oracle: symmetry and periodic patches in one mesh\n");
    std::abort();
  }
  if (symmetry && num->cReconstCells == 1 && num->spaceOrder > 1)
    for (const Patch &p : c->patches)
      if (wallOrInjection(p.bcType) && p.n > 0) {
        std::fprintf(stderr, "oracle: constrained gradients (CRECONSTC 1) with symmetry patches\n");
        std::abort();
      }
  if (symmetry) buildSymmetryImages(c);
  if (num->spaceOrder > 1) {
    buildStencils(c);
    buildMoments(c);
  } else {
    c->stOff.assign(c->nCells + 1, 0);
  }
  buildBFaceStencil(c);
  /* RFLU_DerivedInputValues (libflu/RFLU_DerivedInputValues.F90:309-410) */
  for (int k = 0; k < 5; ++k) c->ark[k] = c->grk[k] = 0.0;
  if (num->rkScheme == 1) {
    c->nrkSteps = 4;
    c->ark[0] = 0.5; c->ark[1] = 0.5; c->ark[2] = 1.0; c->ark[3] = 1.0 / 6.0;
    c->grk[0] = 1.0; c->grk[1] = 2.0; c->grk[2] = 2.0; c->grk[3] = 1.0;
  } else if (num->rkScheme == 2) {
    c->nrkSteps = 3;
    c->ark[0] = 8.0 / 15.0; c->ark[1] = 5.0 / 12.0; c->ark[2] = 0.75;
    c->grk[0] = 0.0; c->grk[1] = 17.0 / 25.0; c->grk[2] = 5.0 / 9.0;
  } else {
    c->nrkSteps = 1;
    c->ark[0] = 1.0; c->grk[0] = 1.0;
  }
  c->refCp = num->cp;
  c->refGamma = num->gamma;
  c->gvMol = MixtPerf_M_R(MixtPerf_R_CpG(num->cp, num->gamma));
  c->gvCp = num->cp;
  const size_t n5 = 5 * (size_t)c->nCells;
  c->cv.assign(n5, 0.0); c->cvOld.assign(n5, 0.0); c->rhs.assign(n5, 0.0);
  c->rhsSum.assign(n5, 0.0); c->diss.assign(n5, 0.0); c->lim.assign(n5, 1.0);
  c->dv.assign(3 * (size_t)c->nCells, 0.0);
  c->grad.assign(15 * (size_t)c->nCells, 0.0);
  return c;
}

void orc_destroy(orc_ctx *c) { delete c; }
int orc_nfaces(orc_ctx *c) { return c->nFaces; }
int orc_patch_nfaces(orc_ctx *c, int ip) { return c->patches[ip].n; }
int orc_stencil_nnz(orc_ctx *c) { return c->stOff[c->nCells]; }
void orc_get_bface_stencil(orc_ctx *c, int *off, int *faces) {
  if (off) std::memcpy(off, c->bfOff.data(), sizeof(int) * (c->nCells + 1));
  if (faces && !c->bfIdx.empty()) std::memcpy(faces, c->bfIdx.data(), sizeof(int) * c->bfIdx.size());
}
int orc_nstages(orc_ctx *c) { return c->nrkSteps; }

void orc_get_faces(orc_ctx *c, int *f2c, int *f2v, double *fn, double *fc) {
  if (f2c) std::memcpy(f2c, c->f2c.data(), sizeof(int) * 2 * c->nFaces);
  if (f2v) std::memcpy(f2v, c->f2v.data(), sizeof(int) * 4 * c->nFaces);
  if (fn) std::memcpy(fn, c->fn.data(), sizeof(double) * 4 * c->nFaces);
  if (fc) std::memcpy(fc, c->fc.data(), sizeof(double) * 3 * c->nFaces);
}
void orc_get_cells(orc_ctx *c, double *vol, double *cofg) {
  if (vol) std::memcpy(vol, c->vol.data(), sizeof(double) * c->nCells);
  if (cofg) std::memcpy(cofg, c->cofg.data(), sizeof(double) * 3 * c->nCells);
}
void orc_get_patch(orc_ctx *c, int ip, int *bf2c, double *fn, double *fc) {
  const Patch &p = c->patches[ip];
  if (bf2c) std::memcpy(bf2c, p.bf2c.data(), sizeof(int) * p.n);
  if (fn) std::memcpy(fn, p.fn.data(), sizeof(double) * 4 * p.n);
  if (fc) std::memcpy(fc, p.fc.data(), sizeof(double) * 3 * p.n);
}
void orc_get_periodic(orc_ctx *c, double *fc2, double *stShift) {
  if (fc2) std::memcpy(fc2, c->fc2.data(), sizeof(double) * 3 * c->nFaces);
  if (stShift)
    for (int i = 0; i < c->nCells; ++i)
      for (int s = c->stOff[i]; s < c->stOff[i + 1]; ++s) {
        const int j = c->stIdx[s];
        double dx, dy, dz;
        memberOffset(c, i, j, dx, dy, dz);
        /* the translation of the member's image, exactly as applied */
        const double px = c->cofg[3 * j] - c->cofg[3 * i], py = c->cofg[3 * j + 1] - c->cofg[3 * i + 1],
                     pz = c->cofg[3 * j + 2] - c->cofg[3 * i + 2];
        stShift[3 * s] = (dx == px) ? 0.0 : dx - px;
        stShift[3 * s + 1] = (dy == py) ? 0.0 : dy - py;
        stShift[3 * s + 2] = (dz == pz) ? 0.0 : dz - pz;
      }
}
int orc_n_reflections(orc_ctx *c) { return (int)c->xfQ.size(); }
void orc_get_symmetry(orc_ctx *c, int *stXf, double *stShift, double *xfQ) {
  const int nc = c->nCells;
  for (int s = 0; s < c->stOff[nc]; ++s) {
    const int j = c->stIdx[s];
    if (j < nc) {
      stXf[s] = -1;
      stShift[3 * s] = stShift[3 * s + 1] = stShift[3 * s + 2] = 0.0;
      continue;
    }
    stXf[s] = c->imgXf[j - nc];
    for (int d = 0; d < 3; ++d) stShift[3 * s + d] = c->imgPos[3 * (size_t)(j - nc) + d] - c->cofg[3 * c->imgCell[j - nc] + d];
  }
  for (size_t t = 0; t < c->xfQ.size(); ++t)
    for (int k = 0; k < 9; ++k) xfQ[9 * t + k] = c->xfQ[t][k];
}
void orc_get_stencil(orc_ctx *c, int *off, int *idx, double *moms) {
  if (off) std::memcpy(off, c->stOff.data(), sizeof(int) * (c->nCells + 1));
  /* a symmetry image as its real cell (orc_get_symmetry gives its reflection) */
  if (idx)
    for (size_t s = 0; s < c->stIdx.size(); ++s) {
      const int j = c->stIdx[s];
      idx[s] = j < c->nCells ? j : c->imgCell[j - c->nCells];
    }
  if (moms && !c->moms.empty()) std::memcpy(moms, c->moms.data(), sizeof(double) * 10 * c->nCells);
}

void orc_set_state(orc_ctx *c, const double *cv) {
  std::memcpy(c->cv.data(), cv, sizeof(double) * 5 * c->nCells);
#pragma omp parallel for schedule(static)
  for (int ic = 0; ic < c->nCells; ++ic) setDependentVars(c, ic);
}
void orc_get_state(orc_ctx *c, double *cv, double *dv) {
  if (cv) std::memcpy(cv, c->cv.data(), sizeof(double) * 5 * c->nCells);
  if (dv) std::memcpy(dv, c->dv.data(), sizeof(double) * 3 * c->nCells);
}
void orc_get_rhs(orc_ctx *c, double *rhs) { std::memcpy(rhs, c->rhs.data(), sizeof(double) * 5 * c->nCells); }
void orc_get_grad(orc_ctx *c, double *grad) { std::memcpy(grad, c->grad.data(), sizeof(double) * 15 * c->nCells); }

void orc_residual(orc_ctx *c, double *rhs, double *grad) {
  std::vector<double> save = c->cv;
  for (double &d : c->diss) d = 0.0;
  cellGradients(c);
  convectiveFluxes(c);
  if (rhs) std::memcpy(rhs, c->rhs.data(), sizeof(double) * 5 * c->nCells);
  if (grad) std::memcpy(grad, c->grad.data(), sizeof(double) * 15 * c->nCells);
  c->cv = save;
}

double orc_timestep(orc_ctx *c, double t) { return timeStep(c, t); }
void orc_rk_init(orc_ctx *c, int iStage) { rkInit(c, iStage); }
void orc_cell_gradients(orc_ctx *c) { cellGradients(c); }
void orc_convective_fluxes(orc_ctx *c) { convectiveFluxes(c); }
void orc_add_rhs(orc_ctx *c, const double *src) {
  for (size_t k = 0; k < 5 * (size_t)c->nCells; ++k) c->rhs[k] = c->rhs[k] + src[k];
}
void orc_rk_update(orc_ctx *c, int iStage, double dtMin) { updateStage(c, iStage, dtMin); }
void orc_rk_stage(orc_ctx *c, int iStage, double dtMin) { rkStage(c, iStage, dtMin); }

int orc_run(orc_ctx *c, int nSteps, double *time, double endTime) {
  int done = 0;
  for (int n = 0; n < nSteps; ++n) {
    double dt = timeStep(c, *time);
    bool finished = false;
    if (endTime > 0.0 && *time + dt > endTime) { dt = endTime - *time; finished = true; }
    for (int s = 1; s <= c->nrkSteps; ++s) rkStage(c, s, dt);
    *time = *time + dt;
    ++done;
    if (finished) break;
  }
  return done;
}

void orc_run_fixed_dt(orc_ctx *c, int nSteps, double dt) {
  for (int n = 0; n < nSteps; ++n)
    for (int s = 1; s <= c->nrkSteps; ++s) rkStage(c, s, dt);
}

void orc_set_dt_imposed(orc_ctx *c, double dt) { c->num.dtImposed = dt; }

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_counters(orc_ctx *c, long long *posFix, long long *negP, long long *nan) {
  if (posFix) *posFix = c->posFixCount;
  if (negP) *negP = c->negPCount;
  if (nan) *nan = c->nanCount;
}

} // extern "C"
