// Device view of one region, shared by the kernel translation units and the
// C ABI.  All per-cell arrays are structure-of-arrays in the renumbered
// (Morton) cell order: component k of cell i sits at a[k*nc + i].  R is the
// storage/arithmetic type of state, gradients and fluxes: double in the FP64
// modes, float in the mixed mode; the master conserved state cv, the
// dependent variables dv and the cell volumes are always double.
#pragma once
#include <cstdint>

namespace rflu {

// Device-side scalars of the time loop and the status counters.
struct Scalars {
  unsigned long long dtBits;  // running min of the per-cell dt (bit pattern of a positive double)
  double dtMin;               // global time step of the current step
  double time;                // current time
  double endTime;             // <= 0: no clip
  int finished;               // set when the last step was clipped to endTime
  int stepsDone;
  unsigned long long nanCells, posFixCells, negPCells;
  int firstBadCell;           // reference (1-based) id, INT_MAX if none
  int pad;
};

struct Params {
  int spaceOrder, spaceDiscr, reconst, rkScheme, piclBuild, precision;
  double refCp, refGamma;     // global%refCp, global%refGamma (flux routines)
  double gvCp, gvMol;         // gv(GV_MIXT_CP), gv(GV_MIXT_MOL) = 8314.3/R
  double gcR, gRT, igcR;      // 8314.3/gvMol, gvCp/(gvCp-gcR), 1/gcR (computed once on the host)
  // FP32 copies for the mixed-mode flux arithmetic (no per-face conversions)
  float refCpF, refGammaF, epsEntrF, dissFactF, gvCpF, gvMolF;
  double epsEntr, dissFact;
  double cfl, dtImposed, dtMinLimit;
  int nrkSteps;
  double ark[5], grk[5];
  float arkF[5], grkF[5];     // FP32 copies for the mixed-mode update
  // mixed mode at 2nd order: no kernel of the step reads T or c, so the stage
  // update stores p only and T, c are formed from cv when dv is read out
  int dvPOnly;
};

// Per-cell record layout of prim, grad and flux.  The FP64 modes keep them as
// structure-of-arrays (component k of cell i at a[k*n + i]).  The mixed mode
// packs each cell's record into float4s so that a neighbour gather is two or
// four 16-byte loads: prim (8 floats per cell) = (rho, u, v, w | p, xc, yc, zc)
// with the cell centroid riding along for the least-squares weights; grad (16
// floats per cell) = the 15 components in the order 3*var + dir and one pad;
// flux = one float4 (mass and momentum) per face followed by the nT energy
// fluxes.
// Per-patch constants of the remaining boundary types, formed on the host
// from the patch's values (pPatch%mixt%vals, uniform distribution) in the
// reference's operation order (rflu_gpu_create, capi.cu: patchConstants), so that no trigonometric
// function or constant power is evaluated per face:
//   outflow         K[0] = p_out
//   farfield        K[0] = M_inf, K[1..6] = (rho, p, q, u, v, w)_inf, K[7] = rho E_inf
//   inflow TOTANG   K[0] = p_tot, K[1] = T_tot, K[2..5] = cos/sin(beta_h), cos/sin(beta_v),
//                   K[6] = BCSWI_INFLOW_FIXED, K[7..12] = the supersonic state (rho, rho u, rho v,
//                   rho w, rho E, p)
//   inflow VELTEMP  K[0..3] = u, v, w, T, K[4] = p, K[5] = rho (not subsonic)
//   injection       K[0] = mass flux, K[1] = T_inj
//   symmetry        K[0..8] = the reflection I - 2 n n^T across the patch's
//                   plane, row-major (RFLU_RELP_TransformMatrix,
//                   modflu/RFLU_ModRelatedPatches.F90:449-514)
constexpr int kPatchK = 16;
constexpr int kBcSymmetry = 100;
// The adjoint's transposed-stencil weights (View::tsW): bit 30 of an
// entry's cell id marks a member seen reflected across symmetry patches.
constexpr int kTsReflected = 1 << 30;
constexpr int kTile = 256;
// Shared-memory footprint of one staged tile of the mixed-mode gradient
// kernel: 8 floats per record, the stencil ids as whole 16-byte words (plus
// one for the misalignment of the first), kTileOffInts stencil offsets, and
// the halo cell ids of the tile two ahead in the pipeline (a multiple of 4
// ints: every tile's halo list starts on a 16-byte boundary).
constexpr int kTileOffInts = kTile + 4;
__host__ __device__ inline size_t tileIdWordsFor(int maxTileSt) { return ((size_t)maxTileSt + 7) / 8 + 1; }
__host__ __device__ inline size_t tileHaloIntsFor(int maxRecs) { return ((size_t)(maxRecs - kTile) + 3) / 4 * 4; }
__host__ __device__ inline size_t tileBufFloatsFor(int maxRecs, int maxTileSt) {
  return 8 * (size_t)maxRecs + 4 * tileIdWordsFor(maxTileSt) + kTileOffInts + tileHaloIntsFor(maxRecs);
}

template <typename R> struct Layout {
  static constexpr bool packed = false;
  static constexpr int prim = 5, grad = 15;
};
template <> struct Layout<float> {
  static constexpr bool packed = true;
  static constexpr int prim = 8, grad = 16;
};

template <typename R>
struct View {
  int nc, nf, nb;             // cells, interior faces, boundary faces
  // interior faces (storage order), renumbered cells; FP64 modes
  const int *fc1, *fc2;
  const R *fnx, *fny, *fnz, *fnm;   // unit normal and area
  const R *dL, *dR;                 // (3, nf): fc - cofg(c1), fc - cofg(c2)
  // the same interior face data in the mixed mode, one 48-byte record per
  // face: (nx, ny, nz, nm), (dLx, dLy, dLz, dRx), (dRy, dRz, c1, c2) with the
  // cell ids stored as int bit patterns
  const float *fpk;
  // boundary faces
  const int *bcell;                 // owning cell
  const int *bpatch;                // patch index
  const R *bnx, *bny, *bnz, *bnm;
  const R *bd;                      // (3, nb): fc - cofg(cell)
  const int *patchType, *patchOutflow, *patchOrder;  // patchOutflow: the BCOPT type switch
  const double *patchK;             // kPatchK constants per patch (physics.cuh)
  // constrained gradients (CRECONSTC 1, constr.h): per cell its slot or -1
  // (null: none), per slot the constraint-row counts of the five variables
  // and its first row, per row three weights and the boundary face of a
  // constraint row (-1: a stencil member's row)
  const int *cSlot, *cNcon, *cRowOff, *cRowFace;
  const R *cW;
  // the adjoint of a burning injection face's constraint values, which
  // follow the pressure of the face's cell: per cell (CSR, null: none) the
  // (constrained cell, 8 * row + variable) pairs of the rows its pressure
  // feeds
  const int *cpOff, *cpEnt;
  // mixed mode on a periodic or symmetry mesh (untiled): each stencil
  // member's translation to its image, added to the centroid difference
  // (null: none)
  const float *stShift;
  // symmetry meshes: each stencil member's reflection (-1: none; null: no
  // member is reflected) and the reflections' 3x3 matrices, row-major; a
  // reflected member's velocity is Q u (its density and pressure its own)
  const int *stXf;
  const R *xfQ;
  // cell -> faces CSR in reference summation order; entry e >= 0: interior
  // face (e >> 1) seen from side (e & 1); e < 0: boundary face -(e+1)
  const int *cfOff, *cfEnt;
  // C2C stencil CSR and per-member least-squares weights
  const int *stOff, *stIdx;
  const R *wx, *wy, *wz;
  const double *vol;
  const R *epsq;                    // Venkatakrishnan eps^2 = (vol^(1/3))^3 per cell
  // mixed mode: the LSQ weights w_j = L d_j / |d_j|^2 of a cell share one
  // symmetric 3x3 matrix L (the product of the R-factor coefficients), so the
  // gradient is L * sum_j (q_j - q_i) d_j / |d_j|^2 with d_j the centroid
  // offset (centroids ride in the packed prim records)
  const R *cgx, *cgy, *cgz;         // cell centroids (FP32), written into prim
  const R *lsq;                     // (6, nc): Lxx, Lxy, Lxz, Lyy, Lyz, Lzz
  const R *ivol;                    // 1/vol (FP32), for the FP32 RK increment
  // mixed mode, tiled gradient kernel: cells in tiles of kTile consecutive
  // (Morton) cells; a tile's CTA stages the prim records of its cells and of
  // the halo (the other cells its stencils and faces reach) in shared memory
  // and addresses them by 16-bit local ids (own cells 0..kTile-1, halo slots
  // after; the plan is tiles.h's planTiles)
  int tiled;                        // 0: the gather kernel instead
  int maxRecs;                      // max staged records over the tiles
  int maxTileSt;                    // max stencil entries of a tile's cells
  // WENO smoothing (RECONST 1, 2): the unsmoothed gradients the gradient
  // kernels write, in the layout of grad, read by kWenoSmooth
  R *gradRaw;
  // mixed mode, adjoint of the LSQ gradient: the transposed stencil entry-
  // major (entry k of cell j at k*nc + j): d/|d|^2 with d = x_j - x_i for
  // the cell i whose stencil holds j, and i as int bits (-1 past the end)
  float *tsW;
  int tsWidth;                      // entries per cell of tsW
  int tileGrid;                     // CTAs of the persistent tiled kernels
  int tileGridDt;                   // ... of the variant with the time-step sum
  int cfW;                          // max faces per cell (entries of feD/feN)
  const int *haloOff, *haloIdx;     // CSR over tiles of global halo cell ids by slot (-1: unused);
                                    // each tile's list starts on a 16-byte boundary
  const int4 *tileDesc;             // per tile: haloOff[t], its halo slots, and the
                                    // 16-byte words [w0, w1) of stLoc its stencils use
  const unsigned short *stLoc;      // local id of each stencil member (stIdx order),
                                    // 16-byte aligned and padded by 8 ids
  // per cell-face entry, entry-major (entry k of cell i at [k*nc + i]), in
  // the reference's face order: (dx, dy, dz, tag) with d = fc - cofg(i) and
  // tag = local id of the neighbour (interior), -(b+1) (boundary face b) or
  // INT_MIN (no entry); and the face's (nx, ny, nz, nm)
  const float *feD, *feN;           // 4 floats per entry
  const int *refId;                 // renumbered -> reference (0-based) cell id
  const int *newId;                 // reference (0-based) -> renumbered cell id
  // transposed stencil (FP64 modes): for cell j, the (cell i, entry s) pairs
  // of the stencils that contain j, for the adjoint of the LSQ gradient
  const int *tsOff, *tsCell, *tsEnt;
  // state
  double *cv;                       // (5, nc)
  double *dv;                       // (3, nc): p, T, c
  R *prim;                          // rho, u, v, w, p (Layout<R>)
  R *grad;                          // component (3*var + dir) (Layout<R>)
  R *rhsSum;                        // (5, nc)
  R *flux;                          // 5 per face, nf + nb faces (Layout<R>)
  R *rhs;                           // (5, nc), residual output only
  Scalars *sc;
  Params p;
};

}  // namespace rflu
