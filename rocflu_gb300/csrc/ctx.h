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
};

template <typename R>
struct View {
  int nc, nf, nb;             // cells, interior faces, boundary faces
  // interior faces (storage order), renumbered cells
  const int *fc1, *fc2;
  const R *fnx, *fny, *fnz, *fnm;   // unit normal and area
  const R *dL, *dR;                 // (3, nf): fc - cofg(c1), fc - cofg(c2)
  // boundary faces
  const int *bcell;                 // owning cell
  const int *bpatch;                // patch index
  const R *bnx, *bny, *bnz, *bnm;
  const R *bd;                      // (3, nb): fc - cofg(cell)
  const int *patchType, *patchOutflow, *patchOrder;
  const double *patchPout;
  // cell -> faces CSR in reference summation order; entry e >= 0: interior
  // face (e >> 1) seen from side (e & 1); e < 0: boundary face -(e+1)
  const int *cfOff, *cfEnt;
  // C2C stencil CSR and per-member least-squares weights
  const int *stOff, *stIdx;
  const R *wx, *wy, *wz;
  const double *vol;
  const R *epsq;                    // Venkatakrishnan eps^2 = (vol^(1/3))^3 per cell
  // mixed mode: LSQ weights are formed on the fly from the cell's R-factor
  // coefficients (c1111, c2222, c3333, c12, c13, c23) and the members'
  // centroids, instead of streaming three weights per stencil member
  const R *cgx, *cgy, *cgz;         // cell centroids (FP32)
  const R *rcf;                     // (6, nc) R-factor coefficients
  const R *ivol;                    // 1/vol (FP32), for the FP32 RK increment
  const int *refId;                 // renumbered -> reference (0-based) cell id
  // transposed stencil (FP64 modes): for cell j, the (cell i, entry s) pairs
  // of the stencils that contain j, for the adjoint of the LSQ gradient
  const int *tsOff, *tsCell, *tsEnt;
  // state
  double *cv;                       // (5, nc)
  double *dv;                       // (3, nc): p, T, c
  R *prim;                          // (5, nc): rho, u, v, w, p
  R *grad;                          // (15, nc): component (3*var + dir)
  R *rhsSum;                        // (5, nc)
  R *flux;                          // (5, nf + nb)
  R *rhs;                           // (5, nc), residual output only
  Scalars *sc;
  Params p;
};

}  // namespace rflu
