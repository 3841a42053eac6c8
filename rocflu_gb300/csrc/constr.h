// Constrained cell gradients (CRECONSTC 1): host-side plan (plain C++).
//
// The reference adds to every cell's stencil the wall and injection faces of
// the cell itself and of its stencil members (RFLU_AddBFaces, modflu/
// RFLU_ModStencilsUtils.F90:134-298: cells in stencil order, patches in
// order, at most 18 faces), keeps the 9 nearest (RFLU_SortBFaces, :1501-1585,
// and the cap nBFaceMembsMax of RFLU_SetInfoC2CStencil, modflu/
// RFLU_ModStencilsCells.F90:2816-2909), and for each cell with such faces
// recomputes the gradient of every variable that one of them constrains
// (RFLU_ComputeGradCellsConstr, modflu/RFLU_ModDifferentiationCells.F90:
// 1180-1563): a least-squares fit to the stencil's differences, rows d/|d|,
// and to the constraint values at the faces, rows cwt d_f/|d_f|, through the
// pseudo-inverse of that matrix.  The constraint types and values are
// RFLU_GetConstrType / RFLU_GetConstrValue (modflu/RFLU_ModConstraintUtils.
// F90:122-745) for a TCPERF gas and the primitive variables (rho, u, v, w,
// p): rho at burning injection faces; a velocity component at slip-wall and
// injection faces whose normal is that axis (within 1e-6) and at every
// no-slip-wall face; p never.
//
// The plan holds, per constrained cell and constrained variable, the final
// weights term * pinv(A)[:, row] of every row (the reference forms
// gx = gx + term*aInv(1,row)*dVar row by row, members first), so that the
// kernels accumulate w * dVar in the same order.  The pseudo-inverse is
// formed as (A^T A)^-1 A^T with the inverse by cofactors (the reference calls
// LAPACK dgesdd; for the full-rank matrices it accepts the two agree to
// rounding); a matrix that its singular-value test would reject is an error
// here as it is a stop there.
#pragma once
#include <vector>

namespace rflu {

struct ConstrPlan {
  // the boundary-face stencil: per cell its faces (global 0-based boundary
  // face index, patch after patch), nearest first
  std::vector<int> bfOff, bfIdx;
  // constrained cells (0-based, the caller's numbering), their variables'
  // constraint-row counts (5 per cell: 0 keeps the least-squares gradient)
  // and rows: per cell the rows of each constrained variable in turn, the
  // stencil members' rows first (face -1), then the constraint rows
  std::vector<int> cells, nCon, rowOff;
  std::vector<double> w;     // 3 per row
  std::vector<int> rowFace;  // per row: boundary face of a constraint row, -1 for a member row
};

struct ConstrInput {
  int nCells;
  const double *cofg;                 // (3, nCells)
  const int *stOff, *stIdx;           // cell stencils, 0-based members
  int nPatches;
  const int *patchFaceOff;            // nPatches + 1
  const int *patchType;               // BC types
  const double *patchMinj;            // per patch: the injection mass flux (injection patches)
  const int *bf2c;                    // 0-based cell of each boundary face
  const double *bfn;                  // (4, nBFaces)
  const double *bfc;                  // (3, nBFaces)
  double cwt;                         // cReconstCellsWeight
};

// Returns 0, or -1 with *bad the first cell whose constrained matrix is
// rank-deficient.  withWeights false: the boundary-face stencil only.
int planConstrained(const ConstrInput &in, ConstrPlan &plan, int *bad, bool withWeights = true);

}  // namespace rflu
