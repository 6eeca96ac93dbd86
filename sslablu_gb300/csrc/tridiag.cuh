// Dense block-tridiagonal solvers (red-black cyclic reduction, block Thomas).
#pragma once
#include "hbs.cuh"

namespace slu {

struct RbLevel {
  int nS = 0;                      // blocks on this level
  DevBuf SiM, SiP, T, LU, piv;     // nS m x m blocks each (piv: nS*m int32)
  // inverses of the pivot blocks, formed once from their LU factors: every
  // solve-phase block solve is then one (batched) GEMM
  DevBuf Inv;
};

struct RbSolver {
  int m = 0, nblk = 0;
  bool mixed = false;              // Schur products on the tensor cores
  std::vector<RbLevel> levels;     // levels[0] = the input system
};

void rb_factor(Handle& h, RbSolver& S, int nblk, int m, const double* SiM, const double* SiP,
               const double* T, bool mixed = false);
// Y = A X for the stored input system (level 0), X and Y nblk*m x nrhs.
void rb_apply(Handle& h, const RbSolver& S, const double* X, int ldx, double* Y, int ldy,
              int nrhs);
// Refinement of A x = b with the (mixed) factors and a float64 residual.
void rb_refine(Handle& h, const RbSolver& S, const double* B, int ldb, double* X, int ldx,
               int nrhs, double tol, int maxit, int* iters, double* relres);
void rb_solve(Handle& h, const RbSolver& S, double* B, int ldb, int nrhs);
void thomas_factor(Handle& h, RbSolver& S, int nblk, int m, const double* SiM, const double* SiP,
                   const double* T);
void thomas_solve(Handle& h, const RbSolver& S, double* B, int ldb, int nrhs);

}  // namespace slu
