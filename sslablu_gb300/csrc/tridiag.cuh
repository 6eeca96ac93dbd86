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
  // fused solve operators (blocks of m <= kRbFusedMax), m x 3m each, built at
  // factor time:  Fop_j = [I | -SiM_{2j} Inv_{2j-1} | -SiP_{2j} Inv_{2j+1}]
  // (reduction of even block 2j, Fop_0's middle block zero) and
  // Bop_j = [Inv_o | -Inv_o SiM_o | -Inv_o SiP_o] (back substitution of odd
  // block o = 2j + 1)
  DevBuf Fop, Bop;
};

// Largest block for the fused red-black solve (a step CTA stages row
// slices of a 3m-wide operator and a 3m-long z tile in 96 KB).
constexpr int kRbFusedMax = 256;

struct RbSolver {
  int m = 0, nblk = 0;
  bool mixed = false;              // Schur products on the tensor cores
  bool fused = false;              // levels carry Fop / Bop (m <= kRbFusedMax)
  bool cyclic = false;             // periodic: SiM[0] couples to the last block, SiP[-1] to the first
  std::vector<RbLevel> levels;     // levels[0] = the input system
};

void rb_factor(Handle& h, RbSolver& S, int nblk, int m, const double* SiM, const double* SiP,
               const double* T, bool mixed = false, bool cyclic = false);
// Y = A X for the stored input system (level 0), X and Y nblk*m x nrhs.
void rb_apply(Handle& h, const RbSolver& S, const double* X, int ldx, double* Y, int ldy,
              int nrhs);
// Refinement of A x = b with the (mixed) factors and a float64 residual.
void rb_refine(Handle& h, const RbSolver& S, const double* B, int ldb, double* X, int ldx,
               int nrhs, double tol, int maxit, int* iters, double* relres);
// tc: the block products as split-BF16x3 tensor-core GEMMs (float32
// accuracy: a preconditioner-grade solve) instead of float64 GEMMs.
void rb_solve(Handle& h, const RbSolver& S, double* B, int ldb, int nrhs, bool tc = false);
void thomas_factor(Handle& h, RbSolver& S, int nblk, int m, const double* SiM, const double* SiP,
                   const double* T);
void thomas_solve(Handle& h, const RbSolver& S, double* B, int ldb, int nrhs);

}  // namespace slu
