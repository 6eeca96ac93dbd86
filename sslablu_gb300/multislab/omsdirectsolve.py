"""Functional block Thomas solvers on the GPU -- drop-in for SslabLU
multislab/omsdirectsolve.py.

    build_block_tridiagonal_solver(S_rk_list)            (omsdirectsolve.py:17-68)
    block_tridiagonal_solve(OMS, T, rhs)                 (70-99)
    build_block_cyclic_tridiagonal_solver(OMS, S_rk_list, rhs_list, Ntot, nc)  (102-145)
    block_cyclic_tridiagonal_solve(OMS, T, smw_block, d) (147-160)

The identity-diagonal system [I S_12; S_21 I S_23; ...] is factored by the
device Thomas elimination (slu_thomas_factor).  ``OMS.glob_target_dofs`` (a
list of index ranges, one per interface) places the blocks in the global
vector, as upstream.
"""
import numpy as np
import torch

from .. import _dev as dv
from ..direct_solve.omsdirectsolve import BlockTridiagonalSolver, _dense_block


class ThomasFactors(tuple):
    """(A, B, C) as upstream returns, carrying the device factorisation."""

    def __new__(cls, solver, S_rk_list):
        obj = super().__new__(cls, ([s[0] for s in S_rk_list[1:]], None,
                                    [s[-1] for s in S_rk_list[:-1]]))
        obj.solver = solver
        return obj


def build_block_tridiagonal_solver(S_rk_list):
    """Factor [I C_0; A_1 I C_1; ...] with S_rk_list rows [A_i, C_i]."""
    m = int(S_rk_list[0][0].shape[0])
    th = BlockTridiagonalSolver(m)
    th.factorize(S_rk_list, None)
    return ThomasFactors(th, S_rk_list)


def _index_tensor(indices):
    idx = np.concatenate([np.asarray(list(r), dtype=np.int64) for r in indices])
    return torch.from_numpy(idx).cuda()


def block_tridiagonal_solve(OMS, T, rhs):
    """Solve with factors from build_block_tridiagonal_solver."""
    d, one = dv.prepare_rhs(rhs)
    idx = _index_tensor(OMS.glob_target_dofs)
    x = torch.zeros_like(d)
    x[idx] = T.solver._solve_dev(d[idx].clone())
    return dv.finish(x, rhs, one)


def build_block_cyclic_tridiagonal_solver(OMS, S_rk_list, rhs_list, Ntot, nc):
    """Periodic system via Sherman-Morrison-Woodbury (omsdirectsolve.py:102-145):
    E = S_rk_list[0][0] couples the first block to the last, F =
    S_rk_list[-1][1] the last to the first."""
    m = int(S_rk_list[0][0].shape[0])
    n = len(S_rk_list)
    E = _dense_block(S_rk_list[0][0], m)
    F = _dense_block(S_rk_list[-1][1], m)
    T = build_block_tridiagonal_solver(S_rk_list)
    U = torch.zeros((n * m, 2 * m), dtype=torch.float64, device="cuda")
    V = torch.zeros((n * m, 2 * m), dtype=torch.float64, device="cuda")
    I = torch.eye(m, dtype=torch.float64, device="cuda")
    U[0:m, 0:m] = E
    U[(n - 1) * m:, m:] = F
    V[(n - 1) * m:, 0:m] = I
    V[0:m, m:] = I
    Z = dv.to_dev(block_tridiagonal_solve(OMS, T, U))
    G = dv.gemm(V, Z, ta=True) + torch.eye(2 * m, dtype=torch.float64, device="cuda")
    W = dv.DenseLU(G).solve(V.t().contiguous())
    smw = dv.gemm(Z, W.contiguous())
    return T, smw


def block_cyclic_tridiagonal_solve(OMS, T, smw_block, d):
    """x = y - smw_block y with y = T^{-1} d (omsdirectsolve.py:147-160)."""
    X, one = dv.prepare_rhs(d)
    y = dv.to_dev(block_tridiagonal_solve(OMS, T, X))
    x = y - dv.gemm(dv.to_dev(smw_block), y)
    return dv.finish(x, d, one)
