"""Dense block-tridiagonal direct solvers on the GPU -- drop-in for SslabLU
direct_solve/omsdirectsolve.py.

    RedBlackSolver(m, cyclic=False).factorize(S_rk_list, T) / .solve(rhs)
    BlockTridiagonalSolver(m, cyclic=False).factorize(S_rk_list, T, glob_target_dofs=None)
                                          / .solve(rhs, glob_target_dofs=None)

S_rk_list rows follow upstream: row i is a sequence whose [0] entry couples
block i to block i-1 and whose [-1] entry couples it to block i+1 (a row of
length 1 carries a single coupling, as the multislab assembly produces at the
two ends).  Blocks may be numpy arrays, torch tensors, or any operator with
``matmat`` (materialised once with the identity, as upstream's dense
assembler does).  Factorisation and solves run in libslablu
(slu_rb_factor / slu_rb_solve, slu_thomas_factor / slu_thomas_solve).

Differences from upstream, all in upstream's favour of generality:
  * solve accepts (N,) and (N, nrhs) right-hand sides (upstream red-black is
    1-D only, omsdirectsolve.py:244);
  * a non-power-of-two block count raises ValueError (upstream constructs the
    exception without raising it, omsdirectsolve.py:201-202, then fails with
    an IndexError).
"""
import ctypes
from abc import ABC, abstractmethod

import numpy as np
import torch

from .. import _dev as dv
from .. import _lib as L


class DirectSolver(ABC):
    """omsdirectsolve.py:13-27."""

    def __init__(self, m, cyclic=False):
        self.m = m
        self.cyclic = cyclic

    @abstractmethod
    def factorize(self, S_rk_list, T):
        pass

    @abstractmethod
    def solve(self, rhs):
        pass


def _dense_block(B, m):
    if B is None:
        return torch.zeros((m, m), dtype=torch.float64, device="cuda")
    if isinstance(B, np.ndarray) or dv.is_torch(B):
        return dv.to_dev(B)
    if hasattr(B, "_dev_apply"):
        return B._dev_apply(torch.eye(m, dtype=torch.float64, device="cuda"), False)
    return dv.to_dev(np.asarray(B @ np.identity(m)))


def stack_blocks(S_rk_list, T, m, cyclic=False):
    """(SiM, SiP, T) as (n, m, m) device tensors; SiM[0] = SiP[-1] = 0 unless
    ``cyclic`` (then they are the periodic couplings of rows of length 2)."""
    n = len(S_rk_list)
    SiM = torch.zeros((n, m, m), dtype=torch.float64, device="cuda")
    SiP = torch.zeros((n, m, m), dtype=torch.float64, device="cuda")
    for i, row in enumerate(S_rk_list):
        if len(row) >= 2:
            if i > 0 or cyclic:
                SiM[i] = _dense_block(row[0], m)
            if i < n - 1 or cyclic:
                SiP[i] = _dense_block(row[-1], m)
        elif len(row) == 1:
            if i == 0:
                SiP[i] = _dense_block(row[0], m)
            else:
                SiM[i] = _dense_block(row[0], m)
    if T is None:
        Td = torch.eye(m, dtype=torch.float64, device="cuda").expand(n, m, m).contiguous()
    else:
        Td = torch.stack([_dense_block(t, m) for t in T]).contiguous()
    return SiM.contiguous(), SiP.contiguous(), Td


def _block_size(S_rk_list):
    B = S_rk_list[0][0]
    return int(B.shape[0])


class _DeviceTridiag:
    _factor_fn = None
    _solve_fn = None

    def _factor(self, S_rk_list, T, periodic=False):
        m = _block_size(S_rk_list)
        self.m = m
        SiM, SiP, Td = stack_blocks(S_rk_list, T, m, periodic)
        self.nblk = SiM.shape[0]
        out = ctypes.c_void_p()
        L.check(getattr(L.lib(), self._factor_fn)(L.handle(), self.nblk, m, L.ptr(SiM),
                                                  L.ptr(SiP), L.ptr(Td), ctypes.byref(out)))
        L.sync()
        self._h = out
        # keep the dense blocks for the periodic (SMW) correction
        self._SiM, self._SiP = SiM, SiP

    def _solve_dev(self, B):
        B = B.contiguous()
        L.check(getattr(L.lib(), self._solve_fn)(L.handle(), self._h, L.ptr(B), B.shape[1],
                                                 B.shape[1]))
        return B

    def __del__(self):
        try:
            if getattr(self, "_h", None) is not None and L._lib is not None:
                L.lib().slu_rb_destroy(self._h)
        except Exception:
            pass


class BlockTridiagonalSolver(_DeviceTridiag, DirectSolver):
    """Block Thomas elimination, omsdirectsolve.py:48-175 (incl. the cyclic
    Sherman-Morrison-Woodbury correction of 143-175)."""

    _factor_fn = "slu_thomas_factor"
    _solve_fn = "slu_thomas_solve"

    def factorize(self, S_rk_list, T, glob_target_dofs=None):
        self._factor(S_rk_list, T)
        self.smw_block = None
        if self.cyclic:
            m, n = self.m, self.nblk
            E = _dense_block(S_rk_list[0][0], m)
            F = _dense_block(S_rk_list[-1][1], m)
            U = torch.zeros((n * m, 2 * m), dtype=torch.float64, device="cuda")
            V = torch.zeros((n * m, 2 * m), dtype=torch.float64, device="cuda")
            U[0:m, 0:m] = E
            U[(n - 1) * m:, m:] = F
            I = torch.eye(m, dtype=torch.float64, device="cuda")
            V[(n - 1) * m:, 0:m] = I
            V[0:m, m:] = I
            Z = self._solve_dev(U.clone())
            G = dv.gemm(V, Z, ta=True)
            G += torch.eye(2 * m, dtype=torch.float64, device="cuda")
            W = dv.DenseLU(G).solve(V.t().contiguous())
            self.smw_block = dv.gemm(Z, W.contiguous())
            self._V = V

    def solve(self, rhs, glob_target_dofs=None):
        B, one = dv.prepare_rhs(rhs)
        x = self._solve_dev(B.clone())
        if self.cyclic:
            x = x - dv.gemm(self.smw_block, x)
        return dv.finish(x, rhs, one)


class RedBlackSolver(_DeviceTridiag, DirectSolver):
    """Red-black cyclic reduction, omsdirectsolve.py:177-333; cyclic=True is
    the periodic system (slu_rb_factor_cyclic: SiM[0] couples block 0 to the
    last block and SiP[-1] the last block to block 0), float64 only.

    precision='mixed' (beyond upstream): the Schur-complement products of the
    elimination run on the tensor cores (split-BF16x3, slu_rb_factor_mixed),
    pivot blocks stay float64, and solve() refines against the float64 system
    until ||b - A x|| / ||b|| <= tol per column (slu_rb_refine); the last
    iteration count and relative residual are kept in .iters / .relres.
    """

    _factor_fn = "slu_rb_factor"
    _solve_fn = "slu_rb_solve"

    def __init__(self, m, cyclic=False, precision="f64", tol=1e-10, maxit=20):
        super().__init__(m, cyclic)
        if precision not in ("f64", "mixed"):
            raise ValueError("precision must be 'f64' or 'mixed'")
        self.precision, self.tol, self.maxit = precision, tol, maxit
        if precision == "mixed":
            self._factor_fn = "slu_rb_factor_mixed"

    def factorize(self, S_rk_list, T):
        n = len(S_rk_list)
        if not (n & (n - 1) == 0 and n != 0):
            raise ValueError("ERROR! Number of slabs is not a power of 2.")
        if self.cyclic:
            if self.precision == "mixed":
                raise NotImplementedError("the periodic red-black solver is float64 only")
            self._factor_fn = "slu_rb_factor_cyclic"
        self._factor(S_rk_list, T, periodic=self.cyclic)
        self.nSlabs = n

    def solve(self, rhs):
        B, one = dv.prepare_rhs(rhs)
        if self.precision == "mixed":
            import ctypes
            X = torch.empty_like(B)
            it, rr = ctypes.c_int(), ctypes.c_double()
            L.check(L.lib().slu_rb_refine(L.handle(), self._h, L.ptr(B), B.shape[1], L.ptr(X),
                                          X.shape[1], B.shape[1], float(self.tol),
                                          int(self.maxit), ctypes.byref(it), ctypes.byref(rr)))
            self.iters, self.relres = it.value, rr.value
            return dv.finish(X, rhs, one)
        return dv.finish(self._solve_dev(B.clone()), rhs, one)

    def solve_tc(self, rhs):
        """Beyond upstream: the solve with its block products on the tensor
        cores (split-BF16x3 GEMMs, float32-level accuracy; slu_rb_solve_tc):
        a fast approximate solve for preconditioning an iterative solve of the
        exact operator."""
        B, one = dv.prepare_rhs(rhs)
        B = B.clone().contiguous()
        L.check(L.lib().slu_rb_solve_tc(L.handle(), self._h, L.ptr(B), B.shape[1], B.shape[1]))
        return dv.finish(B, rhs, one)
