"""Grouped solves over many HBS operators.

The reference solves one operator per call (``HBSnew.HBSMAT.solve``,
matAssembly/HBS/HBSnew.py:393-416); a batch of slab systems calls it once
per operator.  ``solve_grouped`` hands the whole batch to the library, which
runs one kernel launch per tree step for every member together
(``slu_ulv_solve_grouped`` / ``slu_refine_grouped``).  Each member's result is
the result of its own ``HBSMAT.solve`` (float64) or ``HBSMAT.solve_refined``
(mixed precision).
"""
import ctypes

import numpy as np
import torch

from . import _dev as dv
from . import _lib as L


def solve_grouped_device(ops, Bs, precision="f64", tol=1e-10, maxit=10, Xs=None):
    """Grouped solve on contiguous float64 CUDA tensors Bs[i] (N_i x c_i).

    ``'f64'`` solves every Bs[i] in place and returns Bs.  ``'mixed'`` writes
    Xs[i] (allocated when None) and returns ``(Xs, iterations, relres)``."""
    n = len(ops)
    if n == 0:
        return ([], 0, []) if precision == "mixed" else []
    for H, B in zip(ops, Bs):
        if B.dtype != torch.float64 or not B.is_cuda or not B.is_contiguous() or B.dim() != 2:
            raise ValueError("right-hand sides must be contiguous 2-D float64 CUDA tensors")
        if B.shape[0] != H.shape[0]:
            raise ValueError("right-hand side has %d rows, operator %d" % (B.shape[0], H.shape[0]))
    op_arr = (ctypes.c_void_p * n)(*[H._op for H in ops])
    bp = (ctypes.c_void_p * n)(*[t.data_ptr() for t in Bs])
    ld = (ctypes.c_int * n)(*[t.shape[1] for t in Bs])
    lib = L.lib()
    if precision == "f64":
        L.check(lib.slu_ulv_solve_grouped(L.handle(), n, op_arr, bp, ld, ld))
        return Bs
    if precision != "mixed":
        raise ValueError("precision must be 'f64' or 'mixed'")
    if Xs is None:
        Xs = [torch.empty_like(t) for t in Bs]
    xp = (ctypes.c_void_p * n)(*[t.data_ptr() for t in Xs])
    it = ctypes.c_int()
    rr = (ctypes.c_double * n)()
    L.check(lib.slu_refine_grouped(L.handle(), n, op_arr, bp, ld, xp, ld, ld, float(tol),
                                   int(maxit), ctypes.byref(it), rr))
    return Xs, it.value, list(np.frombuffer(rr, dtype=np.float64))


class GroupedSolvePlan:
    """solve_grouped_device(ops, Bs) for fixed blocks, captured once
    (slu_ulv_solve_grouped_plan_create): ``plan()`` solves whatever the Bs
    hold, in place, with one graph launch on the current stream."""

    def __init__(self, ops, Bs):
        n = len(ops)
        for H, B in zip(ops, Bs):
            if B.dtype != torch.float64 or not B.is_cuda or not B.is_contiguous() or B.dim() != 2:
                raise ValueError("right-hand sides must be contiguous 2-D float64 CUDA tensors")
            if B.shape[0] != H.shape[0]:
                raise ValueError("right-hand side has %d rows, operator %d"
                                 % (B.shape[0], H.shape[0]))
        self.ops, self.Bs = list(ops), list(Bs)   # the plan reads and writes these
        op_arr = (ctypes.c_void_p * max(n, 1))(*[H._op for H in ops])
        bp = (ctypes.c_void_p * max(n, 1))(*[t.data_ptr() for t in Bs])
        ld = (ctypes.c_int * max(n, 1))(*[t.shape[1] for t in Bs])
        p = ctypes.c_void_p()
        L.check(L.lib().slu_ulv_solve_grouped_plan_create(L.handle(), n, op_arr, bp, ld, ld,
                                                          ctypes.byref(p)))
        self._p = p
        self._launch = L.lib().slu_ulv_solve_plan_launch

    def __call__(self):
        L.check(self._launch(L.handle(), self._p, 0))
        return self.Bs

    def close(self):
        if getattr(self, "_p", None) is not None and L._lib is not None:
            L.lib().slu_ulv_solve_plan_destroy(self._p)
        self._p = None

    def __del__(self):
        self.close()


class GroupedRefinePlan:
    """solve_grouped_device(ops, Bs, "mixed", ..., Xs=Xs) for fixed blocks,
    made once (slu_refine_grouped_plan_create): ``plan(tol, maxit)`` refines
    whatever the Bs hold into the Xs and returns (Xs, iterations, relres)."""

    def __init__(self, ops, Bs, Xs=None):
        n = len(ops)
        for H, B in zip(ops, Bs):
            if B.dtype != torch.float64 or not B.is_cuda or not B.is_contiguous() or B.dim() != 2:
                raise ValueError("right-hand sides must be contiguous 2-D float64 CUDA tensors")
            if B.shape[0] != H.shape[0]:
                raise ValueError("right-hand side has %d rows, operator %d"
                                 % (B.shape[0], H.shape[0]))
        if Xs is None:
            Xs = [torch.empty_like(t) for t in Bs]
        self.ops, self.Bs, self.Xs = list(ops), list(Bs), list(Xs)
        op_arr = (ctypes.c_void_p * max(n, 1))(*[H._op for H in ops])
        bp = (ctypes.c_void_p * max(n, 1))(*[t.data_ptr() for t in Bs])
        xp = (ctypes.c_void_p * max(n, 1))(*[t.data_ptr() for t in Xs])
        ld = (ctypes.c_int * max(n, 1))(*[t.shape[1] for t in Bs])
        p = ctypes.c_void_p()
        L.check(L.lib().slu_refine_grouped_plan_create(L.handle(), n, op_arr, bp, ld, xp, ld, ld,
                                                       ctypes.byref(p)))
        self._p = p
        self._n = n

    def __call__(self, tol=1e-10, maxit=10):
        it = ctypes.c_int()
        rr = (ctypes.c_double * max(self._n, 1))()
        L.check(L.lib().slu_refine_plan_run(L.handle(), self._p, float(tol), int(maxit),
                                            ctypes.byref(it), rr))
        return self.Xs, it.value, list(np.frombuffer(rr, dtype=np.float64)[:self._n])

    def close(self):
        if getattr(self, "_p", None) is not None and L._lib is not None:
            L.lib().slu_refine_plan_destroy(self._p)
        self._p = None

    def __del__(self):
        self.close()


def apply_grouped(ops, Xs, trans=False, Ys=None):
    """Grouped apply on contiguous float64 CUDA tensors: Ys[i] = A_i Xs[i]
    (or A_i^T Xs[i] where ``trans`` -- one flag, or one per member -- is
    true), one kernel launch per tree step for the whole group.  Each result
    equals the member's own HBSMAT.matmat / rmatmat.  Returns Ys."""
    n = len(ops)
    if Ys is None:
        Ys = [torch.empty_like(t) for t in Xs]
    if n == 0:
        return Ys
    tr = list(trans) if isinstance(trans, (list, tuple)) else [bool(trans)] * n
    for H, X, Y in zip(ops, Xs, Ys):
        for t in (X, Y):
            if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous() or t.dim() != 2:
                raise ValueError("operands must be contiguous 2-D float64 CUDA tensors")
        if X.shape[0] != H.shape[1] or Y.shape != X.shape:
            raise ValueError("operand shape does not match the operator")
    op_arr = (ctypes.c_void_p * n)(*[H._op for H in ops])
    tra = (ctypes.c_int * n)(*[int(bool(t)) for t in tr])
    xp = (ctypes.c_void_p * n)(*[t.data_ptr() for t in Xs])
    yp = (ctypes.c_void_p * n)(*[t.data_ptr() for t in Ys])
    ld = (ctypes.c_int * n)(*[t.shape[1] for t in Xs])
    L.check(L.lib().slu_hbs_apply_grouped(L.handle(), n, op_arr, tra, xp, ld, yp, ld, ld))
    return Ys


def solve_grouped(systems, precision="f64", tol=1e-10, maxit=10):
    """Solve A_i x_i = b_i for every (HBSMAT A_i, b_i) in ``systems``.

    ``b_i`` is 1-D or 2-D, numpy or torch; each x_i comes back in the form of
    its b_i.  ``precision='f64'`` runs the float64 ULV sweep (mode N);
    ``'mixed'`` runs float32 sweeps refined against float64 residuals until
    ||b - A x|| / ||b|| <= tol per column, and returns
    ``(xs, iterations, relres)`` with one worst residual per member.
    """
    if precision not in ("f64", "mixed"):
        raise ValueError("precision must be 'f64' or 'mixed'")
    ops, Bs, meta = [], [], []
    for H, b in systems:
        if getattr(H, "mode", "N") != "N":
            raise NotImplementedError("grouped solves are mode N only")
        B, one = dv.prepare_rhs(b)
        ops.append(H)
        Bs.append(B.clone().contiguous())
        meta.append((one, b))
    if precision == "f64":
        out = solve_grouped_device(ops, Bs)
        return [dv.finish(t, ref, one) for t, (one, ref) in zip(out, meta)]
    Xs, it, rr = solve_grouped_device(ops, Bs, "mixed", tol, maxit)
    return [dv.finish(t, ref, one) for t, (one, ref) in zip(Xs, meta)], it, rr
