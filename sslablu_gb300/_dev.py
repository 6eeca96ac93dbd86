"""Device-side helpers shared by the mirror modules.

Operators on the device expose ``_dev_apply(X, trans)`` and, when invertible,
``_dev_solve(X, trans)`` on (N, c) float64 CUDA tensors.  Anything else that
follows the scipy LinearOperator protocol (``matmat`` / ``rmatmat`` /
``solve(v, mode)``) is a caller-supplied host operator: it is evaluated where
the caller defined it and its result is uploaded, exactly as upstream calls it.
"""
import ctypes

import numpy as np
import torch

from . import _lib as L

F64 = torch.float64


def is_torch(x):
    return isinstance(x, torch.Tensor)


def to_dev(x, dtype=F64):
    """numpy / torch -> contiguous CUDA tensor."""
    if is_torch(x):
        t = x.to(device="cuda", dtype=dtype)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64))).to(
            device="cuda", dtype=dtype)
    return t.contiguous()


def to_host(t):
    return t.detach().cpu().numpy()


def out_like(t, ref):
    """Return device tensor t in the container type of the input ref."""
    return t if is_torch(ref) else to_host(t)


def as_2d(t):
    return t[:, None] if t.dim() == 1 else t


def gemm(A, B, C=None, ta=False, tb=False, alpha=1.0, beta=0.0):
    """C = alpha op(A) op(B) + beta C on contiguous 2-D float64 CUDA tensors."""
    M = A.shape[1] if ta else A.shape[0]
    K = A.shape[0] if ta else A.shape[1]
    N = B.shape[0] if tb else B.shape[1]
    if C is None:
        C = torch.empty((M, N), dtype=F64, device="cuda")
        beta = 0.0
    if M == 0 or N == 0:
        return C
    L.check(L.lib().slu_gemm_batched(L.handle(), int(ta), int(tb), M, N, K, float(alpha),
                                     L.ptr(A), A.shape[1], 0, L.ptr(B), B.shape[1], 0,
                                     float(beta), L.ptr(C), C.shape[1], 0, 1))
    return C


class DenseLU:
    """LU factors of a dense matrix on the device (slu_lu_factor)."""

    def __init__(self, A):
        A = to_dev(A)
        n = A.shape[0]
        self.n = n
        self.lu = A.clone()
        self.piv = torch.empty(n, dtype=torch.int32, device="cuda")
        L.check(L.lib().slu_lu_factor(L.handle(), n, L.ptr(self.lu), n, 0, L.ptr(self.piv), 0, 1,
                                      None))

    def solve(self, X, trans=False):
        X = as_2d(X).contiguous()
        L.check(L.lib().slu_lu_solve(L.handle(), int(trans), self.n, L.ptr(self.lu), self.n, 0,
                                     L.ptr(self.piv), 0, L.ptr(X), X.shape[1], 0, X.shape[1], 1))
        return X


class DenseDev:
    """A dense matrix resident on the device, with the operator protocol."""

    def __init__(self, A):
        self.M = to_dev(A)
        self.shape = tuple(self.M.shape)
        self.dtype = np.float64
        self._lu = None
        self.tree = self.quad = None

    def _dev_apply(self, X, trans=False):
        return gemm(self.M, as_2d(X).contiguous(), ta=trans)

    def _dev_solve(self, X, trans=False):
        if self._lu is None:
            self._lu = DenseLU(self.M)
        return self._lu.solve(as_2d(X).clone(), trans)


def dev_apply(op, X, trans=False):
    """op @ X (or op^T @ X) for a (N, c) CUDA tensor X, returning a CUDA tensor."""
    X = as_2d(X)
    if hasattr(op, "_dev_apply"):
        return op._dev_apply(X, trans)
    if isinstance(op, np.ndarray) or is_torch(op):
        M = to_dev(op)
        return gemm(M, X.contiguous(), ta=trans)
    Xh = to_host(X)
    Yh = op.rmatmat(Xh) if trans else op.matmat(Xh)
    return to_dev(np.asarray(Yh).reshape(-1, Xh.shape[1]))


def dev_solve(op, X, trans=False):
    X = as_2d(X)
    if hasattr(op, "_dev_solve"):
        return op._dev_solve(X, trans)
    if isinstance(op, np.ndarray) or is_torch(op):
        return DenseLU(op).solve(X.clone(), trans)
    Xh = to_host(X)
    Yh = op.solve(Xh, mode="T" if trans else "N")
    return to_dev(np.asarray(Yh).reshape(-1, Xh.shape[1]))


def prepare_rhs(v):
    """Any 1-D/2-D numpy or torch input -> (device 2-D tensor, was_1d)."""
    one = v.ndim == 1
    t = to_dev(v)
    return (t[:, None].contiguous() if one else t), one


def finish(t, ref, one):
    t = t[:, 0] if one else t
    return out_like(t, ref)


def void_p_array(ptrs):
    arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
    return arr
