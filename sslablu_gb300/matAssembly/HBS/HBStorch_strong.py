"""Strong-admissibility HBS on the GPU -- drop-in for SslabLU
matAssembly/HBS/HBStorch_strong.py.

Same constructor and call surface as upstream's HBSMAT (908-1310):
  * ``HBSMAT(A=None, device=None, tree=None, quad=False)``; the tree is a
    slabTree built with ``adjacency='partial'`` or ``'full'`` (or a quad
    tree): ``perm_leaf``, ``nleaves``, ``nlevels`` and ``level_adj_list``;
  * ``construct(rk, Om, Psi, Y, Z, ...)`` compresses from the caller's
    sketches (Y = A Om, Z = A^T Psi, N x s, rows in the caller's ordering,
    permuted into tree order as upstream does, 1000-1031): per level, leaf
    first, while some block still has a far field, the cluster bases
    U, V and the near-field tiles E from the near-field stacks; then the
    dense base B = Y pinv(Om);
  * ``matmat / rmatmat / matvec / rmatvec / @ / T`` (1205-1303): numpy in ->
    numpy out, tensors stay tensors;
  * ``Umats / Vmats`` as (Nb, b, rk) tensors and ``Emats`` (one
    ``BlockSparseE`` per compressed level, then the ``DenseBase``), exported
    on first access; ``nbytes``, ``factor_stats``, ``tConstruct``.
Everything runs in libslablu (csrc/strong.cu): batched blocked Householder
QRs of the near-field stacks, Jacobi SVDs, batched GEMMs and a block-sparse
product kernel, float64.  Upstream's truncated-SVD fallback for numerically
rank-deficient near-field stacks is not built (such a stack raises
SluError); ``group_chunk`` / ``store_device`` / ``profile`` are accepted for
compatibility (all factors stay on the device).
"""
import ctypes
import time

import numpy as np
import torch

from ... import _dev as dv
from ... import _lib as L


def has_farfield(adj_sets):
    """HBStorch_strong.py:849-854: some block's near field (its adjacency
    plus itself) misses part of the level."""
    n = len(adj_sets)
    return any(len(set(adj_sets[r]) | {r}) < n for r in range(n))


class BlockSparseE:
    """Near-field tiles of one level (HBStorch_strong.py:396-600): val
    (nnz, b, b), row, col (nnz,), sorted by (row, col)."""

    def __init__(self, val, row, col, n, b):
        self.val, self.row, self.col, self.n, self.b = val, row, col, n, b

    @property
    def nnz(self):
        return int(self.val.shape[0])

    @property
    def nbytes(self):
        return sum(t.element_size() * t.nelement() for t in (self.val, self.row, self.col))

    @property
    def dtype(self):
        return self.val.dtype

    def to_dense(self):
        n, b = self.n, self.b
        D = torch.zeros((n * b, n * b), dtype=self.val.dtype, device=self.val.device)
        for t in range(self.nnz):
            i, j = int(self.row[t]), int(self.col[t])
            D[i * b:(i + 1) * b, j * b:(j + 1) * b] = self.val[t]
        return D


class DenseBase:
    """The dense base operator B (HBStorch_strong.py:856-895)."""

    def __init__(self, B, n, b):
        self.B, self.n, self.b = B, n, b

    @property
    def shape(self):
        return tuple(self.B.shape)

    @property
    def dtype(self):
        return self.B.dtype

    @property
    def nbytes(self):
        return self.B.element_size() * self.B.nelement()


class HBSMAT:
    """Strong-admissibility HBS matrix, compressed and applied on the GPU."""

    def __init__(self, A=None, device=None, tree=None, quad=False):
        self.mode = "N"
        self.dtype = torch.float64
        self.device = device
        self.store_device = device
        self.group_chunk = None
        self.migrate_after_construct = True
        self.factor_stats = {"qr": 0, "svd": 0}
        self.quad = quad
        self.fac = 4 if quad else 2
        self.Nbvec = []
        self.tSample = 0.0
        self.tConstruct = 0.0
        self._op = None
        self._cache = {}
        self._tree = None
        if A is not None:
            self.A = A
            self.shape = A.shape
        if tree is not None:
            self.tree = tree
            self.perm = np.asarray(tree.perm_leaf, dtype=np.int64)
            self.Nb = int(tree.nleaves)
            self.shape = (len(self.perm), len(self.perm))
            self.nl = self.shape[0] // self.Nb
            self.L = int(tree.nlevels)

    @property
    def tree(self):
        return self._tree

    @tree.setter
    def tree(self, t):
        self._tree = t

    # ------------------------------------------------------------ lifetime
    def _free(self):
        if getattr(self, "_op", None) is not None and L._lib is not None:
            L.lib().slu_strong_destroy(self._op)
        self._op = None

    def __del__(self):
        try:
            if not getattr(self, "_is_view", False):
                self._free()
        except Exception:
            pass

    @property
    def T(self):
        """HBStorch_strong.py:1205-1209: a view applied in mode 'T' by @."""
        view = object.__new__(self.__class__)
        view.__dict__ = self.__dict__.copy()
        view._base = self       # keeps the operator alive; the view never frees it
        view._is_view = True
        view.mode = "T"
        return view

    # ------------------------------------------------------------ construct
    def construct(self, rk, Om, Psi, Y, Z, group_chunk=None, store_device=None,
                  empty_cache=True, fast=None, profile=True, profile_detail=True):
        """HBSMAT.construct (1000-1031) + constructHBS (1033-1107)."""
        if self.tree is None:
            raise ValueError("HBSMAT needs a tree (slabTree with level_adj_list)")
        tic = time.time()
        if group_chunk is not None:
            self.group_chunk = group_chunk
        if store_device is not None:
            self.store_device = store_device
        perm_d = torch.from_numpy(self.perm).to("cuda")
        ins = []
        for M in (Om, Psi, Y, Z):
            Md = dv.to_dev(M)
            ins.append(Md[perm_d].contiguous())
        N, s = ins[0].shape
        if N != self.shape[0] or any(t.shape != (N, s) for t in ins):
            raise ValueError("sketches must be N x s arrays of one shape")
        # levels with a far field, leaf first (1046-1103)
        levels = []
        for lvl in range(self.L - 1, -1, -1):
            adj = self.tree.level_adj_list[lvl]
            if not has_farfield(adj):
                break
            levels.append(adj)
        nb = np.array([len(a) for a in levels], dtype=np.int32)
        ptr, idx = [], []
        for adj in levels:
            cnt = 0
            ptr.append(0)
            for r, a in enumerate(adj):
                nf = sorted(set(a) | {r})
                idx.extend(nf)
                cnt += len(nf)
                ptr.append(cnt)
        ptr = np.array(ptr if ptr else [0], dtype=np.int32)
        idx = np.array(idx if idx else [0], dtype=np.int32)
        self._free()
        self._cache = {}
        h = ctypes.c_void_p()
        perm = np.ascontiguousarray(self.perm)
        L.check(L.lib().slu_strong_create(L.handle(), N, self.Nb, self.fac, L.host_ptr(perm),
                                          ctypes.byref(h)))
        self._op = h
        L.check(L.lib().slu_strong_compress(L.handle(), self._op, int(rk), int(s),
                                            *(L.ptr(t) for t in ins), len(levels),
                                            L.host_ptr(nb), L.host_ptr(ptr), L.host_ptr(idx)))
        L.sync()
        self.rk = rk
        self.nSamples = s
        self.Nbvec = [int(self._info(1, t)) for t in range(self._nlev())]
        self.factor_stats = {"qr": int(self._info(6)), "svd": 0}
        self.tConstruct = time.time() - tic

    def constructHBS(self, rk, Om_blk, Psi_blk, Y_blk, Z_blk, empty_cache=True):
        """HBSMAT.constructHBS (1033-1107) from (Nb, nl, s) block tensors
        already in tree order."""
        flat = lambda B: dv.to_dev(B).reshape(-1, B.shape[-1])
        ip = torch.from_numpy(np.argsort(self.perm)).to("cuda")
        self.construct(rk, *(flat(B)[ip] for B in (Om_blk, Psi_blk, Y_blk, Z_blk)))

    def to_device(self, device=None):
        """HBStorch_strong.py:1109-1119: the factors live on the device."""
        return self

    def print_profile(self, sort_by=None):
        print("strong HBS construct: %.3f s, %d near-field stacks factored"
              % (self.tConstruct, self.factor_stats["qr"]))

    # ------------------------------------------------------------ queries
    def _info(self, what, level=0):
        out = ctypes.c_longlong(0)
        L.check(L.lib().slu_strong_info(self._op, what, level, ctypes.byref(out)))
        return out.value

    def _nlev(self):
        return int(self._info(0))

    def _need(self):
        if self._op is None:
            raise ValueError("construct() first")

    def _export(self, what, level):
        key = (what, level)
        if key not in self._cache:
            Nb, b, r, nnz = (self._info(q, level) for q in (1, 2, 3, 4))
            if what in (0, 1):
                t = torch.empty((Nb, b, r), dtype=torch.float64, device="cuda")
            else:
                t = torch.empty((nnz, b, b), dtype=torch.float64, device="cuda")
            L.check(L.lib().slu_strong_export(L.handle(), self._op, what, level, L.ptr(t)))
            self._cache[key] = t
        return self._cache[key]

    @property
    def Umats(self):
        self._need()
        return [self._export(0, t) for t in range(self._nlev())]

    @property
    def Vmats(self):
        self._need()
        return [self._export(1, t) for t in range(self._nlev())]

    @property
    def Emats(self):
        self._need()
        out = []
        for t in range(self._nlev()):
            nnz = self._info(4, t)
            rc = np.zeros((nnz, 2), dtype=np.int32)
            L.check(L.lib().slu_strong_export(L.handle(), self._op, 3, t, L.host_ptr(rc)))
            out.append(BlockSparseE(self._export(2, t), torch.from_numpy(rc[:, 0].astype(np.int64)),
                                    torch.from_numpy(rc[:, 1].astype(np.int64)),
                                    int(self._info(1, t)), int(self._info(2, t))))
        nB = int(self._info(5))
        if ("B",) not in self._cache:
            B = torch.empty((nB, nB), dtype=torch.float64, device="cuda")
            L.check(L.lib().slu_strong_export(L.handle(), self._op, 4, 0, L.ptr(B)))
            self._cache[("B",)] = B
        nl = self._nlev()
        nblk = int(self._info(1, nl - 1)) // self.fac if nl else self.Nb
        out.append(DenseBase(self._cache[("B",)], nblk, nB // max(nblk, 1)))
        return out

    @property
    def nbytes(self):
        """HBSMAT.nbytes (993-998): bytes of U, V and E (the base included)."""
        self._need()
        return int(self._info(7))

    # ------------------------------------------------------------ apply
    def _dev_apply(self, X, trans=False):
        self._need()
        X = dv.as_2d(X).contiguous()
        Yo = torch.empty_like(X)
        L.check(L.lib().slu_strong_apply(L.handle(), self._op, int(trans), L.ptr(X), X.shape[1],
                                         L.ptr(Yo), Yo.shape[1], X.shape[1]))
        return Yo

    def matvec(self, v):
        return self.matmat(v)

    def rmatvec(self, v):
        return self.rmatmat(v)

    def matmat(self, v):
        """HBStorch_strong.py:1296-1297."""
        X, one = dv.prepare_rhs(v)
        return dv.finish(self._dev_apply(X, False), v, one)

    def rmatmat(self, v):
        """HBStorch_strong.py:1299-1300."""
        X, one = dv.prepare_rhs(v)
        return dv.finish(self._dev_apply(X, True), v, one)

    def __matmul__(self, v):
        """HBStorch_strong.py:1302-1303 (honours the .T view)."""
        X, one = dv.prepare_rhs(v)
        return dv.finish(self._dev_apply(X, self.mode == "T"), v, one)
