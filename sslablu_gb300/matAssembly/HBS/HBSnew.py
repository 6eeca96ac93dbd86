"""HBSMAT on the GPU -- drop-in for SslabLU matAssembly/HBS/HBSnew.py.

Same constructor, methods, attributes and return shapes as upstream
HBSnew.HBSMAT (HBSnew.py:65-416).  The operator's factors live on the device
inside libslablu; the upstream list attributes (Umats, Vmats, Dmats, Qlist,
Wlist, Rlist, Uulist) are exported to numpy on first access.

Sampling follows upstream exactly (HBSnew.py:211-227): the Gaussian sketches
are drawn from numpy's global RNG (Om then Psi, shape (N, s) with
s = 6rk+4nl+5 for quad trees and 4rk+2nl+5 for binary ones), so a seeded run
reproduces upstream's sketches; ``A.matmat`` / ``A.rmatmat`` of a device
operator run on the device, a caller's host LinearOperator is evaluated where
it lives.
"""
import ctypes
import time

import numpy as np
import torch

from ... import _dev as dv
from ... import _lib as L


def samples_for(rk, nl, fac):
    """Sample count of HBSnew.py:213-216."""
    return 6 * rk + 4 * nl + 5 if fac == 4 else 4 * rk + 2 * nl + 5


class HBSMAT:
    """HBS matrix (weak admissibility) with randomized construction and ULV solve."""

    # null-space rule of the compression (slu_hbs_set_null_space): 0 is
    # HBSnew.compute_UV's Q[:, -n:]
    _null_mode = 0

    def __init__(self, A=None, tree=None, quad=True):
        self.mode = "N"
        self._op = None
        self._cache = {}
        self.Nbvec = []
        self.NNvec = None
        self.quad = quad
        self.fac = 4 if quad else 2
        self.blockSolveTime = 0
        self.nullTime = 0
        self.setupTime = 0
        self.DTime = 0
        self.tSample = 0
        self.tConstruct = 0
        if A is not None:
            self.A = A
            self.shape = tuple(A.shape)
            self.dtype = getattr(A, "dtype", np.float64)
        if tree is not None:
            self.perm = np.asarray(tree.perm_leaf, dtype=np.int64)
            self.Nb = int(tree.nleaves)
            self.nl = self.A.shape[0] // self.Nb
            self.L = int(tree.nlevels)
            self.tree = tree

    # ------------------------------------------------------------ set-up
    def set_Nbvec(self, Nbvec):
        """HBSnew.py:119-124."""
        self.Nbvec = Nbvec
        self.Nb = Nbvec[0]
        self.nl = self.A.shape[0] // self.Nb
        self.L = len(Nbvec)
        self.perm = np.arange(self.A.shape[0], dtype=np.int64)

    def set_mats(self, Umats, Dmats, Vmats, Nbvec, fac=4):
        """HBSnew.py:125-133: load given factors (level 0 = leaves)."""
        N = int(Dmats[0].shape[0])
        Lv = len(Dmats)
        self.fac = fac
        self.quad = fac == 4
        self.Nb = Nbvec[0]
        self.Nbvec = list(Nbvec)
        self.L = Lv
        self.perm = np.arange(N, dtype=np.int64)
        self.shape = (N, N)
        self.dtype = np.float64
        self._new_op(N, Lv, None)
        for t in range(Lv):
            Nb = int(Nbvec[t])
            D = dv.to_dev(Dmats[t])
            n = D.shape[0] // Nb
            if t < Lv - 1:
                U = dv.to_dev(Umats[t])
                V = dv.to_dev(Vmats[t])
                k = U.shape[1]
            else:
                U = V = None
                k = 0
            L.check(L.lib().slu_hbs_set_level(L.handle(), self._op, t, Nb, n, k, L.ptr(U),
                                              L.ptr(V), L.ptr(D)))
        L.sync()
        self._refresh()
        return self

    def _new_op(self, N, Lv, perm):
        self._free()
        out = ctypes.c_void_p()
        p = None if perm is None else L.i64(perm)
        L.check(L.lib().slu_hbs_create(L.handle(), int(N), int(Lv), int(self.fac),
                                       None if p is None else L.host_ptr(p), ctypes.byref(out)))
        self._op = out
        self._perm_keep = p

    def _free(self):
        if getattr(self, "_op", None) is not None and L._lib is not None:
            L.lib().slu_hbs_destroy(self._op)
        self._op = None
        self._cache = {}

    def __del__(self):
        try:
            if getattr(self, "_owner", True):
                self._free()
        except Exception:
            pass

    @property
    def T(self):
        """HBSnew.py:134-139: transposed view sharing the factors."""
        view = object.__new__(self.__class__)
        view.__dict__ = self.__dict__.copy()
        view._owner = False
        view.mode = "T"
        return view

    # ------------------------------------------------------------ construction
    def construct(self, rk, compute_ULV=False):
        """HBSnew.py:140-145."""
        if compute_ULV:
            self.constructHBS_ULV(rk)
        else:
            self.constructHBS(rk)

    def _sketches(self, rk, rng=None):
        """Om, Psi (N x s) from numpy's global RNG (upstream's draws), a numpy
        Generator, or a torch.Generator on the device (drawn there: no host
        draws and no upload; not upstream's stream)."""
        s = samples_for(rk, self.nl, self.fac)
        self.nSamples = s
        if isinstance(rng, torch.Generator):
            dev = rng.device if rng.device.type == "cuda" else torch.device("cuda")
            Om = torch.randn((self.shape[1], s), generator=rng, dtype=torch.float64, device=dev)
            Psi = torch.randn((self.shape[0], s), generator=rng, dtype=torch.float64, device=dev)
            return Om, Psi
        if rng is None:
            Om = np.random.standard_normal(size=(self.shape[1], s))
            Psi = np.random.standard_normal(size=(self.shape[0], s))
        else:
            Om = rng.standard_normal(size=(self.shape[1], s))
            Psi = rng.standard_normal(size=(self.shape[0], s))
        return Om, Psi

    def _sample(self, Om, Psi):
        """Y = A Om', Z = A^T Psi' with Om'[perm] = Om, rows back in tree order."""
        perm_d = torch.from_numpy(self.perm).to("cuda")
        Omd = dv.to_dev(Om)
        Psid = dv.to_dev(Psi)
        Omp = torch.empty_like(Omd)
        Omp[perm_d] = Omd
        Psip = torch.empty_like(Psid)
        Psip[perm_d] = Psid
        Y = dv.dev_apply(self.A, Omp, False)[perm_d].contiguous()
        Z = dv.dev_apply(self.A, Psip, True)[perm_d].contiguous()
        return Omd, Psid, Y, Z

    def compress_from_sketches(self, rk, Om, Psi, Y, Z, compute_ULV=True):
        """Compression from given tree-ordered sketches and samples (N x s
        arrays); the sampling-free entry of HBStorch.HBSMAT.construct
        (HBStorch.py:163-168) with HBSnew's algorithm."""
        tic = time.time()
        Omd, Psid, Yd, Zd = (dv.to_dev(x) for x in (Om, Psi, Y, Z))
        s = Omd.shape[1]
        self.nSamples = s
        N = self.shape[0]
        self._new_op(N, self.L, self.perm)
        L.check(L.lib().slu_hbs_set_null_space(self._op, int(self._null_mode)))
        L.check(L.lib().slu_hbs_compress(L.handle(), self._op, int(self.Nb), int(rk), int(s),
                                         L.ptr(Omd), L.ptr(Psid), L.ptr(Yd), L.ptr(Zd),
                                         int(bool(compute_ULV))))
        L.sync()
        self._refresh()
        self.Nbvec += [int(x) for x in self._levels[:, 0]]
        self.tCompress = time.time() - tic
        return self

    def constructHBS(self, rk):
        """HBSnew.py:147-210 (upstream draws from an unseeded default_rng)."""
        tic = time.time()
        Om, Psi = self._sketches(rk, np.random.default_rng())
        Omd, Psid, Y, Z = self._sample(Om, Psi)
        self.tSample += time.time() - tic
        self.compress_from_sketches(rk, Omd, Psid, Y, Z, compute_ULV=False)

    def constructHBS_ULV(self, rk):
        """HBSnew.py:211-295."""
        Om, Psi = self._sketches(rk)
        self.construct_drawn(rk, Om, Psi)

    def construct_drawn(self, rk, Om, Psi, compute_ULV=True):
        """constructHBS_ULV with sketches already drawn (by _sketches): the
        sampling Y = A Om, Z = A^T Psi and the compression, on torch's current
        stream.  Lets a caller draw the sketches of several operators in the
        upstream order and construct them concurrently."""
        tic = time.time()
        Omd, Psid, Y, Z = self._sample(Om, Psi)
        self.tSample += time.time() - tic
        self.compress_from_sketches(rk, Omd, Psid, Y, Z, compute_ULV=compute_ULV)

    def compute_ULV(self):
        """HBSnew.py:390-391."""
        L.check(L.lib().slu_ulv_factor(L.handle(), self._op))
        L.sync()
        self._refresh()

    # ------------------------------------------------------------ metadata
    def _refresh(self):
        self._cache = {}
        Lv = ctypes.c_int()
        N = ctypes.c_int()
        ns = ctypes.c_int()
        lev = np.zeros(4 * 64, dtype=np.int32)
        NN = np.zeros(65, dtype=np.int64)
        L.check(L.lib().slu_hbs_info(self._op, ctypes.byref(Lv), ctypes.byref(N),
                                     L.host_ptr(lev), L.host_ptr(NN), ctypes.byref(ns)))
        self.L = Lv.value
        self._levels = lev[:4 * Lv.value].reshape(Lv.value, 4).astype(np.int64)
        self.NNvec = NN[:Lv.value + 1].copy()

    def _export(self, what, level):
        key = (what, level)
        if key not in self._cache:
            cnt = ctypes.c_size_t()
            L.check(L.lib().slu_hbs_export(L.handle(), self._op, what, level, None, 0,
                                           ctypes.byref(cnt)))
            buf = torch.empty(cnt.value, dtype=torch.float64, device="cuda")
            L.check(L.lib().slu_hbs_export(L.handle(), self._op, what, level, L.ptr(buf),
                                           cnt.value, None))
            Nb, n, k, nu = (int(x) for x in self._levels[level])
            cols = {0: k, 1: k, 2: n, 3: n, 4: n, 5: n}.get(what)
            if what == 6:
                cols = k if level < self.L - 1 else n
            arr = dv.to_host(buf)
            self._cache[key] = arr.reshape(-1, cols) if arr.size else np.zeros((0, cols))
        return self._cache[key]

    def _lists(self, what, levels):
        return [self._export(what, t) for t in levels]

    @property
    def Umats(self):
        return self._lists(0, range(self.L - 1))

    @property
    def Vmats(self):
        return self._lists(1, range(self.L - 1))

    @property
    def Dmats(self):
        return self._lists(2, range(self.L))

    @property
    def Qlist(self):
        return self._lists(3, range(self.L))

    @property
    def Wlist(self):
        return [self._export(4, t) if t < self.L - 1 else None for t in range(self.L)]

    @property
    def Rlist(self):
        return self._lists(5, range(self.L))

    @property
    def Uulist(self):
        lv = [t for t in range(self.L) if self._export_count(6, t) > 0]
        return self._lists(6, lv)

    def _export_count(self, what, level):
        cnt = ctypes.c_size_t()
        L.check(L.lib().slu_hbs_export(L.handle(), self._op, what, level, None, 0,
                                       ctypes.byref(cnt)))
        return cnt.value

    @property
    def nbytes(self):
        """HBSnew.py:296-302 (U, V, D bytes)."""
        out = ctypes.c_size_t()
        L.check(L.lib().slu_hbs_nbytes(self._op, 0, ctypes.byref(out)))
        return out.value

    # ------------------------------------------------------------ apply / solve
    def _dev_apply(self, X, trans=False):
        X = dv.as_2d(X).contiguous()
        Y = torch.empty_like(X)
        L.check(L.lib().slu_hbs_apply(L.handle(), self._op, int(trans), L.ptr(X), X.shape[1],
                                      L.ptr(Y), Y.shape[1], X.shape[1]))
        return Y

    def _dev_solve(self, X, trans=False):
        # out of place: no copy of the right-hand sides
        X = dv.as_2d(X).contiguous()
        Y = torch.empty_like(X)
        L.check(L.lib().slu_ulv_solve_into(L.handle(), self._op, L.ptr(X), X.shape[1],
                                           L.ptr(Y), Y.shape[1], X.shape[1], int(trans)))
        return Y

    def matvec(self, v):
        return self.matmat(v)

    def rmatvec(self, v):
        return self.rmatmat(v)

    def matmat(self, v):
        """HBSnew.py:308-328."""
        X, one = dv.prepare_rhs(v)
        return dv.finish(self._dev_apply(X, False), v, one)

    def rmatmat(self, v):
        """HBSnew.py:330-350."""
        X, one = dv.prepare_rhs(v)
        return dv.finish(self._dev_apply(X, True), v, one)

    def __matmul__(self, v):
        """HBSnew.py:352-388 (honours the .T view)."""
        if self.mode not in ("N", "T"):
            raise ValueError("mode not recognized")
        X, one = dv.prepare_rhs(v)
        return dv.finish(self._dev_apply(X, self.mode == "T"), v, one)

    def solve(self, b, mode="N", out=None):
        """HBSnew.py:393-416.  Beyond upstream: a pinned host tensor b (2-D,
        float64, contiguous) is solved without staging copies --
        the first solve step reads b from host memory and the last writes the
        solution into ``out`` (a pinned host tensor of b's shape, allocated
        when None) -- and the call returns once ``out`` holds the result."""
        if mode not in ("N", "T"):
            raise NotImplementedError("mode not recognized")
        if (isinstance(b, torch.Tensor) and not b.is_cuda and b.is_pinned()
                and b.dim() == 2 and b.dtype == torch.float64 and b.is_contiguous()):
            if out is None:
                out = torch.empty(b.shape, dtype=torch.float64, pin_memory=True)
            if out.shape != b.shape or not out.is_pinned() or not out.is_contiguous():
                raise ValueError("out must be a contiguous pinned host tensor of b's shape")
            c = b.shape[1]
            L.check(L.lib().slu_ulv_solve_into(L.handle(), self._op, L.ptr(b), c, L.ptr(out), c,
                                               c, int(mode == "T")))
            torch.cuda.current_stream().synchronize()
            return out
        X, one = dv.prepare_rhs(b)
        return dv.finish(self._dev_solve(X, mode == "T"), b, one)

    def solve_plan(self, b, out=None, mode="N"):
        """Beyond upstream: the solve of b into out captured once (a CUDA
        graph over the library's step launches, with the launch plans tuned
        for b's column count at this point) for repeated solves through the
        same buffers -- a serving loop's staging blocks, a time-stepping
        loop.  b and out are 2-D contiguous float64 tensors of one shape,
        both on the device or both in pinned host memory (out allocated
        like b when None).  ``plan()`` solves what b holds into out and
        returns out: for host buffers once the result is there, for device
        buffers as soon as the solve is queued on the current stream.  The
        plan refuses to run once this operator is refactored."""
        if mode not in ("N", "T"):
            raise NotImplementedError("mode not recognized")
        if not isinstance(b, torch.Tensor) or b.dim() != 2 or b.dtype != torch.float64 \
                or not b.is_contiguous():
            raise ValueError("b must be a contiguous 2-D float64 tensor")
        host = not b.is_cuda
        if host and not b.is_pinned():
            raise ValueError("a host b must be pinned")
        if out is None:
            out = torch.empty(b.shape, dtype=torch.float64,
                              **({"pin_memory": True} if host else {"device": b.device}))
        if out.shape != b.shape or not out.is_contiguous() or out.dtype != torch.float64 \
                or out.is_cuda == host or (host and not out.is_pinned()):
            raise ValueError("out must be a contiguous float64 tensor of b's shape, "
                             "where b is (device, or pinned host)")
        if b.shape[0] != self.shape[0]:
            raise ValueError("b has %d rows, the operator %d" % (b.shape[0], self.shape[0]))
        return SolvePlan(self, b, out, mode == "T", host)

    def autotune(self, nrhs, precision="f64", reps=9):
        """Times the launches of a mode-N solve of `nrhs` columns under a set
        of launch-plan caps and keeps the fastest per launch for later solves
        of that width (results unchanged).  precision 'f64' (solve) or
        'dfloat' (solve_dfloat).  Returns the caps chosen per launch as
        (target CTAs per SM, row-slice floor, column cap) triples."""
        code = {"f64": 0, "dfloat": 2}[precision]
        cap = 256
        knobs = (ctypes.c_int * (3 * cap))()
        n = ctypes.c_int()
        L.check(L.lib().slu_ulv_autotune(L.handle(), self._op, int(nrhs), code, int(reps), knobs,
                                         cap, ctypes.byref(n)))
        return [tuple(knobs[3 * i:3 * i + 3]) for i in range(min(n.value, cap))]

    # ------------------------------------------------------------ mixed precision
    def solve_dfloat(self, b):
        """Mode-N solve in double-float arithmetic on the float32 units (the
        fused sweep of solve(), every factor a float32 pair hi + lo): about
        1e-14 relative accuracy without refinement."""
        X, one = dv.prepare_rhs(b)
        B = dv.as_2d(X).clone().contiguous()
        L.check(L.lib().slu_ulv_solve_dfloat(L.handle(), self._op, L.ptr(B), B.shape[1],
                                             B.shape[1]))
        return dv.finish(B, b, one)

    def solve_ozaki(self, b, mode="N"):
        """Solve on the tensor cores (slu_ulv_solve_ozaki): every step
        product as bfloat16 tcgen05 products of error-free base-256 digit
        splits of operator and vector (Ozaki scheme), float64-level accuracy;
        double-float vectors between steps.  mode 'T' solves with A^T (the
        transposed steps of the float64 mode-T solve)."""
        if mode not in ("N", "T"):
            raise ValueError("mode not recognized")
        X, one = dv.prepare_rhs(b)
        X = dv.as_2d(X).contiguous()
        Y = torch.empty_like(X)
        L.check(L.lib().slu_ulv_solve_ozaki(L.handle(), self._op, L.ptr(X), X.shape[1],
                                            L.ptr(Y), Y.shape[1], X.shape[1], int(mode == "T")))
        return dv.finish(Y, b, one)

    def apply_ozaki(self, x, trans=False):
        """A x (A^T x with trans) on the tensor cores (slu_hbs_apply_ozaki):
        the apply steps as digit-split bfloat16 products, float64-level
        accuracy."""
        X, one = dv.prepare_rhs(x)
        X = dv.as_2d(X).contiguous()
        Y = torch.empty_like(X)
        L.check(L.lib().slu_hbs_apply_ozaki(L.handle(), self._op, L.ptr(X), X.shape[1],
                                            L.ptr(Y), Y.shape[1], X.shape[1], int(bool(trans))))
        return dv.finish(Y, x, one)

    def solve_refined(self, b, tol=1e-10, maxit=10, inner="dfloat"):
        """Mixed-precision solve: ULV sweeps on the float32 units
        (``inner='dfloat'``: double-float, usually one iteration;
        ``'float32'``: plain float32, two or three) or on the tensor cores
        (``'tensor'``: digit-split bfloat16 products, with the residual from
        the tensor-core apply) corrected by float64-accurate residuals of
        this operator until ||b - A x|| / ||b|| <= tol per column.  Returns
        (x, iterations, worst relative residual)."""
        modes = {"float32": 0, "dfloat": 1, "tensor": 2}
        if inner not in modes:
            raise ValueError("inner must be 'dfloat', 'float32' or 'tensor'")
        L.check(L.lib().slu_hbs_set_refine_inner(self._op, modes[inner]))
        B, one = dv.prepare_rhs(b)
        X = torch.empty_like(B)
        it = ctypes.c_int()
        rr = ctypes.c_double()
        L.check(L.lib().slu_refine(L.handle(), self._op, L.ptr(B), B.shape[1], L.ptr(X),
                                   X.shape[1], B.shape[1], float(tol), int(maxit),
                                   ctypes.byref(it), ctypes.byref(rr)))
        return dv.finish(X, b, one), it.value, rr.value


class SolvePlan:
    """A captured solve of HBSMAT.solve_plan (slu_ulv_solve_plan_*)."""

    def __init__(self, H, b, out, trans, host):
        c = b.shape[1]
        self.b, self.out, self._H = b, out, H     # the plan reads and writes these
        self._host = host
        self._launch = L.lib().slu_ulv_solve_plan_launch
        p = ctypes.c_void_p()
        L.check(L.lib().slu_ulv_solve_plan_create(L.handle(), H._op, L.ptr(b), c, L.ptr(out), c,
                                                  c, int(trans), ctypes.byref(p)))
        self._p = p

    def __call__(self):
        L.check(self._launch(L.handle(), self._p, int(self._host)))
        return self.out

    def close(self):
        if getattr(self, "_p", None) is not None and L._lib is not None:
            L.lib().slu_ulv_solve_plan_destroy(self._p)
        self._p = None

    def __del__(self):
        self.close()
