"""HBS block-tridiagonal solvers on the GPU -- drop-in for SslabLU
direct_solve/omsdirectsolveHBS.py.

    id_op, dense_to_linop, _linop_from_mat,
    STS_linop, RB_linop, Sprime_Linop, Dprime_Linop      (omsdirectsolveHBS.py:12-179)
    ThomasSolverHBS(m, rk, cyclic=False)                 (189-351)
    RedBlackSolverHBS(m, rk, tree, quad, cyclic=False)   (359-558)

Every implicit operator applies on the device (``_dev_apply`` / ``_dev_solve``
on float64 CUDA tensors) and also offers the scipy-style ``matmat`` /
``rmatmat`` / ``solve`` for host callers.  Each Schur complement is
compressed by the GPU HBSMAT with the upstream sketch order (Om then Psi
from numpy's global RNG per compression, compressions in upstream's loop
order), so seeded runs reproduce upstream's sketches.

Beyond upstream: solve accepts (N,) and (N, nrhs) right-hand sides (upstream
RB-HBS is 1-D only, omsdirectsolveHBS.py:503); the compressions of one
red-black level, which are independent, run concurrently on worker streams
(sketches still drawn in upstream's order on the calling thread).
"""
import concurrent.futures as cf
import os
import threading

import numpy as np
import torch

from .. import _dev as dv
from .. import _lib as L
from ..matAssembly.HBS import HBSnew
from .omsdirectsolve import DirectSolver


# ---------------------------------------------------------------------------
# operator helpers
# ---------------------------------------------------------------------------
def _refine(solver, rhs, tol, maxit):
    """Iterative refinement of solver.solve against solver.apply (the exact
    block-tridiagonal operator, float64): x += solve(b - A x) until every
    column's relative residual is at most tol.  Returns (x, solves, relres)."""
    B, one = dv.prepare_rhs(rhs)
    bn = torch.linalg.norm(B, dim=0).clamp_min(np.finfo(np.float64).tiny)
    X = solver.solve(B)
    it, rel = 1, float("inf")
    while True:
        R = B - solver.apply(X)
        rel = float((torch.linalg.norm(R, dim=0) / bn).max())
        if rel <= tol or it >= maxit:
            break
        X = X + solver.solve(R)
        it += 1
    return dv.finish(X, rhs, one), it, rel


class _DevOp:
    """Device operator with the scipy LinearOperator call surface."""

    dtype = np.float64
    tree = None
    quad = None

    def _host_call(self, v, trans):
        X, one = dv.prepare_rhs(v)
        return dv.finish(self._dev_apply(X, trans), v, one)

    def matmat(self, v):
        return self._host_call(v, False)

    def rmatmat(self, v):
        return self._host_call(v, True)

    matvec = matmat
    rmatvec = rmatmat

    def __matmul__(self, v):
        return self.matmat(v)

    def solve(self, v, mode="N"):
        X, one = dv.prepare_rhs(v)
        return dv.finish(self._dev_solve(X, mode == "T"), v, one)


class id_op(_DevOp):
    """Identity operator (omsdirectsolveHBS.py:12-20)."""

    def __init__(self, n, dtype=np.float64):
        self.shape = (n, n)

    def _dev_apply(self, X, trans=False):
        return dv.as_2d(X).clone()

    def _dev_solve(self, X, trans=False):
        return dv.as_2d(X).clone()


class _DenseOp(_DevOp):
    def __init__(self, A):
        self._d = dv.DenseDev(A)
        self.shape = self._d.shape
        self.tree = None
        self.quad = None

    def _dev_apply(self, X, trans=False):
        return self._d._dev_apply(X, trans)

    def _dev_solve(self, X, trans=False):
        return self._d._dev_solve(X, trans)


def dense_to_linop(A):
    """omsdirectsolveHBS.py:22-36: dense matrix as an operator with .solve."""
    return _DenseOp(A)


def _linop_from_mat(A):
    """omsdirectsolveHBS.py:38-54."""
    return _DenseOp(A)


class STS_linop(_DevOp):
    """-Sl T^{-1} Sr (omsdirectsolveHBS.py:162-179)."""

    def __init__(self, Sl, T, Sr):
        self.Sl, self.T, self.Sr = Sl, T, Sr
        self.shape = (T.shape[0], T.shape[1])

    def _dev_apply(self, X, trans=False):
        if not trans:
            return -dv.dev_apply(self.Sl, dv.dev_solve(self.T, dv.dev_apply(self.Sr, X)))
        return -dv.dev_apply(self.Sr, dv.dev_solve(self.T, dv.dev_apply(self.Sl, X, True), True),
                             True)


class RB_linop(_DevOp):
    """Ti - SiPi tp^{-1} smp - SiMi tm^{-1} spm (omsdirectsolveHBS.py:77-106);
    tm, tp, smp, spm may be None at the boundary."""

    def __init__(self, Ti, tm, tp, SiPi, SiMi, smp, spm):
        self.Ti, self.tm, self.tp = Ti, tm, tp
        self.SiPi, self.SiMi, self.smp, self.spm = SiPi, SiMi, smp, spm
        self.shape = (Ti.shape[0], Ti.shape[1])

    def _dev_apply(self, X, trans=False):
        X = dv.as_2d(X)
        if not trans:
            r = dv.dev_apply(self.Ti, X).clone()
            if self.tp is not None:
                r -= dv.dev_apply(self.SiPi, dv.dev_solve(self.tp, dv.dev_apply(self.smp, X)))
            if self.tm is not None:
                r -= dv.dev_apply(self.SiMi, dv.dev_solve(self.tm, dv.dev_apply(self.spm, X)))
        else:
            r = dv.dev_apply(self.Ti, X, True).clone()
            if self.tp is not None:
                r -= dv.dev_apply(self.smp, dv.dev_solve(self.tp, dv.dev_apply(self.SiPi, X, True),
                                                         True), True)
            if self.tm is not None:
                r -= dv.dev_apply(self.spm, dv.dev_solve(self.tm, dv.dev_apply(self.SiMi, X, True),
                                                         True), True)
        return r


class _SumOp(_DevOp):
    """The sum of linear operators (both orientations)."""

    def __init__(self, ops):
        self.ops = ops
        self.shape = tuple(ops[0].shape)

    def _dev_apply(self, X, trans=False):
        X = dv.as_2d(X)
        r = dv.dev_apply(self.ops[0], X, trans).clone()
        for op in self.ops[1:]:
            r += dv.dev_apply(op, X, trans)
        return r


class Sprime_Linop(_DevOp):
    """I - Sl Sp^{-1} Sr, or I - Sl Sr when id=True (omsdirectsolveHBS.py:108-141)."""

    def __init__(self, Sl, Sprime_prev, Sr, id=False):
        self.Sl, self.Sp, self.Sr, self.ident = Sl, Sprime_prev, Sr, id
        self.shape = (Sl.shape[0], Sr.shape[1])

    def _dev_apply(self, X, trans=False):
        X = dv.as_2d(X)
        if not trans:
            inner = dv.dev_apply(self.Sr, X)
            if not self.ident:
                inner = dv.dev_solve(self.Sp, inner)
            return X - dv.dev_apply(self.Sl, inner)
        inner = dv.dev_apply(self.Sl, X, True)
        if not self.ident:
            inner = dv.dev_solve(self.Sp, inner, True)
        return X - dv.dev_apply(self.Sr, inner, True)


class Dprime_Linop(_DevOp):
    """D - A Dprev^{-1} B (omsdirectsolveHBS.py:143-160)."""

    def __init__(self, D, A, B, Dprev):
        self.D, self.A, self.B, self.Dprev = D, A, B, Dprev
        self.shape = (D.shape[0], D.shape[1])

    def _dev_apply(self, X, trans=False):
        X = dv.as_2d(X)
        if not trans:
            return dv.dev_apply(self.D, X) - dv.dev_apply(
                self.A, dv.dev_solve(self.Dprev, dv.dev_apply(self.B, X)))
        return dv.dev_apply(self.D, X, True) - dv.dev_apply(
            self.B, dv.dev_solve(self.Dprev, dv.dev_apply(self.A, X, True), True), True)


def _shape0(op):
    return int(op.shape[0])


# concurrent compressions (worker threads, one stream each), shared by every
# factorisation of the process; SSLABLU_LEVEL_WORKERS sets the count
_LEVEL_WORKERS = max(1, int(os.environ.get("SSLABLU_LEVEL_WORKERS", "12")))
_POOL = None
_POOL_LOCK = threading.Lock()
_TLS = threading.local()


def _blocking_worker():
    """Initializer of factorisation worker threads: their host waits (the
    library's and _wait's) sleep instead of spinning, so a dozen or more
    waiting workers leave the host cores to the ones launching work."""
    L.lib().slu_set_blocking_waits(1)


def _wait(stream):
    """Wait for the work queued on ``stream`` so far, asleep (blocking-sync
    event) rather than spinning."""
    ev = torch.cuda.Event(blocking=True)
    ev.record(stream)
    ev.synchronize()


def _level_pool():
    """The worker threads of the level compressions, made once per process:
    each keeps one stream per device (and so one library handle and scratch
    arena) for every factorisation, however many systems are factored."""
    global _POOL
    with _POOL_LOCK:
        if _POOL is None:
            _POOL = cf.ThreadPoolExecutor(max_workers=_LEVEL_WORKERS,
                                          initializer=_blocking_worker)
        return _POOL


def _worker_stream(dev):
    streams = getattr(_TLS, "streams", None)
    if streams is None:
        streams = _TLS.streams = {}
    if dev not in streams:
        streams[dev] = torch.cuda.Stream(dev)
    return streams[dev]


# ---------------------------------------------------------------------------
# HBS Thomas, omsdirectsolveHBS.py:189-351
# ---------------------------------------------------------------------------
class ThomasSolverHBS(DirectSolver):
    """Block Thomas with identity diagonal; every S'_i = I - S_{i,i-1}
    S'_{i-1}^{-1} S_{i-1,i} compressed to HBS and ULV-factored on the GPU."""

    def __init__(self, m, rk, cyclic=False):
        super().__init__(m, cyclic)
        self.rk = rk
        self.solve_method = None

    def factorize(self, S_rk_list, T=None):
        if T is not None:
            self.factorize_with_diag(S_rk_list, T)
            self.solve_method = "diag"
        else:
            self.factorize_id_diag(S_rk_list)
            self.solve_method = "id_diag"

    def factorize_id_diag(self, S_rk_list):
        """omsdirectsolveHBS.py:202-245."""
        rk = self.rk
        m = _shape0(S_rk_list[0][0])
        n = len(S_rk_list) - 1
        I = id_op(m)
        Sl = [S_rk_list[i][0] for i in range(1, n + 1)]
        Sr = [S_rk_list[i][-1] for i in range(n)]
        Sp = [I]
        for i in range(1, n + 1):
            if i == 1:
                op = Sprime_Linop(Sl[0], I, Sr[0], id=True)
            else:
                op = Sprime_Linop(Sl[i - 1], Sp[i - 1], Sr[i - 1])
            h = HBSnew.HBSMAT(op, Sl[i - 1].tree, Sl[i - 1].quad)
            h.construct(rk, compute_ULV=True)
            Sp.append(h)
        self.A, self.B, self.C = Sl, Sp, Sr

    def factorize_with_diag(self, AB_list, D_list):
        """omsdirectsolveHBS.py:247-273 (upstream passes the tree in the wrong
        argument slot at 267; here the tree of D_list[i] is used)."""
        m = _shape0(D_list[0])
        n = len(D_list) - 1
        A = [AB_list[i][0] for i in range(n)]
        C = [AB_list[i][-1] for i in range(n)]
        B = [D_list[0]]
        for i in range(1, n + 1):
            op = Dprime_Linop(D_list[i], A[i - 1], C[i - 1], B[-1])
            h = HBSnew.HBSMAT(op, D_list[i].tree, D_list[i].quad)
            h.construct(self.rk, compute_ULV=True)
            B.append(h)
        self.A, self.B, self.C = A, B, C

    def _indices(self, glob_target_dofs, count):
        m = self.m
        if glob_target_dofs is None:
            return [slice(l * m, (l + 1) * m) for l in range(count)]
        return [slice(r.start, r.stop) if isinstance(r, range) else r for r in glob_target_dofs]

    def solve(self, rhs, glob_target_dofs=None):
        d, one = dv.prepare_rhs(rhs)
        d = d.clone()
        if self.solve_method == "id_diag":
            Sl, Sp, Sr = self.A, self.B, self.C
            n = len(Sl)
            idx = self._indices(glob_target_dofs, n + 1)
            for i in range(1, n + 1):                                  # 300-304
                if i == 1:
                    d[idx[i]] -= dv.dev_apply(Sl[0], d[idx[0]])
                else:
                    d[idx[i]] -= dv.dev_apply(Sl[i - 1], dv.dev_solve(Sp[i - 1], d[idx[i - 1]]))
            x = torch.zeros_like(d)
            x[idx[n]] = dv.dev_solve(Sp[n], d[idx[n]])                # 307
            for i in range(n - 1, 0, -1):
                x[idx[i]] = dv.dev_solve(Sp[i], d[idx[i]] - dv.dev_apply(Sr[i], x[idx[i + 1]]))
            x[idx[0]] = d[idx[0]] - dv.dev_apply(Sr[0], x[idx[1]])
        elif self.solve_method == "diag":
            A, B, C = self.A, self.B, self.C
            n = len(A)
            idx = self._indices(glob_target_dofs, n + 1)
            for i in range(1, n + 1):                                  # 330-331
                d[idx[i]] -= dv.dev_apply(A[i - 1], dv.dev_solve(B[i], d[idx[i - 1]]))
            x = torch.zeros_like(d)
            x[idx[n]] = dv.dev_solve(B[n], d[idx[n]])
            for i in range(n - 1, 0, -1):
                x[idx[i]] = dv.dev_solve(B[i], d[idx[i]] - dv.dev_apply(C[i], x[idx[i + 1]]))
            x[idx[0]] = dv.dev_solve(B[0], d[idx[0]] - dv.dev_apply(C[0], x[idx[1]]))
        else:
            raise ValueError("Factorization not set")
        return dv.finish(x, rhs, one)

    def apply(self, x):
        """Beyond upstream: the identity-diagonal block-tridiagonal operator
        the solver was factored from (factorize without T), applied with the
        given couplings in float64."""
        if self.solve_method != "id_diag":
            raise NotImplementedError("apply needs the identity-diagonal factorisation")
        X, one = dv.prepare_rhs(x)
        m, n = self.m, len(self.A)
        Y = X.clone()
        for i in range(n + 1):
            blk = slice(i * m, (i + 1) * m)
            if i > 0:
                Y[blk] += dv.dev_apply(self.A[i - 1], X[(i - 1) * m:i * m])
            if i < n:
                Y[blk] += dv.dev_apply(self.C[i], X[(i + 1) * m:(i + 2) * m])
        return dv.finish(Y, x, one)

    def solve_refined(self, rhs, tol=1e-10, maxit=5):
        """Beyond upstream: solve() refined against apply() (float64
        residuals with the exact couplings), which removes the error of the
        HBS compressions.  Returns (x, solves, worst column relative
        residual)."""
        return _refine(self, rhs, tol, maxit)


# ---------------------------------------------------------------------------
# HBS red-black, omsdirectsolveHBS.py:359-558
# ---------------------------------------------------------------------------
class RedBlackSolverHBS(DirectSolver):
    """Cyclic reduction where each new diagonal block and coupling of every
    level is an HBS compression (+ ULV for the diagonal) of an implicit
    operator, all on the GPU."""

    def __init__(self, m, rk, tree, quad, cyclic=False, sketch_seed=None):
        super().__init__(m, cyclic)
        self.rk = rk
        self.tree = tree
        self.quad = quad
        # beyond upstream: with sketch_seed the compressions draw their
        # sketches on the device from one seeded torch generator (no host
        # draws, no uploads); by default numpy's global RNG in upstream's
        # order, so seeded runs reproduce upstream's sketches
        self._gen = None
        if sketch_seed is not None:
            self._gen = torch.Generator(device="cuda")
            self._gen.manual_seed(int(sketch_seed))

    def _hbs(self, linop, rk=None):
        """omsdirectsolveHBS.py:383-391."""
        h = HBSnew.HBSMAT(linop, self.tree, self.quad)
        h.construct(self.rk if rk is None else rk, compute_ULV=True)
        return h

    def _hbs_many(self, linops, rk):
        """_hbs of every operator of a level: sketches drawn here in list
        order (upstream's draw order), then sampling + compression + ULV of
        all of them concurrently, one worker stream each."""
        rk = self.rk if rk is None else rk
        jobs = []
        for op in linops:
            h = HBSnew.HBSMAT(op, self.tree, self.quad)
            jobs.append((h,) + h._sketches(rk, self._gen))
        if len(jobs) == 1:
            h, Om, Psi = jobs[0]
            h.construct_drawn(rk, Om, Psi)
            return [h]
        dev = torch.cuda.current_device()
        _wait(torch.cuda.current_stream(dev))   # inputs ready for every stream

        def run(job):
            h, Om, Psi = job
            torch.cuda.set_device(dev)
            st = _worker_stream(dev)
            with torch.cuda.stream(st):
                h.construct_drawn(rk, Om, Psi)
            _wait(st)
            return h

        return list(_level_pool().map(run, jobs))

    def factorize(self, S_rk_list, T=None):
        """omsdirectsolveHBS.py:397-430."""
        m = _shape0(S_rk_list[0][0])
        nS = len(S_rk_list)
        if not (nS & (nS - 1) == 0 and nS != 0):
            raise ValueError("Number of slabs must be a power of 2.")
        SiM = [s[0] for s in S_rk_list]
        SiP = [s[-1] for s in S_rk_list]
        if not self.cyclic:   # periodic: SiM[0] and SiP[-1] are the wrap couplings
            SiM[0] = _linop_from_mat(np.zeros((m, m)))
            SiP[-1] = _linop_from_mat(np.zeros((m, m)))
        if T is None:
            T = [id_op(m) for _ in range(nS)]
        RB = [(SiM, T, T, SiP)]
        l = nS
        while l > 1:
            RB.append(self._build_level(m, l, RB[-1], self.rk))
            l //= 2
        self.nSlabs = nS
        self.RB = RB

    def _build_level(self, m, nS, lev, rk):
        """omsdirectsolveHBS.py:436-483 (same compression order)."""
        SiM, T, Th, SiP = lev
        B_lin = []
        cyc = self.cyclic
        for i in range(0, nS, 2):
            spm = SiP[(i - 1) % nS] if (i > 0 or cyc) else None
            smp = SiM[(i + 1) % nS] if (i < nS - 1 or cyc) else None
            tm = Th[(i - 1) % nS] if spm is not None else None
            tp = Th[(i + 1) % nS] if smp is not None else None
            B_lin.append(RB_linop(T[i], tm, tp, SiP[i], SiM[i], smp, spm))
        A_lin = [STS_linop(SiM[i], Th[(i - 1) % nS], SiM[(i - 1) % nS]) for i in range(0, nS, 2)]
        C_lin = [STS_linop(SiP[i], Th[(i + 1) % nS], SiP[(i + 1) % nS]) for i in range(0, nS, 2)]
        if cyc and nS == 2:
            # one periodic block left: its couplings A, C act on the block
            # itself, so the diagonal to compress is B + A + C (the dense
            # solver's B_0 += A_0 + C_0, omsdirectsolve.py:326-327; upstream's
            # HBS solver leaves A and C out of its last block)
            B_lin = [_SumOp([B_lin[0], A_lin[0], C_lin[0]])]
        # upstream compresses T_new, then A, then C (one sketch pair each, in
        # that order); the compressions are independent of one another
        hs = self._hbs_many(B_lin + A_lin + C_lin, rk)
        k = len(B_lin)
        T_new, A, C = hs[:k], hs[k:2 * k], hs[2 * k:]
        return (A, B_lin, T_new, C)

    def solve(self, rhs):
        """omsdirectsolveHBS.py:489-558 (multi-column right-hand sides allowed)."""
        m, RB = self.m, self.RB
        v0, one = dv.prepare_rhs(rhs)
        vs = [v0.clone()]
        for l in range(len(RB) - 1):                                   # forward reduction
            SiM, _, Th, SiP = RB[l]
            nS = len(SiM)
            nR = nS // 2
            vp = vs[-1]
            vn = torch.empty((m * nR, vp.shape[1]), dtype=vp.dtype, device=vp.device)
            for j in range(nR):
                i = 2 * j
                c = vp[i * m:(i + 1) * m].clone()
                if i > 0 or self.cyclic:
                    q = (i - 1) % nS
                    c -= dv.dev_apply(SiM[i], dv.dev_solve(Th[q], vp[q * m:(q + 1) * m]))
                if i < nS - 1 or self.cyclic:
                    q = (i + 1) % nS
                    c -= dv.dev_apply(SiP[i], dv.dev_solve(Th[q], vp[q * m:(q + 1) * m]))
                vn[j * m:(j + 1) * m] = c
            vs.append(vn)
        vs[-1] = dv.dev_solve(RB[-1][2][0], vs[-1])                     # coarsest
        for l in range(len(RB) - 1, 0, -1):                             # back substitution
            SiM, _, Th, SiP = RB[l - 1]
            nR = len(SiM) // 2
            for j in range(nR):
                i = 2 * j
                vs[l - 1][i * m:(i + 1) * m] = vs[l][j * m:(j + 1) * m]
                c = dv.dev_apply(SiM[i + 1], vs[l][j * m:(j + 1) * m])
                if j + 1 < nR or self.cyclic:
                    q = (j + 1) % nR
                    c = c + dv.dev_apply(SiP[i + 1], vs[l][q * m:(q + 1) * m])
                blk = vs[l - 1][(i + 1) * m:(i + 2) * m] - c
                vs[l - 1][(i + 1) * m:(i + 2) * m] = dv.dev_solve(Th[i + 1], blk)
        return dv.finish(vs[0], rhs, one)

    def apply(self, x):
        """Beyond upstream: the block-tridiagonal operator the solver was
        factored from (the level-0 couplings and diagonal blocks as given,
        float64)."""
        SiM, T, _, SiP = self.RB[0]
        m, nS = self.m, len(SiM)
        X, one = dv.prepare_rhs(x)
        Y = torch.empty_like(X)
        for i in range(nS):
            y = dv.dev_apply(T[i], X[i * m:(i + 1) * m])
            if i > 0 or self.cyclic:
                q = (i - 1) % nS
                y = y + dv.dev_apply(SiM[i], X[q * m:(q + 1) * m])
            if i < nS - 1 or self.cyclic:
                q = (i + 1) % nS
                y = y + dv.dev_apply(SiP[i], X[q * m:(q + 1) * m])
            Y[i * m:(i + 1) * m] = y
        return dv.finish(Y, x, one)

    def solve_refined(self, rhs, tol=1e-10, maxit=5):
        """Beyond upstream: solve() refined against apply() (float64
        residuals with the exact couplings): the red-black levels compress
        Schur complements sampled through the compressed blocks below them,
        and at large sizes their errors compound (3-5e-7 at 32 slabs x 4096
        points); refinement restores the tolerance.  Returns (x, solves,
        worst column relative residual)."""
        return _refine(self, rhs, tol, maxit)
