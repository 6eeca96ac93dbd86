"""Red-black HBS solves of many block-tridiagonal systems at once.

Upstream solves each interface system with its own
RedBlackSolverHBS.solve (direct_solve/omsdirectsolveHBS.py:489-558): per
red-black level one ULV solve per odd block and one HBS apply per coupling,
each a handful of kernel launches, so a batch of systems costs launches in
proportion to its size.  ``solve_rb_hbs_grouped`` advances all systems of a
batch level by level together: each phase of a level -- the odd blocks'
solves, then the couplings' applies -- is one grouped call over every system
(slu_ulv_solve_grouped / slu_hbs_apply_grouped: one launch per tree step for
all members, whatever their sizes), so the launch count follows the depth of
the deepest system, not the number of systems.  Each system's result is what
its own ``solve`` returns (the same kernels on the same data).

Systems may differ in block size, block count (each a power of two, as
red-black requires), rank and right-hand-side count.  Blocks that are the
identity (``id_op``, the level-0 diagonal of an I + S system) are copies;
operators marked ``_zero`` (decoupled padding) contribute nothing; other
dense operators run one by one.

``factorize_many`` builds the systems of a batch concurrently: the
factorisations are independent, and one system's red-black levels alone
leave the GPU idle between its small launches and host steps.
"""
import concurrent.futures as cf
import threading

import torch

from .. import _dev as dv
from ..grouped import apply_grouped, solve_grouped_device
from .omsdirectsolveHBS import _blocking_worker, _wait, _worker_stream, id_op


_BUILD_POOLS = {}
_BUILD_LOCK = threading.Lock()


def _build_pool(workers):
    """Worker threads for factorize_many, made once per size and kept: each
    thread keeps one stream per device (and so one library handle), however
    many batches are factored."""
    with _BUILD_LOCK:
        if workers not in _BUILD_POOLS:
            _BUILD_POOLS[workers] = cf.ThreadPoolExecutor(max_workers=workers,
                                                          initializer=_blocking_worker)
        return _BUILD_POOLS[workers]


def factorize_many(jobs, workers=6):
    """Run independent factorisation jobs (callables, each building and
    factoring one system) ``workers`` at a time.  Each job runs on a worker
    thread with its own CUDA stream, and so its own library handle and
    scratch arena; its stream is synchronised before the job counts as done,
    so every result is ready for use on any stream.  Returns the results in
    job order.  Jobs that draw from a shared host RNG must serialise those
    draws themselves."""
    dev = torch.cuda.current_device()
    torch.cuda.current_stream(dev).synchronize()   # inputs made on the caller's stream
    if workers <= 1 or len(jobs) <= 1:
        return [j() for j in jobs]

    def run(job):
        torch.cuda.set_device(dev)
        st = _worker_stream(dev)
        with torch.cuda.stream(st):
            out = job()
        _wait(st)
        return out

    return list(_build_pool(workers).map(run, jobs))


def _is_hbs(op):
    return getattr(op, "_op", None) is not None and hasattr(op, "solve_plan") and \
        getattr(op, "mode", "N") == "N"


def _solve_inplace(items):
    """[(op, B)]: B <- op^{-1} B for contiguous 2-D device tensors B
    (identity blocks are left as they are)."""
    g_ops, g_B = [], []
    for op, B in items:
        if isinstance(op, id_op):
            continue
        if _is_hbs(op):
            g_ops.append(op)
            g_B.append(B)
        else:
            B.copy_(dv.dev_solve(op, B))
    if g_ops:
        solve_grouped_device(g_ops, g_B)


def _apply_into(items):
    """[(op, X, Y)]: Y <- op X (Y untouched for operators marked _zero)."""
    g_ops, g_X, g_Y = [], [], []
    for op, X, Y in items:
        if getattr(op, "_zero", False):
            continue
        if isinstance(op, id_op):
            Y.copy_(X)
        elif _is_hbs(op):
            g_ops.append(op)
            g_X.append(X)
            g_Y.append(Y)
        else:
            Y.copy_(dv.dev_apply(op, X))
    if g_ops:
        apply_grouped(g_ops, g_X, Ys=g_Y)


def solve_rb_hbs_grouped(solvers, rhs):
    """x_s = solvers[s].solve(rhs[s]) for every factored RedBlackSolverHBS,
    all systems at once.  rhs[s]: (nS_s m_s,) or (nS_s m_s, c_s), numpy or
    torch; each result comes back in the form of its right-hand side.  Per
    system and level the blocks are handled as one (blocks, m, c) view, so
    the host issues a few tensor operations per system and level and one
    grouped call per phase."""
    st = []
    for S, b in zip(solvers, rhs):
        B, one = dv.prepare_rhs(b)
        st.append({"m": S.m, "RB": S.RB, "cyc": S.cyclic, "vs": [B.clone().contiguous()],
                   "one": one, "ref": b, "depth": len(S.RB) - 1})
    maxd = max((s["depth"] for s in st), default=0)

    def view(s, V):
        return V.view(-1, s["m"], V.shape[1])

    # forward reduction (omsdirectsolveHBS.py:503-530): level l of every system
    for l in range(maxd):
        act = [s for s in st if l < s["depth"]]
        sol = []
        for s in act:
            SiM, _, Th, SiP = s["RB"][l]
            vp = view(s, s["vs"][-1])
            # odd blocks, copied (a lone odd block is already contiguous, and
            # the level keeps its right-hand side for the back substitution)
            s["W"] = vp[1::2].clone(memory_format=torch.contiguous_format)
            sol += [(Th[q], s["W"][q // 2]) for q in range(1, len(SiM), 2)]
        _solve_inplace(sol)
        app = []
        for s in act:
            SiM, _, Th, SiP = s["RB"][l]
            nS, W = len(SiM), s["W"]
            s["Yl"] = torch.zeros_like(W)
            s["Yr"] = torch.zeros_like(W)
            for j in range(nS // 2):
                i = 2 * j
                if i > 0 or s["cyc"]:
                    app.append((SiM[i], W[((i - 1) % nS) // 2], s["Yl"][j]))
                if i < nS - 1 or s["cyc"]:
                    app.append((SiP[i], W[((i + 1) % nS) // 2], s["Yr"][j]))
        _apply_into(app)
        for s in act:
            vp = view(s, s["vs"][-1])
            vn = vp[0::2] - s["Yl"] - s["Yr"]
            s["vs"].append(vn.reshape(-1, vn.shape[2]))
            del s["W"], s["Yl"], s["Yr"]
    # coarsest block of every system
    _solve_inplace([(s["RB"][-1][2][0], s["vs"][-1]) for s in st])
    # back substitution (omsdirectsolveHBS.py:531-556), from each system's top
    for k in range(maxd):
        act = [s for s in st if k < s["depth"]]
        app = []
        for s in act:
            l = s["depth"] - k
            SiM, _, Th, SiP = s["RB"][l - 1]
            nR = len(SiM) // 2
            hi = view(s, s["vs"][l])
            s["Ym"] = torch.zeros_like(hi)
            s["Yp"] = torch.zeros_like(hi)
            for j in range(nR):
                app.append((SiM[2 * j + 1], hi[j], s["Ym"][j]))
                if j + 1 < nR or s["cyc"]:
                    app.append((SiP[2 * j + 1], hi[(j + 1) % nR], s["Yp"][j]))
        _apply_into(app)
        sol = []
        for s in act:
            l = s["depth"] - k
            SiM, _, Th, SiP = s["RB"][l - 1]
            lo, hi = view(s, s["vs"][l - 1]), view(s, s["vs"][l])
            lo[0::2] = hi
            s["R"] = (lo[1::2] - (s["Ym"] + s["Yp"])).contiguous()
            sol += [(Th[2 * j + 1], s["R"][j]) for j in range(len(SiM) // 2)]
        _solve_inplace(sol)
        for s in act:
            l = s["depth"] - k
            view(s, s["vs"][l - 1])[1::2] = s["R"]
            del s["R"], s["Ym"], s["Yp"]
    return [dv.finish(s["vs"][0], s["ref"], s["one"]) for s in st]


class GroupedRBSolvePlan:
    """solve_rb_hbs_grouped for fixed right-hand-side blocks, made once: the
    whole batch's red-black solve -- the copies, grouped solves, grouped
    applies and block updates of every level -- becomes one program of
    grouped phases (slu_grouped_program_create: tables uploaded once, the
    sequence captured as one CUDA graph), so a solve is one graph launch.
    ``plan()`` solves whatever the Bs hold and returns the Xs (the same
    results as each system's own solve).  Bs[s]: contiguous (nS_s m_s, c_s)
    float64 CUDA tensors; the plan keeps them and its buffers alive."""

    def __init__(self, solvers, Bs, Xs=None):
        import ctypes
        from .. import _lib as L
        self.Bs = list(Bs)
        self.Xs = [torch.empty_like(B) for B in self.Bs] if Xs is None else list(Xs)
        self._keep = []
        phases = []       # (kind, [(op, X, Y, ld, c, n)])

        def phase(kind, items):
            items = [it for it in items if it is not None]
            if items:
                phases.append((kind, items))

        def blocks(T, m):
            c = T.shape[1]
            return [T[j * m:(j + 1) * m] for j in range(T.shape[0] // m)]

        def ew(X, Y):
            return (None, X, Y, 0, 0, Y.numel())

        def hbs(op, X, Y=None):
            if isinstance(op, id_op) or getattr(op, "_zero", False):
                return None
            if not _is_hbs(op):
                raise NotImplementedError("grouped red-black plans take HBS operators, the "
                                          "identity and decoupled (_zero) blocks")
            return (op, X, Y, X.shape[1], X.shape[1], 0)

        st = []
        for S, B, X in zip(solvers, self.Bs, self.Xs):
            if B.dtype != torch.float64 or not B.is_cuda or not B.is_contiguous() or B.dim() != 2:
                raise ValueError("right-hand sides must be contiguous 2-D float64 CUDA tensors")
            m, c = S.m, B.shape[1]
            vs = [X]
            W, Yl, Yr = [], [], []
            for l in range(len(S.RB) - 1):
                nR = len(S.RB[l][0]) // 2
                for lst in (W, Yl, Yr):
                    lst.append(torch.empty((nR * m, c), dtype=torch.float64, device=B.device))
                vs.append(torch.empty((nR * m, c), dtype=torch.float64, device=B.device))
            self._keep += vs + W + Yl + Yr
            st.append({"S": S, "m": m, "vs": vs, "W": W, "Yl": Yl, "Yr": Yr,
                       "depth": len(S.RB) - 1})
        maxd = max((s["depth"] for s in st), default=0)
        phase(2, [ew(B, X) for B, X in zip(self.Bs, self.Xs)])
        for l in range(maxd):                                   # forward reduction
            act = [s for s in st if l < s["depth"]]
            cp, sol, zero, app, even, sub = [], [], [], [], [], []
            for s in act:
                SiM, _, Th, SiP = s["S"].RB[l]
                nS, m, cyc = len(SiM), s["m"], s["S"].cyclic
                vp, W = blocks(s["vs"][l], m), blocks(s["W"][l], m)
                Yl, Yr = blocks(s["Yl"][l], m), blocks(s["Yr"][l], m)
                vn = blocks(s["vs"][l + 1], m)
                for j in range(nS // 2):
                    cp.append(ew(vp[2 * j + 1], W[j]))
                    sol.append(hbs(Th[2 * j + 1], W[j]))
                    even.append(ew(vp[2 * j], vn[j]))
                zero += [ew(None, s["Yl"][l]), ew(None, s["Yr"][l])]
                for j in range(nS // 2):
                    i = 2 * j
                    if i > 0 or cyc:
                        app.append(hbs(SiM[i], W[((i - 1) % nS) // 2], Yl[j]))
                    if i < nS - 1 or cyc:
                        app.append(hbs(SiP[i], W[((i + 1) % nS) // 2], Yr[j]))
                sub += [ew(s["Yl"][l], s["vs"][l + 1]), ew(s["Yr"][l], s["vs"][l + 1])]
            phase(2, cp)
            phase(0, sol)
            phase(3, zero)
            phase(1, app)
            phase(2, even)
            phase(5, sub[0::2])
            phase(5, sub[1::2])
        phase(0, [hbs(s["S"].RB[-1][2][0], s["vs"][-1]) for s in st])   # coarsest
        for k in range(maxd):                                   # back substitution
            act = [s for s in st if k < s["depth"]]
            zero, app, cp, add, rsub, sol, back = [], [], [], [], [], [], []
            for s in act:
                l = s["depth"] - k
                SiM, _, Th, SiP = s["S"].RB[l - 1]
                nR, m, cyc = len(SiM) // 2, s["m"], s["S"].cyclic
                hi, lo = blocks(s["vs"][l], m), blocks(s["vs"][l - 1], m)
                Ym, Yp = blocks(s["Yl"][l - 1], m), blocks(s["Yr"][l - 1], m)
                zero += [ew(None, s["Yl"][l - 1]), ew(None, s["Yr"][l - 1])]
                for j in range(nR):
                    app.append(hbs(SiM[2 * j + 1], hi[j], Ym[j]))
                    if j + 1 < nR or cyc:
                        app.append(hbs(SiP[2 * j + 1], hi[(j + 1) % nR], Yp[j]))
                    cp.append(ew(hi[j], lo[2 * j]))
                    rsub.append(ew(lo[2 * j + 1], Ym[j]))
                    sol.append(hbs(Th[2 * j + 1], Ym[j]))
                    back.append(ew(Ym[j], lo[2 * j + 1]))
                add.append(ew(s["Yr"][l - 1], s["Yl"][l - 1]))
            phase(3, zero)
            phase(1, app)
            phase(2, cp)
            phase(4, add)
            phase(6, rsub)
            phase(0, sol)
            phase(2, back)
        kinds = [k for k, _ in phases]
        counts = [len(it) for _, it in phases]
        flat = [it for _, its in phases for it in its]
        nn = len(flat)
        P = ctypes.c_void_p
        ops = (P * nn)(*[(op._op if op is not None else None) for op, *_ in flat])
        xp = (P * nn)(*[(X.data_ptr() if X is not None else None) for _, X, *_ in flat])
        yp = (P * nn)(*[(Y.data_ptr() if Y is not None else None) for _, _, Y, *_ in flat])
        ld = (ctypes.c_int * nn)(*[it[3] for it in flat])
        cc = (ctypes.c_int * nn)(*[it[4] for it in flat])
        ne = (ctypes.c_longlong * nn)(*[it[5] for it in flat])
        self._ops = [it[0] for it in flat if it[0] is not None]      # keeps the operators alive
        self.phases = len(phases)
        self._plan = P()
        L.check(L.lib().slu_grouped_program_create(
            L.handle(), len(phases), (ctypes.c_int * len(phases))(*kinds),
            (ctypes.c_int * len(phases))(*counts), ops, xp, yp, ld, cc, ne,
            ctypes.byref(self._plan)))

    def __call__(self):
        from .. import _lib as L
        L.check(L.lib().slu_ulv_solve_plan_launch(L.handle(), self._plan, 0))
        return self.Xs

    def close(self):
        from .. import _lib as L
        if getattr(self, "_plan", None) is not None and self._plan.value and L._lib is not None:
            L.lib().slu_ulv_solve_plan_destroy(self._plan)
        self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
