"""Block-tridiagonal slab solvers on the GPU against the CPU restatement.

    python -m sslablu_gb300.slabbench dense [--m 256 --slabs 8]
    python -m sslablu_gb300.slabbench hbs   [--m 1024 --slabs 8 --leaf 64 --rank 24]

Workloads (seeded synthetic couplings of the interface system I + S,
sslablu_gb300.synthetic.slab_couplings; the slab PDE pipeline that produces
real S blocks is outside this package):
  dense -- the C1 shape: 8 slabs (7 interfaces padded to a power of two for
           red-black, as upstream requires), 256-point interfaces.  Red-black
           in float64 and in mixed precision (tensor-core Schur products +
           float64 refinement), block Thomas in float64; factor time, solve
           time for 1 and 64 right-hand sides, relative residuals.
  hbs   -- the C3 solve structure at reduced size: red-black and Thomas with
           every block an HBS compression (leaf, rank as given) of an implicit
           operator; factor time, 64-RHS solve time, residual.
GPU times are CUDA-event medians on device-resident data; factor times are
wall-clock around the factorisation (host-driven).  Prints one JSON line.
(`python bench.py --workload c1_dense|c3_hbs` runs the same measurements with
the CPU restatement of the upstream solvers timed beside them.)
"""
import argparse
import json
import os
import statistics
import sys
import time

import numpy as np
import torch


def _events(fn, reps, warmup=2):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        fn()
        b.record(st)
        b.synchronize()
        ts.append(a.elapsed_time(b) * 1e-3)
    return statistics.median(ts)


def _wall(fn, reps=3):
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts), out


def _relres(S, X, B):
    from .synthetic import tridiag_apply
    R = B - tridiag_apply(S, X)
    return float(np.max(np.linalg.norm(R, axis=0) / np.linalg.norm(B, axis=0)))


def dense(a):
    from .direct_solve.omsdirectsolve import BlockTridiagonalSolver, RedBlackSolver
    from .synthetic import slab_couplings
    m, nS = a.m, a.slabs
    S = slab_couplings(m, nS)
    T = [np.eye(m) for _ in range(nS)]
    rng = np.random.default_rng(1)
    B1 = rng.standard_normal((nS * m, 1))
    B64 = rng.standard_normal((nS * m, 64))
    out = {"workload": "dense block-tridiagonal I + S, %d slabs x %d-point interfaces "
                       "(Gaussian-kernel couplings)" % (nS, m)}
    arms = [("rb_f64", lambda: RedBlackSolver(m)), ("rb_mixed", lambda: RedBlackSolver(m, precision="mixed")),
            ("thomas_f64", lambda: BlockTridiagonalSolver(m))]
    for name, make in arms:
        def fac():
            s = make()
            s.factorize(S, T)
            return s
        t_f, solver = _wall(fac)
        res = {"factor_ms": 1e3 * t_f}
        for tag, B in (("1rhs", B1), ("64rhs", B64)):
            Bd = torch.from_numpy(B).cuda()
            t_s = _events(lambda: solver.solve(Bd), a.reps)
            X = solver.solve(Bd).cpu().numpy()
            res["solve_%s_ms" % tag] = 1e3 * t_s
            res["rhs_per_s_%s" % tag] = B.shape[1] / t_s
            res["relres_%s" % tag] = _relres(S, X, B)
        if name == "rb_mixed":
            res["iters"] = solver.iters
        out[name] = res
    return out


def hbs(a):
    import types
    from .direct_solve.omsdirectsolveHBS import RedBlackSolverHBS, ThomasSolverHBS, dense_to_linop
    from .synthetic import slab_couplings
    out = {"workload": "HBS block-tridiagonal I + S, %d slabs x %d-point interfaces, leaf %d, "
                       "rank %d (Gaussian-kernel couplings)" % (a.slabs, a.m, a.leaf, a.rank)}

    def setup(m):
        S = slab_couplings(m, a.slabs)
        nleaves = m // a.leaf
        tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=nleaves,
                                     nlevels=int(np.log2(nleaves)) + 1)
        ops = []
        for A, C in S:
            la, lc = dense_to_linop(A), dense_to_linop(C)
            la.tree = lc.tree = tree
            la.quad = lc.quad = False
            ops.append((la, lc))
        return S, tree, ops

    def gpu_arms(m, reps):
        S, tree, ops = setup(m)
        B = np.random.default_rng(2).standard_normal((a.slabs * m, 64))
        Bd = torch.from_numpy(B).cuda()
        res = {}
        for name in ("rb_hbs", "thomas_hbs"):
            def fac():
                np.random.seed(11)
                if name == "rb_hbs":
                    s = RedBlackSolverHBS(m, a.rank, tree, False)
                else:
                    s = ThomasSolverHBS(m, a.rank)
                s.factorize(ops)
                return s
            t_f, solver = _wall(fac, reps=1)
            t_s = _events(lambda: solver.solve(Bd), reps)
            X = solver.solve(Bd).cpu().numpy()
            res[name] = {"factor_ms": 1e3 * t_f, "solve_64rhs_ms": 1e3 * t_s,
                         "rhs_per_s_64rhs": 64 / t_s, "relres_64rhs": _relres(S, X, B)}
            # refined against the exact couplings to 1e-10
            t_r = _events(lambda: solver.solve_refined(Bd), max(1, reps // 2))
            Xr, it, _ = solver.solve_refined(Bd)
            res[name].update({"refined_solve_64rhs_ms": 1e3 * t_r, "refined_solves": it,
                              "relres_refined_64rhs": _relres(S, Xr.cpu().numpy(), B)})
        return res

    out.update(gpu_arms(a.m, a.reps))
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("kind", choices=["dense", "hbs"])
    ap.add_argument("--m", type=int, default=None)
    ap.add_argument("--slabs", type=int, default=8)
    ap.add_argument("--leaf", type=int, default=64)
    ap.add_argument("--rank", type=int, default=24)
    ap.add_argument("--reps", type=int, default=10)
    a = ap.parse_args()
    if a.m is None:
        a.m = 256 if a.kind == "dense" else 1024
    out = dense(a) if a.kind == "dense" else hbs(a)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
