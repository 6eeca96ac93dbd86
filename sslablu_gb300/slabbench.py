"""Block-tridiagonal slab solvers on the GPU against the CPU restatement.

    python -m sslablu_gb300.slabbench dense [--m 256 --slabs 8]
    python -m sslablu_gb300.slabbench hbs   [--m 1024 --slabs 8 --leaf 64 --rank 24]
    python -m sslablu_gb300.slabbench helmholtz [--slabs 33 --n 64 --leaf 128 --rank 64]

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


def helmholtz(a):
    """The C3 pipeline on real slab operators: 3-D variable-coefficient
    Helmholtz (k = kappa, c = 1 + 0.5 sin 2pi x sin 2pi y sin 2pi z) on
    [0,1]^3 cut into a.slabs slabs, a.n x a.n interface planes, stencil
    discretisation with 5 points across a double slab.
      1. the slab maps S_l, S_r sampled on the GPU through batched slab solves
         (multislab.slabmaps; oms.compute_stmaps) and compressed by the rkHBS
         assembler (leaf a.leaf, rank a.rank; matAssembler.py:104-133);
      2. RedBlackSolverHBS factorisation of the compressed interface system
         of wavenumber a.prec_kappa (the preconditioner's operator);
      3. 64 right-hand sides (smooth seeded interface data) solved by GMRES on
         the exact interface operator of wavenumber a.kappa (slab solves,
         float64) with the red-black HBS solve as preconditioner, to a 1e-10
         relative residual (test/3D/cubeTest.py:158-186).
    With prec_kappa = kappa this is upstream's iterative solve.  At k = 20
    the weak-admissibility red-black HBS factorisation of the Helmholtz
    couplings is unstable at moderate ranks -- the Schur complements it
    compresses are near-singular, and compression errors are amplified by
    their inverses; upstream's algorithm does the same, and its Thomas
    variant is worse -- so the default preconditioner is the red-black HBS
    factorisation of the Laplace interface system (prec_kappa = 0: a
    shifted-Laplacian preconditioner for Helmholtz, after Erlangga, Vuik and
    Oosterlee, Appl. Numer. Math. 50, 2004), which HBS compresses well.
    Reports the stage times, GMRES steps, residual against the exact
    operator, and the residual of the preconditioner alone."""
    from .direct_solve.omsdirectsolveHBS import RedBlackSolverHBS
    from .matAssembly.matAssembler import rkHMatAssembler
    from .multislab.gmres import gmres
    from .multislab.slabmaps import SlabGeometry, StotOperator, slab_stmaps
    g = SlabGeometry(a.slabs, 5, a.n + 2, a.n + 2, kappa=a.kappa, coef=1)
    gp = SlabGeometry(a.slabs, 5, a.n + 2, a.n + 2, kappa=a.prec_kappa, coef=1)
    m, nif = g.m, g.nif
    np.random.seed(20261207)
    asm = rkHMatAssembler(a.leaf, a.rank)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    S_rk = []
    t_sample = 0.0
    for st_l, st_r in slab_stmaps(gp):
        row = []
        for st in (st_l, st_r):
            if st is not None:
                row.append(asm.assemble(st))
                t_sample += asm.stats.timeSample
        S_rk.append(row)
    torch.cuda.synchronize()
    t_compress = time.perf_counter() - t0
    tree = S_rk[0][0].tree
    rb = RedBlackSolverHBS(m, a.rank, tree, False)
    t0 = time.perf_counter()
    rb.factorize(S_rk)
    torch.cuda.synchronize()
    t_factor = time.perf_counter() - t0
    St = StotOperator(g)
    # smooth seeded interface data: low-order trig series per plane
    pts = g.points(0)
    rng = np.random.default_rng(7)
    B = np.zeros((nif * m, a.nrhs))
    for j in range(a.nrhs):
        for i in range(nif):
            coef = rng.standard_normal((4, 4))
            v = np.zeros(m)
            for p in range(4):
                for q in range(4):
                    v += coef[p, q] * np.sin((p + 1) * np.pi * pts[:, 1]) * \
                        np.sin((q + 1) * np.pi * pts[:, 2])
            B[i * m:(i + 1) * m, j] = v
    Bd = torch.from_numpy(B).cuda()
    # the preconditioner alone (one red-black HBS solve)
    Xp = rb.solve(Bd)
    R = Bd - St.dev_matmat(Xp)
    res_pre = float((R.norm(dim=0) / Bd.norm(dim=0)).max())
    torch.cuda.synchronize()
    ts = []
    for _ in range(a.reps):
        t0 = time.perf_counter()
        X, steps, rel = gmres(St.dev_matmat, Bd, rb.solve, tol=1e-10, restart=30, maxiter=200)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    R = Bd - St.dev_matmat(X)
    res = float((R.norm(dim=0) / Bd.norm(dim=0)).max())
    t_solve = statistics.median(ts)
    # one exact interface apply and one preconditioner solve, timed alone
    t_apply = _wall(lambda: St.dev_matmat(Bd), 3)[0]
    t_pre = _wall(lambda: rb.solve(Bd), 3)[0]
    return {"workload": "3-D Helmholtz k=%g, c = 1 + 0.5 sin sin sin, %d slabs, %d x %d "
                        "interfaces (m=%d), 5-point slabs, rkHBS leaf %d rank %d; "
                        "preconditioner: red-black HBS of the k=%g interface system"
                        % (a.kappa, a.slabs, a.n, a.n, m, a.leaf, a.rank, a.prec_kappa),
            "interfaces": nif, "m": m, "nrhs": a.nrhs,
            "maps_sample_compress_s": t_compress, "maps_sample_s": t_sample,
            "chebyshev_steps": St.maps.steps or None,
            "rb_hbs_factor_s": t_factor,
            "preconditioner_relres": res_pre,
            "gmres_steps": steps, "relres": res, "gmres_relres": rel,
            "solve_s": t_solve, "rhs_per_s": a.nrhs / t_solve,
            "stot_apply_ms": 1e3 * t_apply, "rb_hbs_solve_ms": 1e3 * t_pre}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("kind", choices=["dense", "hbs", "helmholtz"])
    ap.add_argument("--m", type=int, default=None)
    ap.add_argument("--slabs", type=int, default=8)
    ap.add_argument("--leaf", type=int, default=64)
    ap.add_argument("--rank", type=int, default=24)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--n", type=int, default=64, help="helmholtz: interface plane n x n")
    ap.add_argument("--kappa", type=float, default=20.0)
    ap.add_argument("--prec-kappa", type=float, default=0.0,
                    help="helmholtz: wavenumber of the preconditioner's interface system")
    ap.add_argument("--nrhs", type=int, default=64)
    a = ap.parse_args()
    if a.m is None:
        a.m = 256 if a.kind == "dense" else 1024
    if a.kind == "helmholtz":
        out = helmholtz(a)
    else:
        out = dense(a) if a.kind == "dense" else hbs(a)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
