"""Block-tridiagonal slab solvers on the GPU against the CPU restatement.

    python -m sslablu_gb300.slabbench dense [--m 256 --slabs 8]
    python -m sslablu_gb300.slabbench hbs   [--m 1024 --slabs 8 --leaf 64 --rank 24]
    python -m sslablu_gb300.slabbench helmholtz [--slabs 33 --n 64 --leaf 128 --rank 64]
    python -m sslablu_gb300.slabbench strong [--n 64 --leaf 128 --rank 32 --adjacency full]

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
  strong -- strong-admissibility HBS of a coupling between two interface
           planes: construct time, apply throughput, accuracy, and the
           weak-admissibility HBS at the same rank beside it.
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
    discretisation with 5 points across a double slab.  64 right-hand sides
    (smooth seeded interface data) are solved by GMRES on the exact interface
    operator Stot (slab solves, float64; multislab/oms.py:258-302) to a 1e-10
    relative residual (test/3D/cubeTest.py:158-186), with one of two
    preconditioners (a.prec):
      hbs   -- upstream's iterative solve: the slab maps sampled on the GPU
               through batched slab solves (oms.compute_stmaps), compressed by
               the rkHBS assembler (leaf a.leaf, rank a.rank;
               matAssembler.py:104-133) and factored by RedBlackSolverHBS (of
               the wavenumber a.prec_kappa: 0 gives a shifted-Laplacian
               preconditioner, after Erlangga, Vuik and Oosterlee, Appl.
               Numer. Math. 50, 2004).  At k = 20 the weak-admissibility
               red-black HBS factorisation is not a usable preconditioner (the
               Schur complements it compresses are near-singular; upstream's
               algorithm does the same even at ranks near the leaf size);
      dense -- the maps formed densely by the same slab solves (identity
               sketches) and factored by the mixed-precision dense red-black
               solver (Schur-complement products on the tcgen05 tensor cores,
               float64 pivot blocks), whose solve -- its block products on the
               tensor cores too -- preconditions GMRES.
    Reports the stage times, GMRES steps, residual against the exact
    operator, and the residual of the preconditioner alone."""
    from .multislab.gmres import gmres
    from .multislab.slabmaps import SlabGeometry, SlabMaps, StotOperator, slab_stmaps
    g = SlabGeometry(a.slabs, 5, a.n + 2, a.n + 2, kappa=a.kappa, coef=1)
    m, nif = g.m, g.nif
    out = {}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if a.prec == "hbs":
        from .direct_solve.omsdirectsolveHBS import RedBlackSolverHBS
        from .matAssembly.matAssembler import rkHMatAssembler
        gp = SlabGeometry(a.slabs, 5, a.n + 2, a.n + 2, kappa=a.prec_kappa, coef=1)
        np.random.seed(20261207)
        asm = rkHMatAssembler(a.leaf, a.rank)
        S_rk = []
        for st_l, st_r in slab_stmaps(gp):
            S_rk.append([asm.assemble(st) for st in (st_l, st_r) if st is not None])
        torch.cuda.synchronize()
        out["maps_sample_compress_s"] = time.perf_counter() - t0
        rb = RedBlackSolverHBS(m, a.rank, S_rk[0][0].tree, False)
        t0 = time.perf_counter()
        rb.factorize(S_rk)
        torch.cuda.synchronize()
        out["factor_s"] = time.perf_counter() - t0
        prec = rb.solve
        desc = "red-black HBS of the k=%g system, rkHBS leaf %d rank %d" % (a.prec_kappa, a.leaf,
                                                                            a.rank)
    else:
        from .direct_solve.omsdirectsolve import RedBlackSolver
        maps = SlabMaps(g, None, 1e-14)
        Id = torch.zeros((nif * m, m), dtype=torch.float64, device="cuda")
        Id.view(nif, m, m)[:] = torch.eye(m, dtype=torch.float64, device="cuda")
        Sl = maps.apply(Id, None).view(nif, m, m)
        Sr = maps.apply(None, Id).view(nif, m, m)
        del Id
        torch.cuda.synchronize()
        out["maps_dense_s"] = time.perf_counter() - t0
        out["chebyshev_steps"] = maps.steps
        rows = [[Sl[i], Sr[i]] for i in range(nif)]
        rb = RedBlackSolver(m, precision="mixed")
        t0 = time.perf_counter()
        rb.factorize(rows, [torch.eye(m, dtype=torch.float64, device="cuda")] * nif)
        torch.cuda.synchronize()
        out["factor_s"] = time.perf_counter() - t0
        del Sl, Sr, rows

        def prec(X):
            return rb.solve_tc(X)
        desc = ("dense red-black of the exact maps, tensor-core Schur products and solve "
                "products (split-BF16x3) with float64 pivot blocks")
    St = StotOperator(g)
    pts = g.points(0)
    rng = np.random.default_rng(7)
    B = np.zeros((nif * m, a.nrhs))
    for j in range(a.nrhs):
        for i in range(nif):
            cf = rng.standard_normal((4, 4))
            v = np.zeros(m)
            for p in range(4):
                for q in range(4):
                    v += cf[p, q] * np.sin((p + 1) * np.pi * pts[:, 1]) * \
                        np.sin((q + 1) * np.pi * pts[:, 2])
            B[i * m:(i + 1) * m, j] = v
    Bd = torch.from_numpy(B).cuda()
    Xp = prec(Bd)
    R = Bd - St.dev_matmat(Xp)
    out["preconditioner_relres"] = float((R.norm(dim=0) / Bd.norm(dim=0)).max())
    gmres(St.dev_matmat, Bd, prec, tol=1e-10, restart=30, maxiter=a.maxiter)   # warm-up
    torch.cuda.synchronize()
    ts = []
    for _ in range(a.reps):
        t0 = time.perf_counter()
        X, steps, rel = gmres(St.dev_matmat, Bd, prec, tol=1e-10, restart=30, maxiter=a.maxiter)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    R = Bd - St.dev_matmat(X)
    t_solve = statistics.median(ts)
    out.update({
        "workload": "3-D Helmholtz k=%g, c = 1 + 0.5 sin sin sin, %d slabs, %d x %d interfaces "
                    "(m=%d), 5-point slabs; GMRES on the exact interface operator; "
                    "preconditioner: %s" % (a.kappa, a.slabs, a.n, a.n, m, desc),
        "interfaces": nif, "m": m, "nrhs": a.nrhs, "chebyshev_steps_stot": St.maps.steps or None,
        "gmres_steps": steps, "relres": float((R.norm(dim=0) / Bd.norm(dim=0)).max()),
        "solve_s": t_solve, "rhs_per_s": a.nrhs / t_solve,
        "stot_apply_ms": 1e3 * _wall(lambda: St.dev_matmat(Bd), 3)[0],
        "preconditioner_ms": 1e3 * _wall(lambda: prec(Bd), 3)[0]})
    return out


def strong(a):
    """Strong-admissibility HBS (HBStorch_strong) of the coupling between two
    nearby n x n interface planes: construct from sketches (warm median of
    reps, the first call separate), apply throughput for nrhs columns,
    accuracy against the dense operator, and the weak-admissibility HBS at
    the same rank for comparison."""
    from .matAssembly.HBS.HBStorch_strong import HBSMAT
    from .matAssembly.HBS import HBStorch
    from .matAssembly.HBS.slabTree import slabTree
    from .synthetic import plane_coupling, plane_points
    XX = plane_points(a.n)
    A = plane_coupling(XX)
    N = A.shape[0]
    kmax = 9 if a.adjacency == "full" else 5
    s = kmax * max(2 * a.rank, a.leaf) + a.rank + 20
    rng = np.random.default_rng(0)
    Ad = torch.from_numpy(A).cuda()
    Om = torch.from_numpy(rng.standard_normal((N, s))).cuda()
    Psi = torch.from_numpy(rng.standard_normal((N, s))).cuda()
    Y, Z = Ad @ Om, Ad.T @ Psi
    tree = slabTree(XX, False, a.leaf, adjacency=a.adjacency)
    H = HBSMAT(device="cuda", tree=tree)
    if getattr(a, "once", False):
        # one construct and one apply, nothing else (for launch lists)
        H.construct(a.rank, Om, Psi, Y, Z)
        X = torch.from_numpy(rng.standard_normal((N, a.nrhs))).cuda()
        H._dev_apply(X)
        torch.cuda.synchronize()
        return {"workload": "strong construct + one apply", "N": N, "samples": s}
    t_cold, _ = _wall(lambda: H.construct(a.rank, Om, Psi, Y, Z), reps=1)
    t_warm, _ = _wall(lambda: H.construct(a.rank, Om, Psi, Y, Z), reps=max(1, a.reps))
    X = torch.from_numpy(rng.standard_normal((N, a.nrhs))).cuda()
    t_apply = _events(lambda: H._dev_apply(X), a.reps)
    err = float(torch.linalg.norm(H._dev_apply(X) - Ad @ X) / torch.linalg.norm(Ad @ X))
    errT = float(torch.linalg.norm(H._dev_apply(X, True) - Ad.T @ X) / torch.linalg.norm(Ad.T @ X))
    t_dense = _events(lambda: Ad @ X, a.reps)
    # weak admissibility at the same rank (the rkHBS assembler's sample count)
    wtree = slabTree(XX, False, a.leaf)
    sw = max(2 * a.rank, a.leaf) + a.rank + 10
    W = HBStorch.HBSMAT(device="cuda", tree=wtree)
    Omw, Psiw = Om[:, :sw].contiguous(), Psi[:, :sw].contiguous()
    W.construct(a.rank, Omw.cpu().numpy(), Psiw.cpu().numpy(), (Ad @ Omw).cpu().numpy(),
                (Ad.T @ Psiw).cpu().numpy())
    werr = float(np.linalg.norm(W.matmat(X.cpu().numpy()) - (Ad @ X).cpu().numpy())
                 / float(torch.linalg.norm(Ad @ X)))
    return {"workload": "strong-admissibility HBS of an exp(-r)/(r+0.02) coupling between "
                        "%d x %d interface planes 0.05 apart, %s adjacency, leaf %d, rank %d"
                        % (a.n, a.n, a.adjacency, a.leaf, a.rank),
            "N": N, "samples": s, "levels": len(H.Umats), "stacks": H.factor_stats["qr"],
            "construct_s": t_warm, "construct_cold_s": t_cold,
            "apply_ms": 1e3 * t_apply, "nrhs": a.nrhs, "apply_rhs_per_s": a.nrhs / t_apply,
            "dense_apply_ms": 1e3 * t_dense, "relerr": err, "relerr_T": errT,
            "nbytes": H.nbytes, "dense_bytes": 8 * N * N,
            "weak_same_rank_relerr": werr}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("kind", choices=["dense", "hbs", "helmholtz", "strong"])
    ap.add_argument("--adjacency", default="full", choices=["full", "partial"],
                    help="strong: near-field rule of the slab tree")
    ap.add_argument("--once", action="store_true",
                    help="strong: one construct and one apply only (for profiling)")
    ap.add_argument("--m", type=int, default=None)
    ap.add_argument("--slabs", type=int, default=8)
    ap.add_argument("--leaf", type=int, default=64)
    ap.add_argument("--rank", type=int, default=24)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--n", type=int, default=64, help="helmholtz: interface plane n x n")
    ap.add_argument("--kappa", type=float, default=20.0)
    ap.add_argument("--prec-kappa", type=float, default=0.0,
                    help="helmholtz: wavenumber of the HBS preconditioner's interface system")
    ap.add_argument("--prec", default="dense", choices=["dense", "hbs"],
                    help="helmholtz: GMRES preconditioner")
    ap.add_argument("--maxiter", type=int, default=100)
    ap.add_argument("--nrhs", type=int, default=64)
    a = ap.parse_args()
    if a.m is None:
        a.m = 256 if a.kind == "dense" else 1024
    if a.kind == "strong":
        out = strong(a)
    elif a.kind == "helmholtz":
        out = helmholtz(a)
    else:
        out = dense(a) if a.kind == "dense" else hbs(a)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
