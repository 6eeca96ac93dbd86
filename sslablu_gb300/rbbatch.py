"""Many uneven slab interface systems solved by red-black HBS, grouped.

    python -m sslablu_gb300.rbbatch [--systems 512 --nrhs 8 --reps 10]

Workload: ``--systems`` seeded 2-D Poisson interface systems (I + S) x = b.
Each is [0,1]^2 cut into nI + 1 slabs (nI ~ U{4..16} interfaces) with
interface size m ~ U{128, 256, 512, 1024, 2048}.  The slab maps S are the
5-point-stencil maps (``synthetic.poisson_slab_map``, closed form, square
cells).  Each system's coupling is compressed once by the rkHBS assembler
(leaf 64, rank ~ U{16..48}) and shared by all its interfaces.  Systems are
padded to a power-of-two block count with decoupled identity blocks, as
red-black requires, and factored by RedBlackSolverHBS (sketches drawn on the
device from a seeded generator); ``--workers`` systems are built at a
time, each on its own stream.  ``--nrhs``
right-hand sides ~ N(0, 1) per system (zero on the padding).

Arms, each timed with CUDA events on the current stream after warm-up:
  * per_system: each system's own RedBlackSolverHBS.solve, one after another;
  * grouped: solve_rb_hbs_grouped over the whole batch (each phase of a
    red-black level one grouped call over every system);
  * grouped_plan: the same program built once (GroupedRBSolvePlan: every
    table uploaded once, the whole solve one CUDA graph launch).
Reported: factorisation time (wall), RHS/s and launches per step of each
arm, the worst relative residual of the grouped solutions against the exact
float64 systems (dense maps), and the largest difference between the two
arms.  Prints one JSON line.
"""
import argparse
import contextlib
import functools
import json
import statistics
import threading
import time
import types

import numpy as np
import torch

from . import _lib as L


def system_specs(systems, seed, sizes=(128, 256, 512, 1024, 2048), ranks=(16, 48),
                 interfaces=(4, 16)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(systems):
        nI = int(rng.integers(interfaces[0], interfaces[1] + 1))
        m = int(rng.choice(sizes))
        rk = int(rng.integers(ranks[0], ranks[1] + 1))
        out.append((nI, m, rk))
    return out


def build_system(nI, m, rk, seed, rng_lock=None):
    """(solver, dense S on the device, padded block count): the factored
    RedBlackSolverHBS of one system and its exact coupling.  ``rng_lock``
    (held while numpy's global RNG is seeded and drawn from) lets systems
    be built on several threads with the draws of a one-by-one build."""
    from .direct_solve.omsdirectsolveHBS import RedBlackSolverHBS, _linop_from_mat
    from .matAssembly.matAssembler import rkHMatAssembler
    from .synthetic import poisson_slab_map
    width = 2.0 / (nI + 1)
    nx = int(round(width * (m + 1))) // 2 * 2 + 1          # square cells, odd
    S = poisson_slab_map(m, max(nx, 3), width)
    XX = np.linspace(0.0, 1.0, m + 2)[1:-1]
    with rng_lock if rng_lock is not None else contextlib.nullcontext():
        np.random.seed(seed)
        H = rkHMatAssembler(64, rk).assemble(types.SimpleNamespace(A=S, XXI=XX))
    Z = _linop_from_mat(np.zeros((m, m)))
    Z._zero = True
    P = 1 << int(np.ceil(np.log2(nI)))
    S_rk = []
    for i in range(P):
        left = H if 0 < i < nI else Z
        right = H if i < nI - 1 else Z
        S_rk.append([left, right])
    rb = RedBlackSolverHBS(m, rk, H.tree, False, sketch_seed=seed)
    rb.factorize(S_rk)
    return rb, torch.from_numpy(S).cuda(), P


def build_systems(specs, seed, workers=6):
    """build_system of every spec (system j seeded seed + 17 j), ``workers``
    systems at a time (grouped_rb.factorize_many: one stream per worker)."""
    from .direct_solve.grouped_rb import factorize_many
    lock = threading.Lock()
    jobs = [functools.partial(build_system, nI, m, rk, seed + 17 * j, lock)
            for j, (nI, m, rk) in enumerate(specs)]
    return factorize_many(jobs, workers)


def exact_apply(S, nI, P, X):
    """(I + S-couplings) X for the padded system (the padding blocks are I)."""
    m = S.shape[0]
    Y = X.clone()
    for i in range(nI):
        if i > 0:
            Y[i * m:(i + 1) * m] += S @ X[(i - 1) * m:i * m]
        if i < nI - 1:
            Y[i * m:(i + 1) * m] += S @ X[(i + 1) * m:(i + 2) * m]
    return Y


def _time(fn, reps, warmup=2):
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


def run(systems=512, nrhs=8, reps=10, seed=20261205, workers=6):
    from .direct_solve.grouped_rb import solve_rb_hbs_grouped
    torch.cuda.set_device(0)
    specs = system_specs(systems, seed)
    t0 = time.perf_counter()
    built = build_systems(specs, seed, workers)
    torch.cuda.synchronize()
    t_factor = time.perf_counter() - t0
    rng = np.random.default_rng(seed + 1)
    Bs = []
    for (nI, m, rk), (rb, S, P) in zip(specs, built):
        b = np.zeros((P * m, nrhs))
        b[:nI * m] = rng.standard_normal((nI * m, nrhs))
        Bs.append(torch.from_numpy(b).cuda())
    solvers = [rb for rb, _, _ in built]
    total = systems * nrhs
    out = {"workload": "%d 2-D Poisson interface systems (I + S), interfaces U{4..16}, "
                       "interface size U{128,...,2048}, stencil slab maps (closed form) "
                       "compressed by rkHBS leaf 64 rank U{16..48}, red-black HBS, %d RHS "
                       "each" % (systems, nrhs),
           "systems": systems, "nrhs": nrhs, "factor_s": t_factor,
           "factor_per_system_ms": 1e3 * t_factor / systems, "factor_workers": workers,
           "sizes": {str(s): sum(1 for sp in specs if sp[1] == s)
                     for s in (128, 256, 512, 1024, 2048)}}
    from .direct_solve.grouped_rb import GroupedRBSolvePlan
    t0 = time.perf_counter()
    plan = GroupedRBSolvePlan(solvers, Bs)
    torch.cuda.synchronize()
    out["plan_build_s"] = time.perf_counter() - t0
    out["plan_phases"] = plan.phases
    arms = {"per_system": lambda: [rb.solve(B) for rb, B in zip(solvers, Bs)],
            "grouped": lambda: solve_rb_hbs_grouped(solvers, Bs),
            "grouped_plan": plan}
    res = {}
    for name, fn in arms.items():
        fn()                                   # first use composes apply operators
        torch.cuda.synchronize()
        # an NVTX range per arm (a profiler can keep one arm's launches)
        with torch.cuda.nvtx.range(name):
            c0 = L.lib().slu_launch_count()
            xs = fn()
            torch.cuda.synchronize()
            launches = L.lib().slu_launch_count() - c0
            t = _time(fn, reps)
        out[name] = {"rhs_per_s": total / t, "ms_per_step": 1e3 * t, "gpu_launches": launches}
        res[name] = xs
    worst, diff = 0.0, 0.0
    for (nI, m, rk), (rb, S, P), B, xg, xq, xp in zip(specs, built, Bs, res["grouped"],
                                                     res["grouped_plan"], res["per_system"]):
        R = B - exact_apply(S, nI, P, xq)
        worst = max(worst, float((torch.linalg.norm(R, dim=0) /
                                  torch.linalg.norm(B, dim=0)).max()))
        for x in (xg, xq):
            diff = max(diff, float(torch.linalg.norm(x - xp) / torch.linalg.norm(xp)))
    out["relres_vs_exact"] = worst
    out["grouped_vs_per_system"] = diff
    for name in ("grouped", "grouped_plan"):
        out["speedup_" + name] = out[name]["rhs_per_s"] / out["per_system"]["rhs_per_s"]
    return out, specs, built, Bs, res


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--systems", type=int, default=512)
    ap.add_argument("--nrhs", type=int, default=8)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--seed", type=int, default=20261205)
    ap.add_argument("--workers", type=int, default=6,
                    help="systems built and factored at a time (one stream each)")
    a = ap.parse_args()
    out = run(a.systems, a.nrhs, a.reps, a.seed, a.workers)[0]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
