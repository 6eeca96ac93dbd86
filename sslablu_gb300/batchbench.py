"""Many uneven systems per launch: grouped vs per-operator HBS solves.

    python -m sslablu_gb300.batchbench [--systems 512 --nrhs 8 --reps 20]

Workload (the solve stage of a batch of slab interface systems of uneven
sizes): ``--systems`` seeded synthetic exact HBS operators, interface size N
drawn from {128, 256, 512, 1024, 2048}, leaf 64, rank drawn from 16..48, a
leaf shift of 16 (the I + S form of the interface systems), ULV-factored on
the device; ``--nrhs`` right-hand sides ~ N(0, 1) per system.  One step
solves every system once.  Arms, each timed with CUDA events on the current
stream after warm-up (the factors of the batch exceed L2, so no flush):
  * per_operator_f64: one ``HBSMAT.solve`` sweep per system (2L-1 launches each, fewer
    where the top levels run as one composed operator);
  * grouped_f64: one grouped sweep for the whole batch (2 maxL - 1 launches);
  * grouped_f64_plan: the same sweep through a grouped solve plan (step
    tables built and uploaded once, the launches replayed as one graph);
  * grouped_mixed: grouped float32 sweeps refined to 1e-10 with double-float
    residuals;
  * grouped_mixed_plan: the same through a grouped refinement plan (buffers
    and task tables built once, each iteration replayed as a CUDA graph).
Prints one JSON line: RHS/s and systems/s per arm, the worst relative
residual of each arm against the float64 operators, and launches per step.
"""
import argparse
import json
import statistics
import time

import numpy as np
import torch

from . import _lib as L


def system_factors(systems, seed, sizes=(128, 256, 512, 1024, 2048), ranks=(16, 48),
                   shift=16.0):
    """(Umats, Dmats, Vmats, Nbvec) of the first `systems` systems of the batch."""
    from .synthetic import random_hbs_factors
    rng = np.random.default_rng(seed)
    out = []
    for j in range(systems):
        N = int(rng.choice(sizes))
        k = int(rng.integers(ranks[0], ranks[1] + 1))
        Lv = int(np.log2(N // 64)) + 1
        out.append(random_hbs_factors(k, 64, Lv, quad=False,
                                      rng=np.random.default_rng(seed + 1000 + j), shift=shift))
    return out


def build_batch(systems, seed):
    from .matAssembly.HBS.HBSnew import HBSMAT
    ops = []
    for U, D, V, Nbvec in system_factors(systems, seed):
        H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
        H.compute_ULV()
        ops.append(H)
    return ops


def _time(fn, reps, warmup=3):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    ts = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        fn()
        b.record(st)
        b.synchronize()
        ts.append(a.elapsed_time(b) * 1e-3)
    return ts


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--systems", type=int, default=512)
    ap.add_argument("--nrhs", type=int, default=8)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--seed", type=int, default=20261205)
    a = ap.parse_args()
    from .grouped import GroupedRefinePlan, GroupedSolvePlan, solve_grouped_device

    t0 = time.perf_counter()
    ops = build_batch(a.systems, a.seed)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    rng = np.random.default_rng(a.seed + 1)
    rhs = [torch.from_numpy(rng.standard_normal((H.shape[0], a.nrhs))).cuda() for H in ops]
    total = a.systems * a.nrhs
    work = [r.clone() for r in rhs]

    # the float64 arms solve in place: timed passes re-solve the previous
    # solution (the work does not depend on the values); the residual check
    # starts from a fresh copy of the right-hand sides
    def per_operator():
        for H, W in zip(ops, work):
            L.check(L.lib().slu_ulv_solve(L.handle(), H._op, L.ptr(W), a.nrhs, a.nrhs, 0))

    def grouped_f64():
        solve_grouped_device(ops, work)

    plan = GroupedSolvePlan(ops, work)

    def grouped_f64_plan():
        plan()

    outs = [torch.empty_like(r) for r in rhs]
    iters = []

    def grouped_mixed():
        _, it, _ = solve_grouped_device(ops, rhs, "mixed", 1e-10, 10, Xs=outs)
        iters.append(it)

    outs_p = [torch.empty_like(r) for r in rhs]
    rplan = GroupedRefinePlan(ops, rhs, outs_p)

    def grouped_mixed_plan():
        rplan(1e-10, 10)

    def worst_residual(xs):
        w = 0.0
        for H, B, X in zip(ops, rhs, xs):
            b = B.cpu().numpy()
            r = b - H.matmat(X.cpu().numpy())
            w = max(w, float(np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0))))
        return w

    def reset():
        for B, W in zip(rhs, work):
            W.copy_(B)

    out = {"workload": "%d synthetic exact HBS systems, N in {128..2048}, leaf 64, rank 16-48, "
                       "leaf shift 16, %d RHS each" % (a.systems, a.nrhs),
           "build_s": t_build, "rhs_per_step": total,
           "sizes": {str(n): int(c) for n, c in
                     zip(*np.unique([H.shape[0] for H in ops], return_counts=True))}}
    for name, fn, xs in [("per_operator_f64", per_operator, work),
                         ("grouped_f64", grouped_f64, work),
                         ("grouped_f64_plan", grouped_f64_plan, work),
                         ("grouped_mixed", grouped_mixed, outs),
                         ("grouped_mixed_plan", grouped_mixed_plan, outs_p)]:
        reset()
        fn()          # first call: one-time preparation (factor copies)
        torch.cuda.synchronize()
        reset()
        n0 = L.launch_count()
        fn()
        torch.cuda.synchronize()
        launches = L.launch_count() - n0
        ts = _time(fn, a.reps)
        med = statistics.median(ts)
        reset()
        fn()
        torch.cuda.synchronize()
        out[name] = {"ms_per_step": 1e3 * med, "rhs_per_s": total / med,
                     "systems_per_s": a.systems / med, "launches_per_step": launches,
                     "worst_relres": worst_residual(xs)}
    out["grouped_mixed"]["iterations"] = int(np.median(iters)) if iters else None
    out["grouped_vs_per_operator_f64"] = (out["grouped_f64"]["rhs_per_s"] /
                                          out["per_operator_f64"]["rhs_per_s"])
    out["grouped_mixed_vs_per_operator_f64"] = (out["grouped_mixed"]["rhs_per_s"] /
                                                out["per_operator_f64"]["rhs_per_s"])
    print(json.dumps(out))


if __name__ == "__main__":
    main()
