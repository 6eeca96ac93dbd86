"""Benchmark of the slab direct-solve hot path on one GB300.

Workload (the HBS configuration the headline metric is quoted on): a
synthetic exact HBS matrix, N = 4096, leaf 64, binary tree of 7 levels
(6 below the root), off-diagonal rank 32, leaf generators scaled so the
singular values decay geometrically from 1 to 1e-12; compressed with the
upstream randomized scheme (s = 4*32 + 2*64 + 5 = 261 Gaussian samples, the
count the upstream algorithm fixes) and ULV-factored on the GPU once, outside
the timed region (factor time reported separately).

A step is one batch of 16 right-hand sides ~ N(0, 1) solved to a relative
residual <= 1e-10 against the stored float64 HBS operator:
  plain  : float64 ULV solve (slu_ulv_solve)
  mixed  : ULV sweeps on the float32 units (double-float arithmetic) refined
           against a float64-accurate residual until every column reaches
           1e-10, the residual check inside every step (slu_refine)
  dfloat : the double-float ULV sweep alone (slu_ulv_solve_dfloat), its
           residual checked after the timed region as for plain
`value` is the plain float64 path's RHS solves/s; the other arms are reported
beside it.  `served` repeats the plain / mixed comparison at the batch widths
continuous batching serves one resident operator with (--served-rhs, default
1024 and 4096 right-hand sides), the mixed path there on the tensor cores
(digit-split bfloat16 tcgen05 products, refined to 1e-10).  Inputs (factors ~ 20 MB) fit in L2, so L2 is flushed (a 256 MB
write) before every timed step, outside the timed events.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the upstream numpy solve
(oracle/, a port: the upstream package does not travel) on the host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RHS solves/sec + p50/p99 latency at 1e-10 rel residual, mixed vs plain FP64"
UNIT = "RHS/s"
N, LEAF, LEVELS, RANK, NRHS = 4096, 64, 7, 32, 16
SEED = 20261205
TOL = 1e-10


def workload_config(extra=None):
    cfg = {"workload": "synthetic exact HBS N=4096 leaf=64 levels=7 rank=32 "
                       "sigma 1->1e-12, 16 RHS per step",
           "N": N, "leaf": LEAF, "levels": LEVELS, "rank": RANK, "nrhs": NRHS,
           "samples": 4 * RANK + 2 * LEAF + 5, "tol": TOL, "l2": "flushed before each step",
           "parallelism": "replicas"}
    if extra:
        cfg.update(extra)
    return cfg


def sigma():
    return 10.0 ** (-12.0 * np.arange(RANK) / (RANK - 1))


def make_problem():
    """(Umats, Dmats, Vmats), Nbvec and the right-hand sides of the workload."""
    from sslablu_gb300.synthetic import random_hbs_factors
    np.random.seed(SEED)
    U, D, V, Nbvec = random_hbs_factors(RANK, LEAF, LEVELS, quad=False, sigma=sigma())
    rhs = np.random.default_rng(SEED + 1).standard_normal((N, NRHS))
    return (U, D, V), Nbvec, rhs


# ---------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev=0, path=None):
        self.dev = dev
        self.proc = None
        self.path = path

    def start(self):
        try:
            if self.path is None:
                import tempfile
                fd, self.path = tempfile.mkstemp(prefix="slablu_clocks_", suffix=".csv")
                os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                stderr=subprocess.DEVNULL)
            # the sampler takes a moment to start: wait (at most 5 s) for its
            # first sample, so the timed region is covered
            t0 = time.time()
            while time.time() - t0 < 5.0 and os.path.getsize(self.path) == 0:
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def fp64_peak():
    """Float64 FMA throughput measured live on this GPU (slu_fp64_peak:
    register-only FMA chains, 8 CTAs per SM, CUDA events), TFLOP/s."""
    import ctypes
    from sslablu_gb300 import _lib
    tf, ms = ctypes.c_double(), ctypes.c_double()
    _lib.check(_lib.lib().slu_fp64_peak(_lib.handle(), 1 << 14, ctypes.byref(tf),
                                        ctypes.byref(ms)))
    return tf.value


# ---------------------------------------------------------------- CPU leg
def cpu_time_solve(O, rhs, reps):
    ts = []
    O.solve(rhs)
    for _ in range(reps):
        t0 = time.perf_counter()
        O.solve(rhs)
        ts.append(time.perf_counter() - t0)
    return ts


def cpu_baseline(mats, Nbvec, rhs, budget_s=15.0):
    """The CPU restatement of the upstream numpy ULV solve on the host cores."""
    from oracle.hbs import OracleHBS
    S = OracleHBS().set_mats(mats[0], mats[1], mats[2], list(Nbvec), fac=2)
    np.random.seed(SEED + 7)
    t0 = time.perf_counter()
    O = OracleHBS(S, None, Nbvec[0], len(Nbvec), 2).construct(RANK)
    t_factor = time.perf_counter() - t0
    one = cpu_time_solve(O, rhs, 1)[0]
    reps = max(3, min(200, int(budget_s / max(one, 1e-4))))
    ts = cpu_time_solve(O, rhs, reps)
    med = statistics.median(ts)
    return {"value": NRHS / med, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "%d solves of the 16-RHS batch (upstream ULVsparse.solve restated in "
                      "numpy), median; factor (compress+ULV) %.2f s" % (reps, t_factor),
            "p50_ms": 1e3 * med, "p99_ms": 1e3 * float(np.percentile(ts, 99)),
            "factor_s": t_factor}


def run_reference(args, rank, world):
    if rank != 0:
        return
    mats, Nbvec, rhs = make_problem()
    base = cpu_baseline(mats, Nbvec, rhs, budget_s=max(5.0, 2.0 * args.steps / 10))
    line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["p50_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference", "config": workload_config(),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------- roofline
# DRAM bytes (read + written) per launch of each solve step group, averaged
# over the group's launches in the ncu launch list of
# `python bench.py --steps 2 --warmup 3` (profiles/ulv_step_c2_launches.txt).
# DRAM bytes per launch from the ncu capture of the step kernels (per-level
# figures in profiles/ulv_step_c2_launches.txt), averaged over the levels the
# C2 chain launches: backward and forward levels 0-3 (the top operator stands
# in for levels 4 .. root)
NCU_TRAFFIC = {"step_kernel<double> (backward)": 2600000,
               "step_kernel<double> (forward)": 1297408,
               "step_kernel<double> (root)": 134016}


def launch_cost(kind, Nb, n, k, nu, c, leaf, single=False, top=False):
    """Algorithmic (bytes, flops) of one fused solve launch: the block
    operators read once, the right-hand-side blocks read and written once."""
    if kind == 1 and top:   # [y; v] = Top x, Top 2M x M for the M = Nb n rows of its level
        M = Nb * n
        return 8 * (2 * M * M + M * c + 2 * M * c), 2 * 2 * M * M * c
    if kind == 0:      # [ru; x_parent] = Q^T x
        rows, w = n, n
    elif kind == 1:    # [y; v] = [R^-1 Q^T; D R^-1 Q^T] x
        rows, w = (n if single else 2 * n), n
    else:              # [y_new; v_new] = [G; H] [ru; v; y_next]
        rows, w = (n if leaf else 2 * n), nu + 2 * k
    return 8 * Nb * (rows * w + w * c + rows * c), 2 * Nb * rows * w * c


def launch_roofline(H, B, flush, hbm, src, reps, fp64_tflops):
    """Per-launch device times of the float64 solve (event pairs around each
    launch, inside the library), the dominant launch, and its roofline.  The
    step kernels are float64-pipe bound (their bytes are ~2% of HBM
    bandwidth), so the roofline is their float64 rate against the measured
    float64 FMA peak; the HBM figure is kept beside it."""
    import ctypes
    import torch
    from sslablu_gb300 import _lib
    lib = _lib.lib()
    nl, nn = ctypes.c_int(), ctypes.c_int()
    geo = (ctypes.c_int * 256)()
    _lib.check(lib.slu_hbs_info(H._op, ctypes.byref(nl), ctypes.byref(nn), geo, None, None))
    cap = 64
    runs, meta = [], None
    c = B.shape[1]
    for _ in range(reps):
        flush.fill_(1.0)
        W = B.clone()
        ms = (ctypes.c_float * cap)()
        lvl = (ctypes.c_int * cap)()
        kind = (ctypes.c_int * cap)()
        cnt = ctypes.c_int()
        _lib.check(lib.slu_ulv_solve_timed(_lib.handle(), H._op, _lib.ptr(W), c, c, ms, lvl, kind,
                                           cap, ctypes.byref(cnt)))
        runs.append([ms[i] for i in range(cnt.value)])
        meta = [(lvl[i], kind[i]) for i in range(cnt.value)]
    med = np.median(np.array(runs), axis=0)
    names = {0: "forward", 1: "root", 2: "backward"}
    launches = []
    for (t, kd), m in zip(meta, med):
        Nb, n, k, nu = (geo[4 * t + j] for j in range(4))
        top = kd == 1 and t < nl.value - 1
        by, fl = launch_cost(kd, Nb, n, k, nu, c, t == 0, nl.value == 1, top)
        label = "top" if top else names[kd]
        launches.append({"kernel": "step_kernel<double> (%s)" % label, "level": t,
                         "ms": float(m), "alg_bytes": int(by), "alg_flops": int(fl)})
    # the dominant kernel: the one with the largest share of the solve; its
    # roofline uses per-launch averages over its launches (one per level)
    groups = {}
    for l in launches:
        groups.setdefault(l["kernel"], []).append(l)
    name, top = max(groups.items(), key=lambda kv: sum(x["ms"] for x in kv[1]))
    nl_ = len(top)
    sec = sum(x["ms"] for x in top) * 1e-3 / nl_
    by = sum(x["alg_bytes"] for x in top) / nl_
    fl = sum(x["alg_flops"] for x in top) / nl_
    achieved = by / sec / 1e9
    tflops = fl / sec / 1e12
    total = float(np.sum(med))
    return {"bound": "fp64", "achieved": tflops, "peak": fp64_tflops, "unit": "TFLOP/s",
            "frac": tflops / fp64_tflops, "traffic": NCU_TRAFFIC.get(name), "kernel": name,
            "launches_per_solve": nl_, "alg_flops_per_launch": int(fl),
            "alg_bytes_per_launch": int(by),
            "launch_ms": sec * 1e3, "share_of_solve": sum(x["ms"] for x in top) / total,
            "peak_source": "float64 FMA peak measured live (slu_fp64_peak)",
            "hbm": {"achieved_gbs": achieved, "peak_gbs": hbm, "frac": achieved / hbm,
                    "peak_source": ("hbm_gbs of measured peaks" if src == "measured"
                                    else "6.8 TB/s of fallback")},
            "device_ms_per_solve": total, "launches": launches}


# ---------------------------------------------------------------- replicas
def max_over_ranks(values, world, device):
    """Element-wise maximum over the ranks of a torch.distributed job (the
    slowest replica's times); the values themselves when world == 1."""
    if world <= 1:
        return list(values)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def replica_throughput(world, units_per_rank, slowest_seconds):
    """Whole-job throughput of `world` independent replicas that each process
    `units_per_rank` units, timed by the slowest one."""
    return world * units_per_rank / slowest_seconds


# ---------------------------------------------------------------- GPU leg
def served_widths(H, args, flush, stream, timed, world):
    """The same operator at served batch widths (continuous batching gathers
    many requests for one resident operator into one solve): plain float64
    solves against the mixed path with the tensor-core sweep and residual
    (HBSMAT.solve_refined(inner='tensor'): every step product as bfloat16
    tcgen05 products of error-free digit splits, refined to 1e-10 against a
    float64-accurate residual of the stored operator).  Per width: RHS/s,
    p50/p99 of the step, iterations, worst residual (float64 apply, after the
    timed region) and the speedup."""
    import torch
    out = []
    for c in args.served_rhs:
        Bc = torch.from_numpy(np.random.default_rng(SEED + c).standard_normal((N, c))).cuda()
        steps = max(3, min(args.steps, 10))
        ts_p, l_p, Xp = timed(lambda: H._dev_solve(Bc, False), steps, args.warmup)
        ts_m, l_m, mo = timed(lambda: H.solve_refined(Bc, tol=TOL, maxit=10, inner="tensor"),
                              steps, args.warmup)
        Xm, iters, _ = mo
        R = Bc - H._dev_apply(Xm, False)
        res = float((R.norm(dim=0) / Bc.norm(dim=0)).max())
        err = float((Xm - Xp).norm() / Xp.norm())
        tp, tm = sum(ts_p), sum(ts_m)
        out.append({"nrhs": c,
                    "plain": {"value": world * c * steps / tp, "unit": UNIT,
                              "p50_ms": 1e3 * statistics.median(ts_p), "gpu_launches": l_p,
                              "arm": "float64 ULV solve (HBSMAT.solve)"},
                    "mixed": {"value": world * c * steps / tm, "unit": UNIT,
                              "p50_ms": 1e3 * statistics.median(ts_m),
                              "p99_ms": 1e3 * float(np.percentile(ts_m, 99)),
                              "iters": iters, "relres": res, "relerr_vs_plain": err,
                              "speedup_vs_plain": tp / tm, "gpu_launches": l_m,
                              "dtype": "bf16 tcgen05 products of error-free digit splits "
                                       "(f32 accumulation) + f64-accurate residual refinement"}})
        del Bc
    return out


def run_gpu(args, rank, world):
    import torch
    import torch.distributed as dist
    from sslablu_gb300 import _lib
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    mats, Nbvec, rhs = make_problem()
    # operator to compress: the exact HBS matrix, resident on the device
    A = HBSMAT().set_mats(mats[0], mats[1], mats[2], list(Nbvec), fac=2)
    np.random.seed(SEED + 7)
    # compression + ULV: the first call pays library and module loading and
    # workspace growth (reported as cold); factor_s is the median of three
    # warm factorisations of the same operator with the same sketches
    t_cold, t_warm = None, []
    for rep in range(4):
        np.random.seed(SEED + 7)
        Hr = HBSMAT(A, tree=None, quad=False)
        Hr.set_Nbvec(list(Nbvec))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Hr.construct(RANK, True)
        torch.cuda.synchronize()
        if rep == 0:
            t_cold = time.perf_counter() - t0
        else:
            t_warm.append(time.perf_counter() - t0)
        H = Hr
    t_factor = statistics.median(t_warm)
    H.solve_refined(rhs[:, :1], tol=TOL, maxit=10)   # prepares the double-float factors
    # launch plans of the 16-column solves picked by the autotuner (untimed)
    tuned = {"f64": H.autotune(NRHS), "dfloat": H.autotune(NRHS, "dfloat")}
    torch.cuda.synchronize()

    B = torch.from_numpy(rhs).cuda()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    # repeated solves through fixed buffers: the solve plan replays the 13
    # step launches (tuned plans) as one CUDA graph
    plan_dev = H.solve_plan(B)

    def plain_step():
        return plan_dev()

    def per_call_step():
        return H._dev_solve(B, False)

    def mixed_step():
        return H.solve_refined(B, tol=TOL, maxit=10)

    def dfloat_step():
        return H.solve_dfloat(B)

    def residual(X):
        R = B - H._dev_apply(X, False)
        return float((R.norm(dim=0) / B.norm(dim=0)).max())

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        ts = []
        n0 = _lib.launch_count()
        for _ in range(steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        launches = _lib.launch_count() - n0
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        return ts, launches, out

    clocks = ClockSampler(dev)
    clocks.start()
    ts_plain, launches_plain, Xp = timed(plain_step, args.steps, args.warmup)
    Xp = Xp.clone()
    ts_call, _, _ = timed(per_call_step, args.steps, args.warmup)
    ts_mixed, launches_mixed, mixed_out = timed(mixed_step, args.steps, args.warmup)
    ts_df, launches_df, Xd = timed(dfloat_step, args.steps, args.warmup)
    # end-to-end through the public API: a solve plan over a pinned host
    # block (the first solve step reads it from host memory over NVLink-C2C,
    # the last writes the solution into the pinned host result; every byte
    # crosses host <-> device once each way inside the timed region, and the
    # call returns when the result is in host memory)
    hp = torch.from_numpy(rhs).pin_memory()
    out_h = torch.empty_like(hp).pin_memory()
    plan_host = H.solve_plan(hp, out_h)

    def e2e_times(fn):
        ts = []
        for i in range(args.warmup + args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            if i >= args.warmup:
                ts.append(time.perf_counter() - t0)
        return ts
    e2e = e2e_times(plan_host)
    e2e_call = e2e_times(lambda: H.solve(hp, out=out_h))
    served = served_widths(H, args, flush, stream, timed, world)
    clk = clocks.stop()

    res_plain = residual(Xp)
    Xm, iters, relres = mixed_out
    res_mixed = residual(Xm)
    res_df = residual(Xd)
    tot_plain, tot_mixed, tot_df, tot_e2e = max_over_ranks(
        [sum(ts_plain), sum(ts_mixed), sum(ts_df), sum(e2e)], world, "cuda")
    value = replica_throughput(world, NRHS * args.steps, tot_plain)
    p50 = statistics.median(ts_plain)
    hbm, src = peaks()
    roof = launch_roofline(H, B, flush, hbm, src, reps=max(5, args.steps),
                           fp64_tflops=fp64_peak())
    line = None
    if rank == 0:
        base = cpu_baseline(mats, Nbvec, rhs)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot_plain / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": workload_config({"factor_s": t_factor, "factor_cold_s": t_cold,
                                       "factor_s_is": "median of 3 warm compress + ULV calls",
                                       "arm": "plain float64 ULV solve through a solve plan "
                                              "(HBSMAT.solve_plan: the 9 step launches "
                                              "replayed as one CUDA graph)",
                                       "launch_plans": "autotuned per launch (target CTAs/SM, "
                                                       "row floor, column cap)",
                                       "tuned": tuned}),
            "p50_ms": 1e3 * p50, "p99_ms": 1e3 * float(np.percentile(ts_plain, 99)),
            "relres": res_plain,
            "per_call": {"value": world * NRHS * args.steps / sum(ts_call), "unit": UNIT,
                         "arm": "HBSMAT solve per call (9 stream launches)",
                         "p50_ms": 1e3 * statistics.median(ts_call),
                         "e2e_value": world * NRHS * args.steps / sum(e2e_call),
                         "e2e_p50_ms": 1e3 * statistics.median(e2e_call)},
            "mixed": {"value": world * NRHS * args.steps / tot_mixed, "unit": UNIT,
                      "dtype": "double-float (f32 pairs) ULV sweep + f64-accurate residual "
                               "refinement to 1e-10",
                      "p50_ms": 1e3 * statistics.median(ts_mixed),
                      "p99_ms": 1e3 * float(np.percentile(ts_mixed, 99)),
                      "iters": iters, "relres": res_mixed,
                      "speedup_vs_plain": tot_plain / tot_mixed,
                      "gpu_launches": launches_mixed},
            "served": served,
            "dfloat": {"value": world * NRHS * args.steps / tot_df, "unit": UNIT,
                       "dtype": "double-float (f32 pairs) ULV sweep, no refinement",
                       "p50_ms": 1e3 * statistics.median(ts_df),
                       "p99_ms": 1e3 * float(np.percentile(ts_df, 99)), "relres": res_df,
                       "speedup_vs_plain": tot_plain / tot_df, "gpu_launches": launches_df},
            "e2e": {"value": world * NRHS * args.steps / tot_e2e, "unit": UNIT,
                    "h2d_bytes_per_step": int(rhs.nbytes), "d2h_bytes_per_step": int(rhs.nbytes),
                    "p50_ms": 1e3 * statistics.median(e2e)},
            "gpu_launches": launches_plain,
            "roofline": roof,
            "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "clocks": clk,
        }
        print(json.dumps(line))
    return line


# ---------------------------------------------------------------- other rows
# `--workload` measures the other slab-solver rows, one JSON line each, with
# the oracle (the numpy restatement of the upstream solver) timed beside the
# GPU path on the host cores.  Single GPU; the headline remains the default.
def run_other(args):
    import types
    import torch
    from oracle import direct as od
    torch.cuda.set_device(0)
    base = {"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic"}
    if args.workload == "c1_dense":
        from sslablu_gb300 import slabbench
        from sslablu_gb300.synthetic import slab_couplings
        m, nS = 256, 8
        g = slabbench.dense(types.SimpleNamespace(m=m, slabs=nS, reps=args.steps))
        S = slab_couplings(m, nS)
        T = [np.eye(m) for _ in range(nS)]
        B = np.random.default_rng(1).standard_normal((nS * m, 64))
        cpu = {}
        for name, cls in (("rb_f64", od.RedBlackDense), ("thomas_f64", od.ThomasDense)):
            t0 = time.perf_counter()
            sv = cls(m).factorize(S, T)
            t_f = time.perf_counter() - t0
            ts = []
            for _ in range(3):
                t0 = time.perf_counter()
                sv.solve(B)
                ts.append(time.perf_counter() - t0)
            cpu[name] = {"factor_ms": 1e3 * t_f, "rhs_per_s_64rhs": 64 / statistics.median(ts)}
        line = dict(base, metric="dense red-black RHS solves/sec, 64 RHS", unit="RHS/s",
                    value=g["rb_f64"]["rhs_per_s_64rhs"],
                    ms_per_step=g["rb_f64"]["solve_64rhs_ms"],
                    config={"workload": g["workload"], "slabs": nS, "m": m, "nrhs": 64},
                    arms=g,
                    cpu_baseline={"value": cpu["rb_f64"]["rhs_per_s_64rhs"], "unit": "RHS/s",
                                  "cores": os.cpu_count(), "kind": "port",
                                  "sample": "upstream RedBlackSolver / BlockTridiagonalSolver "
                                            "restated in numpy, same system, 64 RHS",
                                  "arms": cpu})
    elif args.workload == "c3_hbs":
        from sslablu_gb300 import slabbench
        from sslablu_gb300.synthetic import slab_couplings
        m, nS, leaf, rk, m_cpu = 1024, 8, 64, 24, 256
        ns = types.SimpleNamespace(m=m, slabs=nS, leaf=leaf, rank=rk, reps=max(3, args.steps // 5))
        g = slabbench.hbs(ns)
        g_small = slabbench.hbs(types.SimpleNamespace(m=m_cpu, slabs=nS, leaf=leaf, rank=rk,
                                                      reps=ns.reps))
        S = slab_couplings(m_cpu, nS)
        B = np.random.default_rng(2).standard_normal((nS * m_cpu, 64))
        td = (np.arange(m_cpu), m_cpu // leaf, int(np.log2(m_cpu // leaf)) + 1)
        Sop = [(od.dense_op(x), od.dense_op(y)) for x, y in S]
        cpu = {}
        for name, cls in (("rb_hbs", od.RedBlackHBS), ("thomas_hbs", od.ThomasHBS)):
            np.random.seed(11)
            t0 = time.perf_counter()
            sv = cls(m_cpu, rk, td, False).factorize(Sop)
            t_f = time.perf_counter() - t0
            t0 = time.perf_counter()
            try:
                sv.solve(B)
            except ValueError:   # the upstream red-black HBS solve takes one column
                for j in range(B.shape[1]):
                    sv.solve(B[:, j])
            t_s = time.perf_counter() - t0
            cpu[name] = {"m": m_cpu, "factor_ms": 1e3 * t_f, "rhs_per_s_64rhs": 64 / t_s,
                         "gpu_same_size": g_small[name]}
        line = dict(base, metric="HBS red-black RHS solves/sec, 64 RHS", unit="RHS/s",
                    value=g["rb_hbs"]["rhs_per_s_64rhs"],
                    ms_per_step=g["rb_hbs"]["solve_64rhs_ms"],
                    config={"workload": g["workload"], "slabs": nS, "m": m, "leaf": leaf,
                            "rank": rk, "nrhs": 64},
                    arms=g,
                    cpu_baseline={"value": cpu["rb_hbs"]["rhs_per_s_64rhs"], "unit": "RHS/s",
                                  "cores": os.cpu_count(), "kind": "port",
                                  "sample": "upstream RedBlackSolverHBS / ThomasSolverHBS "
                                            "restated in numpy at %d-point interfaces (the GPU "
                                            "at the same size is in arms.gpu_same_size)" % m_cpu,
                                  "arms": cpu})
    elif args.workload == "c3":
        # the C3 operators themselves: 3-D variable-coefficient Helmholtz slabs
        # (k = 20), 33 slabs, 32 interfaces of 64 x 64 points, GMRES on the
        # exact interface operator with the mixed dense red-black preconditioner
        from sslablu_gb300 import slabbench
        ns = types.SimpleNamespace(slabs=33, n=64, kappa=20.0, prec="dense", prec_kappa=20.0,
                                   leaf=128, rank=64, nrhs=64, reps=max(1, min(3, args.steps)),
                                   maxiter=100)
        g = slabbench.helmholtz(ns)
        # CPU: upstream's pipeline restated (sparse-LU slab maps, dense red-black,
        # GMRES) at 17 slabs x 16 x 16 points, a size it runs in seconds
        from scipy.sparse.linalg import LinearOperator, gmres as sgmres
        from oracle.slabmaps import helmholtz3d_slab_maps
        cs, cn = 17, 16
        H = 1.0 / cs
        t0 = time.perf_counter()
        maps = [helmholtz3d_slab_maps(5, cn + 2, cn + 2, 2 * H, 20.0, x0=i * H)
                for i in range(cs - 1)]
        mm, nif = cn * cn, cs - 1
        Sx = [(maps[i][0] if i > 0 else np.zeros((mm, mm)),
               maps[i][1] if i < nif - 1 else np.zeros((mm, mm))) for i in range(nif)]
        rbc = od.RedBlackDense(mm).factorize(Sx, [np.eye(mm)] * nif)
        t_build = time.perf_counter() - t0
        Mtot = np.eye(nif * mm)
        for i in range(nif):
            if i > 0:
                Mtot[i * mm:(i + 1) * mm, (i - 1) * mm:i * mm] = Sx[i][0]
            if i < nif - 1:
                Mtot[i * mm:(i + 1) * mm, (i + 1) * mm:(i + 2) * mm] = Sx[i][1]
        bc = np.random.default_rng(3).standard_normal((nif * mm, 64))
        Pre = LinearOperator(Mtot.shape, matvec=lambda v: rbc.solve(v[:, None])[:, 0])
        t0 = time.perf_counter()
        for j in range(bc.shape[1]):
            try:
                sgmres(Mtot, bc[:, j], M=Pre, rtol=1e-10, restart=30, maxiter=100)
            except TypeError:   # scipy before 1.12 names it tol
                sgmres(Mtot, bc[:, j], M=Pre, tol=1e-10, restart=30, maxiter=100)
        t_cpu = time.perf_counter() - t0
        line = dict(base, metric="3-D Helmholtz slab system RHS solves/sec at 1e-10 rel residual",
                    unit="RHS/s", value=g["rhs_per_s"], ms_per_step=1e3 * g["solve_s"],
                    config={"workload": g["workload"], "interfaces": g["interfaces"],
                            "m": g["m"], "nrhs": g["nrhs"]},
                    arms=g,
                    cpu_baseline={"value": bc.shape[1] / t_cpu, "unit": "RHS/s",
                                  "cores": os.cpu_count(), "kind": "port",
                                  "sample": "upstream pipeline restated (sparse-LU slab maps, "
                                            "dense red-black preconditioned scipy GMRES) at 17 "
                                            "slabs x 16 x 16 points, 64 RHS; build %.2f s"
                                            % t_build})
    elif args.workload == "c3_strong":
        # strong-admissibility HBS (HBStorch_strong) of a coupling between two
        # 64 x 64 interface planes (C3's interface size), full adjacency
        from sslablu_gb300 import slabbench
        from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
        from sslablu_gb300.synthetic import plane_coupling, plane_points
        from oracle.strong import StrongHBS
        ns = types.SimpleNamespace(n=64, leaf=128, rank=32, adjacency="full", nrhs=64,
                                   reps=max(3, min(10, args.steps)))
        g = slabbench.strong(ns)
        XX = plane_points(ns.n)
        A = plane_coupling(XX)
        N, s = A.shape[0], g["samples"]
        rng = np.random.default_rng(0)
        Om, Psi = rng.standard_normal((N, s)), rng.standard_normal((N, s))
        tree = slabTree(XX, False, ns.leaf, adjacency="full")
        O = StrongHBS(tree.perm_leaf, tree.nleaves, tree.level_adj_list)
        t0 = time.perf_counter()
        O.construct(ns.rank, Om, Psi, A @ Om, A.T @ Psi)
        t_con = time.perf_counter() - t0
        X = rng.standard_normal((N, ns.nrhs))
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            O.apply(X)
            ts.append(time.perf_counter() - t0)
        line = dict(base, metric="strong-admissibility HBS applies (RHS/s), 64 RHS", unit="RHS/s",
                    value=g["apply_rhs_per_s"], ms_per_step=g["apply_ms"],
                    config={"workload": g["workload"], "N": N, "samples": s,
                            "construct_s": g["construct_s"]},
                    arms=g,
                    cpu_baseline={"value": ns.nrhs / statistics.median(ts), "unit": "RHS/s",
                                  "cores": os.cpu_count(), "kind": "port",
                                  "sample": "upstream HBStorch_strong restated in numpy "
                                            "(oracle), same operator and sketches, 64 RHS; "
                                            "construct %.2f s" % t_con,
                                  "construct_s": t_con})
    elif args.workload == "c4_rbhbs":
        # C4 as slab systems: uneven 2-D Poisson interface systems, each red-black
        # HBS factored, solved together through one grouped program per step
        from sslablu_gb300 import rbbatch
        from sslablu_gb300.synthetic import poisson_slab_map
        g, specs, built, Bs, res = rbbatch.run(systems=args.systems, nrhs=8,
                                               reps=max(3, min(10, args.steps)))
        # CPU: the oracle's red-black HBS (upstream's restated in numpy) on
        # the first systems of the batch with 128-point interfaces
        t_f = t_s = 0.0
        nrhs_cpu, used = 0, 0
        for (nI, m, rk), (rb, S, P), B in zip(specs, built, Bs):
            if m != 128 or used >= 3:
                continue
            H = rb.RB[0][0][1]
            td = (np.asarray(H.tree.perm_leaf), H.tree.nleaves, H.tree.nlevels)
            Sd = S.cpu().numpy()
            Z = np.zeros((m, m))
            Sop = [(od.dense_op(Sd if 0 < i < nI else Z), od.dense_op(Sd if i < nI - 1 else Z))
                   for i in range(P)]
            np.random.seed(11)
            t0 = time.perf_counter()
            sv = od.RedBlackHBS(m, rk, td, False).factorize(Sop)
            t_f += time.perf_counter() - t0
            b = B.cpu().numpy()
            t0 = time.perf_counter()
            for j in range(b.shape[1]):
                sv.solve(b[:, j])
            t_s += time.perf_counter() - t0
            nrhs_cpu += b.shape[1]
            used += 1
        line = dict(base, metric="batched red-black HBS RHS solves/sec (uneven 2-D Poisson "
                                 "slab systems x 8 RHS)", unit="RHS/s",
                    value=g["grouped_plan"]["rhs_per_s"],
                    ms_per_step=g["grouped_plan"]["ms_per_step"],
                    config={"workload": g["workload"], "systems": g["systems"],
                            "sizes": g["sizes"], "factor_s": g["factor_s"],
                            "factor_workers": g["factor_workers"],
                            "arm": "every system's red-black solve as one grouped program "
                                   "(GroupedRBSolvePlan: one CUDA graph per step)"},
                    gpu_launches=g["grouped_plan"]["gpu_launches"],
                    arms=g,
                    cpu_baseline={"value": nrhs_cpu / t_s if t_s else None, "unit": "RHS/s",
                                  "cores": os.cpu_count(), "kind": "port",
                                  "sample": "upstream RedBlackSolverHBS restated in numpy, "
                                            "the first %d systems with 128-point interfaces "
                                            "(dense couplings), 8 RHS each; factor %.2f s"
                                            % (used, t_f)})
    else:   # c4_batch
        import subprocess
        out = subprocess.run([sys.executable, "-m", "sslablu_gb300.batchbench", "--reps",
                              str(args.steps)], capture_output=True, text=True, check=True)
        g = json.loads(out.stdout.strip().splitlines()[-1])
        # CPU: the oracle's per-system ULV solve over a sample of the systems
        from sslablu_gb300.batchbench import system_factors
        sample = system_factors(32, 20261205)
        ts = 0.0
        nrhs = 0
        for U, D, V, Nbvec in sample:
            O = od_hbs().set_mats(U, D, V, list(Nbvec), fac=2)
            O.compute_ULV()
            b = np.random.default_rng(3).standard_normal((O.shape[0], 8))
            t0 = time.perf_counter()
            O.solve(b)
            ts += time.perf_counter() - t0
            nrhs += 8
        line = dict(base, metric="batched HBS RHS solves/sec (512 uneven systems x 8 RHS)",
                    unit="RHS/s", value=g["grouped_f64_plan"]["rhs_per_s"],
                    ms_per_step=g["grouped_f64_plan"]["ms_per_step"],
                    config={"workload": g["workload"], "sizes": g["sizes"],
                            "arm": "grouped float64 sweep through a grouped solve plan (step "
                                   "tables built once, launches replayed as one CUDA graph)"},
                    mixed={"value": g["grouped_mixed_plan"]["rhs_per_s"], "unit": "RHS/s",
                           "dtype": "grouped double-float sweeps + double-float residuals, "
                                    "refined to 1e-10 (grouped refinement plan)",
                           "ms_per_step": g["grouped_mixed_plan"]["ms_per_step"],
                           "speedup_vs_plain": g["grouped_mixed_plan"]["rhs_per_s"] /
                           g["grouped_f64_plan"]["rhs_per_s"]},
                    arms=g,
                    cpu_baseline={"value": nrhs / ts, "unit": "RHS/s", "cores": os.cpu_count(),
                                  "kind": "port",
                                  "sample": "upstream ULVsparse.solve restated in numpy, the "
                                            "first 32 of the 512 systems, 8 RHS each"})
    print(json.dumps(line))


def od_hbs():
    from oracle.hbs import OracleHBS
    return OracleHBS()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="c2",
                    choices=["c2", "c1_dense", "c3_hbs", "c3", "c3_strong", "c4_batch",
                             "c4_rbhbs"])
    ap.add_argument("--systems", type=int, default=512,
                    help="c4_rbhbs: number of slab systems in the batch")
    ap.add_argument("--served-rhs", type=lambda v: [int(x) for x in v.split(",") if x],
                    default=[1024, 4096],
                    help="batch widths of the served mixed vs plain comparison (comma separated)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.workload != "c2":
        return run_other(args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "native":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)
    if world > 1 and args.impl == "native":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
