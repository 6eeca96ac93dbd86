"""Kernel micro-benchmarks (CUDA-event timing on the launching stream), beside
bench.py: the commands the kernel summaries under profiles/ were made with.

    python bench_kernels.py tc_gemm [--m 4096 --n 261 --k 4096 --reps 20]
    python bench_kernels.py f64_gemm [...]

    python bench_kernels.py compress [--m 4096 --reps 5]
    python bench_kernels.py solve [--m 4096 --n 16 --reps 20]
    python bench_kernels.py refine [--m 4096 --reps 10]

tc_gemm : slu_gemm_split3 (tcgen05 split-BF16x3, float32 accumulation)
f64_gemm: slu_gemm_batched (float64 CUDA-core GEMM) on the same shape
The default shape is the sketch product of an N = 4096 dense block with the
261 Gaussian samples of the rank-32 / leaf-64 HBS compression.  Prints one
JSON line with the median time, the tensor FLOP rate (6 split products) and
the effective rate (2 m n k).
solve: the float64 ULV solve (mode N) of a synthetic exact HBS operator of
size m (leaf 64, rank 32, ULV from the given factors) with n right-hand
sides, three ways: per-step launches (slu_ulv_solve), the mode-T solve
(the transposed steps) and the grouped sweep of a one-member group; prints
the median time per solve of each.  With
--precision dfloat: the double-float sweep (slu_ulv_solve_dfloat) instead.
refine: float64 ULV solve against the double-float sweep alone and against
mixed-precision refinement to 1e-10 with double-float and with float32 inner
sweeps (double-float residuals) on the same operator, for 16, 64, 256 and
1024 right-hand sides; prints the times, iterations and ratios.
compress: HBSMAT.construct(32, compute_ULV=True) of a synthetic exact HBS
operator of size m (leaf 64, rank 32, singular values 1 -> 1e-12), the
sketches sampled through the resident operator; prints the median time and
the relative error of the compressed operator's apply.
"""
import argparse
import os
import sys
import json
import statistics

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from sslablu_gb300 import _lib


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("kernel", choices=["tc_gemm", "f64_gemm", "compress", "solve", "refine",
                                       "tensor"])
    ap.add_argument("--m", type=int, default=4096)
    ap.add_argument("--n", type=int, default=261)
    ap.add_argument("--k", type=int, default=4096)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--widths", default="", help="refine: right-hand-side counts, comma separated")
    ap.add_argument("--precision", default="f64", choices=["f64", "dfloat"],
                    help="solve: float64 (per-level and grouped) or the double-float sweep")
    a = ap.parse_args()
    if a.kernel == "compress":
        return compress(a)
    if a.kernel == "solve":
        return solve(a)
    if a.kernel == "refine":
        return refine(a)
    if a.kernel == "tensor":
        return tensor_sweep(a)
    m, n, k = a.m, a.n, a.k
    rng = np.random.default_rng(0)
    A = torch.from_numpy(rng.standard_normal((m, k))).cuda()
    B = torch.from_numpy(rng.standard_normal((k, n))).cuda()
    C = torch.zeros((m, n), dtype=torch.float64, device="cuda")
    L, h = _lib.lib(), _lib.handle()

    def run():
        if a.kernel == "tc_gemm":
            _lib.check(L.slu_gemm_split3(h, m, n, k, 1.0, _lib.ptr(A), k, _lib.ptr(B), n, 0.0,
                                         _lib.ptr(C), n))
        else:
            _lib.check(L.slu_gemm_batched(h, 0, 0, m, n, k, 1.0, _lib.ptr(A), k, 0, _lib.ptr(B),
                                          n, 0, 0.0, _lib.ptr(C), n, 0, 1))

    for _ in range(a.warmup):
        run()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    ts = []
    for _ in range(a.reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        run()
        e1.record(st)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    _lib.sync()
    t = statistics.median(ts)
    eff = 2.0 * m * n * k
    tensor = 6 * 2.0 * m * n * (-(-k // 64) * 64) if a.kernel == "tc_gemm" else eff
    ref = (A @ B)
    err = float(torch.linalg.norm(C - ref) / torch.linalg.norm(ref))
    print(json.dumps({"kernel": a.kernel, "m": m, "n": n, "k": k, "median_ms": 1e3 * t,
                      "tensor_tflops": tensor / t / 1e12, "effective_tflops": eff / t / 1e12,
                      "relerr": err}))


def solve(a):
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import decaying_sigma, random_hbs_factors
    N, c = a.m, a.n
    Lv = int(np.log2(N // 64)) + 1
    np.random.seed(1)
    U, D, V, Nbvec = random_hbs_factors(32, 64, Lv, quad=False, sigma=decaying_sigma(32),
                                        shift=16.0)
    H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
    H.compute_ULV()
    B = torch.from_numpy(np.random.default_rng(2).standard_normal((N, c))).cuda()
    W = B.clone()
    L, h = _lib.lib(), _lib.handle()

    import ctypes
    ops = (ctypes.c_void_p * 1)(H._op)
    bp = (ctypes.c_void_p * 1)(W.data_ptr())
    ld = (ctypes.c_int * 1)(c)

    def per_level():
        _lib.check(L.slu_ulv_solve(h, H._op, _lib.ptr(W), c, c, 0))

    def mode_T():
        _lib.check(L.slu_ulv_solve(h, H._op, _lib.ptr(W), c, c, 1))

    def grouped():
        _lib.check(L.slu_ulv_solve_grouped(h, 1, ops, bp, ld, ld))

    def dfloat():
        _lib.check(L.slu_ulv_solve_dfloat(h, H._op, _lib.ptr(W), c, c))

    out = {"kernel": "solve", "N": N, "nrhs": c, "levels": Lv}
    st = torch.cuda.current_stream()
    arms = {"f64": (("per_level", per_level), ("mode_T", mode_T), ("grouped", grouped)),
            "dfloat": (("dfloat", dfloat),)}[a.precision]
    for name, run in arms:
        for _ in range(a.warmup):
            run()
        torch.cuda.synchronize()
        ts = []
        for _ in range(a.reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            run()
            e1.record(st)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        _lib.sync()
        out[name + "_ms"] = 1e3 * statistics.median(ts)
    print(json.dumps(out))


def tensor_sweep(a):
    """The tensor-core sweep (slu_ulv_solve_ozaki) and apply on the N = m,
    leaf 64, rank 32 operator for --n right-hand sides: median times."""
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import decaying_sigma, random_hbs_factors
    N, c = a.m, a.n
    Lv = int(np.log2(N // 64)) + 1
    np.random.seed(1)
    U, D, V, Nbvec = random_hbs_factors(32, 64, Lv, quad=False, sigma=decaying_sigma(32),
                                        shift=16.0)
    H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
    H.compute_ULV()
    B = torch.from_numpy(np.random.default_rng(c).standard_normal((N, c))).cuda()
    st = torch.cuda.current_stream()
    out = {"kernel": "tensor", "N": N, "nrhs": c}
    for name, fn in (("solve", lambda: H.solve_ozaki(B)), ("apply", lambda: H.apply_ozaki(B))):
        for _ in range(a.warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(a.reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        out[name + "_ms"] = statistics.median(ts) if ts else None
    print(json.dumps(out))


def refine(a):
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import decaying_sigma, random_hbs_factors
    N = a.m
    Lv = int(np.log2(N // 64)) + 1
    np.random.seed(1)
    U, D, V, Nbvec = random_hbs_factors(32, 64, Lv, quad=False, sigma=decaying_sigma(32),
                                        shift=16.0)
    H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
    H.compute_ULV()
    st = torch.cuda.current_stream()
    out = {"kernel": "refine", "N": N}

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(a.reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return statistics.median(ts)

    widths = [int(x) for x in a.widths.split(",")] if a.widths else (16, 64, 256, 1024)
    for c in widths:
        B = torch.from_numpy(np.random.default_rng(c).standard_normal((N, c))).cuda()
        t64 = timed(lambda: H._dev_solve(B, False))
        x64 = H._dev_solve(B, False)
        tdf = timed(lambda: H.solve_dfloat(B))
        xdf = H.solve_dfloat(B)
        row = {"f64_ms": 1e3 * t64, "dfloat_ms": 1e3 * tdf, "dfloat_speedup": t64 / tdf,
               "dfloat_vs_f64": float(torch.linalg.norm(xdf - x64) / torch.linalg.norm(x64))}
        # tensor-core sweep (digit-split bfloat16 products) and apply
        toz = timed(lambda: H.solve_ozaki(B))
        xoz = H.solve_ozaki(B)
        row.update({"tensor_ms": 1e3 * toz, "tensor_speedup": t64 / toz,
                    "tensor_vs_f64": float(torch.linalg.norm(xoz - x64) /
                                           torch.linalg.norm(x64))})
        ta64 = timed(lambda: H._dev_apply(x64, False))
        taoz = timed(lambda: H.apply_ozaki(x64))
        row.update({"apply_f64_ms": 1e3 * ta64, "apply_tensor_ms": 1e3 * taoz,
                    "apply_tensor_vs_f64": float(torch.linalg.norm(H.apply_ozaki(x64) -
                                                                   H._dev_apply(x64, False)) /
                                                 torch.linalg.norm(B))})
        for inner in ("dfloat", "float32", "tensor"):
            res = {}
            tmx = timed(lambda: res.update(r=H.solve_refined(B, tol=1e-10, inner=inner)))
            row["mixed_%s_ms" % inner] = 1e3 * tmx
            row["mixed_%s_speedup" % inner] = t64 / tmx
            row["mixed_%s_iters" % inner] = res["r"][1]
            row["mixed_%s_relres" % inner] = res["r"][2]
        out["c%d" % c] = row
    print(json.dumps(out))


def compress(a):
    import time
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import decaying_sigma, random_hbs_factors
    N = a.m
    Lv = int(np.log2(N // 64)) + 1
    np.random.seed(1)
    U, D, V, Nbvec = random_hbs_factors(32, 64, Lv, quad=False, sigma=decaying_sigma(32))
    A = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
    ts = []
    H = None
    for i in range(a.warmup + a.reps):
        H = HBSMAT(A, tree=None, quad=False)
        H.set_Nbvec(list(Nbvec))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        H.construct(32, True)
        torch.cuda.synchronize()
        if i >= a.warmup:
            ts.append(time.perf_counter() - t0)
    x = np.random.default_rng(2).standard_normal((N, 4))
    err = float(np.linalg.norm(H.matmat(x) - A.matmat(x)) / np.linalg.norm(A.matmat(x)))
    print(json.dumps({"kernel": "compress", "N": N, "levels": Lv, "rank": 32,
                      "samples": H.nSamples, "median_ms": 1e3 * statistics.median(ts),
                      "apply_relerr": err}))


if __name__ == "__main__":
    main()
