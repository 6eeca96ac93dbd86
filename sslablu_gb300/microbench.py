"""Kernel micro-benchmarks (CUDA-event timing on the launching stream).

    python -m sslablu_gb300.microbench tc_gemm [--m 4096 --n 261 --k 4096 --reps 20]
    python -m sslablu_gb300.microbench f64_gemm [...]

tc_gemm : slu_gemm_split3 (tcgen05 split-BF16x3, float32 accumulation)
f64_gemm: slu_gemm_batched (float64 CUDA-core GEMM) on the same shape
The default shape is the sketch product of an N = 4096 dense block with the
261 Gaussian samples of the rank-32 / leaf-64 HBS compression.  Prints one
JSON line with the median time, the tensor FLOP rate (6 split products) and
the effective rate (2 m n k).
"""
import argparse
import json
import statistics

import numpy as np
import torch

from . import _lib


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("kernel", choices=["tc_gemm", "f64_gemm"])
    ap.add_argument("--m", type=int, default=4096)
    ap.add_argument("--n", type=int, default=261)
    ap.add_argument("--k", type=int, default=4096)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    a = ap.parse_args()
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


if __name__ == "__main__":
    main()
