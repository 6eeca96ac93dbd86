"""Serving loop for resident factored slab operators.

Factored operators (HBS ULV factors or red-black factors) stay resident in
device memory under a byte budget; solve requests (an operator key and a host
block of right-hand sides) arrive over time and are batched per operator.

    srv = SolveServer(budget_bytes=8 << 30, workers=4, max_batch_rhs=64)
    srv.admit("op0", factory, footprint)      # factory() -> factored operator
    srv.run(requests)                         # requests: [Request(key, B, t_arrival)]
    srv.stats()                               # latency p50/p99, RHS/s

Scheduling (continuous batching):
  * a dispatcher thread admits requests at their arrival time into per-
    operator queues;
  * whenever a worker is idle, the operator whose oldest pending request is
    the oldest gets a batch: its pending requests concatenated up to
    ``max_batch_rhs`` columns; requests that arrive while that batch runs join
    a later one;
  * at most one batch per operator is in flight (a factored operator's
    solve plan is not shared between streams), different operators overlap
    on different CUDA streams;
  * each worker owns one CUDA stream, one library handle and two grow-only
    pinned staging buffers; a batch is assembled column by column straight
    into the input buffer (one host pass), copied host -> device, solved,
    copied device -> the output buffer, and each request's columns are
    copied out of it (one host pass).

Grouped dispatch (``group_solve`` given): an idle worker takes the pending
requests of resident operators that have no batch in flight (each up to
``max_batch_rhs`` columns, oldest operators first) until it holds its share
of the pending columns -- the dispatchable columns divided by the idle
workers, at most ``max_group_rhs`` -- and solves them in one grouped call,
whose launches serve all of those operators at once (sslablu_gb300.grouped).
The share keeps every idle worker fed, so one group's host staging overlaps
another's device solve.  The group's right-hand
sides travel as one flat pinned block each way.

Admission by footprint: ``admit`` factors an operator only when the resident
footprint plus its own fits the budget; otherwise it waits (in FIFO order)
until ``retire`` frees memory.

A request's result is its block of the batch's solution: columns do not mix,
so it equals a solve of the request alone (bit for bit on the float64 path,
within the refinement tolerance on the mixed path, where the batch iterates
until its worst column converges).
"""
import collections
import queue
import threading
import time

import numpy as np
import torch


class Request:
    __slots__ = ("key", "B", "t_arrival", "t_start", "t_done", "X", "rid", "error")

    def __init__(self, key, B, t_arrival=0.0, rid=None):
        self.key = key
        self.B = np.ascontiguousarray(B, dtype=np.float64)
        if self.B.ndim == 1:
            self.B = self.B[:, None]
        self.t_arrival = float(t_arrival)
        self.t_start = self.t_done = None
        self.X = None
        self.rid = rid
        self.error = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_arrival


class Resident:
    def __init__(self, key, op, footprint, solve):
        self.key, self.op, self.footprint, self.solve = key, op, footprint, solve
        self.busy = False
        self.last_used = 0.0


def hbs_solver(H, precision="f64", tol=1e-10, maxit=10):
    """Device solve callable for a factored HBSMAT (ULV).  The mixed paths pad
    a batch to a power-of-two column count (zero columns converge at once) so
    each operator keeps only a few refinement plans.  precision 'tensor'
    refines the tensor-core sweep (it pays from a few hundred columns per
    batch); 'mixed' the double-float sweep."""
    if precision == "f64":
        return lambda X: H._dev_solve(X, False)
    inner = "tensor" if precision == "tensor" else "dfloat"

    def mixed(X):
        c = X.shape[1]
        w = 1 << (c - 1).bit_length()
        if w != c:
            X = torch.cat([X, torch.zeros((X.shape[0], w - c), dtype=X.dtype, device=X.device)], 1)
        x, _, _ = H.solve_refined(X.contiguous(), tol=tol, maxit=maxit, inner=inner)
        return x[:, :c]
    return mixed


def hbs_group_solver(precision="f64", tol=1e-10, maxit=10):
    """Grouped device solve for SolveServer(group_solve=...): given HBSMATs,
    one flat float64 device block and its layout [(offset, N, c)], returns
    the flat block of solutions in the same layout."""
    from .grouped import solve_grouped_device

    def run(ops, flat, layout):
        Bs = [flat[o:o + n * c].view(n, c) for o, n, c in layout]
        if precision == "f64":
            solve_grouped_device(ops, Bs)
            return flat
        out = torch.empty_like(flat)
        Xs = [out[o:o + n * c].view(n, c) for o, n, c in layout]
        solve_grouped_device(ops, Bs, "mixed", tol, maxit, Xs=Xs)
        return out
    return run


def rb_solver(rb):
    """Device solve callable for a factored RedBlackSolver (either precision)."""
    return lambda X: rb.solve(X)


class SolveServer:
    def __init__(self, budget_bytes, workers=4, max_batch_rhs=64, group_solve=None,
                 max_group_rhs=4096):
        self.budget = int(budget_bytes)
        self.max_batch = int(max_batch_rhs)
        self.group_solve = group_solve
        self.max_group = int(max_group_rhs)
        self.resident = collections.OrderedDict()
        self.waiting_admissions = collections.deque()
        self.pending = collections.defaultdict(collections.deque)
        self.done = []
        self._lock = threading.Condition()
        self._jobs = queue.Queue()
        self._nworkers = workers
        self._idle = workers
        self._threads = []
        self._stop = False
        self._t0 = None
        self.batches = 0
        self.batch_rhs = []
        for w in range(workers):
            t = threading.Thread(target=self._worker, args=(w,), daemon=True)
            t.start()
            self._threads.append(t)

    # ---------------------------------------------------------- admission
    @property
    def resident_bytes(self):
        return sum(r.footprint for r in self.resident.values())

    def admit(self, key, factory, footprint, solve_factory):
        """Factor and keep `key` resident when the budget allows, else queue it.
        factory() returns the factored operator; solve_factory(op) returns its
        device solve callable X -> A^{-1} X."""
        with self._lock:
            self.waiting_admissions.append((key, factory, int(footprint), solve_factory))
            self._admit_waiting()

    def _admit_waiting(self):
        while self.waiting_admissions:
            key, factory, fp, sf = self.waiting_admissions[0]
            if self.resident_bytes + fp > self.budget and self.resident:
                return
            self.waiting_admissions.popleft()
            op = factory()
            self.resident[key] = Resident(key, op, fp, sf(op))

    def retire(self, key):
        with self._lock:
            r = self.resident.pop(key, None)
            if r is not None:
                del r.op
            torch.cuda.empty_cache()
            self._admit_waiting()

    # ---------------------------------------------------------- scheduling
    def _now(self):
        return time.perf_counter() - self._t0

    def _take(self, key):
        dq = self.pending[key]
        reqs, cols = [], 0
        while dq and (not reqs or cols + dq[0].B.shape[1] <= self.max_batch):
            r = dq.popleft()
            reqs.append(r)
            cols += r.B.shape[1]
        self.resident[key].busy = True
        return reqs, cols

    def _pick_group(self):
        keys = [k for k, dq in self.pending.items()
                if dq and k in self.resident and not self.resident[k].busy]
        if not keys:
            return None
        keys.sort(key=lambda k: self.pending[k][0].t_arrival)
        # this worker's share of what the idle workers can take now
        avail = sum(min(self.max_batch, sum(r.B.shape[1] for r in self.pending[k]))
                    for k in keys)
        share = min(self.max_group, -(-avail // max(1, self._idle)))
        job, total = [], 0
        for k in keys:
            if job and total >= share:
                break
            reqs, cols = self._take(k)
            job.append((k, reqs))
            total += cols
        return job

    def _pick_batch(self):
        if self.group_solve is not None:
            return self._pick_group()
        best, best_t = None, None
        for key, dq in self.pending.items():
            if not dq:
                continue
            r = self.resident.get(key)
            if r is None or r.busy:
                continue
            if best_t is None or dq[0].t_arrival < best_t:
                best, best_t = key, dq[0].t_arrival
        if best is None:
            return None
        return [(best, self._take(best)[0])]

    @staticmethod
    def _staging(stage, which, n):
        """The worker's pinned float64 buffer `which` with room for n values
        (grow-only)."""
        buf = stage.get(which)
        if buf is None or buf.numel() < n:
            buf = torch.empty(max(n, 1 << 16), dtype=torch.float64, pin_memory=True)
            stage[which] = buf
        return buf[:n]

    @staticmethod
    def _assemble(dst, reqs):
        """Writes the requests' blocks side by side into dst (N x cols)."""
        if len(reqs) == 1:
            dst[...] = reqs[0].B
            return
        c = 0
        for r in reqs:
            k = r.B.shape[1]
            dst[:, c:c + k] = r.B
            c += k

    def _solve_one(self, key, reqs, stream, stage):
        res = self.resident[key]
        N = reqs[0].B.shape[0]
        cols = sum(r.B.shape[1] for r in reqs)
        Bh = self._staging(stage, "in", N * cols).view(N, cols)
        self._assemble(Bh.numpy(), reqs)
        with torch.cuda.stream(stream):
            Bd = Bh.to("cuda", non_blocking=True)
            Xd = res.solve(Bd)
            Xh = self._staging(stage, "out", N * cols).view(N, cols)
            Xh.copy_(Xd, non_blocking=True)
            stream.synchronize()
        return [Xh.numpy()]

    def _solve_group(self, job, stream, stage):
        layout, off = [], 0
        for _, reqs in job:
            n, c = reqs[0].B.shape[0], sum(r.B.shape[1] for r in reqs)
            layout.append((off, n, c))
            off += n * c
        flat_in = self._staging(stage, "in", off)
        fin = flat_in.numpy()
        for (o, n, c), (_, reqs) in zip(layout, job):
            self._assemble(fin[o:o + n * c].reshape(n, c), reqs)
        ops = [self.resident[k].op for k, _ in job]
        with torch.cuda.stream(stream):
            Bd = flat_in.to("cuda", non_blocking=True)
            Xd = self.group_solve(ops, Bd, layout)
            Xh = self._staging(stage, "out", off)
            Xh.copy_(Xd, non_blocking=True)
            stream.synchronize()
        flat = Xh.numpy()
        return [flat[o:o + n * c].reshape(n, c) for o, n, c in layout]

    def _worker(self, w):
        stream = None   # created with the first job (no device work before)
        stage = {}
        while True:
            job = self._jobs.get()
            if job is None:
                return
            t_start = self._now()
            try:
                if stream is None:
                    stream = torch.cuda.Stream()
                if self.group_solve is not None:
                    Xs, err = self._solve_group(job, stream, stage), None
                else:
                    Xs, err = self._solve_one(job[0][0], job[0][1], stream, stage), None
            except Exception as e:   # the requests complete with the error
                Xs, err = [None] * len(job), e
            t_done = self._now()
            done, ncols = [], 0
            for (key, reqs), X in zip(job, Xs):
                c = 0
                for r in reqs:
                    k = r.B.shape[1]
                    r.X = None if X is None else X[:, c:c + k].copy()
                    r.error = err
                    r.t_start, r.t_done = t_start, t_done
                    c += k
                done.extend(reqs)
                ncols += c
            with self._lock:
                for key, _ in job:
                    res = self.resident[key]
                    res.busy = False
                    res.last_used = t_done
                self.done.extend(done)
                self.batches += 1
                self.batch_rhs.append(ncols)
                self._idle += 1
                self._lock.notify_all()

    def run(self, requests):
        """Serve `requests` (sorted by t_arrival, seconds from the start);
        returns when every request is done."""
        reqs = sorted(requests, key=lambda r: r.t_arrival)
        for r in reqs:
            if r.key not in self.resident:
                raise KeyError("operator %r is not resident" % (r.key,))
        self.done = []
        self.batches = 0
        self.batch_rhs = []
        self._t0 = time.perf_counter()
        i, n = 0, len(reqs)
        with self._lock:
            while len(self.done) < n:
                now = self._now()
                while i < n and reqs[i].t_arrival <= now:
                    self.pending[reqs[i].key].append(reqs[i])
                    i += 1
                dispatched = False
                while self._idle > 0:
                    b = self._pick_batch()
                    if b is None:
                        break
                    self._idle -= 1
                    self._jobs.put(b)
                    dispatched = True
                if dispatched:
                    continue
                wait = (reqs[i].t_arrival - now) if i < n else 0.05
                self._lock.wait(timeout=max(1e-4, min(wait, 0.05)))
        self.makespan = self._now()
        return self.done

    def stats(self):
        lat = np.array([r.latency for r in self.done])
        rhs = sum(r.B.shape[1] for r in self.done)
        return {"requests": len(self.done), "rhs": int(rhs),
                "makespan_s": self.makespan, "rhs_per_s": rhs / self.makespan,
                "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                "p99_ms": 1e3 * float(np.percentile(lat, 99)),
                "batches": self.batches,
                "mean_batch_rhs": float(np.mean(self.batch_rhs)) if self.batch_rhs else 0.0}

    def close(self):
        for _ in self._threads:
            self._jobs.put(None)
        for t in self._threads:
            t.join(timeout=10)


def poisson_trace(keys, rate, count, rhs_range=(1, 64), seed=0, sizes=None):
    """Seeded Poisson arrivals: `count` requests at `rate` req/s, each on a
    uniformly chosen operator with U{rhs_range} right-hand sides ~ N(0, 1)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    out = []
    for j in range(count):
        key = keys[int(rng.integers(len(keys)))]
        r = int(rng.integers(rhs_range[0], rhs_range[1] + 1))
        n = sizes[key]
        out.append(Request(key, rng.standard_normal((n, r)), t[j], rid=j))
    return out


# ---------------------------------------------------------------------------
# benchmark: python -m sslablu_gb300.serving [--operators 16 --requests 2000 ...]
# ---------------------------------------------------------------------------
def _build_hbs_ops(count, seed, sizes=(2048, 4096, 8192), shift=16.0):
    """Exact synthetic HBS operators (leaf 64, rank 32, singular values 1 -> 1e-12),
    compressed + ULV-factored on the device with the upstream sampling.  The
    leaf diagonal blocks get `shift` * I (like the I + S interface systems of
    the slab method) so that a 1e-10 relative residual is attainable in
    float64 for every size."""
    from .matAssembly.HBS.HBSnew import HBSMAT
    from .synthetic import decaying_sigma, random_hbs_factors
    sigma = decaying_sigma(32)
    ops = []
    for j in range(count):
        N = sizes[j % len(sizes)]
        L = int(np.log2(N // 64)) + 1
        np.random.seed(seed + j)
        U, D, V, Nbvec = random_hbs_factors(32, 64, L, quad=False, sigma=sigma, shift=shift)
        A = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
        H = HBSMAT(A, tree=None, quad=False)
        H.set_Nbvec(list(Nbvec))
        H.construct(32, True)
        ops.append(("hbs%d_N%d" % (j, N), H, N))
    return ops


def _build_dense_rb_ops(count, sizes=(128, 256)):
    """C1-family operators: red-black factorisations of 2-D Laplace interface
    systems (8 slabs, 7 interfaces of m points padded to 8 blocks, as
    upstream's RedBlackSolver needs), their couplings made on the GPU by the
    slab solves of multislab.slabmaps (every double slab of a uniform
    Laplace geometry has the same maps).  Returns (key, solver, rows,
    footprint)."""
    from .direct_solve.omsdirectsolve import RedBlackSolver
    from .multislab.slabmaps import SlabGeometry, SlabMaps
    maps = {}
    for m in sizes:
        nx = int(round(0.25 * (m + 1))) | 1
        g = SlabGeometry(8, nx, m + 2)
        I = torch.eye(m, dtype=torch.float64, device="cuda")
        sm = SlabMaps(g, [1], tol=1e-13)
        Sl = sm.apply(I, None).cpu().numpy()
        Sr = sm.apply(None, I).cpu().numpy()
        maps[m] = (Sl, Sr)
    ops = []
    for j in range(count):
        m = sizes[j % len(sizes)]
        Sl, Sr = maps[m]
        Z = np.zeros((m, m))
        S = [[Z if i == 0 else Sl, Sr if i < 6 else Z] for i in range(7)] + [[Z, Z]]
        rb = RedBlackSolver(m)
        rb.factorize(S, [np.eye(m)] * 8)
        rb.dense_system = _tridiag_dense(Sl, Sr, 7)   # for the residual check
        ops.append(("rb%d_m%d" % (j, m), rb, 7 * m, 8 * 8 * m * m * 8))
    return ops


def _tridiag_dense(Sl, Sr, n):
    m = Sl.shape[0]
    M = np.eye(n * m)
    for i in range(n):
        if i > 0:
            M[i * m:(i + 1) * m, (i - 1) * m:i * m] = Sl
        if i < n - 1:
            M[i * m:(i + 1) * m, (i + 1) * m:(i + 2) * m] = Sr
    return M


def rb_padded_solver(rb, m):
    """Device solve of a red-black factorisation of 7 interfaces padded to 8."""
    def solve(X):
        Xp = torch.cat([X, torch.zeros((m, X.shape[1]), dtype=X.dtype, device=X.device)], 0)
        return rb.solve(Xp.contiguous())[:7 * m]
    return solve


def mix_main(a):
    """C5: resident operators from the C1 and C2/C3 families under one budget
    (HBS interface operators of 2048-8192 points, red-black factorisations of
    Laplace slab systems), served at several Poisson arrival rates; per rate
    RHS/s, p50 / p99 latency and the worst residual of every result."""
    import json
    n_hbs = a.operators // 2
    hbs = _build_hbs_ops(n_hbs, a.seed, shift=a.shift)
    rbs = _build_dense_rb_ops(a.operators - n_hbs)
    solvers = {}
    sizes = {}
    for key, H, n in hbs:
        solvers[key] = (H, n, H.nbytes, "hbs")
        sizes[key] = n
    for key, rb, n, fp in rbs:
        solvers[key] = (rb, n, fp, "rb")
        sizes[key] = n
    out = {"workload": "%d resident operators: %d exact-HBS interface operators (N in "
                       "2048/4096/8192, leaf 64, rank 32) and %d red-black factorisations of "
                       "2-D Laplace slab systems (7 x 128 / 7 x 256 points, couplings from the "
                       "GPU slab solves); Poisson arrivals, 1-64 RHS per request"
                       % (a.operators, n_hbs, a.operators - n_hbs),
           "hbs_precision": a.hbs_precision, "max_batch_rhs": a.max_batch, "rates": []}
    for rate in a.rates:
        srv = SolveServer(budget_bytes=64 << 30, workers=a.workers, max_batch_rhs=a.max_batch)
        try:
            for key, (op, n, fp, kind) in solvers.items():
                if kind == "hbs":
                    srv.admit(key, lambda op=op: op, fp,
                              lambda o: hbs_solver(o, a.hbs_precision))
                else:
                    m = n // 7
                    srv.admit(key, lambda op=op: op, fp, lambda o, m=m: rb_padded_solver(o, m))
            count = int(min(a.requests, max(200, rate * a.seconds)))
            srv.run(poisson_trace(list(sizes), rate, min(200, count), seed=a.seed + 1,
                                  sizes=sizes))
            done = srv.run(poisson_trace(list(sizes), rate, count, seed=a.seed, sizes=sizes))
            st = srv.stats()
            worst = 0.0
            for r in done:
                if r.error is not None:
                    continue
                op, n, fp, kind = solvers[r.key]
                if kind == "hbs":
                    R = r.B - op.matmat(r.X)
                else:
                    R = r.B - op.dense_system @ r.X
                worst = max(worst, float(np.max(np.linalg.norm(R, axis=0) /
                                                np.linalg.norm(r.B, axis=0))))
            st.update(rate=rate, worst_relres=worst,
                      errors=sum(r.error is not None for r in done),
                      offered_rhs_per_s=rate * 32.5)
            out["rates"].append(st)
        finally:
            srv.close()
    print(json.dumps(out))


def main():
    import argparse
    import json
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--operators", type=int, default=16)
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=20000.0)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--shift", type=float, default=16.0)
    ap.add_argument("--max-batch", type=int, default=64)
    ap.add_argument("--group-workers", type=int, default=8)
    ap.add_argument("--seed", type=int, default=20261205)
    ap.add_argument("--mix", action="store_true",
                    help="C5: operators of the C1 and C2/C3 families, swept over --rates")
    ap.add_argument("--rates", type=lambda v: [float(x) for x in v.split(",")],
                    default=[2000.0, 10000.0, 50000.0])
    ap.add_argument("--seconds", type=float, default=1.0,
                    help="--mix: trace length per rate (requests = rate * seconds)")
    ap.add_argument("--hbs-precision", default="f64", choices=["f64", "mixed", "tensor"],
                    help="--mix: solve path of the HBS operators")
    a = ap.parse_args()
    if a.mix:
        return mix_main(a)
    ops = _build_hbs_ops(a.operators, a.seed, shift=a.shift)
    sizes = {k: n for k, _, n in ops}
    out = {"workload": "%d resident exact-HBS operators (N in 2048/4096/8192, leaf 64, rank 32, "
                       "leaf shift %g), Poisson arrivals %.0f req/s, %d requests, 1-64 RHS each, "
                       "%d worker streams per-operator, %d grouped"
                       % (a.operators, a.shift, a.rate, a.requests, a.workers, a.group_workers)}
    # a short trace warms each arm first, then every arm serves the same trace
    arms = [("f64", False), ("mixed", False), ("f64", True), ("mixed", True)]
    for precision, grouped in arms:
        name = ("grouped_" if grouped else "") + precision
        gs = hbs_group_solver(precision) if grouped else None
        srv = SolveServer(budget_bytes=64 << 30, workers=a.group_workers if grouped else a.workers,
                          max_batch_rhs=a.max_batch, group_solve=gs)
        try:
            for key, H, n in ops:
                srv.admit(key, lambda H=H: H, H.nbytes, lambda op, p=precision: hbs_solver(op, p))
            warm = poisson_trace(list(sizes), a.rate, min(200, a.requests), seed=a.seed + 1,
                                 sizes=sizes)
            srv.run(warm)
            trace = poisson_trace(list(sizes), a.rate, a.requests, seed=a.seed, sizes=sizes)
            done = srv.run(trace)
            st = srv.stats()
            # relative residual of every served result against its operator
            worst = 0.0
            errs = [r.error for r in done if r.error is not None]
            if errs:
                st["first_error"] = repr(errs[0])
            for r in done:
                if r.error is not None:
                    continue
                H = dict((k, h) for k, h, _ in ops)[r.key]
                R = r.B - H.matmat(r.X)
                worst = max(worst, float(np.max(np.linalg.norm(R, axis=0) /
                                                np.linalg.norm(r.B, axis=0))))
            st["worst_relres"] = worst
            st["errors"] = sum(r.error is not None for r in done)
            out[name] = st
        finally:
            srv.close()
    out["mixed_vs_f64_rhs_per_s"] = out["mixed"]["rhs_per_s"] / out["f64"]["rhs_per_s"]
    out["grouped_mixed_vs_f64_rhs_per_s"] = (out["grouped_mixed"]["rhs_per_s"] /
                                             out["f64"]["rhs_per_s"])
    print(json.dumps(out))


if __name__ == "__main__":
    main()
