"""Host-side logic that needs no GPU: the grouped serving dispatch policy and
the argument checks of HBSMAT.solve_plan."""
import numpy as np
import pytest
import torch

from sslablu_gb300.serving import Request, SolveServer


def _server_with_pending(cols_per_op, workers):
    srv = SolveServer(budget_bytes=1 << 40, workers=workers, max_batch_rhs=64,
                      group_solve=lambda ops, flat, layout: flat)
    for k, cols in enumerate(cols_per_op):
        srv.admit("op%d" % k, lambda: object(), 1, lambda op: (lambda X: X))
        t = 0.0
        for c in cols:
            srv.pending["op%d" % k].append(Request("op%d" % k, np.zeros((4, c)), t))
            t += 1e-3
    return srv


def test_grouped_dispatch_shares_columns_among_idle_workers():
    """Each idle worker takes its share of the dispatchable columns (at most
    max_batch_rhs per operator, operators oldest first), so several grouped
    jobs run at once instead of one job holding every operator."""
    srv = _server_with_pending([[32, 32], [40], [8, 8], [64], [16]], workers=4)
    try:
        jobs = []
        while srv._idle > 0:
            job = srv._pick_batch()
            if job is None:
                break
            srv._idle -= 1
            jobs.append(job)
        # 64 + 40 + 16 + 64 + 16 = 200 dispatchable columns over 4 workers:
        # shares of ceil(200/4) = 50, then the rest over the remaining workers
        keys = [[k for k, _ in job] for job in jobs]
        assert len(jobs) >= 3
        assert sorted(k for ks in keys for k in ks) == ["op%d" % i for i in range(5)]
        for job in jobs:   # every operator is in one job only, each batch <= 64 columns
            for _, reqs in job:
                assert sum(r.B.shape[1] for r in reqs) <= 64
        assert all(srv.resident[k].busy for k in srv.resident)
    finally:
        srv.close()


def test_grouped_dispatch_single_worker_takes_everything():
    srv = _server_with_pending([[10], [20], [30]], workers=1)
    try:
        job = srv._pick_batch()
        assert [k for k, _ in job] == ["op0", "op1", "op2"]
        assert srv._pick_batch() is None      # every operator now has a batch in flight
    finally:
        srv.close()


def test_solve_plan_argument_checks():
    """solve_plan refuses unpinned host blocks, mixed placements and shape or
    dtype mismatches before touching the library."""
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    H = HBSMAT()
    H.shape = (8, 8)
    b = torch.zeros((8, 2), dtype=torch.float64)
    with pytest.raises(ValueError):
        H.solve_plan(b)                                    # host but not pinned
    with pytest.raises(ValueError):
        H.solve_plan(b.float())                            # not float64
    with pytest.raises(ValueError):
        H.solve_plan(torch.zeros(8, dtype=torch.float64))  # not 2-D
    with pytest.raises(NotImplementedError):
        H.solve_plan(b, mode="X")
