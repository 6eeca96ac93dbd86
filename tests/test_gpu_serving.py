"""Serving loop: each request's result equals a solve of that request alone
(float64 path: to rounding, 1e-14; mixed path: both meet the 1e-10 relative
residual and agree to 1e-8), with requests batched across arrivals and
operators overlapping on several streams or grouped into shared launches;
admission by footprint.  Every result is also checked against the CPU
oracle's float64 solve of its operator (oracle/hbs.py, ULVsparse.solve
restated): 1e-12 for the float64 path; for the mixed path a 1e-10 relative
residual measured with the oracle's float64 apply and 1e-10 agreement."""
import numpy as np
import pytest

from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu


def _operators(precision):
    from oracle.hbs import OracleHBS, gen_random_hbs
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.serving import hbs_solver
    ops, orcs = {}, {}
    for j, (k, nl, L) in enumerate([(8, 16, 5), (16, 32, 4), (8, 32, 4), (16, 16, 6)]):
        np.random.seed(100 + j)
        S, Nbvec = gen_random_hbs(k, nl, L, quad=False)
        H = HBSMAT().set_mats(S.Umats, S.Dmats, S.Vmats, list(Nbvec), fac=2)
        H.compute_ULV()
        O = OracleHBS().set_mats(S.Umats, S.Dmats, S.Vmats, list(Nbvec), fac=2)
        O.compute_ULV()
        ops["hbs%d" % j] = (H, hbs_solver(H, precision), S.shape[0])
        orcs["hbs%d" % j] = O
    return ops, orcs


@pytest.mark.parametrize("grouped", [False, True])
@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_served_results_equal_solo(precision, grouped):
    need_gpu()
    from sslablu_gb300.serving import SolveServer, hbs_group_solver, poisson_trace
    ops, orcs = _operators(precision)
    gs = hbs_group_solver(precision) if grouped else None
    srv = SolveServer(budget_bytes=1 << 34, workers=2 if grouped else 3, max_batch_rhs=24,
                      group_solve=gs)
    try:
        for key, (H, solve, n) in ops.items():
            srv.admit(key, lambda H=H: H, H.nbytes, lambda op, s=solve: s)
        sizes = {k: v[2] for k, v in ops.items()}
        reqs = poisson_trace(list(ops), rate=20000.0, count=60, rhs_range=(1, 8), seed=4,
                             sizes=sizes)
        done = srv.run(reqs)
        st = srv.stats()
    finally:
        srv.close()
    assert len(done) == 60 and all(r.error is None for r in done)
    assert st["batches"] < 60          # requests were batched
    for r in done:
        H, solve, n = ops[r.key]
        O = orcs[r.key]
        B, X = np.asarray(r.B), np.asarray(r.X)
        if precision == "f64":
            solo = H.solve(r.B)
            assert relerr(r.X, solo) < 1e-14
            assert relerr(X, O.solve(B)) < 1e-12
        else:
            res = B - O.matmat(X)
            nb = np.linalg.norm(B, axis=0)
            assert np.all(np.linalg.norm(res, axis=0) <= 1e-10 * nb)
            assert relerr(X, O.solve(B)) <= 1e-10
            solo, _, rr = H.solve_refined(r.B, tol=1e-10)
            assert rr <= 1e-10
            assert relerr(r.X, solo) < 1e-8


def test_admission_by_footprint():
    need_gpu()
    from sslablu_gb300.serving import SolveServer
    built = []

    def factory(name):
        def f():
            built.append(name)
            return name
        return f
    srv = SolveServer(budget_bytes=100, workers=1)
    try:
        srv.admit("a", factory("a"), 60, lambda op: None)
        srv.admit("b", factory("b"), 30, lambda op: None)
        srv.admit("c", factory("c"), 40, lambda op: None)   # 60 + 30 + 40 > 100: waits
        assert built == ["a", "b"] and set(srv.resident) == {"a", "b"}
        srv.retire("a")
        assert built == ["a", "b", "c"] and set(srv.resident) == {"b", "c"}
    finally:
        srv.close()
