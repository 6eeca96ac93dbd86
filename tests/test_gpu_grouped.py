"""Grouped solves over many HBS operators of uneven sizes and depths
(slu_ulv_solve_grouped / slu_refine_grouped through sslablu_gb300.grouped):
every member's result equals the result of its own solve.

Float64: each column runs the same sequence of operations as the
per-operator solve, whatever the column chunking, so the bound is 1e-15
(relative); every member also matches the CPU oracle's float64 solve of the
same operator (oracle/hbs.py: ULVsparse.solve restated, with the same random
sketches when the operator is compressed) to 1e-12.  Mixed: every member
reaches the 1e-10 relative residual measured with the oracle's float64 apply
and matches the oracle's solution to 1e-10."""
import numpy as np
import pytest

from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu

# (k, leaf, levels, quad): N = leaf * fac**(levels-1)
SHAPES = [(8, 16, 5, False), (16, 32, 4, False), (8, 32, 3, False), (16, 16, 6, False),
          (32, 64, 5, False), (8, 16, 3, True), (12, 24, 2, False)]


def _operators(shift=4.0, compress=False, oracle=False):
    """The GPU operators, and with ``oracle`` also their CPU oracle twins
    (the same factors, or the same compression from the same sketches)."""
    from oracle.hbs import OracleHBS
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    ops, orcs = [], []
    for j, (k, nl, L, quad) in enumerate(SHAPES):
        np.random.seed(300 + j)
        U, D, V, Nbvec = random_hbs_factors(k, nl, L, quad=quad, shift=shift)
        fac = 4 if quad else 2
        A = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=fac)
        O = OracleHBS().set_mats(U, D, V, list(Nbvec), fac=fac)
        nsamp = (6 * k + 4 * nl + 5) if quad else (4 * k + 2 * nl + 5)
        if compress and nsamp < A.shape[0]:
            H = HBSMAT(A, tree=None, quad=quad)
            H.set_Nbvec(list(Nbvec))
            state = np.random.get_state()
            H.construct(k, True)
            if oracle:
                np.random.set_state(state)
                O = OracleHBS(O, None, Nbvec[0], len(Nbvec), fac).construct(k)
                O.compute_ULV()
        else:
            A.compute_ULV()
            H = A
            if oracle:
                O.compute_ULV()
        ops.append(H)
        orcs.append(O)
    return (ops, orcs) if oracle else ops


def _oracle_residual(O, x, b):
    """Worst column of ||b - A x|| / ||b|| with the oracle's float64 apply."""
    r = np.asarray(b) - O.matmat(np.asarray(x))
    return float(np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)))


def _rhs(ops, counts, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((H.shape[0], c)) for H, c in zip(ops, counts)]


@pytest.mark.parametrize("compress", [False, True])
def test_grouped_f64_equals_solo(compress):
    need_gpu()
    from sslablu_gb300.grouped import solve_grouped
    ops, orcs = _operators(compress=compress, oracle=True)
    counts = [1, 3, 8, 16, 5, 2, 7]
    bs = _rhs(ops, counts, 1)
    xs = solve_grouped(list(zip(ops, bs)))
    for H, O, b, x in zip(ops, orcs, bs, xs):
        assert x.shape == b.shape
        assert relerr(x, H.solve(b)) <= 1e-15
        assert relerr(x, O.solve(b)) <= 1e-12


def test_grouped_f64_repeated_members_and_edges():
    """The same operator several times with different right-hand sides, a 1-D
    right-hand side, a member with no columns and an empty group."""
    need_gpu()
    from sslablu_gb300.grouped import solve_grouped
    ops, orcs = _operators(oracle=True)
    group = []
    rng = np.random.default_rng(2)
    for rep in range(9):
        for H in ops:
            c = int(rng.integers(1, 24))
            group.append((H, rng.standard_normal((H.shape[0], c))))
    group.append((ops[0], rng.standard_normal(ops[0].shape[0])))     # 1-D
    group.append((ops[1], np.zeros((ops[1].shape[0], 0))))           # no columns
    xs = solve_grouped(group)
    assert len(xs) == len(group)
    twin = {id(H): O for H, O in zip(ops, orcs)}
    for (H, b), x in zip(group, xs):
        assert x.shape == b.shape
        if b.size:
            assert relerr(x, H.solve(b)) <= 1e-15
            assert relerr(x, twin[id(H)].solve(b)) <= 1e-12
    assert solve_grouped([]) == []


def test_grouped_mixed_refinement():
    need_gpu()
    from sslablu_gb300.grouped import solve_grouped
    ops, orcs = _operators(compress=True, oracle=True)
    counts = [4, 1, 16, 8, 3, 5, 2]
    bs = _rhs(ops, counts, 3)
    xs, iters, rr = solve_grouped(list(zip(ops, bs)), precision="mixed", tol=1e-10)
    assert 1 <= iters <= 10 and len(rr) == len(ops)
    for H, O, b, x, r in zip(ops, orcs, bs, xs, rr):
        assert r <= 1e-10
        assert _oracle_residual(O, x, b) <= 1e-10
        assert relerr(x, O.solve(b)) <= 1e-10
        solo, _, rs = H.solve_refined(b, tol=1e-10)
        assert rs <= 1e-10
        assert relerr(x, solo) < 1e-8


@pytest.mark.parametrize("k", [16, 24, 33, 40, 48])
def test_per_level_solve_equals_grouped_for_uneven_ranks(k):
    """Ranks up to 3/4 of the leaf size and levels of 1-3 blocks: the
    per-level kernels (which switch to one-batch prefetching of the block
    matrices on small levels) agree with the grouped sweep to rounding."""
    need_gpu()
    from oracle.hbs import OracleHBS
    from sslablu_gb300.grouped import solve_grouped
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    for N in (128, 256, 512):
        Lv = int(np.log2(N // 64)) + 1
        U, D, V, Nbvec = random_hbs_factors(k, 64, Lv, quad=False,
                                            rng=np.random.default_rng(N + k), shift=16.0)
        H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
        H.compute_ULV()
        O = OracleHBS().set_mats(U, D, V, list(Nbvec), fac=2)
        O.compute_ULV()
        b = np.random.default_rng(k).standard_normal((N, 8))
        x_solo = H.solve(b)
        x_grp = solve_grouped([(H, b)])[0]
        assert _oracle_residual(O, x_grp, b) < 1e-12, (N, k)
        assert relerr(x_grp, O.solve(b)) < 1e-12, (N, k)
        assert relerr(x_solo, x_grp) < 1e-13, (N, k)


def test_grouped_apply_equals_solo():
    """Grouped applies (mode N and T mixed, uneven sizes and depths, a
    one-level member) equal each member's own matmat / rmatmat bitwise."""
    need_gpu()
    import torch
    from sslablu_gb300.grouped import apply_grouped
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    ops = []
    for N, k in ((64, 16), (256, 24), (1024, 32), (512, 16)):
        Lv = int(np.log2(N // 64)) + 1
        U, D, V, Nbvec = random_hbs_factors(k, 64, Lv, quad=False,
                                            rng=np.random.default_rng(N + k), shift=4.0)
        ops.append(HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2))
    rng = np.random.default_rng(3)
    Xs = [torch.from_numpy(rng.standard_normal((H.shape[0], c))).cuda()
          for H, c in zip(ops, (3, 8, 1, 5))]
    trans = [False, True, False, True]
    Ys = apply_grouped(ops, Xs, trans)
    for H, X, Y, t in zip(ops, Xs, Ys, trans):
        ref = H._dev_apply(X, t)
        assert torch.equal(Y, ref)


def test_grouped_solve_plan_equals_grouped_solve():
    """A grouped solve plan (step tables built once, launches replayed as one
    graph) gives the grouped solve's results bitwise, with new data in the
    blocks on every call, and refuses to run after a member is refactored."""
    need_gpu()
    import torch
    from sslablu_gb300 import _lib as L
    from sslablu_gb300.grouped import GroupedSolvePlan, solve_grouped_device
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    ops = []
    for j, (N, k) in enumerate([(128, 16), (512, 24), (256, 33), (1024, 16)]):
        Lv = int(np.log2(N // 64)) + 1
        U, D, V, Nbvec = random_hbs_factors(k, 64, Lv, quad=False,
                                            rng=np.random.default_rng(j), shift=16.0)
        ops.append(HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2))
        ops[-1].compute_ULV()
    cols = [3, 8, 1, 5]
    Bs = [torch.empty((H.shape[0], c), dtype=torch.float64, device="cuda")
          for H, c in zip(ops, cols)]
    plan = GroupedSolvePlan(ops, Bs)
    rng = np.random.default_rng(7)
    for _ in range(3):
        data = [rng.standard_normal(tuple(B.shape)) for B in Bs]
        for B, d in zip(Bs, data):
            B.copy_(torch.from_numpy(d))
        plan()
        ref = [torch.from_numpy(d).cuda() for d in data]
        solve_grouped_device(ops, ref)
        torch.cuda.synchronize()
        for B, R in zip(Bs, ref):
            assert torch.equal(B, R)
    ops[1].compute_ULV()
    with pytest.raises(L.SluError):
        plan()
    plan.close()


def test_grouped_refine_plan_equals_grouped_refinement():
    """A grouped refinement plan (buffers and tables built once, iterations
    replayed as CUDA graphs) gives the per-call grouped refinement's results
    bitwise, with the same iteration count and residuals, on new data every
    call; it refuses to run after a member is refactored."""
    need_gpu()
    import torch
    from sslablu_gb300 import _lib as L
    from sslablu_gb300.grouped import GroupedRefinePlan, solve_grouped_device
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    ops = []
    for j, (N, k) in enumerate([(256, 16), (512, 24), (128, 16)]):
        Lv = int(np.log2(N // 64)) + 1
        U, D, V, Nbvec = random_hbs_factors(k, 64, Lv, quad=False,
                                            rng=np.random.default_rng(j + 5), shift=16.0)
        ops.append(HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2))
        ops[-1].compute_ULV()
    cols = [4, 2, 7]
    Bs = [torch.empty((H.shape[0], c), dtype=torch.float64, device="cuda")
          for H, c in zip(ops, cols)]
    plan = GroupedRefinePlan(ops, Bs)
    rng = np.random.default_rng(9)
    for _ in range(2):
        data = [rng.standard_normal(tuple(B.shape)) for B in Bs]
        for B, d in zip(Bs, data):
            B.copy_(torch.from_numpy(d))
        Xs, it, rr = plan(1e-10, 10)
        ref = [torch.from_numpy(d).cuda() for d in data]
        Xr, it_r, rr_r = solve_grouped_device(ops, ref, "mixed", 1e-10, 10)
        torch.cuda.synchronize()
        assert it == it_r and np.allclose(rr, rr_r, rtol=0, atol=0)
        for X, R in zip(Xs, Xr):
            assert torch.equal(X, R)
        assert max(rr) <= 1e-10
    ops[0].compute_ULV()
    with pytest.raises(L.SluError):
        plan(1e-10, 10)
    plan.close()
