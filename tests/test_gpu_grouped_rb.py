"""Grouped red-black HBS solves (direct_solve/grouped_rb.py) of uneven 2-D
Poisson interface systems against each system's own RedBlackSolverHBS.solve
(itself pinned to upstream in test_gpu_hbs_solvers.py) and against the
exact float64 systems built from the stencil slab maps, and one such system
against the oracle's red-black HBS on the same draws."""
import numpy as np
import pytest

from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu


def test_grouped_rb_hbs_matches_per_system_solves():
    """Eight systems of 4..11 interfaces (padded to 4, 8, 16 blocks) and
    128 / 256-point interfaces, 3 RHS each: the grouped solve equals every
    system's own solve to 1e-12 and solves the exact system to the
    compression accuracy."""
    need_gpu()
    import torch
    from sslablu_gb300.direct_solve.grouped_rb import solve_rb_hbs_grouped
    from sslablu_gb300.rbbatch import build_system, exact_apply
    specs = [(4, 128, 16), (5, 256, 24), (8, 128, 20), (11, 256, 32), (6, 128, 48),
             (9, 256, 16), (4, 256, 40), (7, 128, 28)]
    built = [build_system(nI, m, rk, 100 + j) for j, (nI, m, rk) in enumerate(specs)]
    rng = np.random.default_rng(3)
    Bs = []
    for (nI, m, rk), (rb, S, P) in zip(specs, built):
        b = np.zeros((P * m, 3))
        b[:nI * m] = rng.standard_normal((nI * m, 3))
        Bs.append(torch.from_numpy(b).cuda())
    from sslablu_gb300.direct_solve.grouped_rb import GroupedRBSolvePlan
    xg = solve_rb_hbs_grouped([b[0] for b in built], Bs)
    plan = GroupedRBSolvePlan([b[0] for b in built], Bs)
    xq = [x.clone() for x in plan()]
    for B in Bs:                                  # the plan reads whatever Bs hold
        B.mul_(2.0)
    xq2 = plan()
    for (nI, m, rk), (rb, S, P), B, x, y, y2 in zip(specs, built, Bs, xg, xq, xq2):
        xp = rb.solve(B) / 2.0
        for z in (x, y, y2 / 2.0):
            assert float(torch.linalg.norm(z - xp) / torch.linalg.norm(xp)) <= 1e-12
        R = B / 2.0 - exact_apply(S, nI, P, x)
        rel = torch.linalg.norm(R, dim=0) / torch.linalg.norm(B / 2.0, dim=0)
        assert float(rel.max()) <= 1e-6, (nI, m, rk)
    plan.close()


def test_grouped_rb_hbs_one_dimensional_and_cyclic():
    """1-D right-hand sides come back 1-D, and a periodic system (cyclic
    red-black, wrap-around couplings) solved in a group equals its own
    solve."""
    need_gpu()
    import torch
    from sslablu_gb300.direct_solve.grouped_rb import solve_rb_hbs_grouped
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS
    from sslablu_gb300.rbbatch import build_system
    rb0, S0, P0 = build_system(4, 128, 16, 7)
    H = rb0.RB[0][0][1]                        # the compressed coupling of that system
    per = RedBlackSolverHBS(128, 16, H.tree, False, cyclic=True)
    per.factorize([[H, H] for _ in range(4)])
    rng = np.random.default_rng(5)
    b0 = rng.standard_normal(P0 * 128)
    b1 = rng.standard_normal((4 * 128, 2))
    x0, x1 = solve_rb_hbs_grouped([rb0, per], [b0, b1])
    from sslablu_gb300.direct_solve.grouped_rb import GroupedRBSolvePlan
    Bq = [torch.from_numpy(b0[:, None].copy()).cuda(), torch.from_numpy(b1.copy()).cuda()]
    q0, q1 = GroupedRBSolvePlan([rb0, per], Bq)()
    assert isinstance(x0, np.ndarray) and x0.shape == b0.shape
    r0 = rb0.solve(b0)
    r1 = per.solve(b1)
    assert np.linalg.norm(x0 - r0) <= 1e-12 * np.linalg.norm(r0)
    assert np.linalg.norm(x1 - r1) <= 1e-12 * np.linalg.norm(r1)
    assert np.linalg.norm(q0.cpu().numpy()[:, 0] - r0) <= 1e-12 * np.linalg.norm(r0)
    assert np.linalg.norm(q1.cpu().numpy() - r1) <= 1e-12 * np.linalg.norm(r1)


def test_device_sketches_factor_to_the_same_accuracy():
    """RedBlackSolverHBS(sketch_seed=...) draws its compressions' sketches on
    the device (beyond upstream); the factorisation is as accurate as with
    upstream's host draws, and reproducible for a seed."""
    need_gpu()
    import torch
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS
    from sslablu_gb300.rbbatch import build_system, exact_apply
    rb, S, P = build_system(6, 256, 24, 11)
    H = rb.RB[0][0][1]
    S_rk = [[rb.RB[0][0][i], rb.RB[0][3][i]] for i in range(P)]
    b = torch.from_numpy(np.random.default_rng(2).standard_normal((P * 256, 2))).cuda()
    b[6 * 256:] = 0.0
    xs = []
    for _ in range(2):
        d = RedBlackSolverHBS(256, 24, H.tree, False, sketch_seed=5)
        d.factorize(S_rk)
        xs.append(d.solve(b))
    assert torch.equal(xs[0], xs[1])
    for x in (xs[0], rb.solve(b)):
        r = torch.linalg.norm(b - exact_apply(S, 6, P, x), dim=0) / torch.linalg.norm(b, dim=0)
        assert float(r.max()) <= 1e-6


def test_concurrent_builds_equal_one_by_one_builds():
    """rbbatch.build_systems (grouped_rb.factorize_many: four systems at a
    time, each on its own stream, the assembler's RNG draws serialised)
    factors every system as the one-by-one build does: the solutions agree
    to 1e-13 (the same draws and the same kernels on the same data)."""
    need_gpu()
    import torch
    from sslablu_gb300.rbbatch import build_system, build_systems
    specs = [(4, 128, 16), (6, 256, 24), (9, 128, 32), (5, 256, 20), (8, 128, 40)]
    seed = 500
    par = build_systems(specs, seed, workers=4)
    seq = [build_system(nI, m, rk, seed + 17 * j) for j, (nI, m, rk) in enumerate(specs)]
    rng = np.random.default_rng(5)
    for (nI, m, rk), (rb_p, S_p, P_p), (rb_s, S_s, P_s) in zip(specs, par, seq):
        assert P_p == P_s
        assert torch.equal(S_p, S_s)
        b = np.zeros((P_s * m, 4))
        b[:nI * m] = rng.standard_normal((nI * m, 4))
        B = torch.from_numpy(b).cuda()
        xp, xs = rb_p.solve(B), rb_s.solve(B)
        assert float(torch.linalg.norm(xp - xs) / torch.linalg.norm(xs)) <= 1e-13, (nI, m, rk)


def test_c4_system_matches_the_oracle():
    """One system of the C4 batch's kind (5 interfaces of 128 points padded
    to 8 blocks, stencil slab map compressed by the rkHBS assembler at rank
    16), red-black HBS factored with upstream's sketch draws (numpy's global
    RNG), against the oracle's red-black HBS (upstream's restated) on the
    same coupling operator and the same draws: the solutions agree to 1e-9
    and both solve the exact system to 1e-9."""
    need_gpu()
    import types
    import torch
    from oracle import direct as od
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS, _linop_from_mat
    from sslablu_gb300.matAssembly.matAssembler import rkHMatAssembler
    from sslablu_gb300.rbbatch import exact_apply
    from sslablu_gb300.synthetic import poisson_slab_map
    nI, m, rk, P = 5, 128, 16, 8
    width = 2.0 / (nI + 1)
    nx = int(round(width * (m + 1))) // 2 * 2 + 1
    S = poisson_slab_map(m, max(nx, 3), width)
    np.random.seed(31)
    H = rkHMatAssembler(64, rk).assemble(
        types.SimpleNamespace(A=S, XXI=np.linspace(0.0, 1.0, m + 2)[1:-1]))
    Hd = np.asarray(H.matmat(np.eye(m)))
    Z = _linop_from_mat(np.zeros((m, m)))
    Z._zero = True
    rb = RedBlackSolverHBS(m, rk, H.tree, False)
    np.random.seed(32)
    rb.factorize([[H if 0 < i < nI else Z, H if i < nI - 1 else Z] for i in range(P)])
    Zd = np.zeros((m, m))
    tree = H.tree
    ov = od.RedBlackHBS(m, rk, (np.asarray(tree.perm_leaf), tree.nleaves, tree.nlevels), False)
    np.random.seed(32)
    ov.factorize([(od.dense_op(Hd if 0 < i < nI else Zd), od.dense_op(Hd if i < nI - 1 else Zd))
                  for i in range(P)])
    b = np.zeros((P * m, 3))
    b[:nI * m] = np.random.default_rng(4).standard_normal((nI * m, 3))
    x = np.asarray(rb.solve(b))
    xo = np.stack([np.asarray(ov.solve(b[:, j])) for j in range(3)], axis=1)
    assert relerr(x, xo) <= 1e-9
    Sd = torch.from_numpy(S).cuda()
    for sol in (x, xo):
        R = b - exact_apply(Sd, nI, P, torch.from_numpy(sol).cuda()).cpu().numpy()
        assert float((np.linalg.norm(R, axis=0) / np.linalg.norm(b, axis=0)).max()) <= 1e-9
