"""The CPU oracle reproduces the upstream golden vectors (no GPU)."""
import numpy as np
import pytest

from oracle import direct as od
from oracle import hbs as oh
from tests._cases import hbs_from_fixture, kernel_system, relerr, test_rb_system


def test_rb_dense_cases(golden):
    g = golden("rb_dense")
    for nS, m in g["cases"]:
        S, T, mat, rhs = test_rb_system(int(nS), int(m))
        key = "%d_%d" % (nS, m)
        x = od.RedBlackDense(int(m)).factorize(S, T).solve(rhs)
        assert relerr(x, g["x_rb_" + key]) < 1e-14
        assert relerr(x, g["x_np_" + key]) < 1e-8      # upstream test_RB bar
        xt = od.ThomasDense(int(m)).factorize(S, T).solve(rhs)
        assert relerr(xt, g["x_th_" + key]) < 1e-14


def test_thomas_cyclic(golden):
    g = golden("thomas_cyclic")
    S = [tuple(p) for p in g["S"]]
    x = od.ThomasDense(4, cyclic=True).factorize(S, list(g["T"])).solve(g["rhs"])
    assert relerr(x, g["x"]) < 1e-14


@pytest.mark.parametrize("name", ["hbs_binary_k8", "hbs_quad_k8"])
def test_hbs_construct_factors(golden, name):
    g = golden(name)
    S, Nbvec = hbs_from_fixture(g)
    O = oh.OracleHBS(S, None, Nbvec[0], len(Nbvec), 4 if g["quad"] else 2)
    O.construct(int(g["k"]))          # draws Om, Psi from the global RNG, as upstream
    assert np.array_equal(O.NNvec, g["NNvec"])
    for nm in ["Umats", "Vmats", "Dmats", "Qlist", "Rlist", "Uulist"]:
        for i, M in enumerate(getattr(O, nm)):
            ref = g["%s_%d" % (nm, i)]
            assert M.shape == ref.shape
            if ref.size == 0:
                continue
            assert np.abs(M - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    x = g["x"]
    assert relerr(O.matmat(x), g["mm"]) < 1e-13
    assert relerr(O.rmatmat(x), g["rmm"]) < 1e-13
    assert relerr(O.solve(x), g["sol"]) < 1e-13
    assert relerr(O.solve(x, "T"), g["solT"]) < 1e-13
    assert relerr(O.solve(x[:, 0]), g["sol1"]) < 1e-13
    # exactness of the round trip (upstream HBSnewTest.py:93-110 bars)
    assert relerr(O.matmat(x), g["Ax_true"]) < 1e-12
    # standalone ULV of the generator factors
    Ql, Wl, Uul, Rl, NNv = oh.compute_ULV(S.Umats, S.Dmats, S.Vmats, Nbvec)
    assert np.array_equal(NNv, g["ulv_NNvec"])
    y = oh.ulv_solve(S.Umats, S.Dmats, Ql, Wl, Uul, Rl, NNv, Nbvec, x.copy())
    yt = oh.ulv_solve(S.Umats, S.Dmats, Ql, Wl, Uul, Rl, NNv, Nbvec, x.copy(), "T")
    assert relerr(y, g["ulv_sol"]) < 1e-13
    assert relerr(yt, g["ulv_solT"]) < 1e-13


def test_hbs_c2_shape(golden):
    g = golden("hbs_c2_n512")
    S, Nbvec = hbs_from_fixture(g)
    O = oh.OracleHBS(S, None, Nbvec[0], len(Nbvec), 2)
    O.construct(int(g["k"]))
    assert O.nSamples == int(g["nSamples"]) == 4 * 32 + 2 * 64 + 5
    x = g["x"]
    assert relerr(O.matmat(x), g["mm"]) < 1e-13
    assert relerr(O.solve(x), g["sol"]) < 1e-12
    assert relerr(O.solve(x, "T"), g["solT"]) < 1e-12
    assert relerr(O.matmat(x), g["Ax_true"]) < 1e-12


def test_c1_poisson(golden):
    g = golden("c1_poisson64")
    n = g["Sl"].shape[0]
    nc = int(g["nc"])
    S = [[g["Sr"][0]]] + [[g["Sl"][i], g["Sr"][i]] for i in range(1, n - 1)] + [[g["Sl"][n - 1]]]
    T = [np.eye(nc)] * n
    x = od.ThomasDense(nc).factorize(S, T).solve(g["rhs"])
    assert relerr(x, g["x_th"]) < 1e-14
    Sp = [[g["Sl"][i], g["Sr"][i]] for i in range(n)] + [[np.zeros((nc, nc))] * 2]
    xr = od.RedBlackDense(nc).factorize(Sp, [np.eye(nc)] * (n + 1)).solve(
        np.concatenate([g["rhs"], np.zeros(nc)]))
    assert relerr(xr, g["x_rb"]) < 1e-13
    A, B, C = od.build_block_tridiagonal_solver(S)
    idx = [range(i * nc, (i + 1) * nc) for i in range(n)]
    assert relerr(od.block_tridiagonal_solve(idx, (A, B, C), g["rhs"]), g["x_f"]) < 1e-14


@pytest.mark.parametrize("rk", [16, 24])
def test_rbhbs_kernel(golden, rk):
    g = golden("rbhbs_kernel")
    m, nS, leaf, nlev = int(g["m"]), int(g["nS"]), int(g["leaf"]), int(g["nlev"])
    S = [(od.dense_op(a), od.dense_op(c)) for a, c in kernel_system(m, nS)]
    td = (np.arange(m), m // leaf, nlev)
    np.random.seed(11)
    x = od.RedBlackHBS(m, rk, td, False).factorize(S).solve(g["b"])
    assert relerr(x, g["x_rb_%d" % rk]) < 1e-12
    np.random.seed(12)
    y = od.ThomasHBS(m, rk, td, False).factorize(S).solve(g["b"])
    assert relerr(y, g["x_th_%d" % rk]) < 1e-12


def test_rbhbs_gauss(golden):
    from tests._cases import gauss_system, tridiag_matrix
    g = golden("rbhbs_gauss")
    m, nS, leaf, nlev, rk = (int(g[k]) for k in ("m", "nS", "leaf", "nlev", "rk"))
    S = gauss_system(m, nS)
    Sop = [(od.dense_op(a), od.dense_op(c)) for a, c in S]
    td = (np.arange(m), m // leaf, nlev)
    np.random.seed(11)
    x = od.RedBlackHBS(m, rk, td, False).factorize(Sop).solve(g["b"])
    assert relerr(x, g["x_rb"]) < 1e-12
    np.random.seed(12)
    y = od.ThomasHBS(m, rk, td, False).factorize(Sop).solve(g["b"])
    assert relerr(y, g["x_th"]) < 1e-12
    M = tridiag_matrix(S, m)
    assert relerr(M @ g["x_rb"], g["b"]) < 1e-12


def test_package_generator_matches_oracle_generator():
    """sslablu_gb300.synthetic (benchmarks, serving CLI) draws the same
    operator as the oracle's generator for the same seed."""
    from oracle.hbs import gen_random_hbs
    from sslablu_gb300.synthetic import decaying_sigma, random_hbs_factors
    for k, nl, L, quad in [(8, 16, 4, False), (4, 8, 3, True)]:
        sig = decaying_sigma(k)
        np.random.seed(5)
        S, nb = gen_random_hbs(k, nl, L, quad=quad, sigma=sig)
        np.random.seed(5)
        U, D, V, nb2 = random_hbs_factors(k, nl, L, quad=quad, sigma=sig)
        assert list(nb) == list(nb2)
        for a, b in zip(S.Umats + S.Vmats + S.Dmats, U + V + D):
            assert np.array_equal(a, b)


def _exact_in_tree_order(k, nl, L, seed, perm):
    """The operator of the hbstorch / assembler fixtures (see make_golden.py)."""
    np.random.seed(seed)
    S, _ = oh.gen_random_hbs(k, nl, L, quad=False)
    M = S.matmat(np.eye(S.shape[0]))
    A = np.zeros_like(M)
    A[np.ix_(perm, perm)] = M
    return A


def test_slab_tree_mirror_matches_upstream(golden):
    """sslablu_gb300's slabTree (host code of the tree protocol) against
    upstream slabTree: perm_leaf, nleaves, nlevels, leaf boundary DOFs and
    interface DOFs, on lines, rectangles (binary, quad) and a plane in 3-D,
    including split lines that hold points (which both halves keep)."""
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    g = golden("slab_trees")
    cases = [("line256", "line", 256, False, 32), ("rect16_bin", "rect16", 0, False, 16),
             ("rect16_quad", "rect16", 0, True, 16), ("plane3d_bin", "plane32", 0, False, 128),
             ("plane3d_quad", "plane32", 0, True, 64), ("line2d", "line2d", 128, False, 8),
             ("rect17_bin", "rect17", 0, False, 20), ("rect17_quad", "rect17", 0, True, 20)]
    for name, kind, n, quad, leaf in cases:
        t = slabTree(_cloud(kind, n), quad, leaf)
        p = name + "_"
        assert np.array_equal(t.perm_leaf, g[p + "perm"]), name
        assert [t.nleaves, t.nlevels] == list(g[p + "shape"]), name
        sides = [np.asarray(t.get_node(b).bDOFs[sd]) if t.get_node(b).bDOFs is not None
                 else np.zeros(0, np.int64)
                 for b in t.get_leaves() for sd in ("left", "down", "up", "right")]
        bd = np.concatenate(sides).astype(np.int64)
        assert np.array_equal(bd, g[p + "bdofs"]), name
        il = [len(t.get_node(b).iDOFs) if t.get_node(b).iDOFs is not None else -1
              for b in sorted(t._boxes)]
        assert il == list(g[p + "ilen"]), name
        idofs = [np.asarray(t.get_node(b).iDOFs) for b in sorted(t._boxes)
                 if t.get_node(b).iDOFs is not None]
        cat = np.concatenate(idofs).astype(np.int64) if idofs else np.zeros(0, np.int64)
        assert np.array_equal(cat, g[p + "idofs"]), name


def _cloud(kind, n=0):
    if kind == "line":
        return np.linspace(0, 1, n)
    if kind == "line2d":
        return np.stack([np.linspace(0, 1, n), np.full(n, 0.25)], 1)
    if kind == "rect16":
        return np.stack(np.meshgrid(np.linspace(0, 1, 16), np.linspace(0, 2, 16), indexing="ij"),
                        -1).reshape(-1, 2)
    if kind == "rect17":
        return np.stack(np.meshgrid(np.linspace(0, 1, 17), np.linspace(0, 1, 17), indexing="ij"),
                        -1).reshape(-1, 2)
    g = np.stack(np.meshgrid(np.linspace(0, 1, 32), np.linspace(0, 1, 32), indexing="ij"),
                 -1).reshape(-1, 2)
    return np.concatenate([np.full((g.shape[0], 1), 0.5), g], 1)


def test_oracle_hbstorch_rule_matches_upstream(golden):
    """The oracle with HBStorch's null-space rule (s < 2n at the leaves)
    reproduces upstream HBStorch's factors (D, and U/V up to column signs) and
    outputs; the ULV solve of those factors matches upstream ULVsparse."""
    g = golden("hbstorch")
    perm = g["perm"]
    k = int(g["k"])
    A = _exact_in_tree_order(k, 16, 5, 7, perm)
    O = oh.OracleHBS(A, perm, 16, 5, 2)
    Om, Psi = g["Om"], g["Psi"]
    O.compress_from_sketches(k, Om[perm], Psi[perm], (A @ Om)[perm], (A.T @ Psi)[perm],
                             null_after_n=True)
    # leaf D exactly; above the leaves the blocks are expressed in the child
    # bases, which an SVD fixes only up to column signs
    for t in range(5):
        ref = g["D%d" % t].reshape(O.Dmats[t].shape)
        got = O.Dmats[t] if t == 0 else np.abs(O.Dmats[t])
        assert relerr(got, ref if t == 0 else np.abs(ref)) < 1e-12
    for t in range(4):
        for nm, mats in (("U", O.Umats), ("V", O.Vmats)):
            ref = g["%s%d" % (nm, t)].reshape(mats[t].shape)
            assert relerr(np.abs(mats[t]), np.abs(ref)) < 1e-12
    x = g["x"]
    assert relerr(O.matmat(x), g["Ax"]) < 1e-13
    assert relerr(O.rmatmat(x), g["ATx"]) < 1e-13
    assert relerr(O.solve(g["b"]), g["sol"]) < 1e-12
    # HBSnew's rule spans part of the sketch's range here (s < 2n): different factors
    O2 = oh.OracleHBS(A, perm, 16, 5, 2)
    O2.compress_from_sketches(k, Om[perm], Psi[perm], (A @ Om)[perm], (A.T @ Psi)[perm])
    assert relerr(O2.matmat(x), g["Ax"]) > 1e-8


def test_poisson2d_slab_maps_match_upstream(golden):
    """The DST closed form of the 2-D stencil slab maps (oracle/slabmaps.py)
    against upstream's own maps: the 64-point C1-layout blocks entry by
    entry, and at C1's full 256-point interfaces a stored fingerprint, the
    block norms and the interface operator's action on upstream's solution."""
    from oracle.slabmaps import poisson2d_couplings
    g = golden("c1_poisson64")
    S = poisson2d_couplings(64, 8, 17)
    for i in range(7):
        assert np.abs(S[i][0] - g["Sl"][i]).max() < 1e-15
        assert np.abs(S[i][1] - g["Sr"][i]).max() < 1e-15
    g = golden("c1_poisson256")
    m = int(g["nc"])
    S = poisson2d_couplings(m, int(g["nslabs"]), int(g["nx"]))
    fp = g["fingerprint"]
    assert np.abs(S[1][0][:8, :8] - fp[0]).max() < 1e-15
    assert np.abs(S[1][1][:8, :8] - fp[1]).max() < 1e-15
    assert np.abs(S[1][0][-8:, -8:] - fp[2]).max() < 1e-15
    norms = np.array([[np.linalg.norm(a), np.linalg.norm(b)] for a, b in S])
    assert np.abs(norms - g["norms"]).max() < 1e-13
    x = g["x_th"]
    n = len(S)
    Sx = x.copy()
    for i in range(n):
        if i > 0:
            Sx[i * m:(i + 1) * m] += S[i][0] @ x[(i - 1) * m:i * m]
        if i < n - 1:
            Sx[i * m:(i + 1) * m] += S[i][1] @ x[(i + 1) * m:(i + 2) * m]
    assert relerr(Sx, g["Stot_x"]) < 1e-13


def test_helmholtz3d_slab_maps_match_upstream(golden):
    """The 3-D variable-coefficient Helmholtz slab maps (7-point stencil,
    sparse LU of the slab interior) against upstream's oms + stencil solver
    on 4 interfaces of 8 x 8 points; the sampled form (one sparse solve per
    sketch, both orientations) against the dense maps."""
    from oracle.slabmaps import helmholtz3d_sample, helmholtz3d_slab_maps
    g = golden("c3_helmholtz_small")
    ns = int(g["nslabs"])
    H = 1.0 / ns
    geo = (int(g["nx"]), int(g["ny"]), int(g["nz"]), 2 * H, float(g["kappa"]))
    for i in range(ns - 1):
        L, R = helmholtz3d_slab_maps(*geo, x0=(i + 1) * H - H)
        if i > 0:
            assert np.abs(L - g["Sl"][i]).max() < 1e-11 * np.abs(g["Sl"][i]).max()
        if i < ns - 2:
            assert np.abs(R - g["Sr"][i]).max() < 1e-11 * np.abs(g["Sr"][i]).max()
    Om = np.random.default_rng(0).standard_normal((L.shape[0], 5))
    x0 = (ns - 1) * H - H
    assert relerr(helmholtz3d_sample(*geo, x0, Om, 0), L @ Om) < 1e-13
    assert relerr(helmholtz3d_sample(*geo, x0, Om, 1, trans=True), R.T @ Om) < 1e-13


def _periodic_matrix(S, T):
    nS, m = S.shape[0], S.shape[2]
    M = np.zeros((nS * m, nS * m))
    for i in range(nS):
        M[i * m:(i + 1) * m, i * m:(i + 1) * m] = T[i]
        j = (i - 1) % nS
        M[i * m:(i + 1) * m, j * m:(j + 1) * m] += S[i][0]
        j = (i + 1) % nS
        M[i * m:(i + 1) * m, j * m:(j + 1) * m] += S[i][1]
    return M


def test_rb_cyclic_fixture_is_the_periodic_system(golden):
    """Upstream's RedBlackSolver(cyclic=True) solves the periodic system in
    which SiM[0] couples block 0 to the last block and SiP[-1] the last
    block to block 0 (with two blocks both couplings land on the other
    block): the fixture agrees with a dense solve of that system."""
    g = golden("rb_cyclic")
    for key in ("2_5", "4_6", "8_16"):
        M = _periodic_matrix(g["S_" + key], g["T_" + key])
        assert relerr(np.linalg.solve(M, g["rhs_" + key]), g["x_" + key]) < 1e-14


def test_slab_adjacency_mirror_matches_upstream(golden):
    """slabTree.level_adj_list (the strong-admissibility near field) against
    upstream's: binary trees with 'partial' and 'full' adjacency, quad trees,
    on lines, rectangles and a plane in 3-D."""
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    from tests.golden.make_golden import SLAB_TREE_CASES, adjacency_record, slab_cloud
    g = golden("slab_adjacency")
    for name, kind, n, quad, leaf in SLAB_TREE_CASES:
        for adj in (("partial",) if quad else ("partial", "full")):
            t = slabTree(slab_cloud(kind, n), quad, leaf, adjacency=adj)
            lv, cnt, nbr = adjacency_record(t)
            k = "%s_%s_" % (name, adj)
            assert np.array_equal(lv, g[k + "levels"]), k
            assert np.array_equal(cnt, g[k + "count"]), k
            assert np.array_equal(nbr, g[k + "nbr"]), k


def test_strong_oracle_matches_upstream(golden):
    """oracle.strong (HBStorch_strong restated in numpy) against upstream's
    own construct + sweep on the same sketches: apply in both orientations
    to 1e-12, the leaf near-field tiles (norms) to 1e-9, the level count."""
    from oracle.strong import StrongHBS
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    from tests.golden.make_golden import STRONG_CASES, strong_samples
    g = golden("hbs_strong")
    for case in STRONG_CASES:
        name, kind, quad, leaf, adj, rk, seed = case
        XX, A, Om, Psi, x = strong_samples(*case)
        t = slabTree(XX, quad, leaf, adjacency=adj)
        O = StrongHBS(t.perm_leaf, t.nleaves, t.level_adj_list, 4 if quad else 2)
        O.construct(rk, Om, Psi, A @ Om, A.T @ Psi)
        p = name + "_"
        for got, ref in ((O.apply(x), g[p + "Ax"]), (O.apply(x, True), g[p + "ATx"])):
            assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), name
        rc = g[p + "tile_rc"]
        norms = np.array([np.linalg.norm(O.E[0].tiles[(int(i), int(j))]) for i, j in rc])
        assert len(O.E[0].tiles) == len(rc), name
        assert np.allclose(norms, g[p + "tile_norms"], rtol=1e-9, atol=0), name
        assert [len(O.U), len(O.E) + 1] == list(g[p + "nlev"]), name


def test_poisson_slab_map_closed_form():
    """The closed-form Poisson slab map of the workload generator equals the
    oracle's (pinned to upstream's stencil pipeline) on both edges."""
    from oracle.slabmaps import poisson2d_slab_maps
    from sslablu_gb300.synthetic import poisson_slab_map
    for m, nx, w in [(64, 5, 0.25), (128, 41, 2 / 9), (200, 17, 0.1)]:
        S = poisson_slab_map(m, nx, w)
        for ref in poisson2d_slab_maps(m, nx, w):
            assert np.abs(S - ref).max() <= 1e-13 * np.abs(ref).max()
