"""Strong-admissibility HBS on the GPU (slu_strong_* through
sslablu_gb300.matAssembly.HBS.HBStorch_strong) against upstream's own
HBStorch_strong outputs on the same sketches (tests/golden/hbs_strong.npz:
planes of points with 'partial', 'full' and quad adjacency) and against the
CPU oracle (oracle/strong.py, pinned to the same fixture).  The compressed
operator is unique given the sketches, so its apply must agree to 1e-12;
the leaf bases agree through their projectors U U^T (singular vectors are
unique up to sign) and the near-field tiles one by one."""
import numpy as np
import pytest

from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu


def _build(case):
    from sslablu_gb300.matAssembly.HBS.HBStorch_strong import HBSMAT
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    from tests.golden.make_golden import strong_samples
    name, kind, quad, leaf, adj, rk, seed = case
    XX, A, Om, Psi, x = strong_samples(*case)
    tree = slabTree(XX, quad, leaf, adjacency=adj)
    H = HBSMAT(device="cuda", tree=tree, quad=quad)
    H.construct(rk, Om, Psi, A @ Om, A.T @ Psi)
    return H, tree, A, Om, Psi, x


@pytest.mark.parametrize("ci", range(4))
def test_strong_matches_upstream(ci):
    """matmat / rmatmat / @ of the T view vs upstream HBStorch_strong
    (1e-12), every leaf near-field tile's norm (1e-9), the level count and
    nbytes."""
    need_gpu()
    from tests.golden.make_golden import STRONG_CASES
    g = np.load("tests/golden/hbs_strong.npz")
    case = STRONG_CASES[ci]
    H, tree, A, Om, Psi, x = _build(case)
    p = case[0] + "_"
    Ax, ATx = g[p + "Ax"], g[p + "ATx"]
    assert np.linalg.norm(H.matmat(x) - Ax) <= 1e-12 * np.linalg.norm(Ax)
    assert np.linalg.norm(H.rmatmat(x) - ATx) <= 1e-12 * np.linalg.norm(ATx)
    assert np.linalg.norm((H.T @ x) - ATx) <= 1e-12 * np.linalg.norm(ATx)
    y1 = H.matvec(x[:, 0])
    assert y1.shape == (x.shape[0],)
    assert np.linalg.norm(y1 - Ax[:, 0]) <= 1e-12 * np.linalg.norm(Ax[:, 0])
    E0 = H.Emats[0]
    norms = np.linalg.norm(E0.val.cpu().numpy(), axis=(1, 2))
    got = {(int(i), int(j)): v for i, j, v in zip(E0.row, E0.col, norms)}
    ref = {(int(i), int(j)): v for (i, j), v in zip(g[p + "tile_rc"], g[p + "tile_norms"])}
    assert sorted(got) == sorted(ref)
    for key, v in ref.items():
        assert abs(got[key] - v) <= 1e-9 * v, key
    assert [len(H.Umats), len(H.Emats)] == list(g[p + "nlev"])
    assert H.nbytes == int(g[p + "nbytes"])


def test_strong_factors_match_oracle():
    """Leaf projectors U U^T, V V^T vs the oracle's (1e-10) and the leaf
    tiles (1e-8: each tile carries R^-1 of a near-field stack of ~600 rows,
    so its rounding is the stack's condition number times 1e-16; the oracle
    and upstream differ by 3e-10 there), full adjacency on a 32 x 32 plane."""
    need_gpu()
    from oracle.strong import StrongHBS
    from tests.golden.make_golden import STRONG_CASES
    case = STRONG_CASES[1]
    H, tree, A, Om, Psi, x = _build(case)
    O = StrongHBS(tree.perm_leaf, tree.nleaves, tree.level_adj_list)
    O.construct(case[5], Om, Psi, A @ Om, A.T @ Psi)
    for got, ref in ((H.Umats[0], O.U[0]), (H.Vmats[0], O.V[0])):
        got = got.cpu().numpy()
        pg = np.einsum("nbk,nck->nbc", got, got)
        pr = np.einsum("nbk,nck->nbc", ref, ref)
        assert np.abs(pg - pr).max() <= 1e-10
    E0 = H.Emats[0]
    val = E0.val.cpu().numpy()
    for t in range(E0.nnz):
        ref = O.E[0].tiles[(int(E0.row[t]), int(E0.col[t]))]
        assert np.linalg.norm(val[t] - ref) <= 1e-8 * max(np.linalg.norm(ref), 1e-300)


def test_strong_accuracy_against_the_operator():
    """The compressed operator against the dense operator it compresses:
    full adjacency resolves the kernel far better than partial at the same
    rank (the reason for strong admissibility), and both stay below
    upstream's own errors on these cases (recorded in the fixture)."""
    need_gpu()
    from tests.golden.make_golden import STRONG_CASES
    g = np.load("tests/golden/hbs_strong.npz")
    errs = {}
    for case in STRONG_CASES[:2]:
        H, tree, A, Om, Psi, x = _build(case)
        errs[case[0]] = np.linalg.norm(H.matmat(x) - A @ x) / np.linalg.norm(A @ x)
        assert errs[case[0]] <= 1.01 * float(g[case[0] + "_relerr"])
    assert errs["plane_full"] < 0.05 * errs["plane_partial"]


def test_strong_rank_deficient_stack_is_reported():
    """A near-field stack without full row rank (a zero sketch block) is
    reported as an error, where upstream switches to a truncated SVD."""
    need_gpu()
    from sslablu_gb300._lib import SluError
    from sslablu_gb300.matAssembly.HBS.HBStorch_strong import HBSMAT
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    from tests.golden.make_golden import STRONG_CASES, strong_samples
    case = STRONG_CASES[3]
    name, kind, quad, leaf, adj, rk, seed = case
    XX, A, Om, Psi, x = strong_samples(*case)
    tree = slabTree(XX, quad, leaf, adjacency=adj)
    Om = Om.copy()
    Om[np.asarray(tree.perm_leaf)[:leaf]] = 0.0      # the first leaf's sketch rows
    H = HBSMAT(device="cuda", tree=tree, quad=quad)
    with pytest.raises(SluError, match="rank deficient"):
        H.construct(rk, Om, Psi, A @ Om, A.T @ Psi)
