"""HBS red-black and Thomas solvers on the GPU vs upstream golden vectors.

rbhbs_gauss: rank 16 resolves the Schur complements to a ~1e-13 residual, so
the GPU result must match upstream to 1e-10 (float64 rounding of the two
implementations, amplified only by the conditioning of the compressions).
rbhbs_kernel: the exponential-kernel couplings are truncation dominated at
ranks 16/24 (upstream residual 4e-5 / 1e-5).  The singular values near the
cut decay slowly, so the retained subspace of each truncated SVD is fixed only
up to the near-degenerate cluster at the cut: float64 rounding differences
between any two implementations (LAPACK vs this library) move the truncated
approximation within its own error.  There parity is equal solution quality:
the GPU residual within 2x of upstream's, and the two solutions no further
apart than 100x that residual.  (Thomas-HBS at these ranks is well resolved
and must match to 1e-10.)
"""
import numpy as np
import pytest
import types

from tests._cases import gauss_system, kernel_system, relerr, tridiag_matrix
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu


def _ops(S, tree):
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import dense_to_linop
    out = []
    for a, c in S:
        la, lc = dense_to_linop(a), dense_to_linop(c)
        la.tree = lc.tree = tree
        la.quad = lc.quad = False
        out.append((la, lc))
    return out


def test_rbhbs_gauss(golden):
    need_gpu()
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS, ThomasSolverHBS
    g = golden("rbhbs_gauss")
    m, nS, leaf, nlev, rk = (int(g[k]) for k in ("m", "nS", "leaf", "nlev", "rk"))
    tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=m // leaf, nlevels=nlev)
    S = gauss_system(m, nS)
    M = tridiag_matrix(S, m)
    np.random.seed(11)
    R = RedBlackSolverHBS(m, rk, tree, False)
    R.factorize(_ops(S, tree))
    x = R.solve(g["b"])
    assert x.shape == g["b"].shape
    assert relerr(x, g["x_rb"]) < 1e-10
    assert relerr(M @ x, g["b"]) < 1e-11
    np.random.seed(12)
    T = ThomasSolverHBS(m, rk)
    T.factorize(_ops(S, tree))
    y = T.solve(g["b"])
    assert relerr(y, g["x_th"]) < 1e-10
    assert relerr(M @ y, g["b"]) < 1e-11
    # multi-RHS through the same factors
    B = np.stack([g["b"], -g["b"]], axis=1)
    X = R.solve(B)
    assert relerr(X[:, 1], -x) < 1e-12


@pytest.mark.parametrize("rk", [16, 24])
def test_rbhbs_kernel(golden, rk):
    need_gpu()
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS, ThomasSolverHBS
    g = golden("rbhbs_kernel")
    m, nS, leaf, nlev = int(g["m"]), int(g["nS"]), int(g["leaf"]), int(g["nlev"])
    tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=m // leaf, nlevels=nlev)
    S = kernel_system(m, nS)
    M = tridiag_matrix(S, m)
    np.random.seed(11)
    R = RedBlackSolverHBS(m, rk, tree, False)
    R.factorize(_ops(S, tree))
    x = R.solve(g["b"])
    res_ref = relerr(M @ g["x_rb_%d" % rk], g["b"])
    assert relerr(M @ x, g["b"]) < 2 * res_ref
    assert relerr(x, g["x_rb_%d" % rk]) < 100 * res_ref
    np.random.seed(12)
    T = ThomasSolverHBS(m, rk)
    T.factorize(_ops(S, tree))
    y = T.solve(g["b"])
    assert relerr(y, g["x_th_%d" % rk]) < 1e-10


def test_hbs_slab_solvers_refined(golden):
    """solve_refined on the exponential-kernel system at rank 16: the
    red-black solve is truncation bound (plain residual ~1e-5) and refinement
    against the exact couplings brings it to 1e-10; Thomas is resolved
    already (one solve); apply() is the dense block-tridiagonal matrix."""
    need_gpu()
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS, ThomasSolverHBS
    g = golden("rbhbs_kernel")
    m, nS, leaf, nlev = int(g["m"]), int(g["nS"]), int(g["leaf"]), int(g["nlev"])
    tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=m // leaf, nlevels=nlev)
    S = kernel_system(m, nS)
    M = tridiag_matrix(S, m)
    b = g["b"]
    x0 = np.random.default_rng(3).standard_normal(M.shape[0])
    for seed, make, bound in ((11, lambda: RedBlackSolverHBS(m, 16, tree, False), True),
                              (12, lambda: ThomasSolverHBS(m, 16), False)):
        np.random.seed(seed)
        sv = make()
        sv.factorize(_ops(S, tree))
        assert relerr(sv.apply(x0), M @ x0) < 1e-13
        x, it, rel = sv.solve_refined(b, tol=1e-10, maxit=8)
        if bound:
            assert relerr(M @ sv.solve(b), b) > 1e-8      # the plain solve is truncation bound
            assert 2 <= it <= 8
        assert x.shape == b.shape and it >= 1
        assert rel <= 1e-10 and relerr(M @ x, b) < 1e-10


def test_rbhbs_concurrent_compressions_repeat(golden):
    """One red-black level's compressions run on worker threads, each at its
    own tree level and so its own shared-memory size for the panel QR and
    Jacobi kernels (omsdirectsolveHBS.py:436-483 _build_level: three
    compressions per kept node).  Repeated factorisations with the same
    seed must all succeed and give the same solution to rounding."""
    need_gpu()
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS
    g = golden("rbhbs_kernel")
    m, nS, leaf, nlev = int(g["m"]), int(g["nS"]), int(g["leaf"]), int(g["nlev"])
    tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=m // leaf, nlevels=nlev)
    S = kernel_system(m, nS)
    M = tridiag_matrix(S, m)
    res_ref = relerr(M @ g["x_rb_24"], g["b"])
    xs = []
    for _ in range(4):
        np.random.seed(11)
        R = RedBlackSolverHBS(m, 24, tree, False)
        R.factorize(_ops(S, tree))
        xs.append(R.solve(g["b"]))
        assert relerr(M @ xs[-1], g["b"]) < 2 * res_ref
    for x in xs[1:]:
        assert relerr(x, xs[0]) < 1e-8


def test_rbhbs_cyclic_periodic_system():
    """Periodic red-black HBS (RedBlackSolverHBS(cyclic=True),
    omsdirectsolveHBS.py:375-558 with modular neighbours) on Gaussian-kernel
    couplings that rank 16 resolves, 4 and 8 blocks, against the dense solve
    of the periodic system.  When a level reduces to one block its couplings
    act on that block itself and are added to its diagonal, as upstream's
    dense cyclic solver does (omsdirectsolve.py:326-327); upstream's HBS
    solver leaves them out and misses this system by a residual of 0.38 (a
    defect not reproduced)."""
    need_gpu()
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS
    m, leaf, nlev, rk = 128, 32, 3, 16
    tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=m // leaf, nlevels=nlev)
    x = np.linspace(0, 1, m)

    def blk(shift):
        return 0.3 * np.exp(-20.0 * (x[:, None] - x[None, :] - shift) ** 2)
    for nS in (4, 8):
        S = [(blk(0.2 + 0.01 * i), blk(-0.2 - 0.01 * i)) for i in range(nS)]
        M = np.eye(nS * m)
        for i in range(nS):
            j = (i - 1) % nS
            M[i * m:(i + 1) * m, j * m:(j + 1) * m] += S[i][0]
            j = (i + 1) % nS
            M[i * m:(i + 1) * m, j * m:(j + 1) * m] += S[i][1]
        b = np.random.default_rng(nS).standard_normal((nS * m, 3))
        np.random.seed(11)
        R = RedBlackSolverHBS(m, rk, tree, False, cyclic=True)
        R.factorize([[la, lc] for la, lc in _ops(S, tree)])
        xs = R.solve(b)
        assert relerr(M @ xs, b) < 1e-10, nS
        assert relerr(xs, np.linalg.solve(M, b)) < 1e-10, nS
        assert relerr(R.apply(xs), M @ xs) < 1e-13, nS
