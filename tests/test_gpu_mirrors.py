"""Functional mirrors (ULVsparse, multislab) on the GPU vs upstream golden vectors."""
import types

import numpy as np
import pytest

from tests._cases import gauss_system, hbs_from_fixture, relerr, tridiag_matrix
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["hbs_binary_k8", "hbs_quad_k8"])
def test_ulvsparse_functions(golden, name):
    need_gpu()
    from sslablu_gb300.matAssembly.HBS import ULVsparse
    g = golden(name)
    S, Nbvec = hbs_from_fixture(g)
    Ql, Wl, Uul, Rl, NNv = ULVsparse.compute_ULV(S.Umats, S.Dmats, S.Vmats, Nbvec)
    assert np.array_equal(NNv, g["ulv_NNvec"])
    x = g["x"]
    y = ULVsparse.solve(S.Umats, S.Dmats, Ql, Wl, Uul, Rl, NNv, Nbvec, x.copy())
    yt = ULVsparse.solve(S.Umats, S.Dmats, Ql, Wl, Uul, Rl, NNv, Nbvec, x.copy(), mode="T")
    assert relerr(y, g["ulv_sol"]) < 1e-12
    assert relerr(yt, g["ulv_solT"]) < 1e-12


def test_multislab_thomas_c1(golden):
    need_gpu()
    from sslablu_gb300.multislab import omsdirectsolve as mods
    g = golden("c1_poisson64")
    n = g["Sl"].shape[0]
    nc = int(g["nc"])
    S = [[g["Sr"][0]]] + [[g["Sl"][i], g["Sr"][i]] for i in range(1, n - 1)] + [[g["Sl"][n - 1]]]
    OMS = types.SimpleNamespace(glob_target_dofs=[range(i * nc, (i + 1) * nc) for i in range(n)])
    T = mods.build_block_tridiagonal_solver(S)
    x = mods.block_tridiagonal_solve(OMS, T, g["rhs"])
    assert relerr(x, g["x_f"]) < 1e-12
    assert relerr(x, g["x_th"]) < 1e-12


def test_multislab_cyclic_matches_dense(golden):
    need_gpu()
    from sslablu_gb300.multislab import omsdirectsolve as mods
    rng = np.random.default_rng(9)
    nS, m = 5, 6
    S = [[0.1 * rng.standard_normal((m, m)), 0.1 * rng.standard_normal((m, m))] for _ in range(nS)]
    M = np.eye(nS * m)
    for i in range(nS):
        if i > 0:
            M[i * m:(i + 1) * m, (i - 1) * m:i * m] = S[i][0]
        if i < nS - 1:
            M[i * m:(i + 1) * m, (i + 1) * m:(i + 2) * m] = S[i][1]
    M[0:m, (nS - 1) * m:] = S[0][0]
    M[(nS - 1) * m:, 0:m] = S[-1][1]
    OMS = types.SimpleNamespace(glob_target_dofs=[range(i * m, (i + 1) * m) for i in range(nS)])
    T, smw = mods.build_block_cyclic_tridiagonal_solver(OMS, S, None, nS * m, m)
    b = rng.standard_normal(nS * m)
    x = mods.block_cyclic_tridiagonal_solve(OMS, T, smw, b)
    assert relerr(x, np.linalg.solve(M, b)) < 1e-12


def test_multislab_hbs_thomas_gauss(golden):
    need_gpu()
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import dense_to_linop
    from sslablu_gb300.multislab import omsdirectsolveHBS as modh
    g = golden("rbhbs_gauss")
    m, nS, leaf, nlev, rk = (int(g[k]) for k in ("m", "nS", "leaf", "nlev", "rk"))
    tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=m // leaf, nlevels=nlev)
    S = gauss_system(m, nS)
    ops = [(dense_to_linop(a), dense_to_linop(c)) for a, c in S]
    np.random.seed(12)
    T = modh.build_block_tridiagonal_solver(ops, tree, False, rk)
    OMS = types.SimpleNamespace(glob_target_dofs=[range(i * m, (i + 1) * m) for i in range(nS)])
    x = modh.block_tridiagonal_solve(OMS, T, g["b"])
    # same algorithm and sketches as direct_solve.ThomasSolverHBS
    assert relerr(x, g["x_th"]) < 1e-10
    assert relerr(tridiag_matrix(S, m) @ x, g["b"]) < 1e-11
