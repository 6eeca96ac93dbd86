"""The tensor-core (tcgen05) sweep and apply: bfloat16 products of error-free
digit splits (Ozaki scheme) against the CPU oracle's float64 ULV solve
(ULVsparse.solve, matAssembly/HBS/ULVsparse.py:296-327) and HBS apply
(HBSnew.HBSMAT.matmat, matAssembly/HBS/HBSnew.py:308-350).

Seven digits per operand and every digit pair of weight >= 2^-64 leave a
relative error of ~2^-50 of |S| |z| per step product, so the results must
agree with the float64 oracle as closely as a float64 implementation does:
1e-12 relative for solves and applies (the plain float64 path's tolerance),
and the refined solve must reach a 1e-10 relative residual measured with the
oracle's float64 apply."""
import numpy as np
import pytest

from oracle.hbs import OracleHBS, gen_random_hbs
from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _pair(k, nl, L, quad, seed, sigma=None):
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    np.random.seed(seed)
    S, Nbvec = gen_random_hbs(k, nl, L, quad=quad, sigma=sigma)
    fac = 4 if quad else 2
    G = HBSMAT().set_mats(S.Umats, S.Dmats, S.Vmats, list(Nbvec), fac=fac)
    G.compute_ULV()
    O = OracleHBS().set_mats(S.Umats, S.Dmats, S.Vmats, list(Nbvec), fac=fac)
    O.compute_ULV()
    return G, O


@pytest.mark.parametrize("k,nl,L,quad,nrhs", [(8, 16, 4, False, 1), (8, 16, 4, False, 130),
                                              (16, 32, 5, False, 64), (8, 16, 3, True, 7),
                                              (32, 64, 4, False, 300)])
def test_ozaki_apply_and_solve_match_oracle(k, nl, L, quad, nrhs):
    need_gpu()
    G, O = _pair(k, nl, L, quad, seed=k + nl + L + nrhs)
    x = np.random.default_rng(nrhs).standard_normal((G.shape[0], nrhs))
    assert relerr(G.apply_ozaki(x), O.matmat(x)) < TOL
    assert relerr(G.solve_ozaki(x), O.solve(x)) < TOL


def test_ozaki_wide_dynamic_range():
    """Columns of very different magnitude (beyond the float32 range), and a
    zero column: each column is normalised by its largest power of two on
    entry, so every column keeps its relative accuracy."""
    need_gpu()
    G, O = _pair(16, 32, 4, False, seed=5)
    scales = np.array([1.0, 1e-20, 1e25, 0.0, 3e-8, 1e-200, 1e200, 1.0])
    x = np.random.default_rng(9).standard_normal((G.shape[0], scales.size)) * scales
    xs = G.solve_ozaki(x)
    xo = O.solve(x)
    ya = G.apply_ozaki(x)
    yo = O.matmat(x)
    for j in range(scales.size):
        if scales[j] == 0.0:
            assert not xs[:, j].any() and not ya[:, j].any()
            continue
        sc = scales[j]   # compared after rescaling (the norms of 1e200 columns overflow)
        assert relerr(xs[:, j] / sc, xo[:, j] / sc) < TOL, j
        assert relerr(ya[:, j] / sc, yo[:, j] / sc) < TOL, j


def test_ozaki_c2_operator_refined():
    """The N = 4096, leaf 64, rank 32 operator with singular values decaying
    from 1 to 1e-12 (the HBS benchmark's shape): the tensor-core solve agrees
    with the float64 GPU solve, and refinement driven by the tensor-core
    residual reaches 1e-10 against the oracle's float64 apply."""
    need_gpu()
    sigma = 10.0 ** (-12.0 * np.arange(32) / 31)
    G, O = _pair(32, 64, 7, False, seed=20261205, sigma=sigma)
    b = np.random.default_rng(1).standard_normal((G.shape[0], 96))
    x64 = G.solve(b)
    xt = G.solve_ozaki(b)
    assert relerr(xt, x64) < TOL
    xr, it, rel = G.solve_refined(b, tol=1e-10, maxit=4, inner="tensor")
    assert it >= 1 and rel <= 1e-10
    r = b - O.matmat(xr)
    res = np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)
    assert res.max() <= 1e-10
    assert relerr(xr, O.solve(b)) < 1e-10


@pytest.mark.parametrize("k,nl,L,quad,nrhs", [(8, 16, 4, False, 5), (16, 32, 5, False, 64),
                                              (8, 16, 3, True, 7), (32, 64, 4, False, 300)])
def test_ozaki_transposed_apply_and_solve(k, nl, L, quad, nrhs):
    """A^T x and A^{-T} b on the tensor cores: the apply against the oracle's
    rmatmat and the solve against the float64 mode-T solve (the same
    transposed steps, pinned to upstream in test_gpu_hbs.py), 1e-12; at
    rank 32 / leaf 64 the transposed backward steps read 128 rows per block
    (the widest step the digit sums keep exact)."""
    need_gpu()
    G, O = _pair(k, nl, L, quad, seed=3 * k + nl + L + nrhs)
    x = np.random.default_rng(nrhs + 1).standard_normal((G.shape[0], nrhs))
    assert relerr(G.apply_ozaki(x, trans=True), O.rmatmat(x)) < TOL
    assert relerr(G.solve_ozaki(x, mode="T"), G.solve(x, mode="T")) < TOL
    assert relerr(G.solve_ozaki(x[:, 0], mode="T"), G.solve(x[:, 0], mode="T")) < TOL


def test_ozaki_refactor_rebuilds_digits():
    """A refactored operator's tensor-core solve uses the new factors (the
    digit forms are rebuilt, not reused)."""
    need_gpu()
    G, O = _pair(16, 32, 4, False, seed=9)
    x = np.random.default_rng(2).standard_normal((G.shape[0], 40))
    import torch
    from sslablu_gb300 import _lib as L
    G.solve_ozaki(x)                     # builds the digit forms
    G2, O2 = _pair(16, 32, 4, False, seed=10)
    keep = []
    Lv = len(O2.Dmats)
    for t in range(Lv):                  # new factors into the same operator
        Nb = int(O2.Nbvec[t])
        D = torch.from_numpy(np.ascontiguousarray(O2.Dmats[t])).cuda()
        n = D.shape[0] // Nb
        U = V = None
        k = 0
        if t < Lv - 1:
            U = torch.from_numpy(np.ascontiguousarray(O2.Umats[t])).cuda()
            V = torch.from_numpy(np.ascontiguousarray(O2.Vmats[t])).cuda()
            k = U.shape[1]
        keep += [U, V, D]
        L.check(L.lib().slu_hbs_set_level(L.handle(), G._op, t, Nb, n, k, L.ptr(U), L.ptr(V),
                                          L.ptr(D)))
    G.compute_ULV()
    assert relerr(G.solve_ozaki(x), O2.solve(x)) < TOL
