"""The assembler side of the path on the GPU: HBStorch.HBSMAT (compression
from given sketches with HBStorch's null-space rule), ULVsparse_torch, and
matAssembler's rkHBS / dense methods, against upstream outputs frozen in
tests/golden/hbstorch.npz and assembler.npz."""
import numpy as np
import pytest

from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _exact_in_tree_order(k, nl, L, seed, perm):
    from oracle.hbs import gen_random_hbs
    np.random.seed(seed)
    S, _ = gen_random_hbs(k, nl, L, quad=False)
    M = S.matmat(np.eye(S.shape[0]))
    A = np.zeros_like(M)
    A[np.ix_(perm, perm)] = M
    return A


def _grid16():
    return np.stack(np.meshgrid(np.linspace(0, 1, 16), np.linspace(0, 2, 16), indexing="ij"),
                    -1).reshape(-1, 2)


def _hbstorch(g):
    from sslablu_gb300.matAssembly.HBS.HBStorch import HBSMAT
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    tree = slabTree(_grid16(), False, 16)
    assert np.array_equal(tree.perm_leaf, g["perm"])
    A = _exact_in_tree_order(int(g["k"]), 16, tree.nlevels, 7, tree.perm_leaf)
    H = HBSMAT(device="cuda", tree=tree, quad=False)
    H.construct(int(g["k"]), g["Om"], g["Psi"], A @ g["Om"], A.T @ g["Psi"])
    return H, A


def test_hbstorch_construct_from_sketches(golden):
    need_gpu()
    g = golden("hbstorch")
    H, A = _hbstorch(g)
    assert list(H.Nbvec) == list(g["Nbvec"]) and H.nSamples == int(g["nSamples"])
    assert H.nbytes == int(g["nbytes"])
    x = g["x"]
    assert relerr(H.matmat(x), g["Ax"]) < TOL
    assert relerr(H.rmatmat(x), g["ATx"]) < TOL
    assert relerr(H @ x, g["Ax"]) < TOL and relerr(H.T @ x, g["ATx"]) < TOL
    D = H.Dmats
    assert tuple(D[0].shape) == g["D0"].shape
    assert relerr(D[0].cpu().numpy(), g["D0"]) < TOL
    assert D[-1].device.type == "cpu"               # root D on the host, as upstream
    for t, U in enumerate(H.Umats):
        assert relerr(np.abs(U.cpu().numpy()), np.abs(g["U%d" % t])) < TOL
    # the intended compute_ULV / solve of the compressed operator
    H.compute_ULV()
    assert relerr(H.solve(g["b"], "cuda"), g["sol"]) < TOL


def test_ulvsparse_torch_mirror(golden):
    need_gpu()
    import torch
    from sslablu_gb300.matAssembly.HBS import ULVsparse_torch as UT
    g = golden("hbstorch")
    H, _ = _hbstorch(g)
    Nbvec = [int(d.shape[0]) for d in H.Dmats]
    Q, W, Uu, R, NN = UT.compute_ULV(H.Umats, H.Dmats, H.Vmats, Nbvec, "cuda")
    assert [int(q.shape[0]) for q in Q] == Nbvec and len(W) == len(Uu) == len(Nbvec) - 1
    perm = g["perm"]
    rhs = torch.from_numpy(g["b"][perm]).cuda()
    y = UT.solve(H.Umats, H.Dmats, Q, W, Uu, R, NN, rhs, "cuda")
    assert relerr(y.cpu().numpy(), g["sol"][perm]) < TOL
    y1 = UT.solve(H.Umats, H.Dmats, Q, W, Uu, R, NN, rhs[:, 0], "cuda")
    assert y1.dim() == 1 and relerr(y1.cpu().numpy(), g["sol"][perm, 0]) < TOL
    blk = UT.convert_to_torch_tens(g["b"], 16, "cuda")
    assert tuple(blk.shape) == (16, 16, 3)
    assert np.array_equal(UT.convert_to_blkdiag(blk).cpu().numpy(), g["b"])


def test_mat_assembler_rkhbs_and_dense(golden):
    need_gpu()
    import types
    import scipy.sparse.linalg as sla
    from sslablu_gb300.matAssembly import matAssembler as MA
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    g = golden("assembler")
    XX = _grid16()
    perm = slabTree(XX, False, 8).perm_leaf
    assert np.array_equal(perm, g["perm"])
    A = _exact_in_tree_order(3, 8, 6, 9, perm)
    stmap = types.SimpleNamespace(A=sla.aslinearoperator(A), XXI=XX)
    np.random.seed(11)
    asm = MA.rkHMatAssembler(8, 3)
    H = asm.assemble(stmap)
    assert H.nSamples == int(g["nSamples"]) and asm.stats.nbytes == int(g["nbytes"])
    x = g["x"]
    assert relerr(H.matmat(x), g["Ax"]) < TOL
    assert relerr(H.rmatmat(x), g["ATx"]) < TOL
    M = MA.denseMatAssembler().assemble(stmap)
    assert bool(g["dense_ok"]) and np.array_equal(M, A)
    assert isinstance(MA.tolHMatAssembler(1e-6, 8, 3).assemble(stmap), TypeError)


def test_hbstorch_construct_with_ulv_sampling():
    """constructHBS_ULV: device-drawn sketches through a device operator; an
    exact HBS operator is recovered to rounding and solved."""
    need_gpu()
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT as Exact
    from sslablu_gb300.matAssembly.HBS.HBStorch import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    np.random.seed(21)
    U, D, V, Nbvec = random_hbs_factors(8, 32, 4, quad=False, shift=4.0)
    A = Exact().set_mats(U, D, V, list(Nbvec), fac=2)
    H = HBSMAT(A=A, device="cuda", quad=False)
    H.set_Nbvec(list(Nbvec))
    H.construct(8, compute_ULV=True)
    x = np.random.default_rng(3).standard_normal((A.shape[0], 2))
    assert relerr(H.matmat(x), A.matmat(x)) < 1e-10
    assert relerr(A.matmat(H.solve(x, "cuda")), x) < 1e-10


def test_mat_assembler_mixed_sampling(golden):
    """precision='mixed' takes the samples of an explicit matrix on the
    tensor cores (split-BF16x3, ~1e-7 relative); the compressed operator of
    the upstream assembler case then agrees with upstream's float64 result to
    the sampling accuracy (1e-5), and the float64 default stays at 1e-12."""
    need_gpu()
    import types
    from sslablu_gb300.matAssembly import matAssembler as MA
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    g = golden("assembler")
    XX = _grid16()
    perm = slabTree(XX, False, 8).perm_leaf
    A = _exact_in_tree_order(3, 8, 6, 9, perm)
    stmap = types.SimpleNamespace(A=A, XXI=XX)
    for prec, tol in (("f64", TOL), ("mixed", 1e-5)):
        np.random.seed(11)
        asm = MA.matAssembler(MA.matAssemblerOptions("rkHBS", 0, 8, 3, precision=prec))
        H = asm.assemble(stmap)
        assert relerr(H.matmat(g["x"]), g["Ax"]) < tol, prec
        assert relerr(H.rmatmat(g["x"]), g["ATx"]) < tol, prec


def test_mat_assembler_rkhbs_strong():
    """rkHMatAssembler_strong (upstream's rkHBS_strong names a class its
    module lacks): the assembled strong-admissibility operator equals the
    oracle's compression from the same draws (1e-12) and resolves the
    coupling far better than the weak rkHBS at the same rank."""
    need_gpu()
    import types
    from oracle.strong import StrongHBS
    from sslablu_gb300.matAssembly import matAssembler as MA
    from sslablu_gb300.matAssembly.HBS.slabTree import slabTree
    from sslablu_gb300.synthetic import plane_coupling, plane_points
    XX = plane_points(32)
    A = plane_coupling(XX)
    N, rk, leaf = A.shape[0], 16, 64
    stmap = types.SimpleNamespace(A=A, XXI=XX)
    np.random.seed(5)
    asm = MA.rkHMatAssembler_strong(leaf, rk)
    H = asm.assemble(stmap)
    s = 5 * max(2 * rk, leaf) + rk + 20
    np.random.seed(5)
    Om = np.random.standard_normal((N, s))
    Psi = np.random.standard_normal((N, s))
    t = slabTree(XX, False, leaf)
    O = StrongHBS(t.perm_leaf, t.nleaves, t.level_adj_list).construct(rk, Om, Psi, A @ Om,
                                                                      A.T @ Psi)
    x = np.random.default_rng(6).standard_normal((N, 3))
    assert relerr(H.matmat(x), O.apply(x)) < TOL
    assert relerr(H.rmatmat(x), O.apply(x, True)) < TOL
    assert asm.stats.nbytes == H.nbytes > 0
    np.random.seed(5)
    W = MA.rkHMatAssembler(leaf, rk).assemble(stmap)
    assert relerr(H.matmat(x), A @ x) < 0.2 * relerr(W.matmat(x), A @ x)
