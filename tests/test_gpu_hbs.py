"""HBS compression, ULV factor/solve and apply on the GPU vs the upstream
golden vectors (tests/golden/hbs_*.npz) and the CPU oracle."""
import numpy as np
import pytest

from tests._cases import hbs_from_fixture, relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu

TOL = 1e-12   # plain float64 path vs upstream float64 (relative, per array)


def _oracle_residual(S, Nbvec, x, b):
    """Worst column of ||b - A x|| / ||b||, A applied by the oracle in float64."""
    from oracle.hbs import OracleHBS
    O = OracleHBS().set_mats(S.Umats, S.Dmats, S.Vmats, list(Nbvec), fac=2)
    r = b - O.matmat(x)
    return float(np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)))


def _gpu_hbs_from_oracle(S, Nbvec, fac):
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    G = HBSMAT()
    G.set_mats(S.Umats, S.Dmats, S.Vmats, list(Nbvec), fac=fac)
    return G


@pytest.mark.parametrize("name", ["hbs_binary_k8", "hbs_quad_k8"])
def test_apply_and_standalone_ulv(golden, name):
    need_gpu()
    g = golden(name)
    S, Nbvec = hbs_from_fixture(g)
    fac = 4 if g["quad"] else 2
    G = _gpu_hbs_from_oracle(S, Nbvec, fac)
    x = g["x"]
    assert relerr(G.matmat(x), g["Ax_true"]) < TOL
    assert relerr(G.rmatmat(x), g["ATx_true"]) < TOL
    assert relerr(G @ x, g["Ax_true"]) < TOL
    assert relerr(G.T @ x, g["ATx_true"]) < TOL
    G.compute_ULV()
    assert np.array_equal(G.NNvec, g["ulv_NNvec"])
    assert relerr(G.solve(x), g["ulv_sol"]) < TOL
    assert relerr(G.solve(x, mode="T"), g["ulv_solT"]) < TOL
    # 1-D in, 1-D out
    y1 = G.solve(x[:, 0])
    assert y1.shape == (x.shape[0],)
    assert relerr(y1, g["ulv_sol"][:, 0]) < TOL


@pytest.mark.parametrize("name", ["hbs_binary_k8", "hbs_quad_k8", "hbs_c2_n512"])
def test_construct_ulv(golden, name):
    """HBSMAT(A).construct(k, True) with upstream's seeded sketches."""
    need_gpu()
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    g = golden(name)
    S, Nbvec = hbs_from_fixture(g)      # leaves the global RNG where upstream drew from
    fac = 4 if g["quad"] else 2
    import numpy.random as npr
    state = npr.get_state()
    A = _gpu_hbs_from_oracle(S, Nbvec, fac)
    npr.set_state(state)
    H = HBSMAT(A, tree=None, quad=bool(g["quad"]))
    H.set_Nbvec(list(Nbvec))
    H.construct(int(g["k"]), True)
    assert H.nSamples == int(g["nSamples"])
    assert np.array_equal(H.NNvec, g["NNvec"])
    x = g["x"]
    assert relerr(H.matmat(x), g["mm"]) < TOL
    assert relerr(H.rmatmat(x), g["rmm"]) < TOL
    assert relerr(H.solve(x), g["sol"]) < TOL
    assert relerr(H.solve(x, mode="T"), g["solT"]) < TOL
    assert relerr(H.solve(x[:, 0]), g["sol1"]) < TOL


def test_construct_factors_match(golden):
    """Stored factors equal upstream's up to column signs of U/V."""
    need_gpu()
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    g = golden("hbs_binary_k8")
    S, Nbvec = hbs_from_fixture(g)
    import numpy.random as npr
    state = npr.get_state()
    A = _gpu_hbs_from_oracle(S, Nbvec, 2)
    npr.set_state(state)
    H = HBSMAT(A, tree=None, quad=False)
    H.set_Nbvec(list(Nbvec))
    H.construct(int(g["k"]), True)
    # leaf D is basis independent; above the leaves D is written in the
    # children's U/V bases, whose column signs are the SVD's free choice
    Ds = H.Dmats
    assert relerr(Ds[0], g["Dmats_0"]) < 1e-11
    for t in range(1, len(Ds)):
        assert relerr(np.abs(Ds[t]), np.abs(g["Dmats_%d" % t])) < 1e-11
    for t, U in enumerate(H.Umats):
        Ur = g["Umats_%d" % t]
        Nb = Nbvec[t]
        n = U.shape[0] // Nb
        for b in range(Nb):
            Pg = U[b * n:(b + 1) * n] @ U[b * n:(b + 1) * n].T
            Pr = Ur[b * n:(b + 1) * n] @ Ur[b * n:(b + 1) * n].T
            if t > 0:   # rows are child skeleton coordinates (sign choice of the child SVD)
                Pg, Pr = np.abs(Pg), np.abs(Pr)
            assert np.abs(Pg - Pr).max() < 1e-11


@pytest.mark.parametrize("inner", ["dfloat", "float32"])
def test_mixed_refinement_reaches_tolerance(golden, inner):
    """ULV sweeps on the float32 units + double-float residuals reach 1e-10
    (checked with the float64 apply) and agree with the float64 solve: one
    iteration with the double-float sweep, two or more with float32."""
    need_gpu()
    g = golden("hbs_c2_n512")
    S, Nbvec = hbs_from_fixture(g)
    G = _gpu_hbs_from_oracle(S, Nbvec, 2)
    G.compute_ULV()
    x = g["x"]
    xm, iters, rr = G.solve_refined(x, tol=1e-10, maxit=10, inner=inner)
    assert rr <= 1e-10
    assert iters == 1 if inner == "dfloat" else iters >= 2
    # residual with the oracle's float64 apply, solution vs upstream's own
    assert _oracle_residual(S, Nbvec, xm, x) <= 1e-10
    assert relerr(xm, g["sol"]) < 1e-9


def test_dfloat_solve_matches_float64(golden):
    """The double-float sweep (float32 pairs, 48-bit significands) against
    the float64 sweep and the oracle's solution of the golden C2 operator:
    within 1e-12 relative (the operator's condition number times 2^-47)."""
    need_gpu()
    g = golden("hbs_c2_n512")
    S, Nbvec = hbs_from_fixture(g)
    G = _gpu_hbs_from_oracle(S, Nbvec, 2)
    G.compute_ULV()
    x = g["x"]
    xd = G.solve_dfloat(x)
    assert relerr(xd, G.solve(x)) < 1e-12
    assert relerr(xd, g["sol"]) < 1e-12
    assert _oracle_residual(S, Nbvec, xd, x) < 1e-12
    x1 = G.solve_dfloat(x[:, 0])
    assert x1.ndim == 1 and relerr(x1, g["sol1"]) < 1e-12


@pytest.mark.parametrize("k", [16, 33, 48])
def test_dfloat_solve_uneven_ranks_and_chunks(k):
    """Uneven ranks (odd pitches, the one-batch prefetch variants on small
    levels) and right-hand-side counts that split into ragged column chunks."""
    need_gpu()
    from oracle.hbs import OracleHBS
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    for N, c in ((128, 1), (256, 7), (512, 300)):
        Lv = int(np.log2(N // 64)) + 1
        U, D, V, Nbvec = random_hbs_factors(k, 64, Lv, quad=False,
                                            rng=np.random.default_rng(N + k), shift=16.0)
        H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
        H.compute_ULV()
        O = OracleHBS().set_mats(U, D, V, list(Nbvec), fac=2)
        O.compute_ULV()
        b = np.random.default_rng(k + c).standard_normal((N, c))
        xd = H.solve_dfloat(b)
        assert relerr(xd, H.solve(b)) < 1e-12, (N, k, c)
        assert relerr(xd, O.solve(b)) < 1e-12, (N, k, c)
        assert relerr(O.matmat(xd), b) < 1e-12, (N, k, c)


def test_autotuned_plans_keep_results():
    """The launch-plan autotuner moves work between CTAs only: solves after
    tuning (float64 and double-float) are bitwise equal to untuned ones."""
    need_gpu()
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    U, D, V, Nbvec = random_hbs_factors(32, 64, 4, quad=False, rng=np.random.default_rng(4),
                                        shift=16.0)
    H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
    H.compute_ULV()
    b = np.random.default_rng(5).standard_normal((H.shape[0], 16))
    x0, xd0 = H.solve(b), H.solve_dfloat(b)
    kn = H.autotune(16, reps=3)
    # one cap set per launch: 2 L - 1 steps, or fewer where the top levels
    # run as one composed operator
    assert len(kn) % 2 == 1 and 3 <= len(kn) <= 2 * len(Nbvec) - 1
    assert all(len(k) == 3 and min(k) >= 1 for k in kn)
    H.autotune(16, "dfloat", reps=3)
    assert np.array_equal(H.solve(b), x0)
    assert np.array_equal(H.solve_dfloat(b), xd0)
    # a column's result does not depend on how many columns are solved with it
    assert np.array_equal(H.solve(b[:, :7]), x0[:, :7])


def test_out_of_place_solve_matches_in_place():
    """slu_ulv_solve_into reads X and writes Y (leading dimensions wider than
    the column count; one-level and multi-level trees; modes N and T): X is
    unchanged and Y equals the in-place solve bitwise."""
    need_gpu()
    import torch
    from sslablu_gb300 import _lib as L
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    for Lv in (1, 4):
        U, D, V, Nbvec = random_hbs_factors(16, 64, Lv, quad=False,
                                            rng=np.random.default_rng(Lv), shift=16.0)
        H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
        H.compute_ULV()
        N, c = H.shape[0], 5
        Xw = torch.from_numpy(np.random.default_rng(9).standard_normal((N, 8))).cuda()
        X0 = Xw.clone()
        for trans in (0, 1):
            Yw = torch.full((N, 7), 7.0, dtype=torch.float64, device="cuda")
            L.check(L.lib().slu_ulv_solve_into(L.handle(), H._op, L.ptr(Xw), 8, L.ptr(Yw), 7, c,
                                               trans))
            B = Xw[:, :c].clone().contiguous()
            L.check(L.lib().slu_ulv_solve(L.handle(), H._op, L.ptr(B), c, c, trans))
            torch.cuda.synchronize()
            assert torch.equal(Xw, X0)
            assert torch.equal(Yw[:, :c], B) and bool((Yw[:, c:] == 7.0).all())


def test_pinned_host_solve_reads_and_writes_host_memory():
    """HBSMAT.solve on a pinned host block: the solve steps read the block and
    write the result in host memory directly; equal to the device solve."""
    need_gpu()
    import torch
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    from sslablu_gb300.synthetic import random_hbs_factors
    U, D, V, Nbvec = random_hbs_factors(16, 64, 4, quad=False, rng=np.random.default_rng(6),
                                        shift=16.0)
    H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=2)
    H.compute_ULV()
    hp = torch.from_numpy(np.random.default_rng(7).standard_normal((H.shape[0], 6))).pin_memory()
    out = torch.empty_like(hp).pin_memory()
    y = H.solve(hp, out=out)
    assert y is out and not y.is_cuda
    assert torch.equal(y, H.solve(hp.cuda()).cpu())
    assert torch.equal(H.solve(hp), y)     # output allocated when not given


def _hbs_with_perm(U, D, V, Nbvec, perm, fac=2):
    """An HBSMAT over the given factors whose tree ordering is `perm`
    (the ordering construct() takes from a slabTree's perm_leaf)."""
    from sslablu_gb300 import _lib as L
    from sslablu_gb300 import _dev as dv
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    H = HBSMAT().set_mats(U, D, V, list(Nbvec), fac=fac)
    N, Lv = H.shape[0], len(D)
    H._new_op(N, Lv, perm)
    H.perm = np.asarray(perm, dtype=np.int64)
    for t in range(Lv):
        Nb = int(Nbvec[t])
        Dd = dv.to_dev(D[t])
        n = Dd.shape[0] // Nb
        Ud = dv.to_dev(U[t]) if t < Lv - 1 else None
        Vd = dv.to_dev(V[t]) if t < Lv - 1 else None
        k = Ud.shape[1] if Ud is not None else 0
        L.check(L.lib().slu_hbs_set_level(L.handle(), H._op, t, Nb, n, k, L.ptr(Ud), L.ptr(Vd),
                                          L.ptr(Dd)))
    L.sync()
    H.compute_ULV()
    return H


@pytest.mark.parametrize("k,nl,Lv,quad,c", [(16, 64, 4, False, 3), (16, 64, 3, True, 5),
                                            (33, 64, 3, False, 70), (16, 64, 1, False, 2),
                                            (48, 64, 2, False, 1)])
def test_mode_T_solve_matches_oracle_with_permutation(k, nl, Lv, quad, c):
    """Mode-T solve (the transposed steps) vs the oracle's ULVsparse.solve
    mode T, through a random non-involutory tree ordering applied as
    HBSnew.solve does (scatter in, gather out); one-level trees, quad trees,
    uneven ranks, ragged column counts.  Mode N
    on the same operator as a check of the ordering."""
    need_gpu()
    from oracle import hbs as oh
    from sslablu_gb300.synthetic import random_hbs_factors
    U, D, V, Nbvec = random_hbs_factors(k, nl, Lv, quad=quad,
                                        rng=np.random.default_rng(k + Lv), shift=16.0)
    N = D[0].shape[0]
    rng = np.random.default_rng(N + k)
    perm = rng.permutation(N)
    while np.array_equal(perm[perm], np.arange(N)):
        perm = rng.permutation(N)
    H = _hbs_with_perm(U, D, V, Nbvec, perm, fac=4 if quad else 2)
    Ql, Wl, Uul, Rl, NNv = oh.compute_ULV(U, D, V, list(Nbvec))
    b = rng.standard_normal((N, c))
    rhs = np.zeros_like(b)
    rhs[perm] = b
    refT = oh.ulv_solve(U, D, Ql, Wl, Uul, Rl, NNv, list(Nbvec), rhs, "T")[perm]
    assert relerr(H.solve(b, mode="T"), refT) < TOL
    refN = np.zeros_like(b)
    refN[perm] = oh.ulv_solve(U, D, Ql, Wl, Uul, Rl, NNv, list(Nbvec), b[perm])
    assert relerr(H.solve(b), refN) < TOL
    # 1-D in, 1-D out
    assert relerr(H.solve(b[:, 0], mode="T"), refT[:, 0]) < TOL


def test_mode_T_float32_and_pinned_host():
    """The float32 mode-T solve (the same transposed steps on the float32
    operator copies) is within float32 accuracy of float64, and a pinned host
    block solved in mode T equals the device solve bitwise."""
    need_gpu()
    import torch
    from sslablu_gb300 import _lib as L
    from sslablu_gb300.synthetic import random_hbs_factors
    U, D, V, Nbvec = random_hbs_factors(16, 64, 4, quad=False, rng=np.random.default_rng(3),
                                        shift=16.0)
    N = D[0].shape[0]
    H = _hbs_with_perm(U, D, V, Nbvec, np.random.default_rng(4).permutation(N))
    b = np.random.default_rng(5).standard_normal((N, 6))
    x64 = H.solve(b, mode="T")
    L.check(L.lib().slu_hbs_prepare_f32(L.handle(), H._op))
    B32 = torch.from_numpy(b).float().cuda().contiguous()
    L.check(L.lib().slu_ulv_solve_f32(L.handle(), H._op, L.ptr(B32), 6, 6, 1))
    torch.cuda.synchronize()
    assert relerr(B32.double().cpu().numpy(), x64) < 1e-5
    hp = torch.from_numpy(b).pin_memory()
    y = H.solve(hp, mode="T")
    assert not y.is_cuda and y.is_pinned()
    assert torch.equal(y, H.solve(hp.cuda(), mode="T").cpu())
    assert relerr(y.numpy(), x64) < TOL


def test_solve_plan_matches_solve_and_refuses_after_refactor():
    """HBSMAT.solve_plan (one CUDA graph per solve) equals the solve through
    slu_ulv_solve_into bitwise for modes N and T, on device buffers and on
    pinned host buffers, with new data in b on every call and with tuned
    launch plans; a refactored operator's plan refuses to run."""
    need_gpu()
    import torch
    from sslablu_gb300 import _lib as L
    from sslablu_gb300.synthetic import random_hbs_factors
    U, D, V, Nbvec = random_hbs_factors(16, 64, 4, quad=False, rng=np.random.default_rng(8),
                                        shift=16.0)
    N = D[0].shape[0]
    H = _hbs_with_perm(U, D, V, Nbvec, np.random.default_rng(9).permutation(N))
    rng = np.random.default_rng(10)
    for mode in ("N", "T"):
        bd = torch.empty((N, 5), dtype=torch.float64, device="cuda")
        plan = H.solve_plan(bd, mode=mode)
        bh = torch.empty((N, 5), dtype=torch.float64).pin_memory()
        hplan = H.solve_plan(bh, mode=mode)
        assert hplan.out.is_pinned() and not hplan.out.is_cuda
        for _ in range(3):
            x = rng.standard_normal((N, 5))
            bd.copy_(torch.from_numpy(x))
            bh.copy_(torch.from_numpy(x))
            y = plan()
            torch.cuda.synchronize()
            ref = H.solve(bd, mode=mode)
            assert torch.equal(y, ref)
            assert torch.equal(hplan(), ref.cpu())
        plan.close()
        hplan.close()
    H.autotune(5)
    bd = torch.from_numpy(rng.standard_normal((N, 5))).cuda()
    plan = H.solve_plan(bd)
    y = plan().clone()
    torch.cuda.synchronize()
    assert torch.equal(y, H.solve(bd))
    H.compute_ULV()
    with pytest.raises(L.SluError):
        plan()
    plan.close()
