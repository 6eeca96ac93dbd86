"""Freeze golden vectors by running the upstream SslabLU modules themselves.

Run in a container that has the upstream tree (default /root/reference, or
$SSLABLU_REF_ROOT):

    python tests/golden/make_golden.py

Every random input is drawn from numpy's legacy global RNG after
``np.random.seed(seed)`` (a stream numpy keeps stable across versions) or from
``default_rng(seed)``, so tests can regenerate inputs instead of storing them;
the large outputs are stored.  Fixtures written (all small):

  rb_dense.npz       upstream direct_solve/test_RB.py cases: RedBlackSolver and
                     BlockTridiagonalSolver solutions
  thomas_cyclic.npz  BlockTridiagonalSolver(cyclic=True) on a periodic system
  rb_cyclic.npz      RedBlackSolver(cyclic=True) on periodic systems of 2, 4, 8 blocks
  hbs_*.npz          HBSnew.HBSMAT(...).construct(k, True) of exact random HBS
                     matrices (test/rkprop/HBSnewTest.py generator): factors,
                     matmat/rmatmat and solve (N and T) outputs
  c1_poisson64.npz   multislab.oms + stencil 2D Poisson, 8 slabs, 64-point
                     interfaces (the C1 layout at reduced size): S blocks, rhs
                     and the Thomas / red-black / functional-Thomas solutions
  c1_poisson256.npz  the same at C1's 256-point interfaces: rhs, solutions and
                     a fingerprint of the S blocks (regenerated by the oracle)
  c3_helmholtz_small.npz  multislab.oms + 3-D stencil variable-coefficient
                     Helmholtz (k = 20), 4 interfaces of 8 x 8 points: S blocks,
                     rhs, Thomas / red-black solutions
  rbhbs_kernel.npz   RedBlackSolverHBS / ThomasSolverHBS on an exponential-
                     kernel block-tridiagonal system (truncation dominated)
  rbhbs_gauss.npz    the same on a Gaussian-kernel system that rank 16
                     resolves to a ~1e-13 residual
  slab_trees.npz     slabTree on lines, rectangles (binary and quad) and a plane
                     in 3-D: perm_leaf, nleaves, nlevels, leaf boundary DOFs and
                     interface DOFs
  slab_adjacency.npz slabTree.level_adj_list of the same trees ('partial' and
                     'full' adjacency for the binary ones)
  hbs_strong.npz     HBStorch_strong.HBSMAT (strong admissibility) on planes
                     of points with partial, full and quad adjacency:
                     matmat / rmatmat, leaf near-field tile norms, nbytes
  hbstorch.npz       HBStorch.HBSMAT(tree=slabTree).construct(k, Om, Psi, Y, Z)
                     of an exact HBS matrix in a rectangle tree's ordering, with
                     the rkHBS assembler's sample count (s < 2n at the leaves):
                     factors, matmat / rmatmat, and the ULVsparse solution of
                     the compressed operator (HBStorch's own compute_ULV and
                     solve do not run upstream)
  assembler.npz      matAssembler rkHBS and dense assembly of a stMap-like
                     operator (exact HBS in tree order on a 16 x 16 grid)

Run one group with ``python tests/golden/make_golden.py <name> ...``.
"""
import contextlib
import io
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import refshim  # noqa: E402
from oracle.hbs import gen_random_hbs  # noqa: E402

QUIET = io.StringIO()


def rb_dense(ref):
    sys.path.insert(0, os.path.join(refshim.REF_ROOT, "direct_solve"))
    with contextlib.redirect_stdout(QUIET):
        import test_RB
    out = {}
    cases = [(8, 3), (2, 1), (2, 5), (4, 3), (8, 1), (8, 5), (8, 10), (16, 3), (32, 3)]
    out["cases"] = np.array(cases)
    for nS, m in cases:
        S, T, mat, rhs = test_RB.make_block_tridiagonal(nS, m, 42)
        with contextlib.redirect_stdout(QUIET):
            rb = ref.omsdirectsolve.RedBlackSolver(m)
            rb.factorize(S, T)
            x_rb = rb.solve(rhs)
        th = ref.omsdirectsolve.BlockTridiagonalSolver(m)
        th.factorize(S, T)
        x_th = th.solve(rhs)
        key = "%d_%d" % (nS, m)
        out["x_rb_" + key] = x_rb
        out["x_th_" + key] = x_th
        out["x_np_" + key] = np.linalg.solve(mat, rhs)
    np.savez_compressed(os.path.join(HERE, "rb_dense.npz"), **out)


def thomas_cyclic(ref):
    nS, m = 6, 4
    rng = np.random.default_rng(3)
    S = [(0.1 * rng.standard_normal((m, m)), 0.1 * rng.standard_normal((m, m))) for _ in range(nS)]
    T = [rng.standard_normal((m, m)) + 8 * np.eye(m) for _ in range(nS)]
    rhs = rng.standard_normal((nS * m, 2))
    th = ref.omsdirectsolve.BlockTridiagonalSolver(m, cyclic=True)
    th.factorize(S, T)
    np.savez_compressed(os.path.join(HERE, "thomas_cyclic.npz"),
                        S=np.array(S), T=np.array(T), rhs=rhs, x=th.solve(rhs))


def rb_cyclic(ref):
    """RedBlackSolver(cyclic=True) on periodic block-tridiagonal systems of
    2, 4 and 8 blocks (upstream's solve is 1-D: one column each)."""
    out = {}
    for nS, m, seed in ((2, 5, 11), (4, 6, 12), (8, 16, 13)):
        rng = np.random.default_rng(seed)
        S = [[0.2 * rng.standard_normal((m, m)), 0.2 * rng.standard_normal((m, m))]
             for _ in range(nS)]
        T = [rng.standard_normal((m, m)) + 6 * np.eye(m) for _ in range(nS)]
        rhs = rng.standard_normal(nS * m)
        with contextlib.redirect_stdout(QUIET):
            rb = ref.omsdirectsolve.RedBlackSolver(m, cyclic=True)
            rb.factorize(S, T)
            x = rb.solve(rhs)
        key = "%d_%d" % (nS, m)
        out["S_" + key] = np.array(S)
        out["T_" + key] = np.array(T)
        out["rhs_" + key] = rhs
        out["x_" + key] = x
    np.savez_compressed(os.path.join(HERE, "rb_cyclic.npz"), **out)


def hbs_case(ref, name, k, nl, L, quad, seed, sigma=None, nrhs=3, store_factors=True):
    """Exact random HBS -> upstream compression + ULV -> outputs."""
    np.random.seed(seed)
    S, Nbvec = gen_random_hbs(k, nl, L, quad, sigma=sigma)
    fac = 4 if quad else 2
    src = ref.HBSnew.HBSMAT()
    src.set_mats(S.Umats, S.Dmats, S.Vmats, list(Nbvec), fac=fac)
    with contextlib.redirect_stdout(QUIET):
        H = ref.HBSnew.HBSMAT(src, tree=None, quad=quad)
        H.set_Nbvec(list(Nbvec))
        H.construct(k, True)
    rng = np.random.default_rng(seed + 1)
    x = rng.standard_normal((S.shape[0], nrhs))
    out = dict(k=k, nl=nl, L=L, quad=int(quad), seed=seed, Nbvec=np.array(Nbvec),
               NNvec=np.array(H.NNvec), nSamples=H.nSamples,
               x=x, Ax_true=src.matmat(x), ATx_true=src.rmatmat(x),
               mm=H.matmat(x), rmm=H.rmatmat(x),
               sol=H.solve(x), solT=H.solve(x, mode="T"),
               sol1=H.solve(x[:, 0]))
    if sigma is not None:
        out["sigma"] = np.asarray(sigma)
    if store_factors:
        for nm in ["Umats", "Vmats", "Dmats", "Qlist", "Rlist", "Uulist"]:
            for i, M in enumerate(getattr(H, nm)):
                out["%s_%d" % (nm, i)] = M
        for i, M in enumerate(H.Wlist):
            if M is not None:
                out["Wlist_%d" % i] = M
        # the standalone factorisation of the generator's own factors
        Ql, Wl, Uul, Rl, NNv = ref.ULVsparse.compute_ULV(S.Umats, S.Dmats, S.Vmats, Nbvec)
        out["ulv_NNvec"] = np.array(NNv)
        out["ulv_sol"] = ref.ULVsparse.solve(S.Umats, S.Dmats, Ql, Wl, Uul, Rl, NNv, Nbvec, x.copy())
        out["ulv_solT"] = ref.ULVsparse.solve(S.Umats, S.Dmats, Ql, Wl, Uul, Rl, NNv, Nbvec,
                                               x.copy(), mode="T")
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def c1_poisson(ref, P):
    sq = P.square
    nslabs, nx, ny = 8, 17, 66
    slabs, conn, H = sq.dSlabs(nslabs)
    gb = lambda p: sq.gb(p, jax_avail=False)
    pdo = P.pdo.PDO2d(c11=P.pdo.const(1.0), c22=P.pdo.const(1.0))
    opts = P.solver.solverOptions("stencil", [nx, ny])
    O = P.oms.oms(slabs, pdo, gb, opts, conn)
    bc = lambda p: np.sin(np.pi * p[:, 0]) * np.sinh(np.pi * p[:, 1])
    import warnings
    with contextlib.redirect_stdout(QUIET), warnings.catch_warnings():
        warnings.simplefilter("ignore")
        S, rhs_list, Ntot, nc = O.construct_Stot_helper(bc, P.matAssembler.denseMatAssembler())
        Stot, rhs = O.construct_Stot_and_rhstot_linearOperator(S, rhs_list, Ntot, nc)
    n = len(S)
    Sl = np.zeros((n, nc, nc))
    Sr = np.zeros((n, nc, nc))
    for i, row in enumerate(S):
        if i > 0:
            Sl[i] = row[0]
        if i < n - 1:
            Sr[i] = row[-1]
    T = [np.eye(nc) for _ in range(n)]
    th = ref.omsdirectsolve.BlockTridiagonalSolver(nc)
    th.factorize(S, T)
    x_th = th.solve(rhs)
    # red-black needs 2^p blocks: pad with one decoupled identity block
    Sp = [[Sl[i], Sr[i]] for i in range(n)] + [[np.zeros((nc, nc)), np.zeros((nc, nc))]]
    rhs_p = np.concatenate([rhs, np.zeros(nc)])
    with contextlib.redirect_stdout(QUIET):
        rb = ref.omsdirectsolve.RedBlackSolver(nc)
        rb.factorize(Sp, [np.eye(nc)] * (n + 1))
        x_rb = rb.solve(rhs_p)
    # functional Thomas of multislab/omsdirectsolve.py
    with contextlib.redirect_stdout(QUIET):
        import multislab.omsdirectsolve as mods
    Tf = mods.build_block_tridiagonal_solver(S)
    x_f = mods.block_tridiagonal_solve(O, Tf, rhs)
    np.savez_compressed(os.path.join(HERE, "c1_poisson64.npz"),
                        Sl=Sl, Sr=Sr, rhs=rhs, x_th=x_th, x_rb=x_rb, x_f=x_f,
                        Stot_x=Stot @ x_th, nc=nc)


def c1_poisson256(ref, P):
    """The C1 layout at its full interface size: 8 slabs, 7 interfaces of
    256 points (Ny = 258; Nx = 65 per double slab, hx = hy ~ 1/256).  The S
    blocks are not stored (the oracle's closed form regenerates them; a
    fingerprint pins it): rhs, the Thomas and padded red-black solutions."""
    sq = P.square
    nslabs, nx, ny = 8, 65, 258
    slabs, conn, H = sq.dSlabs(nslabs)
    gb = lambda p: sq.gb(p, jax_avail=False)
    pdo = P.pdo.PDO2d(c11=P.pdo.const(1.0), c22=P.pdo.const(1.0))
    opts = P.solver.solverOptions("stencil", [nx, ny])
    O = P.oms.oms(slabs, pdo, gb, opts, conn)
    bc = lambda p: np.sin(np.pi * p[:, 0]) * np.sinh(np.pi * p[:, 1])
    import warnings
    with contextlib.redirect_stdout(QUIET), warnings.catch_warnings():
        warnings.simplefilter("ignore")
        S, rhs_list, Ntot, nc = O.construct_Stot_helper(bc, P.matAssembler.denseMatAssembler())
        Stot, rhs = O.construct_Stot_and_rhstot_linearOperator(S, rhs_list, Ntot, nc)
    n = len(S)
    T = [np.eye(nc) for _ in range(n)]
    th = ref.omsdirectsolve.BlockTridiagonalSolver(nc)
    th.factorize(S, T)
    x_th = th.solve(rhs)
    Sp = [[S[i][0] if i > 0 else np.zeros((nc, nc)), S[i][-1] if i < n - 1 else np.zeros((nc, nc))]
          for i in range(n)] + [[np.zeros((nc, nc)), np.zeros((nc, nc))]]
    with contextlib.redirect_stdout(QUIET):
        rb = ref.omsdirectsolve.RedBlackSolver(nc)
        rb.factorize(Sp, [np.eye(nc)] * (n + 1))
        x_rb = rb.solve(np.concatenate([rhs, np.zeros(nc)]))
    fp = np.stack([S[1][0][:8, :8], S[1][-1][:8, :8], S[1][0][-8:, -8:]])
    norms = np.array([[np.linalg.norm(S[i][0]) if i > 0 else 0.0,
                       np.linalg.norm(S[i][-1]) if i < n - 1 else 0.0] for i in range(n)])
    np.savez_compressed(os.path.join(HERE, "c1_poisson256.npz"), rhs=rhs, x_th=x_th, x_rb=x_rb,
                        Stot_x=Stot @ x_th, nc=nc, nx=nx, nslabs=nslabs, fingerprint=fp,
                        norms=norms)


def c3_helmholtz_small(ref, P):
    """The C3 operator family at a size upstream solves in seconds: 3-D
    variable-coefficient Helmholtz (Delta u + k^2 c(x) u, k = 20,
    c = 1 + 0.5 sin(2 pi x) sin(2 pi y) sin(2 pi z)) on [0,1]^3 cut into 5
    slabs (4 interfaces of 8 x 8 points: Ny = Nz = 10, Nx = 5 per double
    slab), stencil discretisation, dense S blocks.  Stores the couplings,
    rhs (Dirichlet data of a smooth field) and the Thomas / red-black
    solutions."""
    cube = P.cube
    nslabs, nx, ny, nz, kappa = 5, 5, 10, 10, 20.0
    slabs, conn, H = cube.dSlabs(nslabs)
    gb = lambda p: cube.gb(p, jax_avail=False)
    one = lambda p: np.ones_like(p[:, 0])
    cfun = lambda p: kappa ** 2 * (1.0 + 0.5 * np.sin(2 * np.pi * p[:, 0]) *
                                   np.sin(2 * np.pi * p[:, 1]) * np.sin(2 * np.pi * p[:, 2]))
    pdo = P.pdo.PDO3d(c11=one, c22=one, c33=one, c=cfun)
    opts = P.solver.solverOptions("stencil", [nx, ny, nz])
    O = P.oms.oms(slabs, pdo, gb, opts, conn)
    bc = lambda p: np.sin(np.pi * p[:, 0] + 0.3) * np.cos(2 * p[:, 1]) * np.cosh(p[:, 2])
    import warnings
    with contextlib.redirect_stdout(QUIET), warnings.catch_warnings():
        warnings.simplefilter("ignore")
        S, rhs_list, Ntot, nc = O.construct_Stot_helper(bc, P.matAssembler.denseMatAssembler())
        Stot, rhs = O.construct_Stot_and_rhstot_linearOperator(S, rhs_list, Ntot, nc)
    n = len(S)
    Sl = np.zeros((n, nc, nc))
    Sr = np.zeros((n, nc, nc))
    for i, row in enumerate(S):
        if i > 0:
            Sl[i] = row[0]
        if i < n - 1:
            Sr[i] = row[-1]
    th = ref.omsdirectsolve.BlockTridiagonalSolver(nc)
    th.factorize(S, [np.eye(nc) for _ in range(n)])
    x_th = th.solve(rhs)
    with contextlib.redirect_stdout(QUIET):
        rb = ref.omsdirectsolve.RedBlackSolver(nc)
        rb.factorize([[Sl[i], Sr[i]] for i in range(n)], [np.eye(nc)] * n)
        x_rb = rb.solve(rhs)
    np.savez_compressed(os.path.join(HERE, "c3_helmholtz_small.npz"), Sl=Sl, Sr=Sr, rhs=rhs,
                        x_th=x_th, x_rb=x_rb, Stot_x=Stot @ x_th, nc=nc, nx=nx, ny=ny, nz=nz,
                        nslabs=nslabs, kappa=kappa)


def kernel_system(m=64, nS=4):
    x = np.linspace(0, 1, m)

    def blk(shift):
        return 0.3 * np.exp(-np.abs(x[:, None] - x[None, :] - shift) * 3)
    S = []
    for i in range(nS):
        A = blk(0.2 + 0.01 * i) if i > 0 else np.zeros((m, m))
        C = blk(-0.2 - 0.01 * i) if i < nS - 1 else np.zeros((m, m))
        S.append((A, C))
    return S


def gauss_system(m=128, nS=4, c=20.0):
    x = np.linspace(0, 1, m)

    def blk(shift):
        return 0.3 * np.exp(-c * (x[:, None] - x[None, :] - shift) ** 2)
    S = []
    for i in range(nS):
        A = blk(0.2 + 0.01 * i) if i > 0 else np.zeros((m, m))
        C = blk(-0.2 - 0.01 * i) if i < nS - 1 else np.zeros((m, m))
        S.append((A, C))
    return S


def rbhbs_gauss(ref):
    """Well-resolved HBS red-black / Thomas (residual ~1e-13 at rank 16)."""
    m, nS, leaf, nlev, rk = 128, 4, 32, 3, 16
    tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=m // leaf, nlevels=nlev)
    S = gauss_system(m, nS)

    def lo(A):
        o = ref.omsdirectsolveHBS.dense_to_linop(A)
        o.tree, o.quad = tree, False
        return o
    Slo = [(lo(a), lo(c)) for a, c in S]
    b = np.random.default_rng(7).standard_normal(nS * m)
    out = dict(m=m, nS=nS, leaf=leaf, nlev=nlev, rk=rk, b=b)
    np.random.seed(11)
    with contextlib.redirect_stdout(QUIET):
        R = ref.omsdirectsolveHBS.RedBlackSolverHBS(m, rk, tree, False)
        R.factorize(Slo)
        out["x_rb"] = R.solve(b)
    np.random.seed(12)
    with contextlib.redirect_stdout(QUIET):
        T = ref.omsdirectsolveHBS.ThomasSolverHBS(m, rk)
        T.factorize(Slo)
        out["x_th"] = T.solve(b)
    np.savez_compressed(os.path.join(HERE, "rbhbs_gauss.npz"), **out)


def rbhbs(ref):
    m, nS, leaf, nlev = 64, 4, 16, 3
    tree = types.SimpleNamespace(perm_leaf=np.arange(m), nleaves=m // leaf, nlevels=nlev)
    S = kernel_system(m, nS)

    def lo(A):
        o = ref.omsdirectsolveHBS.dense_to_linop(A)
        o.tree, o.quad = tree, False
        return o
    Slo = [(lo(a), lo(c)) for a, c in S]
    b = np.random.default_rng(7).standard_normal(nS * m)
    out = dict(m=m, nS=nS, leaf=leaf, nlev=nlev, b=b)
    for rk in (16, 24):
        np.random.seed(11)
        with contextlib.redirect_stdout(QUIET):
            R = ref.omsdirectsolveHBS.RedBlackSolverHBS(m, rk, tree, False)
            R.factorize(Slo)
            out["x_rb_%d" % rk] = R.solve(b)
        np.random.seed(12)
        with contextlib.redirect_stdout(QUIET):
            T = ref.omsdirectsolveHBS.ThomasSolverHBS(m, rk)
            T.factorize(Slo)
            out["x_th_%d" % rk] = T.solve(b)
    np.savez_compressed(os.path.join(HERE, "rbhbs_kernel.npz"), **out)


SLAB_TREE_CASES = [
    ("line256", "line", 256, False, 32),
    ("rect16_bin", "rect16", 0, False, 16),
    ("rect16_quad", "rect16", 0, True, 16),
    ("plane3d_bin", "plane32", 0, False, 128),
    ("plane3d_quad", "plane32", 0, True, 64),
    ("line2d", "line2d", 128, False, 8),
    ("rect17_bin", "rect17", 0, False, 20),
    ("rect17_quad", "rect17", 0, True, 20),
]


def slab_cloud(kind, n=0):
    """Point clouds of the slab tree cases (regenerated by the tests)."""
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
    if kind == "plane32":
        g = np.stack(np.meshgrid(np.linspace(0, 1, 32), np.linspace(0, 1, 32), indexing="ij"),
                     -1).reshape(-1, 2)
        return np.concatenate([np.full((g.shape[0], 1), 0.5), g], 1)
    raise ValueError(kind)


def tree_record(t, prefix, out):
    """perm/nleaves/nlevels and the DOF lists of a built slabTree."""
    out[prefix + "perm"] = np.asarray(t.perm_leaf)
    out[prefix + "shape"] = np.array([t.nleaves, t.nlevels])
    bd, bl, idofs, il = [], [], [], []
    for b in t.get_leaves():
        node = t.get_node(b)
        for side in ("left", "down", "up", "right"):
            v = np.asarray(node.bDOFs[side]) if node.bDOFs is not None else np.zeros(0, int)
            bd.append(v)
            bl.append(len(v))
    for b in sorted(t._boxes):
        node = t.get_node(b)
        v = np.asarray(node.iDOFs) if node.iDOFs is not None else np.zeros(0, int)
        idofs.append(v)
        il.append(len(v) if node.iDOFs is not None else -1)
    out[prefix + "bdofs"] = np.concatenate(bd).astype(np.int64)
    out[prefix + "blen"] = np.array(bl)
    out[prefix + "idofs"] = np.concatenate(idofs).astype(np.int64)
    out[prefix + "ilen"] = np.array(il)


def slab_trees(ref):
    import matAssembly.HBS.slabTree as ST
    out = {}
    for name, kind, n, quad, leaf in SLAB_TREE_CASES:
        with contextlib.redirect_stdout(QUIET):
            t = ST.slabTree(slab_cloud(kind, n), quad, leaf)
        tree_record(t, name + "_", out)
    np.savez_compressed(os.path.join(HERE, "slab_trees.npz"), **out)


def adjacency_record(t):
    """level_adj_list flattened: per level, per rank, the sorted neighbours
    (counts and concatenated ranks)."""
    cnt, nbr = [], []
    for adj in t.level_adj_list:
        for a in adj:
            cnt.append(len(a))
            nbr.extend(sorted(a))
    return np.array([len(a) for a in t.level_adj_list]), np.array(cnt), np.array(nbr, dtype=np.int64)


def slab_adjacency(ref):
    """slabTree.level_adj_list of the slab tree cases, binary trees with
    'partial' and 'full' adjacency, quad trees with their own rule."""
    import matAssembly.HBS.slabTree as ST
    out = {}
    for name, kind, n, quad, leaf in SLAB_TREE_CASES:
        for adj in (("partial",) if quad else ("partial", "full")):
            with contextlib.redirect_stdout(QUIET):
                t = ST.slabTree(slab_cloud(kind, n), quad, leaf, adjacency=adj)
            lv, cnt, nbr = adjacency_record(t)
            key = "%s_%s_" % (name, adj)
            out[key + "levels"], out[key + "count"], out[key + "nbr"] = lv, cnt, nbr
    np.savez_compressed(os.path.join(HERE, "slab_adjacency.npz"), **out)


def strong_kernel(XX, shift=0.05, eps=0.02):
    """exp(-r) / (r + eps) between a plane of points and its copy shifted by
    `shift` along x: a smooth operator whose near field decays slowly, the
    shape of a slab coupling between neighbouring interfaces."""
    D = np.linalg.norm(XX[:, None, :] - XX[None, :, :] - np.array([shift, 0.0, 0.0]), axis=2)
    return np.exp(-D) / (D + eps)


STRONG_CASES = [
    # name, cloud, quad, leaf, adjacency, rank, seed
    ("plane_partial", "plane32", False, 64, "partial", 16, 31),
    ("plane_full", "plane32", False, 64, "full", 16, 32),
    ("plane_quad", "plane32", True, 64, "partial", 16, 33),
    ("rect_full", "rect16z", False, 16, "full", 6, 34),
]


def strong_cloud(kind):
    if kind == "rect16z":
        g = slab_cloud("rect16")
        return np.concatenate([np.zeros((g.shape[0], 1)), g], 1)
    return slab_cloud(kind)


def strong_samples(name, kind, quad, leaf, adj, rk, seed):
    """Inputs of a strong-admissibility case (regenerated by the tests):
    the tree, the operator, sketches with upstream's thinSlab3D sample count
    s = kmax max(2 rk, leaf) + rk + 20 (kmax 9 full, 5 partial), and x."""
    XX = strong_cloud(kind)
    A = strong_kernel(XX)
    kmax = 9 if adj == "full" else 5
    s = kmax * max(2 * rk, leaf) + rk + 20
    rng = np.random.default_rng(seed)
    N = A.shape[0]
    Om, Psi = rng.standard_normal((N, s)), rng.standard_normal((N, s))
    x = rng.standard_normal((N, 3))
    return XX, A, Om, Psi, x


def hbs_strong(ref):
    """HBStorch_strong.HBSMAT(tree=slabTree(adjacency=...)).construct(rk, Om,
    Psi, Y, Z): matmat / rmatmat of the compressed operator, the Frobenius
    norm of every leaf-level near-field tile (sorted by (row, col)), nbytes."""
    import matAssembly.HBS.slabTree as ST
    import matAssembly.HBS.HBStorch_strong as HS
    out = {}
    for name, kind, quad, leaf, adj, rk, seed in STRONG_CASES:
        XX, A, Om, Psi, x = strong_samples(name, kind, quad, leaf, adj, rk, seed)
        with contextlib.redirect_stdout(QUIET):
            tree = ST.slabTree(XX, quad, leaf, adjacency=adj)
            H = HS.HBSMAT(device="cpu", tree=tree, quad=quad)
            H.construct(rk, Om, Psi, A @ Om, A.T @ Psi, profile=False)
        E0 = H.Emats[0]
        order = np.lexsort((E0.col.numpy(), E0.row.numpy()))
        p = name + "_"
        out[p + "Ax"] = np.asarray(H.matmat(x))
        out[p + "ATx"] = np.asarray(H.rmatmat(x))
        out[p + "tile_norms"] = np.linalg.norm(E0.val.numpy()[order], axis=(1, 2))
        out[p + "tile_rc"] = np.stack([E0.row.numpy()[order], E0.col.numpy()[order]], 1)
        out[p + "nlev"] = np.array([len(H.Umats), len(H.Emats)])
        out[p + "nbytes"] = np.array(H.nbytes)
        out[p + "relerr"] = np.array(np.linalg.norm(out[p + "Ax"] - A @ x) / np.linalg.norm(A @ x))
    np.savez_compressed(os.path.join(HERE, "hbs_strong.npz"), **out)


def exact_in_tree_order(k, nl, L, seed, perm):
    """Dense A with A[perm][:, perm] equal to an exact random HBS matrix."""
    np.random.seed(seed)
    S, _ = gen_random_hbs(k, nl, L, quad=False)
    M = S.matmat(np.eye(S.shape[0]))
    A = np.zeros_like(M)
    A[np.ix_(perm, perm)] = M
    return A


def hbstorch(ref):
    import torch
    import matAssembly.HBS.slabTree as ST
    import matAssembly.HBS.HBStorch as HT
    import matAssembly.HBS.ULVsparse as US
    with contextlib.redirect_stdout(QUIET):
        tree = ST.slabTree(slab_cloud("rect16"), False, 16)
    perm = np.asarray(tree.perm_leaf)
    k, leaf = 4, 16
    A = exact_in_tree_order(k, leaf, tree.nlevels, 7, perm)
    s = max(2 * k, leaf) + k + 10
    rng = np.random.default_rng(5)
    Om = rng.standard_normal((256, s))
    Psi = rng.standard_normal((256, s))
    x = rng.standard_normal((256, 3))
    H = HT.HBSMAT(device="cpu", tree=tree, quad=False)
    with contextlib.redirect_stdout(QUIET):
        H.construct(k, Om, Psi, A @ Om, A.T @ Psi)
    out = {"perm": perm, "k": k, "s": s, "Om": Om, "Psi": Psi, "x": x,
           "Nbvec": np.array(H.Nbvec), "nSamples": H.nSamples, "nbytes": H.nbytes,
           "Ax": H.matmat(x), "ATx": H.rmatmat(x)}
    for name, lst in (("U", H.Umats), ("V", H.Vmats), ("D", H.Dmats)):
        for t, m in enumerate(lst):
            out["%s%d" % (name, t)] = np.asarray(m.detach().cpu().numpy())
    # ULV solve of the compressed operator through upstream ULVsparse (numpy)
    flat = lambda m: m.detach().cpu().numpy().reshape(-1, m.shape[2])
    Umats = [flat(u) for u in H.Umats]
    Vmats = [flat(v) for v in H.Vmats]
    Dmats = [flat(d) for d in H.Dmats]
    Nbvec = [int(d.shape[0]) for d in H.Dmats]
    with contextlib.redirect_stdout(QUIET):
        Q, W, Uu, R, NN = US.compute_ULV(Umats, Dmats, Vmats, Nbvec)
        b = A @ x
        uh = US.solve(Umats, Dmats, Q, W, Uu, R, NN, Nbvec, b[perm, :])
    u = np.zeros_like(uh)
    u[perm, :] = uh
    out["b"] = b
    out["sol"] = u
    np.savez_compressed(os.path.join(HERE, "hbstorch.npz"), **out)


def assembler(ref):
    import scipy.sparse.linalg as sla
    import matAssembly.matAssembler as MA
    import matAssembly.HBS.slabTree as ST
    XX = slab_cloud("rect16")
    with contextlib.redirect_stdout(QUIET):
        tree = ST.slabTree(XX, False, 8)
    perm = np.asarray(tree.perm_leaf)
    A = exact_in_tree_order(3, 8, tree.nlevels, 9, perm)
    lin = sla.aslinearoperator(A)
    stmap = types.SimpleNamespace(A=lin, XXI=XX)
    np.random.seed(11)
    with contextlib.redirect_stdout(QUIET):
        H = MA.rkHMatAssembler(8, 3).assemble(stmap)
    x = np.random.default_rng(12).standard_normal((256, 2))
    with contextlib.redirect_stdout(QUIET):
        M = MA.denseMatAssembler().assemble(stmap)
    np.savez_compressed(os.path.join(HERE, "assembler.npz"), perm=perm, x=x, Ax=H.matmat(x),
                        ATx=H.rmatmat(x), nSamples=H.nSamples, nbytes=H.nbytes,
                        dense_ok=np.array(np.array_equal(M, A)))


def main():
    only = sys.argv[1:]
    if only:
        refshim.install()
        with contextlib.redirect_stdout(QUIET):
            P = refshim.import_pipeline()
        for name in only:
            globals()[name](P)
        return
    ref = refshim.import_hot_path()
    P = refshim.import_pipeline()
    rb_dense(ref)
    thomas_cyclic(ref)
    rb_cyclic(ref)
    hbs_case(ref, "hbs_binary_k8", 8, 16, 4, False, 101)
    hbs_case(ref, "hbs_quad_k8", 8, 8, 3, True, 102)
    sig = 10.0 ** (-12.0 * np.arange(32) / 31.0)
    hbs_case(ref, "hbs_c2_n512", 32, 64, 4, False, 103, sigma=sig, nrhs=4, store_factors=False)
    c1_poisson(ref, P)
    c1_poisson256(ref, P)
    c3_helmholtz_small(ref, P)
    rbhbs(ref)
    rbhbs_gauss(ref)
    slab_trees(ref)
    slab_adjacency(ref)
    hbs_strong(ref)
    hbstorch(ref)
    assembler(ref)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
