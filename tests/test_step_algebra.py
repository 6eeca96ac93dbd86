"""The algebra of the composed step operators, on the CPU with the oracle.

The device solve runs ULVsparse.solve as one block product per tree step
with operators composed at factor time (sweep_ops.cu).  These tests restate
that composition in numpy -- mode N: Qt = Q^T, [G; H] from W, R, Uu, U, D;
mode T: the same steps transposed, in reverse order, with the columns of
[G; H]^T reordered to the children's [v; y] ranges (the index map of
transpose_children_kernel) -- and check both against the oracle's
ULVsparse.solve on random exact HBS operators, binary and quad trees; and
the top of the chain composed into one operator (hbs_make_sweep's top step)."""
import numpy as np
import pytest

from oracle import hbs as oh


def _compose(U, D, Qs, Ws, Uus, Rs, Nbvec):
    L = len(D)
    Sw = []
    for t in range(L - 1):
        Nb, n, k = Nbvec[t], D[t].shape[1], U[t].shape[1]
        nu = n - k
        blocks = []
        for b in range(Nb):
            R = Rs[t][b * nu:(b + 1) * nu]
            M = np.linalg.solve(R[:, :nu], np.hstack([np.eye(nu), -Uus[t][b * nu:(b + 1) * nu],
                                                      -R[:, nu:]]))
            W = Ws[t][b * n:(b + 1) * n]
            G = W[:, :nu] @ M
            G[:, nu + k:] += W[:, nu:]
            if t == 0:
                blocks.append(G)
            else:
                Hm = D[t][b * n:(b + 1) * n] @ G
                Hm[:, nu:nu + k] += U[t][b * n:(b + 1) * n]
                blocks.append(np.vstack([G, Hm]))
        Sw.append(np.stack(blocks))
    G = np.linalg.solve(Rs[L - 1], Qs[L - 1].T)
    root = G if L == 1 else np.vstack([G, D[L - 1] @ G])
    return Sw, root


def _children_order(n, kc):
    """Row of [G; H] feeding column j of [G; H]^T: child c's [v; y] range."""
    sig = []
    for c in range(n // kc):
        sig += [n + c * kc + i for i in range(kc)] + [c * kc + i for i in range(kc)]
    return sig


def _solve_N(U, D, Qs, Nbvec, Sw, root, b):
    L = len(D)
    x, ru = b, []
    for t in range(L - 1):
        Nb, n, k = Nbvec[t], D[t].shape[1], U[t].shape[1]
        z = np.einsum("bij,bjc->bic", Qs[t].reshape(Nb, n, n).transpose(0, 2, 1),
                      x.reshape(Nb, n, -1))
        ru.append(z[:, :n - k])
        x = z[:, n - k:].reshape(-1, b.shape[1])
    yv = root @ x
    if L == 1:
        return yv
    n = D[L - 1].shape[1]
    y, v = yv[:n], yv[n:]
    for t in range(L - 2, -1, -1):
        Nb, k = Nbvec[t], U[t].shape[1]
        z = np.concatenate([ru[t], v.reshape(Nb, k, -1), y.reshape(Nb, k, -1)], axis=1)
        out = np.einsum("bij,bjc->bic", Sw[t], z)
        n = D[t].shape[1]
        y = out[:, :n].reshape(-1, b.shape[1])
        v = out[:, n:].reshape(-1, b.shape[1]) if t > 0 else None
    return y


def _solve_T(U, D, Qs, Nbvec, Sw, root, b):
    L = len(D)
    if L == 1:
        return root.T @ b
    z, ru = b, []
    for t in range(L - 1):   # backward^T, leaf -> root-1
        Nb, n, k = Nbvec[t], D[t].shape[1], U[t].shape[1]
        S = Sw[t]
        if t > 0:
            S = S[:, _children_order(n, U[t - 1].shape[1]), :]
        out = np.einsum("bij,bjc->bic", S.transpose(0, 2, 1), z.reshape(Nb, S.shape[1], -1))
        ru.append(out[:, :n - k])
        z = out[:, n - k:].reshape(-1, b.shape[1])   # [v'; y'] per block, child after child
    n = D[L - 1].shape[1]
    x = root[_children_order(n, U[L - 2].shape[1])].T @ z
    for t in range(L - 2, -1, -1):   # forward^T, root-1 -> leaf
        Nb, n, k = Nbvec[t], D[t].shape[1], U[t].shape[1]
        zz = np.concatenate([ru[t], x.reshape(Nb, k, -1)], axis=1)
        x = np.einsum("bij,bjc->bic", Qs[t].reshape(Nb, n, n), zz).reshape(-1, b.shape[1])
    return x


def _chain(U, D, Qs, Nbvec, Sw, root, x, t0):
    """Forward steps t0 .. L-2, root, backward steps L-2 .. t0 on the level-t0
    vector x: returns [y_t0; v_t0] (t0 >= 1), or the solution (t0 = 0)."""
    L = len(D)
    ru = {}
    for t in range(t0, L - 1):
        Nb, n, k = Nbvec[t], D[t].shape[1], U[t].shape[1]
        z = np.einsum("bij,bjc->bic", Qs[t].reshape(Nb, n, n).transpose(0, 2, 1),
                      x.reshape(Nb, n, -1))
        ru[t] = z[:, :n - k]
        x = z[:, n - k:].reshape(-1, z.shape[2])
    yv = root @ x
    n = D[L - 1].shape[1]
    y, v = yv[:n], yv[n:]
    for t in range(L - 2, t0 - 1, -1):
        Nb, k = Nbvec[t], U[t].shape[1]
        z = np.concatenate([ru[t], v.reshape(Nb, k, -1), y.reshape(Nb, k, -1)], axis=1)
        out = np.einsum("bij,bjc->bic", Sw[t], z)
        n = D[t].shape[1]
        y = out[:, :n].reshape(-1, z.shape[2])
        v = out[:, n:].reshape(-1, z.shape[2]) if t > 0 else None
    return y if t0 == 0 else np.vstack([y, v])


@pytest.mark.parametrize("k,nl,L,quad", [(8, 16, 5, False), (8, 16, 4, True), (16, 32, 4, False)])
def test_top_operator_matches_ulv_solve(k, nl, L, quad):
    """The top of the chain as one operator (levels t0 .. root, composed by
    running those steps on the identity) reproduces ULVsparse.solve when the
    solve runs forward steps below t0, the top product, backward steps below
    t0."""
    rng = np.random.default_rng(k + nl + L)
    np.random.seed(k * 3 + L)
    S, Nbvec = oh.gen_random_hbs(k, nl, L, quad=quad)
    U, D, V = S.Umats, S.Dmats, S.Vmats
    Qs, Ws, Uus, Rs, NN = oh.compute_ULV(U, D, V, Nbvec)
    Nbvec = list(Nbvec)
    Sw, root = _compose(U, D, Qs, Ws, Uus, Rs, Nbvec)
    b = rng.standard_normal((D[0].shape[0], 2))
    ref = oh.ulv_solve(U, D, Qs, Ws, Uus, Rs, NN, Nbvec, b.copy())
    for t0 in range(1, L - 1):
        M = Nbvec[t0] * D[t0].shape[1]
        Top = _chain(U, D, Qs, Nbvec, Sw, root, np.eye(M), t0)      # 2M x M
        x, ru = b, []
        for t in range(t0):
            Nb, n, kk = Nbvec[t], D[t].shape[1], U[t].shape[1]
            z = np.einsum("bij,bjc->bic", Qs[t].reshape(Nb, n, n).transpose(0, 2, 1),
                          x.reshape(Nb, n, -1))
            ru.append(z[:, :n - kk])
            x = z[:, n - kk:].reshape(-1, b.shape[1])
        yv = Top @ x
        y, v = yv[:M], yv[M:]
        for t in range(t0 - 1, -1, -1):
            Nb, kk = Nbvec[t], U[t].shape[1]
            z = np.concatenate([ru[t], v.reshape(Nb, kk, -1), y.reshape(Nb, kk, -1)], axis=1)
            out = np.einsum("bij,bjc->bic", Sw[t], z)
            n = D[t].shape[1]
            y = out[:, :n].reshape(-1, b.shape[1])
            v = out[:, n:].reshape(-1, b.shape[1]) if t > 0 else None
        assert np.linalg.norm(y - ref) <= 1e-11 * np.linalg.norm(ref), t0


@pytest.mark.parametrize("k,nl,L,quad", [(8, 16, 4, False), (8, 16, 3, True), (5, 16, 3, False),
                                         (8, 16, 1, False), (8, 8, 3, False), (16, 32, 2, False)])
def test_composed_steps_match_ulv_solve(k, nl, L, quad):
    rng = np.random.default_rng(k * 100 + nl + L)
    np.random.seed(k + L)
    S, Nbvec = oh.gen_random_hbs(k, nl, L, quad=quad)
    U, D, V = S.Umats, S.Dmats, S.Vmats
    Qs, Ws, Uus, Rs, NN = oh.compute_ULV(U, D, V, Nbvec)
    b = rng.standard_normal((D[0].shape[0], 3))
    Sw, root = _compose(U, D, Qs, Ws, Uus, Rs, list(Nbvec))
    refN = oh.ulv_solve(U, D, Qs, Ws, Uus, Rs, NN, Nbvec, b.copy())
    refT = oh.ulv_solve(U, D, Qs, Ws, Uus, Rs, NN, Nbvec, b.copy(), "T")
    xN = _solve_N(U, D, Qs, list(Nbvec), Sw, root, b)
    xT = _solve_T(U, D, Qs, list(Nbvec), Sw, root, b)
    assert np.linalg.norm(xN - refN) <= 1e-11 * np.linalg.norm(refN)
    assert np.linalg.norm(xT - refT) <= 1e-11 * np.linalg.norm(refT)
