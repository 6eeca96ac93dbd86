"""Strong-admissibility HBS -- CPU restatement (numpy), test infrastructure.

This module is the oracle for sslablu_gb300's strong-admissibility HBS; only
tests, the smoke check and the CPU legs of the benchmarks import it.  It
restates upstream's matAssembly/HBS/HBStorch_strong.py:

  * NearField (183-246): near field of block r = its level adjacency plus r,
    blocks grouped by near-field size;
  * _factor_nf / _rowspace / _pinv_rhs (261-315): per block, a QR of the
    transposed near-field Gaussian stack S_nf^T (s x m, m = |NF| b), with a
    truncated-SVD fallback when m > s or min |R_ii| <= 1e-12 max |R_ii|;
  * _range_via_projection (318-332): U_i = leading left singular vectors of
    Y_i (I - Q Q^T);
  * compute_bases_and_E_strong (687-797): the near-field tiles
    E_ij = (I - U_i U_i^T) A_ij + U_i U_i^T A_ij (I - V_j V_j^T), recovered
    from the sketches by right-solves against the near-field stacks;
  * HBSMAT.constructHBS (1033-1107): per level (leaf first) the sketch
    reduction Y <- U^T (Y - E Om), Z <- V^T (Z - E^T Psi), Om <- V^T Om,
    Psi <- U^T Psi, children regrouped by fac; when no block has a far field
    left, the dense base B = Y pinv(Om) (compute_final_E, 897-906);
  * HBSMAT._sweep (1232-1293): down-sweep V^T, dense base, up-sweep
    U (coarse) + E (this level); mode 'T' swaps U and V and transposes E, B.

Singular vectors are unique only up to sign (and rotation inside repeated
singular values), so parity is checked on what does not depend on that
choice: the operator's apply, the projectors U U^T, the tiles E_ij and B.
Pinned against upstream's own outputs (tests/golden/hbs_strong.npz).
"""
import numpy as np
import scipy.linalg as sl

RCOND = 1e-12


def near_field(adj):
    """HBStorch_strong.py:199-246: (nf lists incl. self, [(k, ranks)])."""
    nf = [sorted(set(a) | {r}) for r, a in enumerate(adj)]
    groups = {}
    for r in range(len(adj)):
        groups.setdefault(len(nf[r]), []).append(r)
    return nf, sorted(groups.items())


def has_farfield(adj):
    """HBStorch_strong.py:849-854."""
    n = len(adj)
    return any(len(set(a) | {r}) < n for r, a in enumerate(adj))


def factor_nf(Snf):
    """HBStorch_strong.py:261-287 for one block: ('qr', Q, R) or ('svd', U, S, Vh)."""
    m, s = Snf.shape
    if m <= s:
        Q, R = np.linalg.qr(Snf.T)
        d = np.abs(np.diag(R))
        if d.min() > RCOND * max(d.max(), 0.0):
            return ("qr", Q, R)
    U, S, Vh = np.linalg.svd(Snf, full_matrices=False)
    return ("svd", U, S, Vh)


def rowspace(fac):
    if fac[0] == "qr":
        return fac[1]
    _, U, S, Vh = fac
    keep = (S > RCOND * S[0]).astype(float)
    return (Vh * keep[:, None]).T


def pinv_rhs(rhs, fac):
    """rhs @ pinv(S_nf) (HBStorch_strong.py:303-315)."""
    if fac[0] == "qr":
        _, Q, R = fac
        return sl.solve_triangular(R, (rhs @ Q).T, lower=False).T
    _, U, S, Vh = fac
    sinv = np.where(S > RCOND * S[0], 1.0 / np.where(S > 0, S, 1.0), 0.0)
    return ((rhs @ Vh.T) * sinv) @ U.T


def far_range(Yi, Q, rk):
    """Leading rk left singular vectors of Y_i (I - Q Q^T) (318-332)."""
    Yp = Yi - (Yi @ Q) @ Q.T
    U = np.linalg.svd(Yp, full_matrices=False)[0]
    return U[:, :rk]


class BlockSparse:
    """Near-field tiles: dict (i, j) -> b x b."""

    def __init__(self, tiles, n, b):
        self.tiles, self.n, self.b = tiles, n, b

    def apply(self, X, trans=False):
        """X: (n, b, c) blocks -> E X (or E^T X)."""
        out = np.zeros((self.n, self.b, X.shape[2]))
        for (i, j), T in self.tiles.items():
            if trans:
                out[j] += T.T @ X[i]
            else:
                out[i] += T @ X[j]
        return out


def bases_and_E(Om, Psi, Y, Z, adj, rk):
    """compute_bases_and_E_strong (687-797) for one level; blocks (Nb, b, s)."""
    Nb, b, s = Om.shape
    nf, groups = near_field(adj)
    rg = min(rk, b)
    U = np.zeros((Nb, b, rk))
    V = np.zeros((Nb, b, rk))
    tiles = {}
    stats = {"qr": 0, "svd": 0}
    for k, ranks in groups:                       # pass 1: Omega stacks
        for i in ranks:
            fac = factor_nf(Om[nf[i]].reshape(k * b, s))
            stats[fac[0]] += 1
            Ui = far_range(Y[i], rowspace(fac), rg)
            U[i, :, :rg] = Ui
            X1 = pinv_rhs(Y[i] - Ui @ (Ui.T @ Y[i]), fac)
            for a, j in enumerate(nf[i]):
                tiles[(i, j)] = X1[:, a * b:(a + 1) * b].copy()
    for k, ranks in groups:                       # pass 2: Psi stacks
        for j in ranks:
            fac = factor_nf(Psi[nf[j]].reshape(k * b, s))
            stats[fac[0]] += 1
            Vj = far_range(Z[j], rowspace(fac), rg)
            V[j, :, :rg] = Vj
            X2 = pinv_rhs(Z[j] - Vj @ (Vj.T @ Z[j]), fac)
            for a, i in enumerate(nf[j]):
                Ui = U[i]
                tiles[(i, j)] = tiles[(i, j)] + Ui @ (Ui.T @ X2[:, a * b:(a + 1) * b].T)
    return U, V, BlockSparse(tiles, Nb, b), stats


class StrongHBS:
    """HBStorch_strong.HBSMAT restated: construct from sketches, apply."""

    def __init__(self, perm, Nb, level_adj_list, fac=2):
        self.perm = np.asarray(perm)
        self.Nb = int(Nb)
        self.adj = level_adj_list
        self.fac = fac
        self.U, self.V, self.E = [], [], []
        self.B = None
        self.stats = {"qr": 0, "svd": 0}

    def construct(self, rk, Om, Psi, Y, Z):
        """HBSMAT.construct + constructHBS (1000-1107); Om, Psi, Y, Z are
        N x s in the caller's ordering."""
        N, s = Om.shape
        Nb, nl = self.Nb, N // self.Nb
        p = self.perm
        blk = lambda M: M[p].reshape(Nb, nl, s)
        Om, Psi, Y, Z = blk(Om), blk(Psi), blk(Y), blk(Z)
        rkm = min(rk, nl)
        L = len(self.adj)
        for lvl in range(L - 1, -1, -1):
            adj = self.adj[lvl]
            if not has_farfield(adj):
                b = Y.shape[1]
                self.B = Y.reshape(-1, s) @ np.linalg.pinv(Om.reshape(-1, s))
                return self
            U, V, E, st = bases_and_E(Om, Psi, Y, Z, adj, rkm)
            for key in st:
                self.stats[key] += st[key]
            Nb //= self.fac
            r = U.shape[2]
            T = lambda A, M: np.einsum("nbk,nbs->nks", A, M).reshape(Nb, self.fac * r, s)
            Y = T(U, Y - E.apply(Om))
            Z = T(V, Z - E.apply(Psi, True))
            Om, Psi = T(V, Om), T(U, Psi)
            self.U.append(U)
            self.V.append(V)
            self.E.append(E)
            rkm = rk
        raise ValueError("the tree's levels end before the near field covers a level")

    def apply(self, x, trans=False):
        """HBSMAT._sweep (1232-1293)."""
        x = np.asarray(x, dtype=float)
        one = x.ndim == 1
        X = x[:, None] if one else x
        c = X.shape[1]
        down, up = (self.U, self.V) if trans else (self.V, self.U)
        VV = [X[self.perm].reshape(self.Nb, -1, c)]
        for A in down:
            P = np.einsum("nbk,nbc->nkc", A, VV[-1])
            VV.append(P.reshape(A.shape[0] // self.fac, self.fac * A.shape[2], c))
        B = self.B.T if trans else self.B
        u = (B @ VV[-1].reshape(-1, c))
        for lvl in range(len(up) - 1, -1, -1):
            A = up[lvl]
            u = np.einsum("nbk,nkc->nbc", A, u.reshape(A.shape[0], A.shape[2], c))
            u = u + self.E[lvl].apply(VV[lvl], trans)
        out = np.zeros_like(X)
        out[self.perm] = u.reshape(-1, c)
        return out[:, 0] if one else out
