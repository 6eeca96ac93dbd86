"""Oracle (test infrastructure only): HBS compression, HBS apply, ULV factor/solve.

Vectorised numpy restatement of
  * matAssembly/HBS/HBSnew.py   (compute_UV 20-28, block_solve_r 11-19,
    block_mult 32-47, construct_D 48-62, HBSMAT.constructHBS_ULV 211-295,
    matmat 308-328, rmatmat 330-350, solve 393-416)
  * matAssembly/HBS/ULVsparse.py (block_qr 18-25, block_Q_and_R 51-61,
    compute_QRW_sparse 64-100, sparse_block_mult 101-156,
    block_diag_add 158-183, apply_sparse_block 185-203, block_solve 213-226,
    compute_ULV 231-293, solve 295-358)

Upstream loops over blocks; here each level is one stacked (Nb, n, c) array
and numpy's stacked LAPACK calls (qr/svd/pinv/solve) run the same routines per
block.  Stored layout is the upstream "reduced block-diagonal" one: a level
with Nb blocks of n rows is an (Nb*n, c) row-major array.

Parity pinned against tests/golden/*.npz, produced by the upstream code.
Never imported by the product package.
"""
import numpy as np


# --------------------------------------------------------------------------
# stacked-block helpers
# --------------------------------------------------------------------------
def bv(X, Nb):
    """(Nb*n, c) -> (Nb, n, c) view."""
    return X.reshape(Nb, X.shape[0] // Nb, X.shape[1])


def ub(B):
    """(Nb, n, c) -> (Nb*n, c)."""
    return B.reshape(B.shape[0] * B.shape[1], B.shape[2])


def tr(B):
    return np.swapaxes(B, -1, -2)


def block_mult(A, B, Nb, mode="N"):
    """HBSnew.py:32-47 (== ULVsparse.apply_sparse_block, ULVsparse.py:185-203)."""
    if mode == "N":
        return ub(bv(A, Nb) @ bv(B, Nb))
    if mode == "T":
        return ub(tr(bv(A, Nb)) @ bv(B, Nb))
    raise ValueError("mode not recognized")


def sparse_block_mult(A, B, NbA, NbB, mode="N"):
    """ULVsparse.py:101-156, for the block-count ratios upstream uses.

    N, NbB <  NbA: C_{i*f+j} = A_{i*f+j} @ B_i[j*ka:(j+1)*ka]       (121-136)
    N, NbB == NbA: C_i = A_i @ B_i
    T, NbB == NbA: C_i = A_i^T @ B_i                               (137-150)
    """
    if mode == "N":
        if NbB == NbA:
            return block_mult(A, B, NbA, "N")
        if NbB < NbA:
            f = NbA // NbB
            Ab = bv(A, NbA)
            ka = Ab.shape[2]
            Bs = B.reshape(NbB * f, ka, B.shape[1])
            return ub(Ab @ Bs)
        raise NotImplementedError("NbB > NbA not used on this path")
    if mode == "T":
        if NbB != NbA:
            raise NotImplementedError("only equal block counts used on this path")
        return block_mult(A, B, NbA, "T")
    raise ValueError("mode not recognized")


def block_diag_add(A, B, NbA, NbB):
    """ULVsparse.py:158-183: add child blocks B (NbB blocks of k x k) onto the
    diagonal sub-blocks of the parent blocks A (NbA blocks of f*k x f*k)."""
    kA, kB = A.shape[1], B.shape[1]
    f = kA // kB
    if kA < kB:
        raise ValueError("put smol frist")
    C = A
    Cb = C.reshape(NbA, f, kB, f, kB)
    Bb = B.reshape(NbA, f, kB, kB)
    for j in range(f):
        Cb[:, j, :, j, :] += Bb[:, j]
    return C


def block_solve(A, B, Nb, mode="N"):
    """ULVsparse.py:213-226 (np.linalg.solve per block)."""
    Ab = bv(A, Nb)
    if mode == "T":
        Ab = tr(Ab)
    elif mode != "N":
        raise ValueError("Mode not recognized")
    return ub(np.linalg.solve(Ab, bv(B, Nb)))


# --------------------------------------------------------------------------
# compression kernels
# --------------------------------------------------------------------------
def compute_UV(Om, Y, rk, Nb, after_n=False):
    """HBSnew.py:20-28: complete QR of each Om block^T, project Y onto the
    trailing n columns of Q, keep the rk leading left singular vectors.
    ``after_n`` projects on every column after the first n instead
    (HBStorch.py:73-82)."""
    Omb = bv(Om, Nb)                 # (Nb, n, s)
    n = Omb.shape[1]
    Q = np.linalg.qr(tr(Omb), mode="complete")[0]   # (Nb, s, s)
    M = bv(Y, Nb) @ (Q[:, :, n:] if after_n else Q[:, :, -n:])
    U = np.linalg.svd(M)[0][:, :, :rk]
    return ub(np.ascontiguousarray(U))


def construct_D(U, V, Y, Z, Om, Psi, Nb):
    """HBSnew.py:48-62."""
    Ub, Vb = bv(U, Nb), bv(V, Nb)
    Yb, Zb = bv(Y, Nb), bv(Z, Nb)
    t1 = (Yb - Ub @ (tr(Ub) @ Yb)) @ np.linalg.pinv(bv(Om, Nb))
    inner = (Zb - Vb @ (tr(Vb) @ Zb)) @ np.linalg.pinv(bv(Psi, Nb))
    t2 = Ub @ (tr(Ub) @ tr(inner))
    return ub(t1 + t2)


def block_solve_r(A, B, Nb):
    """HBSnew.py:11-19: A_blk @ pinv(B_blk, rcond=1e-15)."""
    return ub(bv(A, Nb) @ np.linalg.pinv(bv(B, Nb), rcond=1e-15))


# --------------------------------------------------------------------------
# ULV pieces
# --------------------------------------------------------------------------
def block_qr(V, Nb):
    """ULVsparse.py:18-25: trailing n-k columns of the complete QR of V_blk."""
    Vb = bv(V, Nb)
    k = Vb.shape[2]
    Q = np.linalg.qr(Vb, mode="complete")[0]
    return ub(np.ascontiguousarray(Q[:, :, k:]))


def compute_QRW_sparse(Dtot, Vtot, Nb):
    """ULVsparse.py:64-100 -> Q, W12, Ru, R22, NN."""
    if Nb == 1:
        Q, Ru = np.linalg.qr(Dtot, mode="reduced")
        return Q, None, Ru, 0, Ru.shape[1]
    k = Vtot.shape[1]
    n = Vtot.shape[0] // Nb
    NN = (n - k) * Nb
    if n > k:
        W1 = block_qr(Vtot, Nb)
    else:
        W1 = np.zeros((Nb * n, 0))
    W12 = np.append(W1, Vtot, axis=1)
    # block_Q_and_R, ULVsparse.py:51-61
    Qb, Rb = np.linalg.qr(bv(Dtot, Nb) @ bv(W12, Nb))
    Ru = ub(np.ascontiguousarray(Rb[:, : n - k, :]))
    R22 = ub(np.ascontiguousarray(Rb[:, n - k:, n - k:]))
    return ub(Qb), W12, Ru, R22, NN


def compute_ULV(Umats, Dmats, Vmats, Nbvec):
    """ULVsparse.py:231-293 (standalone factorisation of given HBS factors)."""
    NNvec = [0]
    Qlist, Wlist, Uulist, Rlist = [], [], [], []
    Uhat = R22 = None
    for i in range(len(Dmats)):
        if i == 0:
            Q, W, Ru, R22, NN = compute_QRW_sparse(Dmats[0], Vmats[0], Nbvec[0])
        else:
            Rhat = sparse_block_mult(Uhat, Dmats[i], Nbvec[i - 1], Nbvec[i])
            Rhat = block_diag_add(Rhat, R22, Nbvec[i], Nbvec[i - 1])
            Vi = Vmats[i] if i < len(Vmats) else None
            Q, W, Ru, R22, NN = compute_QRW_sparse(Rhat, Vi, Nbvec[i])
        NNvec.append(NNvec[-1] + NN)
        if i < len(Umats):
            n = Umats[i].shape[0] // Nbvec[i]
            k = Umats[i].shape[1]
            if i > 0:
                Uhat = sparse_block_mult(Uhat, Umats[i], Nbvec[i - 1], Nbvec[i])
            else:
                Uhat = Umats[0]
            Uulist.append(sparse_block_mult(Q[:, : n - k], Uhat, Nbvec[i], Nbvec[i], "T"))
            Uhat = sparse_block_mult(Q[:, n - k:], Uhat, Nbvec[i], Nbvec[i], "T")
        Qlist.append(Q)
        Wlist.append(W)
        Rlist.append(Ru)
    return Qlist, Wlist, Uulist, Rlist, np.array(NNvec, dtype=np.int64)


def ulv_solve(Umats, Dmats, Qlist, Wlist, Uulist, Rlist, NNvec, Nbvec, rhs, mode="N"):
    """ULVsparse.py:295-358 (block-ordered right-hand side, no permutation)."""
    L = len(Dmats)
    r = rhs[:, None].copy() if rhs.ndim == 1 else rhs.copy()
    NN = [int(x) for x in NNvec]
    if mode == "N":
        # forward sweep, 302-310
        for i in range(L):
            Nb = Nbvec[i]
            t = tr(bv(Qlist[i], Nb)) @ bv(r[NN[i]:], Nb)
            if i < L - 1:
                n = Umats[i].shape[0] // Nb
                k = Umats[i].shape[1]
                r[NN[i]:NN[i + 1]] = ub(t[:, : n - k])
                r[NN[i + 1]:] = ub(t[:, n - k:])
            else:
                r[NN[i]:NN[i + 1]] = ub(t)
        # root solve and backward sweep, 312-327
        y = np.zeros(r.shape)
        y[NN[L - 1]:] = block_solve(Rlist[L - 1], r[NN[L - 1]:], Nbvec[L - 1])
        v = block_mult(Dmats[L - 1], y[NN[L - 1]:], Nbvec[L - 1])
        for i in range(L - 2, -1, -1):
            Nb = Nbvec[i]
            n = Umats[i].shape[0] // Nb
            k = Umats[i].shape[1]
            R = bv(Rlist[i], Nb)
            rhs0 = (r[NN[i]:NN[i + 1]] - block_mult(Uulist[i], v, Nb)
                    - ub(R[:, :, n - k:] @ bv(y[NN[i + 1]:], Nb)))
            y[NN[i]:NN[i + 1]] = ub(np.linalg.solve(R[:, :, : n - k], bv(rhs0, Nb)))
            Wb = bv(Wlist[i], Nb)
            y[NN[i]:] = ub(Wb[:, :, : n - k] @ bv(y[NN[i]:NN[i + 1]], Nb)
                           + Wb[:, :, n - k:] @ bv(y[NN[i + 1]:], Nb))
            v = block_mult(Umats[i], v, Nb) + block_mult(Dmats[i], y[NN[i]:], Nb)
    elif mode == "T":
        # 328-353
        y = r.copy()
        v = np.zeros((Umats[0].shape[0], r.shape[1]))
        for i in range(L - 1):
            Nb = Nbvec[i]
            n = Umats[i].shape[0] // Nb
            k = Umats[i].shape[1]
            Wb = bv(Wlist[i], Nb)
            rb = bv(r, Nb)
            top = ub(tr(Wb[:, :, : n - k]) @ rb)
            bot = ub(tr(Wb[:, :, n - k:]) @ rb)
            R = bv(Rlist[i], Nb)
            yi = ub(np.linalg.solve(tr(R[:, :, : n - k]), bv(top, Nb)))
            y[NN[i]:NN[i + 1]] = yi
            v = block_mult(Uulist[i], yi, Nb, "T") + block_mult(Umats[i], v, Nb, "T")
            r = (bot - ub(tr(R[:, :, n - k:]) @ bv(yi, Nb))
                 - block_mult(Dmats[i + 1], v, Nbvec[i + 1], "T"))
        y[NN[L - 1]:] = block_solve(Rlist[L - 1], r, 1, "T")
        for i in range(L - 1, -1, -1):
            Nb = Nbvec[i]
            Qb = bv(Qlist[i], Nb)
            if i < L - 1:
                n = Umats[i].shape[0] // Nb
                k = Umats[i].shape[1]
                y[NN[i]:] = ub(Qb[:, :, : n - k] @ bv(y[NN[i]:NN[i + 1]], Nb)
                               + Qb[:, :, n - k:] @ bv(y[NN[i + 1]:], Nb))
            else:
                y[NN[i]:NN[i + 1]] = Qb[0] @ y[NN[i]:NN[i + 1]]
    else:
        raise NotImplementedError("mode not recognized")
    if rhs.ndim == 1:
        y = y.flatten()
    return y


# --------------------------------------------------------------------------
# HBS operator
# --------------------------------------------------------------------------
def samples_for(rk, nl, fac):
    """HBSnew.py:213-216."""
    return 6 * rk + 4 * nl + 5 if fac == 4 else 4 * rk + 2 * nl + 5


class OracleHBS:
    """State of upstream HBSnew.HBSMAT after construct(rk, compute_ULV=True).

    Built from an operator ``A`` (``.shape``, ``.matmat``, ``.rmatmat``) and the
    tree data (perm, Nb at the leaves, number of levels L, fac 2|4).
    """

    def __init__(self, A=None, perm=None, Nb=None, L=None, fac=2):
        self.A = A
        self.fac = fac
        self.Umats, self.Vmats, self.Dmats = [], [], []
        self.Qlist, self.Wlist, self.Rlist, self.Uulist = [], [], [], []
        self.Nbvec = []
        if A is not None:
            self.shape = tuple(A.shape)
            self.perm = np.arange(A.shape[0]) if perm is None else np.asarray(perm)
            self.Nb, self.L = Nb, L
            self.nl = A.shape[0] // Nb

    @classmethod
    def from_tree(cls, A, tree, quad):
        """HBSnew.py:82-118."""
        return cls(A, tree.perm_leaf, tree.nleaves, tree.nlevels, 4 if quad else 2)

    def set_mats(self, Umats, Dmats, Vmats, Nbvec, fac=4):
        """HBSnew.py:125-133."""
        self.Umats, self.Dmats, self.Vmats = Umats, Dmats, Vmats
        self.perm = np.arange(Dmats[0].shape[0])
        self.fac = fac
        self.Nb = Nbvec[0]
        self.Nbvec = list(Nbvec)
        self.shape = (Dmats[0].shape[0], Dmats[0].shape[0])
        return self

    # -- compression + interleaved ULV, HBSnew.py:211-295 ---------------------
    def draw_sketches(self, rk):
        """HBSnew.py:213-219: draws from the global numpy RNG, Om then Psi."""
        s = samples_for(rk, self.nl, self.fac)
        Om = np.random.standard_normal(size=(self.shape[1], s))
        Psi = np.random.standard_normal(size=(self.shape[0], s))
        return Om, Psi

    def construct(self, rk, Om=None, Psi=None):
        if Om is None:
            Om, Psi = self.draw_sketches(rk)
        s = Om.shape[1]
        self.nSamples = s
        perm = self.perm
        Omp = np.zeros(Om.shape)
        Omp[perm] = Om
        Psip = np.zeros(Psi.shape)
        Psip[perm] = Psi
        Y = np.asarray(self.A.matmat(Omp))[perm]
        Z = np.asarray(self.A.rmatmat(Psip))[perm]
        self.compress_from_sketches(rk, Om, Psi, Y, Z)
        return self

    def compress_from_sketches(self, rk, Om, Psi, Y, Z, null_after_n=False):
        """Levels leaf -> root (HBSnew.py:234-294), sketches in tree order;
        ``null_after_n`` selects HBStorch's null-space rule (HBStorch.py:73-82,
        its level loop 184-229 being the same)."""
        fac, L, nl = self.fac, self.L, self.nl
        Nb = self.Nb
        self.Nbvec = []
        NNvec = [0]
        Y = Y.copy()
        Z = Z.copy()
        Om_l, Psi_l, Y_l, Z_l = Om, Psi, Y, Z
        U_l = V_l = D_l = None
        Uhat = R22 = None
        for lvl in range(L - 1, -1, -1):
            if lvl == L - 1:
                rkm = min(rk, nl)
            else:
                Y_l = Y_l - block_mult(D_l, Om_l, Nb)
                Y_l = block_mult(U_l, Y_l, Nb, "T")
                Z_l = Z_l - block_mult(D_l, Psi_l, Nb, "T")
                Z_l = block_mult(V_l, Z_l, Nb, "T")
                Om_l = block_mult(V_l, Om_l, Nb, "T")
                Psi_l = block_mult(U_l, Psi_l, Nb, "T")
                Nb = Nb // fac
                rkm = min(rk, nl * fac ** (L - 1 - lvl))
            self.Nbvec.append(Nb)
            if lvl > 0:
                U_l = compute_UV(Om_l, Y_l, rkm, Nb, null_after_n)
                V_l = compute_UV(Psi_l, Z_l, rkm, Nb, null_after_n)
                D_l = construct_D(U_l, V_l, Y_l, Z_l, Om_l, Psi_l, Nb)
                self.Umats.append(U_l)
                self.Vmats.append(V_l)
            else:
                D_l = block_solve_r(Y_l, Om_l, Nb)
                U_l = np.identity(D_l.shape[0])
            self.Dmats.append(D_l)
            if lvl == L - 1:
                Rhat = D_l
            else:
                Rhat = sparse_block_mult(Uhat, D_l, self.Nbvec[-2], self.Nbvec[-1])
                Rhat = block_diag_add(Rhat, R22, self.Nbvec[-1], self.Nbvec[-2])
            Q, W, Ru, R22, NN = compute_QRW_sparse(Rhat, V_l, self.Nbvec[-1])
            self.Qlist.append(Q)
            self.Wlist.append(W)
            self.Rlist.append(Ru)
            NNvec.append(NNvec[-1] + NN)
            if lvl == L - 1:
                Uhat = U_l
            else:
                Uhat = sparse_block_mult(Uhat, U_l, self.Nbvec[-2], self.Nbvec[-1])
            Nbl = self.Nbvec[-1]
            self.Uulist.append(sparse_block_mult(Q[:, :-rk], Uhat, Nbl, Nbl, "T"))
            Uhat = sparse_block_mult(Q[:, -rk:], Uhat, Nbl, Nbl, "T")
        self.NNvec = np.array(NNvec, dtype=np.int64)
        return self

    def compute_ULV(self):
        """HBSnew.py:390-391."""
        (self.Qlist, self.Wlist, self.Uulist, self.Rlist,
         self.NNvec) = compute_ULV(self.Umats, self.Dmats, self.Vmats, self.Nbvec)

    # -- apply, HBSnew.py:308-350 -------------------------------------------
    def _apply(self, v, trans):
        one = v.ndim == 1
        vp = v[self.perm, None] if one else v[self.perm, :]
        first, second = (self.Umats, self.Vmats) if trans else (self.Vmats, self.Umats)
        dm = "T" if trans else "N"
        Nb = self.Nb
        VV = [vp]
        for lvl in range(len(first)):
            VV.append(block_mult(first[lvl], VV[lvl], Nb, "T"))
            Nb //= self.fac
        up = block_mult(self.Dmats[-1], VV[-1], Nb, dm)
        for lvl in range(len(second) - 1, -1, -1):
            up = (block_mult(second[lvl], up, self.fac * Nb)
                  + block_mult(self.Dmats[lvl], VV[lvl], self.fac * Nb, dm))
            Nb *= self.fac
        u = np.zeros(up.shape)
        u[self.perm] = up
        return u.flatten() if one else u

    def matmat(self, v):
        return self._apply(v, False)

    def rmatmat(self, v):
        return self._apply(v, True)

    matvec = matmat
    rmatvec = rmatmat

    def __matmul__(self, v):
        return self._apply(v, getattr(self, "mode", "N") == "T")

    # -- solve, HBSnew.py:393-416 -------------------------------------------
    def solve(self, b, mode="N"):
        one = b.ndim == 1
        args = (self.Umats, self.Dmats, self.Qlist, self.Wlist, self.Uulist,
                self.Rlist, self.NNvec, self.Nbvec)
        if mode == "N":
            bp = b[self.perm, None] if one else b[self.perm, :]
            uh = ulv_solve(*args, bp.copy())
            u = np.zeros(uh.shape)
            u[self.perm] = uh
        elif mode == "T":
            # upstream scatters the input and gathers the output (404-411)
            rhs = np.zeros((b.shape[0], 1) if one else b.shape)
            rhs[self.perm] = b[:, None] if one else b
            uh = ulv_solve(*args, rhs, mode="T")
            u = uh[self.perm]
        else:
            raise NotImplementedError("mode not recognized")
        return u.flatten() if one else u


def gen_random_hbs(k, nl, L, quad=True, sigma=None, rng=None):
    """Exact synthetic HBS in the layout of test/rkprop/HBSnewTest.py:15-73.

    Each U/V block is an orthonormalised Gaussian; D is projected off the U/V
    ranges on all but the root level.  ``sigma`` (length k), when given,
    scales the columns of every U block so the off-diagonal singular values
    decay as prescribed (the decaying-spectrum variant of the generator).
    ``rng`` defaults to the global numpy RNG, as upstream.
    """
    normal = (rng.standard_normal if rng is not None else np.random.standard_normal)
    fac = 4 if quad else 2
    N = nl * fac ** (L - 1)
    Nb = N // nl
    Nbvec = [Nb]
    k0 = min(k, nl)

    def level(nb, n, kk, project, scale=None):
        U = np.zeros((nb * n, kk))
        V = np.zeros((nb * n, kk))
        D = np.zeros((nb * n, n))
        for i in range(nb):
            Ui = np.linalg.qr(normal(size=(n, kk)), mode="reduced")[0]
            Vi = np.linalg.qr(normal(size=(n, kk)), mode="reduced")[0]
            Di = normal(size=(n, n))
            if project:
                Di = Di - Ui @ (Ui.T @ Di @ Vi) @ Vi.T
            if scale is not None:
                Ui = Ui * np.asarray(scale)[:kk]
            U[i * n:(i + 1) * n] = Ui
            V[i * n:(i + 1) * n] = Vi
            D[i * n:(i + 1) * n] = Di
        return U, V, D

    U, V, D = level(Nb, nl, k0, True, sigma)
    Umats, Vmats, Dmats = [U], [V], [D]
    for ind in range(1, L):
        Nb //= fac
        Nbvec.append(Nb)
        n = fac * (k0 if ind == 1 else k)
        U, V, D = level(Nb, n, k, ind < L - 1)
        if ind < L - 1:
            Umats.append(U)
            Vmats.append(V)
        Dmats.append(D)
    return OracleHBS().set_mats(Umats, Dmats, Vmats, Nbvec, fac=fac), Nbvec
