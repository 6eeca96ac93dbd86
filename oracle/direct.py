"""Oracle (test infrastructure only): block-tridiagonal direct solvers.

numpy/scipy restatement of
  * direct_solve/omsdirectsolve.py: BlockTridiagonalSolver 48-175 (Thomas with
    LU-factored diagonal, cyclic SMW 143-175), RedBlackSolver 177-333
    (cyclic reduction; the LU->dense rebuild of 31-46/314 is replaced by
    keeping T, which is the same matrix up to rounding).
  * multislab/omsdirectsolve.py 17-160 (functional Thomas with identity
    diagonal, cyclic SMW).
  * direct_solve/omsdirectsolveHBS.py: id_op 12-20, STS_linop 162-179,
    RB_linop 77-106, Sprime_Linop 108-141, ThomasSolverHBS 189-351,
    RedBlackSolverHBS 359-558, with oracle.hbs.OracleHBS in place of
    HBSnew.HBSMAT.

Parity pinned against tests/golden/*.npz (produced by the upstream code).
Never imported by the product package.
"""
import numpy as np
from scipy.linalg import lu_factor, lu_solve

from .hbs import OracleHBS


# --------------------------------------------------------------------------
# dense Thomas, omsdirectsolve.py:48-175
# --------------------------------------------------------------------------
class ThomasDense:
    def __init__(self, m, cyclic=False):
        self.m, self.cyclic = m, cyclic

    def factorize(self, S_rk_list, T, glob_target_dofs=None):
        m = S_rk_list[0][0].shape[0]
        n = len(S_rk_list) - 1
        I = np.eye(m)
        self.A, self.B = [], [lu_factor(T[0])]
        self.C = [S_rk_list[i][-1] for i in range(n)]
        for i in range(1, n + 1):
            Ai = S_rk_list[i][0] @ lu_solve(self.B[-1], I)          # 89-91
            Bi = T[i] - Ai @ self.C[i - 1]                          # 94
            self.A.append(Ai)
            self.B.append(lu_factor(Bi))
        self.smw_block = None
        if self.cyclic:                                              # 148-166
            E, F = S_rk_list[0][0], S_rk_list[-1][1]
            nb = len(S_rk_list)
            U = np.zeros((nb * m, 2 * m))
            V = np.zeros((nb * m, 2 * m))
            U[0:m, 0:m] = E
            U[(nb - 1) * m:, m:] = F
            V[(nb - 1) * m:, 0:m] = I
            V[0:m, m:] = I
            Z = self._solve(U, glob_target_dofs)
            self.smw_block = Z @ np.linalg.solve(np.eye(2 * m) + V.T @ Z, V.T)
        return self

    def _solve(self, rhs, glob_target_dofs=None):                    # 105-141
        m = self.m
        n = len(self.A)
        d = rhs.copy()
        idx = ([range(l * m, (l + 1) * m) for l in range(len(self.B))]
               if glob_target_dofs is None else glob_target_dofs)
        for i in range(1, n + 1):
            d[idx[i]] = d[idx[i]] - self.A[i - 1] @ d[idx[i - 1]]
        x = np.zeros(d.shape)
        x[idx[n]] = lu_solve(self.B[n], d[idx[n]])
        for i in range(n - 1, -1, -1):
            x[idx[i]] = lu_solve(self.B[i], d[idx[i]] - self.C[i] @ x[idx[i + 1]])
        return x

    def solve(self, rhs, glob_target_dofs=None):
        x = self._solve(rhs, glob_target_dofs)
        if self.cyclic:
            x = x - self.smw_block @ x
        return x


# --------------------------------------------------------------------------
# dense red-black, omsdirectsolve.py:177-333
# --------------------------------------------------------------------------
class RedBlackDense:
    def __init__(self, m, cyclic=False):
        self.m, self.cyclic = m, cyclic

    def factorize(self, S_rk_list, T):
        m = S_rk_list[0][0].shape[0]
        nS = len(S_rk_list)
        SiM = [s[0] for s in S_rk_list]
        SiP = [s[-1] for s in S_rk_list]
        if not self.cyclic:
            SiM[0] = np.zeros((m, m))
            SiP[-1] = np.zeros((m, m))
        RB = [(SiM, list(T), [lu_factor(t) for t in T], SiP)]
        l = nS
        while l > 1:
            RB.append(self._level(m, l, RB[-1]))
            l //= 2
        self.RB, self.nSlabs = RB, nS
        return self

    def _level(self, m, nS, lev):                                     # 283-333
        SiM, T, Tinv, SiP = lev
        cyc = self.cyclic
        Bs, As, Cs = [], [], []
        for i in range(0, nS, 2):
            B = T[i].copy()
            if i > 0 or cyc:
                B -= SiM[i] @ lu_solve(Tinv[i - 1], SiP[(i - 1) % nS])
            if i < nS - 1 or cyc:
                B -= SiP[i] @ lu_solve(Tinv[i + 1], SiM[(i + 1) % nS])
            Bs.append(B)
            As.append(-SiM[i] @ lu_solve(Tinv[i - 1], SiM[(i - 1) % nS]))
            Cs.append(-SiP[i] @ lu_solve(Tinv[(i + 1) % nS], SiP[(i + 1) % nS]))
        if len(Bs) == 1 and cyc:
            Bs[0] = Bs[0] + As[0] + Cs[0]
        return (As, Bs, [lu_factor(b) for b in Bs], Cs)

    def solve(self, rhs):                                             # 221-279
        m, RB = self.m, self.RB
        cyc = self.cyclic
        vs = [rhs.copy()]
        for l in range(len(RB) - 1):
            SiM, _, Tinv, SiP = RB[l]
            nS = len(SiM)
            nR = nS // 2
            vp = vs[-1]
            vn = np.zeros((m * nR,) + rhs.shape[1:])
            for j in range(nR):
                i = 2 * j
                c = vp[i * m:(i + 1) * m].copy()
                if cyc or i > 0:
                    p = (i - 1) % nS
                    c -= SiM[i] @ lu_solve(Tinv[p], vp[p * m:(p + 1) * m])
                if cyc or i < nS - 1:
                    q = (i + 1) % nS
                    c -= SiP[i] @ lu_solve(Tinv[q], vp[q * m:(q + 1) * m])
                vn[j * m:(j + 1) * m] = c
            vs.append(vn)
        vs[-1] = lu_solve(RB[-1][2][0], vs[-1])
        for l in range(len(RB) - 1, 0, -1):
            SiM, _, Tinv, SiP = RB[l - 1]
            nR = len(SiM) // 2
            for j in range(nR):
                i = 2 * j
                vs[l - 1][i * m:(i + 1) * m] = vs[l][j * m:(j + 1) * m]
                c = SiM[i + 1] @ vs[l][j * m:(j + 1) * m]
                if cyc or j + 1 < nR:
                    q = (j + 1) % nR
                    c = c + SiP[i + 1] @ vs[l][q * m:(q + 1) * m]
                blk = vs[l - 1][(i + 1) * m:(i + 2) * m] - c
                vs[l - 1][(i + 1) * m:(i + 2) * m] = lu_solve(Tinv[i + 1], blk)
        return vs[0]


# --------------------------------------------------------------------------
# functional Thomas with identity diagonal, multislab/omsdirectsolve.py:17-160
# --------------------------------------------------------------------------
def build_block_tridiagonal_solver(S_rk_list):
    m = S_rk_list[0][0].shape[0]
    n = len(S_rk_list) - 1
    I = np.eye(m)
    A, B = [], [I]
    C = [S_rk_list[i][-1] for i in range(n)]
    for i in range(1, n + 1):
        Ai = S_rk_list[i][0] @ (B[-1] if i == 1 else lu_solve(B[-1], I))
        A.append(Ai)
        B.append(lu_factor(I - Ai @ C[i - 1]))
    return A, B, C


def block_tridiagonal_solve(indices, T, rhs):
    A, B, C = T
    n = len(A)
    d = rhs.copy()
    for i in range(1, n + 1):
        d[indices[i]] = d[indices[i]] - A[i - 1] @ d[indices[i - 1]]
    x = np.zeros(d.shape)
    x[indices[n]] = lu_solve(B[n], d[indices[n]])
    for i in range(n - 1, 0, -1):
        x[indices[i]] = lu_solve(B[i], d[indices[i]] - C[i] @ x[indices[i + 1]])
    x[indices[0]] = d[indices[0]] - C[0] @ x[indices[1]]
    return x


# --------------------------------------------------------------------------
# implicit operators, omsdirectsolveHBS.py:12-179
# --------------------------------------------------------------------------
class Op:
    """Minimal LinearOperator: matmat/rmatmat (+ optional solve)."""

    def __init__(self, n, mm, rmm, solve=None, tree=None, quad=None):
        self.shape = (n, n)
        self.dtype = np.float64
        self._mm, self._rmm, self._solve = mm, rmm, solve
        self.tree, self.quad = tree, quad

    def matmat(self, v):
        return self._mm(v)

    def rmatmat(self, v):
        return self._rmm(v)

    def solve(self, v, mode="N"):
        return self._solve(v, mode)

    def __matmul__(self, v):
        return self._mm(v)


def id_op(n):
    return Op(n, lambda v: v.copy(), lambda v: v.copy(), lambda v, mode="N": v.copy())


def dense_op(A):
    A = np.asarray(A)
    return Op(A.shape[0], lambda v: A @ v, lambda v: A.T @ v,
              lambda v, mode="N": np.linalg.solve(A if mode == "N" else A.T, v))


def _col(v):
    return v[:, None] if v.ndim == 1 else v


def _back(r, v):
    return r.flatten() if v.ndim == 1 else r


def sts_op(Sl, T, Sr):
    """-Sl T^{-1} Sr, omsdirectsolveHBS.py:162-179."""
    return Op(T.shape[0],
              lambda v: _back(-Sl.matmat(T.solve(Sr.matmat(_col(v)))), v),
              lambda v: _back(-Sr.rmatmat(T.solve(Sl.rmatmat(_col(v)), mode="T")), v))


def rb_op(Ti, tm, tp, SiPi, SiMi, smp, spm):
    """Ti - SiPi tp^{-1} smp - SiMi tm^{-1} spm, omsdirectsolveHBS.py:77-106."""
    def mm(v):
        w = _col(v)
        r = Ti.matmat(w)
        if tp is not None:
            r = r - SiPi.matmat(tp.solve(smp.matmat(w)))
        if tm is not None:
            r = r - SiMi.matmat(tm.solve(spm.matmat(w)))
        return _back(r, v)

    def rmm(v):
        w = _col(v)
        r = Ti.rmatmat(w)
        if tp is not None:
            r = r - smp.rmatmat(tp.solve(SiPi.rmatmat(w), mode="T"))
        if tm is not None:
            r = r - spm.rmatmat(tm.solve(SiMi.rmatmat(w), mode="T"))
        return _back(r, v)
    return Op(Ti.shape[0], mm, rmm)


def sprime_op(Sl, Sp, Sr, ident=False):
    """I - Sl Sp^{-1} Sr, omsdirectsolveHBS.py:108-141."""
    if ident:
        return Op(Sl.shape[0],
                  lambda v: _back(_col(v) - Sl.matmat(Sr.matmat(_col(v))), v),
                  lambda v: _back(_col(v) - Sr.rmatmat(Sl.rmatmat(_col(v))), v))
    return Op(Sl.shape[0],
              lambda v: _back(_col(v) - Sl.matmat(Sp.solve(Sr.matmat(_col(v)))), v),
              lambda v: _back(_col(v) - Sr.rmatmat(Sp.solve(Sl.rmatmat(_col(v)), mode="T")), v))


def _hbs(linop, perm, nleaves, nlevels, quad, rk):
    h = OracleHBS(linop, perm, nleaves, nlevels, 4 if quad else 2)
    return h.construct(rk)


# --------------------------------------------------------------------------
# HBS Thomas, omsdirectsolveHBS.py:189-351 (identity-diagonal branch)
# --------------------------------------------------------------------------
class ThomasHBS:
    def __init__(self, m, rk, tree_data, quad):
        self.m, self.rk, self.tree_data, self.quad = m, rk, tree_data, quad

    def factorize(self, S_rk_list):
        n = len(S_rk_list) - 1
        I = id_op(self.m)
        Sl = [S_rk_list[i][0] for i in range(1, n + 1)]
        Sr = [S_rk_list[i][-1] for i in range(n)]
        Sp = [I]
        for i in range(1, n + 1):
            op = (sprime_op(Sl[0], I, Sr[0], ident=True) if i == 1
                  else sprime_op(Sl[i - 1], Sp[i - 1], Sr[i - 1]))
            Sp.append(_hbs(op, *self.tree_data, self.quad, self.rk))
        self.Sl, self.Sp, self.Sr = Sl, Sp, Sr
        return self

    def solve(self, rhs, glob_target_dofs=None):                     # 283-314
        m = self.m
        n = len(self.Sl)
        d = rhs.copy()
        if rhs.ndim == 1:
            d = d[:, None]
        idx = ([range(l * m, (l + 1) * m) for l in range(n + 1)]
               if glob_target_dofs is None else glob_target_dofs)
        for i in range(1, n + 1):
            if i == 1:
                d[idx[i]] = d[idx[i]] - self.Sl[0] @ d[idx[0]]
            else:
                d[idx[i]] = d[idx[i]] - self.Sl[i - 1] @ self.Sp[i - 1].solve(d[idx[i - 1]])
        x = np.zeros(d.shape)
        x[idx[n]] = self.Sp[n].solve(d[idx[n]])
        for i in range(n - 1, 0, -1):
            x[idx[i]] = self.Sp[i].solve(d[idx[i]] - self.Sr[i] @ x[idx[i + 1]])
        x[idx[0]] = d[idx[0]] - self.Sr[0] @ x[idx[1]]
        return x.flatten() if rhs.ndim == 1 else x


# --------------------------------------------------------------------------
# HBS red-black, omsdirectsolveHBS.py:359-558
# --------------------------------------------------------------------------
class RedBlackHBS:
    def __init__(self, m, rk, tree_data, quad):
        self.m, self.rk, self.tree_data, self.quad = m, rk, tree_data, quad

    def _hbs(self, op):
        return _hbs(op, *self.tree_data, self.quad, self.rk)

    def factorize(self, S_rk_list, T=None):
        m = S_rk_list[0][0].shape[0]
        nS = len(S_rk_list)
        if not (nS & (nS - 1) == 0 and nS != 0):
            raise ValueError("Number of slabs must be a power of 2.")
        SiM = [s[0] for s in S_rk_list]
        SiP = [s[-1] for s in S_rk_list]
        SiM[0] = dense_op(np.zeros((m, m)))
        SiP[-1] = dense_op(np.zeros((m, m)))
        if T is None:
            T = [id_op(m) for _ in range(nS)]
        RB = [(SiM, T, T, SiP)]
        l = nS
        while l > 1:
            RB.append(self._level(l, RB[-1]))
            l //= 2
        self.RB = RB
        return self

    def _level(self, nS, lev):                                        # 436-483
        SiM, T, Th, SiP = lev
        Bl, Bh = [], []
        for i in range(0, nS, 2):
            spm = SiP[i - 1] if i > 0 else None
            smp = SiM[i + 1] if i < nS - 1 else None
            tm = Th[i - 1] if spm is not None else None
            tp = Th[i + 1] if smp is not None else None
            op = rb_op(T[i], tm, tp, SiP[i], SiM[i], smp, spm)
            Bl.append(op)
            Bh.append(self._hbs(op))
        A = [self._hbs(sts_op(SiM[i], Th[(i - 1) % nS], SiM[(i - 1) % nS]))
             for i in range(0, nS, 2)]
        C = [self._hbs(sts_op(SiP[i], Th[(i + 1) % nS], SiP[(i + 1) % nS]))
             for i in range(0, nS, 2)]
        return (A, Bl, Bh, C)

    def solve(self, rhs):                                             # 489-558
        m, RB = self.m, self.RB
        vs = [rhs.copy()]
        for l in range(len(RB) - 1):
            SiM, _, Th, SiP = RB[l]
            nS = len(SiM)
            nR = nS // 2
            vp = vs[-1]
            vn = np.zeros(m * nR)
            for j in range(nR):
                i = 2 * j
                c = vp[i * m:(i + 1) * m].copy()
                if i > 0:
                    c -= SiM[i].matmat(Th[i - 1].solve(vp[(i - 1) * m:i * m, None]))[:, 0]
                if i < nS - 1:
                    c -= SiP[i].matmat(Th[i + 1].solve(vp[(i + 1) * m:(i + 2) * m, None]))[:, 0]
                vn[j * m:(j + 1) * m] = c
            vs.append(vn)
        vs[-1] = RB[-1][2][0].solve(vs[-1])
        for l in range(len(RB) - 1, 0, -1):
            SiM, _, Th, SiP = RB[l - 1]
            nR = len(SiM) // 2
            for j in range(nR):
                i = 2 * j
                vs[l - 1][i * m:(i + 1) * m] = vs[l][j * m:(j + 1) * m]
                c = SiM[i + 1].matmat(vs[l][j * m:(j + 1) * m, None])[:, 0]
                if j + 1 < nR:
                    c += SiP[i + 1].matmat(vs[l][(j + 1) * m:(j + 2) * m, None])[:, 0]
                vs[l - 1][(i + 1) * m:(i + 2) * m] -= c
                vs[l - 1][(i + 1) * m:(i + 2) * m] = Th[i + 1].solve(vs[l - 1][(i + 1) * m:(i + 2) * m])
        return vs[0]
