"""Right-preconditioned restarted GMRES on the GPU for blocks of right-hand
sides: the outer loop of upstream's iterative interface solve
(test/3D/cubeTest.py:158-186 and multislab/oms.py:258-302: scipy's gmres on
the interface operator Stot, preconditioned by a RedBlackSolverHBS or
ThomasSolverHBS solve).

Every column runs its own Krylov space (modified Gram-Schmidt Arnoldi, Givens
rotations), but the operator and the preconditioner are applied to all
columns in one call each, so a step costs one batched Stot apply and one
batched preconditioner solve.  The iteration stops per column when
||b - A x|| / ||b|| <= tol (the true residual of the right-preconditioned
system); after each cycle the residual is recomputed with the operator, and
that true residual decides convergence.
"""
import numpy as np
import torch

from .. import _dev as dv


def _colnorm(X):
    return torch.linalg.vector_norm(X, dim=0)


def gmres(A, B, M=None, tol=1e-10, restart=30, maxiter=500):
    """Solve A X = B.  ``A(X)`` and ``M(X)`` act on (n, c) float64 CUDA
    tensors (M approximates A^{-1}; None means no preconditioner).  Returns
    (X, iterations, worst relative residual); X has B's type and shape."""
    Bd, one = dv.prepare_rhs(B)
    n, c = Bd.shape
    Mf = M if M is not None else (lambda X: X)
    X = torch.zeros_like(Bd)
    bn = _colnorm(Bd)
    bn = torch.where(bn > 0, bn, torch.ones_like(bn))
    total = 0
    R = Bd.clone()
    while True:
        beta = _colnorm(R)
        rel = (beta / bn).cpu().numpy()
        if rel.max() <= tol or total >= maxiter:
            relres = float(rel.max())
            break
        active = beta > 0
        safe = torch.where(active, beta, torch.ones_like(beta))
        V = [R / safe]
        Hh = np.zeros((restart + 1, restart, c))
        cs = np.zeros((restart, c))
        sn = np.zeros((restart, c))
        g = np.zeros((restart + 1, c))
        g[0] = beta.cpu().numpy()
        Z = []
        j_done = 0
        for j in range(restart):
            Zj = Mf(V[j])
            Z.append(Zj)
            W = A(Zj)
            hcol = []
            for i in range(j + 1):
                hij = (V[i] * W).sum(0)
                W = W - V[i] * hij
                hcol.append(hij)
            hn = _colnorm(W)
            hcol = torch.stack(hcol).cpu().numpy()
            hnn = hn.cpu().numpy()
            Hh[:j + 1, j] = hcol
            Hh[j + 1, j] = hnn
            V.append(W / torch.where(hn > 0, hn, torch.ones_like(hn)))
            # Givens rotations, per column
            for i in range(j):
                t = cs[i] * Hh[i, j] + sn[i] * Hh[i + 1, j]
                Hh[i + 1, j] = -sn[i] * Hh[i, j] + cs[i] * Hh[i + 1, j]
                Hh[i, j] = t
            den = np.hypot(Hh[j, j], Hh[j + 1, j])
            den = np.where(den > 0, den, 1.0)
            cs[j] = Hh[j, j] / den
            sn[j] = Hh[j + 1, j] / den
            Hh[j, j] = cs[j] * Hh[j, j] + sn[j] * Hh[j + 1, j]
            Hh[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            total += 1
            j_done = j + 1
            if np.max(np.abs(g[j + 1]) / bn.cpu().numpy()) <= tol or total >= maxiter:
                break
        # y = H^{-1} g per column, X += sum_j Z_j y_j
        k = j_done
        Y = np.zeros((k, c))
        for col in range(c):
            Hc = Hh[:k, :k, col]
            gc = g[:k, col]
            yc = np.zeros(k)
            for i in range(k - 1, -1, -1):
                d = Hc[i, i]
                yc[i] = (gc[i] - Hc[i, i + 1:] @ yc[i + 1:]) / d if d != 0 else 0.0
            Y[:, col] = yc
        Yd = torch.from_numpy(Y).to(device=Bd.device)
        for jj in range(k):
            X = X + Z[jj] * Yd[jj]
        R = Bd - A(X)
    return dv.finish(X, B, one), total, relres
