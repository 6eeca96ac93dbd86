"""Seeded synthetic HBS operators for benchmarks and the serving CLI.

Exact HBS matrices in the layout of the reference's test generator
(test/rkprop/HBSnewTest.py:15-73): every U/V block is an orthonormalised
Gaussian, every D block Gaussian and, below the root, projected off the U/V
ranges.  ``sigma`` scales the columns of the leaf U blocks so the
off-diagonal singular values follow a prescribed decay; ``shift`` adds a
multiple of the identity to the leaf D blocks (the I + S form of the slab
interface systems), which keeps the operator well conditioned at every size.
Draws come from ``rng`` (a numpy Generator) or, when it is None, from the
global numpy RNG in the reference generator's order.
"""
import numpy as np


def random_hbs_factors(k, nl, L, quad=False, sigma=None, rng=None, shift=0.0):
    """Returns (Umats, Dmats, Vmats, Nbvec) of an N = nl * fac**(L-1) operator."""
    normal = rng.standard_normal if rng is not None else np.random.standard_normal
    fac = 4 if quad else 2
    Nb = nl * fac ** (L - 1) // nl
    k0 = min(k, nl)

    def level(nb, n, kk, project, scale=None):
        U = np.zeros((nb * n, kk))
        V = np.zeros((nb * n, kk))
        D = np.zeros((nb * n, n))
        for b in range(nb):
            Ub = np.linalg.qr(normal(size=(n, kk)), mode="reduced")[0]
            Vb = np.linalg.qr(normal(size=(n, kk)), mode="reduced")[0]
            Db = normal(size=(n, n))
            if project:
                Db = Db - Ub @ (Ub.T @ Db @ Vb) @ Vb.T
            if scale is not None:
                Ub = Ub * np.asarray(scale)[:kk]
            rows = slice(b * n, (b + 1) * n)
            U[rows], V[rows], D[rows] = Ub, Vb, Db
        return U, V, D

    U, V, D = level(Nb, nl, k0, True, sigma)
    if shift:
        D.reshape(-1, nl, nl)[:] += shift * np.eye(nl)
    Umats, Vmats, Dmats, Nbvec = [U], [V], [D], [Nb]
    for t in range(1, L):
        Nb //= fac
        Nbvec.append(Nb)
        n = fac * (k0 if t == 1 else k)
        U, V, D = level(Nb, n, k, t < L - 1)
        if t < L - 1:
            Umats.append(U)
            Vmats.append(V)
        Dmats.append(D)
    return Umats, Dmats, Vmats, Nbvec


def decaying_sigma(k, smallest=1e-12):
    """Singular values 1 -> smallest, geometric over k columns."""
    return 10.0 ** (np.log10(smallest) * np.arange(k) / max(k - 1, 1))
