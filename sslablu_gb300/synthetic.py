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


def slab_couplings(m, nS, c=20.0):
    """Block-tridiagonal interface couplings of nS slabs with m-point
    interfaces: S_{i,i-1} and S_{i,i+1} are Gaussian kernels of the interface
    coordinate, shifted by +-0.2 (+-0.01 per slab), scaled by 0.3, so that
    I + S is well conditioned and its blocks are HBS compressible.  Returns
    [(S_{i,i-1}, S_{i,i+1})], with zero outer blocks."""
    x = np.linspace(0, 1, m)

    def blk(shift):
        return 0.3 * np.exp(-c * (x[:, None] - x[None, :] - shift) ** 2)
    out = []
    for i in range(nS):
        A = blk(0.2 + 0.01 * i) if i > 0 else np.zeros((m, m))
        C = blk(-0.2 - 0.01 * i) if i < nS - 1 else np.zeros((m, m))
        out.append((A, C))
    return out


def tridiag_apply(S, X):
    """(I + block off-diagonals of S) X for X of shape (nS * m, r), numpy."""
    nS = len(S)
    m = S[0][0].shape[0]
    Y = X.copy()
    for i in range(nS):
        if i > 0:
            Y[i * m:(i + 1) * m] += S[i][0] @ X[(i - 1) * m:i * m]
        if i < nS - 1:
            Y[i * m:(i + 1) * m] += S[i][1] @ X[(i + 1) * m:(i + 2) * m]
    return Y


def plane_points(n, x=0.5):
    """n x n grid on the plane x = const of the unit cube (the interface
    plane of a 3-D slab), as an (n*n, 3) point cloud."""
    g = np.stack(np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="ij"),
                 -1).reshape(-1, 2)
    return np.concatenate([np.full((g.shape[0], 1), x), g], 1)


def plane_coupling(XX, shift=0.05, eps=0.02):
    """exp(-r) / (r + eps) between the points and their copy moved by `shift`
    along x: a smooth coupling between two nearby interfaces whose near
    field decays slowly (the case strong admissibility is built for).
    Returns a float64 numpy array."""
    D = np.linalg.norm(XX[:, None, :] - XX[None, :, :] - np.array([shift, 0.0, 0.0]), axis=2)
    return np.exp(-D) / (D + eps)


def poisson_slab_map(m, nx, width, height=1.0):
    """The slab map S = (A_ii^{-1} A_ib[:, J])[Ic, :] of a double slab of the
    5-point Poisson stencil (c11 = c22 = 1): m interior points along the
    interface (spacing height / (m + 1)), nx grid points across the slab of
    the given width (odd, so the centre line is a grid line).  With Dirichlet
    ends the operator separates: in the sine basis Q of the interface
    direction, mode q decouples into a three-term recurrence across the slab
    whose solution from one edge to the centre is -1 / (2 cosh(M theta_q)),
    M = (nx - 1) / 2, cosh theta_q = 1 + 2 (hx / hy)^2 sin^2(pi q / (2 (m + 1))).
    The left and the right map are equal.  Returns S (m x m float64)."""
    if nx % 2 == 0 or nx < 3:
        raise ValueError("nx must be odd and >= 3")
    hx = width / (nx - 1)
    hy = height / (m + 1)
    q = np.arange(1, m + 1)
    t = 2.0 * (hx / hy) ** 2 * np.sin(np.pi * q / (2 * (m + 1))) ** 2
    theta = np.log1p(t + np.sqrt(t * (t + 2.0)))           # arccosh(1 + t)
    x = 0.5 * (nx - 1) * theta
    sig = -np.exp(-x) / (1.0 + np.exp(-2.0 * x))            # -1 / (2 cosh x)
    Q = np.sqrt(2.0 / (m + 1)) * np.sin(np.pi * np.outer(q, q) / (m + 1))
    return (Q * sig) @ Q.T
