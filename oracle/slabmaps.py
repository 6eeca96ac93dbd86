"""Slab source-target maps of the stencil discretisation (test infrastructure).

This module is part of the CPU oracle: only tests/, __graft_entry__.smoke()
and bench.py's CPU legs may import it.

Upstream builds the interface couplings of the overlapping multislab method
(multislab/oms.py:96-125, ``oms.compute_stmaps``) as

    S_J = (A_ii^{-1} A_ib[:, J])[Ic, :]

for a double-wide slab: A_ii the interior rows of the stencil operator on the
slab, A_ib its couplings to the slab's boundary points, J the points of the
left (J = Il) or right (J = Ir) slab edge that are not on the global
Dirichlet boundary, and Ic the interior points on the slab's centre line
(``slab.compute_idxs_and_pts``, multislab/oms.py:40-53).  The stencil is the
5-point operator of solver/stencil/stencilSolver.py:40-120
(``_constructPDO2D_csr``: c11 u_xx + c22 u_yy [+ c u], interior rows
-2/hx^2 - 2/hy^2 on the diagonal, 1/hx^2 and 1/hy^2 to the neighbours) or
the 7-point one of stencilSolver.py:221-420 (``_constructPDO3D_csr``).

For constant coefficients the interior operator separates: with Dirichlet
ends the second difference along y is diagonalised by the discrete sine
transform, so S_J = Q diag(sigma) Q^T with sigma_q the centre value of one
tridiagonal solve along x per transverse mode q.  The closed form agrees
with upstream's stencil maps to ~1e-16 (tests/test_oracle_golden.py).  The
3-D variable-coefficient maps are formed by a sparse LU of A_ii, as
upstream's stencilSolver.solver_Aii does.
"""
import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import splu


def dst_basis(m):
    """Orthonormal DST-I basis: Q[i, j] = sqrt(2/(m+1)) sin(pi (i+1)(j+1)/(m+1))."""
    j = np.arange(1, m + 1)
    return np.sqrt(2.0 / (m + 1)) * np.sin(np.pi * np.outer(j, j) / (m + 1))


def dst_eigs(m, h):
    """Eigenvalues of the Dirichlet second difference (1/h^2) tridiag(1, -2, 1)."""
    j = np.arange(1, m + 1)
    return -4.0 * np.sin(np.pi * j / (2 * (m + 1))) ** 2 / h ** 2


def _centre_responses(lam, nx, hx):
    """For each transverse eigenvalue lam_q: the centre value of the solution
    of ((1/hx^2) T_x + lam_q I) w = e_edge / hx^2 along the nx - 2 interior x
    points, for the left and for the right edge (Thomas, all modes at once)."""
    nxi = nx - 2
    ic = (nx - 1) // 2 - 1
    a = 1.0 / hx ** 2
    d = -2.0 * a + lam
    q = lam.size
    res = []
    for edge in (0, nxi - 1):
        rhs = np.zeros((nxi, q))
        rhs[edge] = a
        cp = np.zeros((nxi, q))
        dp = np.zeros((nxi, q))
        cp[0] = a / d
        dp[0] = rhs[0] / d
        for i in range(1, nxi):
            den = d - a * cp[i - 1]
            cp[i] = a / den
            dp[i] = (rhs[i] - a * dp[i - 1]) / den
        w = np.zeros((nxi, q))
        w[-1] = dp[-1]
        for i in range(nxi - 2, -1, -1):
            w[i] = dp[i] - cp[i] * w[i + 1]
        res.append(w[ic])
    return res[0], res[1]


def poisson2d_slab_maps(m, nx, width, height=1.0):
    """(S_l, S_r), each m x m: the left / right edge -> centre line maps of a
    double slab of the given width with nx grid points across (odd, so the
    centre line is a grid line) and m interior points along y (Ny = m + 2),
    for the Laplacian (c11 = c22 = 1, no zeroth-order term)."""
    if nx % 2 == 0 or nx < 3:
        raise ValueError("nx must be odd and >= 3 (the centre line is a grid line)")
    hx = width / (nx - 1)
    hy = height / (m + 1)
    Q = dst_basis(m)
    sl, sr = _centre_responses(dst_eigs(m, hy), nx, hx)
    return (Q * sl) @ Q.T, (Q * sr) @ Q.T


def poisson2d_couplings(m, nslabs, nx):
    """The coupling list of the interface system of [0,1]^2 cut into nslabs
    slabs (nslabs - 1 interfaces of m points, double slabs of width
    2/nslabs, upstream's geometry.geom_2D.square.dSlabs): entry i is
    (S_l, S_r) of double slab i, zero where the slab's edge is the global
    boundary, as construct_Stot_helper builds them (multislab/oms.py:140-250)."""
    Sl, Sr = poisson2d_slab_maps(m, nx, 2.0 / nslabs)
    n = nslabs - 1
    Z = np.zeros((m, m))
    return [(Sl if i > 0 else Z, Sr if i < n - 1 else Z) for i in range(n)]


# --------------------------------------------------------------------------
# 3-D variable-coefficient Helmholtz slabs
def c3_coefficient(x, y, z):
    """c(x) = 1 + 0.5 sin(2 pi x) sin(2 pi y) sin(2 pi z)."""
    return 1.0 + 0.5 * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * z)


def helmholtz3d_interior(nx, ny, nz, width, kappa, x0=0.0, coef=c3_coefficient):
    """Interior operator of the double slab [x0, x0 + width] x [0,1]^2 under
    the 7-point stencil of stencilSolver.py:221-420 with c11 = c22 = c33 = 1
    and zeroth-order term c = kappa^2 coef(x, y, z) (Helmholtz
    Delta u + k^2 c u): returns (A_ii as CSC, hx, interior shape).

    Interior points are numbered x fastest, then z, then y:
    idx = (iy * nzi + iz) * nxi + ix."""
    hx = width / (nx - 1)
    hy = 1.0 / (ny - 1)
    hz = 1.0 / (nz - 1)
    nxi, nyi, nzi = nx - 2, ny - 2, nz - 2
    xs = x0 + hx * np.arange(1, nx - 1)
    ys = hy * np.arange(1, ny - 1)
    zs = hz * np.arange(1, nz - 1)
    Y, Z, X = np.meshgrid(ys, zs, xs, indexing="ij")     # (nyi, nzi, nxi)
    c0 = kappa ** 2 * coef(X, Y, Z)
    diag = (-2.0 / hx ** 2 - 2.0 / hy ** 2 - 2.0 / hz ** 2) + c0.ravel()
    N = nxi * nyi * nzi
    idx = np.arange(N).reshape(nyi, nzi, nxi)
    rows, cols, vals = [np.arange(N)], [np.arange(N)], [diag]
    for ax, h in ((2, hx), (1, hz), (0, hy)):
        a = np.take(idx, np.arange(idx.shape[ax] - 1), axis=ax).ravel()
        b = np.take(idx, np.arange(1, idx.shape[ax]), axis=ax).ravel()
        w = np.full(a.size, 1.0 / h ** 2)
        rows += [a, b]
        cols += [b, a]
        vals += [w, w]
    A = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(N, N))
    return A, hx, (nyi, nzi, nxi)


def helmholtz3d_slab_maps(nx, ny, nz, width, kappa, x0=0.0, coef=c3_coefficient):
    """(S_l, S_r) of one 3-D double slab, each (nyi nzi) x (nyi nzi), rows
    and columns in the interface plane's (y, z) order with z fastest (the
    order of upstream's flat grid index k = ix Ny Nz + iy Nz + iz)."""
    A, hx, (nyi, nzi, nxi) = helmholtz3d_interior(nx, ny, nz, width, kappa, x0, coef)
    lu = splu(A)
    m = nyi * nzi
    plane = np.arange(m)
    ic = (nx - 1) // 2 - 1
    out = []
    for edge in (0, nxi - 1):
        rhs = np.zeros((A.shape[0], m))
        rhs[plane * nxi + edge, plane] = 1.0 / hx ** 2
        sol = lu.solve(rhs)
        out.append(sol[plane * nxi + ic, :])
    return out[0], out[1]


def helmholtz3d_sample(nx, ny, nz, width, kappa, x0, Om, edge, trans=False,
                       coef=c3_coefficient):
    """S_edge @ Om (or S_edge^T @ Om with ``trans``) through one sparse solve
    per call, as upstream's compute_stmaps linear operator does
    (multislab/oms.py:99-118): edge 0 = left, 1 = right."""
    A, hx, (nyi, nzi, nxi) = helmholtz3d_interior(nx, ny, nz, width, kappa, x0, coef)
    lu = splu(A)
    m = nyi * nzi
    plane = np.arange(m)
    ic = (nx - 1) // 2 - 1
    e = 0 if edge == 0 else nxi - 1
    rhs = np.zeros((A.shape[0], Om.shape[1]))
    if not trans:
        rhs[plane * nxi + e] = Om / hx ** 2
        return lu.solve(rhs)[plane * nxi + ic]
    rhs[plane * nxi + ic] = Om
    return lu.solve(rhs, trans="T")[plane * nxi + e] / hx ** 2
