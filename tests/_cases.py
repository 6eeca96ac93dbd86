"""Shared input builders for the parity tests (regenerate fixture inputs)."""
import numpy as np

from oracle.hbs import gen_random_hbs


def relerr(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0)


def test_rb_system(nS, m, seed=42):
    """Restates direct_solve/test_RB.py:319-350 (make_block_tridiagonal)."""
    rng = np.random.default_rng(seed)
    N = nS * m
    mat = np.zeros((N, N))
    T, S = [], []
    for i in range(nS):
        B = rng.standard_normal((m, m)) + nS * m * np.eye(m)
        T.append(B)
        mat[i * m:(i + 1) * m, i * m:(i + 1) * m] = B
        A = 0.1 * rng.standard_normal((m, m)) if i > 0 else np.zeros((m, m))
        C = 0.1 * rng.standard_normal((m, m)) if i < nS - 1 else np.zeros((m, m))
        if i > 0:
            mat[i * m:(i + 1) * m, (i - 1) * m:i * m] = A
        if i < nS - 1:
            mat[i * m:(i + 1) * m, (i + 1) * m:(i + 2) * m] = C
        S.append((A, C))
    rhs = rng.standard_normal(N)
    return S, T, mat, rhs


test_rb_system.__test__ = False


def hbs_from_fixture(g):
    """Regenerate the exact random HBS of a golden hbs_*.npz fixture."""
    np.random.seed(int(g["seed"]))
    sigma = g.get("sigma")
    S, Nbvec = gen_random_hbs(int(g["k"]), int(g["nl"]), int(g["L"]), bool(g["quad"]),
                              sigma=sigma)
    return S, Nbvec


def kernel_system(m=64, nS=4):
    """Smooth-kernel block-tridiagonal couplings (tests/golden/make_golden.py)."""
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
    """Gaussian-kernel couplings (tests/golden/make_golden.py)."""
    x = np.linspace(0, 1, m)

    def blk(shift):
        return 0.3 * np.exp(-c * (x[:, None] - x[None, :] - shift) ** 2)
    S = []
    for i in range(nS):
        A = blk(0.2 + 0.01 * i) if i > 0 else np.zeros((m, m))
        C = blk(-0.2 - 0.01 * i) if i < nS - 1 else np.zeros((m, m))
        S.append((A, C))
    return S


def tridiag_matrix(S, m):
    """Assemble I + block off-diagonals of a coupling list."""
    nS = len(S)
    M = np.eye(nS * m)
    for i in range(nS):
        if i > 0:
            M[i * m:(i + 1) * m, (i - 1) * m:i * m] = S[i][0]
        if i < nS - 1:
            M[i * m:(i + 1) * m, (i + 1) * m:(i + 2) * m] = S[i][1]
    return M
