"""GPU slab source-target maps (slu_slab_maps_apply through
sslablu_gb300.multislab.slabmaps) against the CPU oracle's maps
(oracle/slabmaps.py: the 2-D DST closed form and the 3-D sparse-LU maps, both
pinned to upstream's multislab/oms.py + stencil solver in
tests/test_oracle_golden.py).  The GPU solves are Chebyshev iterations run to
a relative accuracy of 1e-14, so maps, transposed maps and the interface
operator must agree with the oracle to 1e-12."""
import numpy as np
import pytest

from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_helmholtz3d_maps_match_oracle():
    """3-D variable-coefficient Helmholtz (k = 20, the C3 coefficient) on 16
    interfaces of 8 x 8 points: S_l X + S_r X' and both transposed maps of
    every slab in one batched call."""
    need_gpu()
    from oracle.slabmaps import helmholtz3d_slab_maps
    from sslablu_gb300.multislab.slabmaps import SlabGeometry, SlabMaps
    g = SlabGeometry(17, 5, 10, 10, kappa=20.0, coef=1)
    m, n = g.m, g.nif
    rng = np.random.default_rng(0)
    XL = rng.standard_normal((n * m, 6))
    XR = rng.standard_normal((n * m, 6))
    maps = SlabMaps(g)
    Y = maps.apply(_dev(XL), _dev(XR)).cpu().numpy()
    YL, YR = maps.apply_t(_dev(XL))
    YL, YR = YL.cpu().numpy(), YR.cpu().numpy()
    assert maps.steps > 10
    for s in range(n):
        Sl, Sr = helmholtz3d_slab_maps(g.nx, g.ny, g.nz, g.width, g.kappa, x0=s * g.H)
        r = slice(s * m, (s + 1) * m)
        assert relerr(Y[r], Sl @ XL[r] + Sr @ XR[r]) < 1e-12, s
        assert relerr(YL[r], Sl.T @ XL[r]) < 1e-12, s
        assert relerr(YR[r], Sr.T @ XL[r]) < 1e-12, s


def test_poisson2d_maps_and_interface_operator():
    """2-D Laplace slabs in the C1 layout (8 slabs, 64-point interfaces):
    one slab's stMap operator, and the interface operator Stot and its
    transpose against the system assembled from the oracle's closed form."""
    need_gpu()
    from oracle.slabmaps import poisson2d_couplings
    from sslablu_gb300.multislab.slabmaps import SlabGeometry, StotOperator, slab_stmaps
    g = SlabGeometry(8, 17, 66)
    m, n = g.m, g.nif
    C = poisson2d_couplings(m, 8, 17)
    M = np.eye(n * m)
    for i in range(n):
        if i > 0:
            M[i * m:(i + 1) * m, (i - 1) * m:i * m] = C[i][0]
        if i < n - 1:
            M[i * m:(i + 1) * m, (i + 1) * m:(i + 2) * m] = C[i][1]
    x = np.random.default_rng(1).standard_normal((n * m, 5))
    St = StotOperator(g)
    assert relerr(St @ x, M @ x) < 1e-12
    assert relerr(St.rmatmat(x), M.T @ x) < 1e-12
    assert relerr(St @ x[:, 0], M @ x[:, 0]) < 1e-12            # 1-D in, 1-D out
    st = slab_stmaps(g)
    assert st[0][0] is None and st[-1][1] is None
    A = st[3][1].A
    v = x[:m, :3]
    assert relerr(A @ v, C[3][1] @ v) < 1e-12
    assert relerr(A.T @ v, C[3][1].T @ v) < 1e-12
    assert relerr(A.rmatmat(v), C[3][1].T @ v) < 1e-12


def test_indefinite_slab_is_refused():
    """Slabs too wide for the Helmholtz shift (upstream's 5-slab 8 x 8 case
    at k = 20): the interior operator is indefinite, so the Chebyshev solve
    does not apply and the call is refused before any launch."""
    need_gpu()
    from sslablu_gb300 import _lib as L
    from sslablu_gb300.multislab.slabmaps import SlabGeometry, SlabMaps
    g = SlabGeometry(5, 5, 10, 10, kappa=20.0, coef=1)
    X = _dev(np.ones((g.nif * g.m, 1)))
    with pytest.raises(L.SluError):
        SlabMaps(g).apply(X, X)
