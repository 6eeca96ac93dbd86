"""tcgen05 split-BF16x3 GEMM (slu_gemm_split3) vs a float64 product.

The kernel accumulates the six split products in float32 within chunks of
512 terms of the leading product (1024 with 256-column tiles) and adds the
chunks in float32, so its relative error is about that of a float32 GEMM of
depth 512-1024 whatever K is: the bound here is 3e-6 (Frobenius, relative).
Shapes cover both tile widths (256 columns when the grid has at least one
tile per SM) and ragged edges in M, N and K."""
import numpy as np
import pytest

from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu


def _run(M, N, K, alpha=1.0, beta=0.0, seed=0):
    import torch
    from sslablu_gb300 import _lib
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((K, N))
    C0 = rng.standard_normal((M, N))
    Ad, Bd = (torch.from_numpy(x).cuda() for x in (A, B))
    Cd = torch.from_numpy(C0.copy()).cuda()
    _lib.check(_lib.lib().slu_gemm_split3(_lib.handle(), M, N, K, alpha, _lib.ptr(Ad), K,
                                          _lib.ptr(Bd), N, beta, _lib.ptr(Cd), N))
    _lib.sync()
    return Cd.cpu().numpy(), alpha * (A @ B) + beta * C0


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 500), (1024, 512, 2048),
                                   (129, 1, 65), (4096, 261, 4096), (2000, 4000, 300),
                                   (2048, 4096, 1024)])
def test_split3_gemm_accuracy(M, N, K):
    need_gpu()
    got, ref = _run(M, N, K)
    assert relerr(got, ref) < 3e-6


def test_split3_gemm_alpha_beta():
    need_gpu()
    got, ref = _run(200, 300, 256, alpha=-0.5, beta=2.0, seed=3)
    assert relerr(got, ref) < 3e-6
