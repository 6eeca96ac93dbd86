"""The allocation-free ULV solve (slu_ulv_solve_noalloc) gives the same
result as slu_ulv_solve.

slu_ulv_solve_noalloc serves callers that cannot let a library allocate
device memory while they solve (a serving runtime owning the GPU memory
budget, or a latency-critical loop that cannot absorb cudaMalloc's implicit
synchronisation); it takes its scratch from a fixed array inside the library.
This file is collected last so that a failure here leaves every other test
already run.  It builds its own operator, so it also passes alone in a fresh
process.
"""
import ctypes

import numpy as np
import pytest

from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _factored_hbs(seed=31):
    from oracle.hbs import gen_random_hbs
    from sslablu_gb300.matAssembly.HBS.HBSnew import HBSMAT
    np.random.seed(seed)
    S, Nbvec = gen_random_hbs(16, 32, 5, quad=False)   # N = 512
    H = HBSMAT().set_mats(S.Umats, S.Dmats, S.Vmats, list(Nbvec), fac=2)
    H.compute_ULV()
    return H


def _solve(fn_name, H, b, trans=0):
    import torch
    from sslablu_gb300 import _lib
    B = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    status = getattr(_lib.lib(), fn_name)(_lib.handle(), H._op, _lib.ptr(B), B.shape[1],
                                          B.shape[1], int(trans))
    torch.cuda.synchronize()
    return status, B.cpu().numpy()


def test_noalloc_matches_allocating_solve_twice():
    need_gpu()
    H = _factored_hbs()
    rng = np.random.default_rng(3)
    N = H.shape[0]
    for call, (nrhs, trans) in enumerate([(16, 0), (5, 1)]):   # two calls in a row
        b = rng.standard_normal((N, nrhs))
        st_ref, x_ref = _solve("slu_ulv_solve", H, b, trans)
        st_new, x_new = _solve("slu_ulv_solve_noalloc", H, b, trans)
        assert st_ref == 0 and st_new == 0, "call %d: status %d / %d" % (call, st_ref, st_new)
        assert relerr(x_new, x_ref) < TOL, "call %d" % call


def _pool_used_bytes():
    """Bytes in use from the current device's default stream-ordered memory
    pool, the pool the library's handles take their workspaces from
    (cudaMallocAsync); read through the driver API."""
    import torch
    cu = ctypes.CDLL("libcuda.so.1")
    dev = ctypes.c_int()
    assert cu.cuDeviceGet(ctypes.byref(dev), torch.cuda.current_device()) == 0
    pool = ctypes.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0
    used = ctypes.c_uint64()
    CU_MEMPOOL_ATTR_USED_MEM_CURRENT = 7
    assert cu.cuMemPoolGetAttribute(pool, CU_MEMPOOL_ATTR_USED_MEM_CURRENT,
                                    ctypes.byref(used)) == 0
    return used.value


def test_noalloc_allocates_nothing():
    """On a fresh stream (so a fresh handle with no workspace yet) the
    allocation-free solve leaves the pool's in-use bytes unchanged, while the
    ordinary solve on the same handle grows them (so the measurement can see
    an allocation)."""
    need_gpu()
    import torch
    from sslablu_gb300 import _lib
    H = _factored_hbs(seed=37)
    N = H.shape[0]
    b = np.random.default_rng(5).standard_normal((N, 24))
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        h = _lib.handle()                       # created here: allocates its status words
        torch.cuda.synchronize()
        B = torch.from_numpy(b).cuda()
        B2 = B.clone()
        torch.cuda.synchronize()
        before = _pool_used_bytes()
        for _ in range(2):
            assert _lib.lib().slu_ulv_solve_noalloc(h, H._op, _lib.ptr(B), 24, 24, 0) == 0
        torch.cuda.synchronize()
        after_noalloc = _pool_used_bytes()
        assert _lib.lib().slu_ulv_solve(h, H._op, _lib.ptr(B2), 24, 24, 0) == 0
        torch.cuda.synchronize()
        after_solve = _pool_used_bytes()
    assert after_noalloc == before, (before, after_noalloc)
    assert after_solve > after_noalloc, (after_noalloc, after_solve)


def test_noalloc_rejects_oversize():
    need_gpu()
    from sslablu_gb300 import _lib
    H = _factored_hbs()
    N = H.shape[0]
    nrhs = (16 << 20) // (8 * N) + 1      # five buffers of N x nrhs cannot fit in 16 MiB
    import torch
    B = torch.zeros((N, nrhs), dtype=torch.float64, device="cuda")
    st = _lib.lib().slu_ulv_solve_noalloc(_lib.handle(), H._op, _lib.ptr(B), nrhs, nrhs, 0)
    assert st == 1   # SLU_ERR_ARG
    assert "limit" in _lib.last_error()
