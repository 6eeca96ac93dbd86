"""Matrix assembly of slab interface maps -- drop-in for SslabLU
matAssembly/matAssembler.py (the dense and rkHBS methods).

    matAssembler(matAssemblerOptions(method, tol, leaf_size, maxRank, ...))
        .assemble(stMap) -> dense ndarray (method 'dense')
                         -> HBStorch.HBSMAT on the GPU (method 'rkHBS')

rkHBS follows matAssembler.py:104-133 step for step: a binary slabTree of the
interface points ``stMap.XXI`` with ``leaf_size`` points per leaf, the sample
count s = max(2 maxRank, leaf_size) + maxRank + 10, Gaussian sketches Om then
Psi from numpy's global RNG, the samples Y = A Om and Z = A^T Psi through
the caller's operator ``stMap.A`` (evaluated wherever it lives), and the
compression HBSMAT.construct(maxRank, Om, Psi, Y, Z), which runs in
libslablu.  ``stats`` carries the sample / compression times and the bytes of
the result, as upstream.

'rkHBS_strong' (matAssembler.py:134-150) names a class upstream's
HBSnew_strong does not define, so upstream cannot run it; here it builds
the strong-admissibility HBStorch_strong.HBSMAT the way upstream's
test/rkprop/thinSlab3D.py drives it: the same slabTree (default 'partial'
adjacency), sketches Om then Psi from numpy's global RNG with thinSlab3D's
sample count s = 5 max(2 maxRank, leaf_size) + maxRank + 20.

Beyond upstream: ``matAssemblerOptions(precision='mixed')`` takes the samples
Y = A Om, Z = A^T Psi of an explicit matrix A (numpy or torch) on the
tcgen05 tensor cores (slu_gemm_split3: split-BF16x3 products, float32
accumulation, ~1e-7 relative -- below any rank truncation the compression
keeps); the default 'f64' evaluates them in float64 as upstream.

Not built: 'rkHBSold' (the legacy HBSTree) and 'epsHBS', which upstream
returns as a TypeError object rather than an operator -- kept as is.
"""
import time

import numpy as np

from .HBS import HBStorch
from .HBS import slabTree as _slabTree


def compute_c0_L0(XX):
    """matAssembler.py:21-33: centre and characteristic length of a cloud."""
    XX_np = XX.detach().cpu().numpy() if hasattr(XX, "detach") else np.asarray(XX)
    N = XX_np.shape[0]
    c0 = np.sum(XX_np, axis=0) / N
    L0 = np.max(np.max(XX_np, axis=0) - np.min(XX_np, axis=0))
    return c0, L0 + 1e-5


class matAssemblerOptions:
    """matAssembler.py:34-59."""

    def __init__(self, method="dense", tol=1e-5, leaf_size=8, maxRank=8, tree=None, ndim=3,
                 quad=False, reduced=False, precision="f64"):
        if precision not in ("f64", "mixed"):
            raise ValueError("precision must be 'f64' or 'mixed'")
        self.precision = precision
        self.method = method
        self.tol = tol
        self.maxRank = maxRank
        self.tree = tree
        self.leaf_size = leaf_size
        self.ndim = ndim
        self.reduced = reduced
        self.quad = quad


class matAssemblerStats:
    """matAssembler.py:60-69."""

    def __init__(self):
        self.timeSample = 0
        self.timeCompress = 0
        self.nbytes = 0


class matAssembler:
    """matAssembler.py:72-133."""

    def __init__(self, matOpts=None):
        self.matOpts = matOpts if matOpts is not None else matAssemblerOptions()
        self.nbytes = 0
        self.stats = matAssemblerStats()

    def assemble(self, stMap, dbg=0):
        linOp = stMap.A
        if dbg > 0:
            print("MAT ASSEMBLER METHOD=%s" % self.matOpts.method)
        method = self.matOpts.method
        if method == "dense":
            tic = time.time()
            M = linOp @ np.identity(linOp.shape[1])
            self.stats.timeSample = time.time() - tic
            self.stats.nbytes = M.nbytes
            return M
        if method == "epsHBS":
            return TypeError("epsHBS currently not implemented")
        if method == "rkHBS":
            quad = False   # binary trees only, as upstream
            opts = self.matOpts
            opts.tree = _slabTree.slabTree(stMap.XXI, quad, opts.leaf_size)
            device = "cuda"
            H = HBStorch.HBSMAT(device=device, tree=opts.tree, quad=quad)
            s = max(2 * opts.maxRank, opts.leaf_size) + opts.maxRank + 10
            Om = np.random.standard_normal((linOp.shape[0], s))
            Psi = np.random.standard_normal((linOp.shape[1], s))
            Y, Z = self._samples(linOp, Om, Psi)
            H.construct(opts.maxRank, Om, Psi, Y, Z)
            self.stats.timeSample = H.tSample   # upstream reports the set-up time only
            self.stats.nbytes = H.nbytes
            self.stats.timeCompress = H.tCompress
            if dbg > 0:
                print("\t Toc solve %d random pdes %.2e s" % (H.nSamples, self.stats.timeSample))
                print("\t Toc HBS construction %.2e s" % self.stats.timeCompress)
                print("\t HBS mem = %5.2f MB" % (self.stats.nbytes / 1e6))
            return H
        if method == "rkHBS_strong":
            from .HBS import HBStorch_strong
            opts = self.matOpts
            opts.tree = _slabTree.slabTree(stMap.XXI, False, opts.leaf_size)
            H = HBStorch_strong.HBSMAT(device="cuda", tree=opts.tree, quad=False)
            s = 5 * max(2 * opts.maxRank, opts.leaf_size) + opts.maxRank + 20
            Om = np.random.standard_normal((linOp.shape[0], s))
            Psi = np.random.standard_normal((linOp.shape[1], s))
            tic = time.time()
            Y, Z = self._samples(linOp, Om, Psi)
            self.stats.timeSample = time.time() - tic
            H.construct(opts.maxRank, Om, Psi, Y, Z)
            self.stats.nbytes = H.nbytes
            self.stats.timeCompress = H.tConstruct
            return H
        raise NotImplementedError("matAssembler method %r is not built" % method)

    def _samples(self, linOp, Om, Psi):
        """Y = A Om, Z = A^T Psi: through the caller's operator, or for an
        explicit matrix with precision 'mixed' on the tensor cores."""
        import torch
        explicit = isinstance(linOp, np.ndarray) or isinstance(linOp, torch.Tensor)
        if self.matOpts.precision == "mixed" and explicit:
            from .. import _dev as dv
            from .. import _lib as L
            A = dv.to_dev(linOp).contiguous()
            out = []
            for M, X in ((A, Om), (A.T.contiguous(), Psi)):
                Xd = dv.to_dev(X).contiguous()
                R = torch.empty((M.shape[0], Xd.shape[1]), dtype=torch.float64, device="cuda")
                L.check(L.lib().slu_gemm_split3(L.handle(), M.shape[0], Xd.shape[1], M.shape[1],
                                                1.0, L.ptr(M), M.shape[1], L.ptr(Xd), Xd.shape[1],
                                                0.0, L.ptr(R), R.shape[1]))
                out.append(R)
            L.sync()
            return out[0], out[1]
        return linOp @ Om, linOp.T @ Psi


class denseMatAssembler(matAssembler):
    def __init__(self):
        super().__init__(matAssemblerOptions())


class rkHMatAssembler(matAssembler):
    def __init__(self, leaf_size, rk, tree=None, ndim=3, quad=False):
        super().__init__(matAssemblerOptions("rkHBS", 0, leaf_size, rk, tree, ndim, quad))


class rkHMatAssembler_strong(matAssembler):
    """matAssembler.py:220-222."""

    def __init__(self, leaf_size, rk, tree=None, ndim=3, quad=False):
        super().__init__(matAssemblerOptions("rkHBS_strong", 0, leaf_size, rk, tree, ndim, quad))


class tolHMatAssembler(matAssembler):
    def __init__(self, tol, leaf_size, rk, ndim=3):
        super().__init__(matAssemblerOptions("epsHBS", tol, leaf_size, rk, ndim))
