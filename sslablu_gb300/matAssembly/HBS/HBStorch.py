"""HBSMAT (torch variant) on the GPU -- drop-in for SslabLU
matAssembly/HBS/HBStorch.py, the engine of the rkHBS assembler.

Same constructor, methods and attribute layout as upstream HBStorch.HBSMAT
(HBStorch.py:85-492):
  * ``HBSMAT(A=None, device=None, tree=None, quad=False)``; a tree supplies
    ``perm_leaf``, ``nleaves`` and ``nlevels`` and fixes the shape;
  * ``construct(rk, Om, Psi, Y, Z, compute_ULV=False, fast=False)`` compresses
    from the caller's sketches (Om, Psi, Y = A Om, Z = A^T Psi, rows in the
    caller's ordering, permuted into tree order as upstream does,
    HBStorch.py:163-168);
  * factor lists ``Umats / Vmats / Dmats`` as (Nb, n, k) block tensors, leaves
    first, the root D on the host (HBStorch.py:230-239);
  * ``matmat / rmatmat / matvec / rmatvec / @ / T`` (354-457), numpy in ->
    numpy out, tensors stay tensors;
  * ``nbytes``, ``nSamples``, the timers.
The compression runs in libslablu with HBStorch's null-space rule
(``compute_UV`` projects each sketch block on every column of the complete Q
after the first n, HBStorch.py:73-82, which is valid for s < 2n as the
assembler's s = max(2k, leaf) + k + 10 requires); pseudo-inverses are taken
through the same QR (``fast`` selects between two formulations of that
pseudo-inverse upstream and is accepted here for compatibility).

Upstream defects not reproduced: HBStorch.compute_ULV calls
ULVsparse_torch.compute_ULV without its ``device`` argument and HBStorch.solve
passes Nbvec in place of the right-hand side (HBStorch.py:467-492); both
raise upstream.  Here ``compute_ULV()`` factors the stored operator and
``solve(b, device, mode)`` solves with it, with HBSnew.solve's permutation
convention for both modes.
"""
import time

import numpy as np
import torch

from ... import _dev as dv
from .HBSnew import HBSMAT as _HBSCore
from .HBSnew import samples_for


class HBSMAT(_HBSCore):
    _null_mode = 1   # HBStorch.compute_UV: Q[:, n:]

    def __init__(self, A=None, device=None, tree=None, quad=False):
        super().__init__(A=A, tree=None, quad=quad)
        self.device = device
        self.Nbvec = []
        if tree is not None:
            self.tree = tree
            self.perm = np.asarray(tree.perm_leaf, dtype=np.int64)
            self.Nb = int(tree.nleaves)
            self.nl = len(self.perm) // self.Nb
            self.L = int(tree.nlevels)
            self.shape = (len(self.perm), len(self.perm))

    def set_Nbvec(self, Nbvec):
        """HBStorch.py:132-137."""
        super().set_Nbvec(Nbvec)

    def set_mats(self, Umats, Dmats, Vmats, Nbvec, fac=4):
        """HBStorch.py:138-145; blocks given as (Nb, n, k) tensors or stacked
        (Nb*n, k) arrays, leaves first."""
        flat = [self._flat(m) for m in Dmats]
        return super().set_mats([self._flat(m) for m in Umats], flat,
                                [self._flat(m) for m in Vmats], list(Nbvec), fac=fac)

    @staticmethod
    def _flat(m):
        if isinstance(m, torch.Tensor):
            m = m.detach()
            return m.reshape(-1, m.shape[-1]).to(torch.float64)
        m = np.asarray(m, dtype=np.float64)
        return m.reshape(-1, m.shape[-1])

    # ------------------------------------------------------------ construction
    def construct(self, rk, Om=None, Psi=None, Y=None, Z=None, compute_ULV=False, fast=False):
        """HBStorch.py:155-159."""
        if compute_ULV:
            self.constructHBS_ULV(rk, fast=fast)
        else:
            self.constructHBS(rk, Om, Psi, Y, Z, fast=fast)

    def constructHBS(self, rk, Om0, Psi0, Y0, Z0, fast=False):
        """HBStorch.py:161-241: compression from given sketches."""
        tic = time.time()
        p = torch.from_numpy(self.perm).to("cuda")
        Om, Psi, Y, Z = (dv.to_dev(x)[p].contiguous() for x in (Om0, Psi0, Y0, Z0))
        self.setupTime += time.time() - tic
        self.tSample += time.time() - tic
        self.Nbvec = [int(self.Nb)]
        self.compress_from_sketches(rk, Om, Psi, Y, Z, compute_ULV=False)

    def constructHBS_ULV(self, rk, fast=False):
        """HBStorch.py:242-324: Gaussian sketches drawn on the device
        (torch.randn, as upstream), samples through the operator, compression
        with the interleaved ULV."""
        s = samples_for(rk, self.nl, self.fac)
        self.nSamples = s
        tic = time.time()
        N = self.shape[0]
        Om = torch.randn(N, s, dtype=torch.float64, device="cuda")
        Psi = torch.randn(N, s, dtype=torch.float64, device="cuda")
        p = torch.from_numpy(self.perm).to("cuda")
        Omp = torch.zeros_like(Om)
        Omp[p] = Om
        Psip = torch.zeros_like(Psi)
        Psip[p] = Psi
        Y = dv.dev_apply(self.A, Omp, False)[p].contiguous()
        Z = dv.dev_apply(self.A, Psip, True)[p].contiguous()
        self.setupTime += time.time() - tic
        self.tSample += time.time() - tic
        self.Nbvec = []
        self.compress_from_sketches(rk, Om, Psi, Y, Z, compute_ULV=True)

    # ------------------------------------------------------------ factors
    def _tens(self, what, t):
        Nb, n, k, nu = (int(x) for x in self._levels[t])
        arr = self._export(what, t)
        T = torch.from_numpy(np.ascontiguousarray(arr)).reshape(Nb, n, arr.shape[1])
        return T if (what == 2 and t == self.L - 1) else T.to("cuda")

    @property
    def Umats(self):
        return [self._tens(0, t) for t in range(self.L - 1)]

    @property
    def Vmats(self):
        return [self._tens(1, t) for t in range(self.L - 1)]

    @property
    def Dmats(self):
        return [self._tens(2, t) for t in range(self.L)]

    # ------------------------------------------------------------ solve
    def solve(self, b, device=None, mode="N"):
        """HBStorch.py:470-492 (intended semantics; see the module notes)."""
        return super().solve(b, mode=mode)
