"""Slab source-target maps and the interface operator on the GPU.

Drop-in for the operators upstream's overlapping multislab driver builds
(multislab/oms.py): ``oms.compute_stmaps`` (96-125) wraps each double slab's
maps S_l, S_r = (A_ii^{-1} A_ib[:, J])[Ic, :] as ``stMap`` linear operators
(solver/solver.py:30-37) for the matrix assembler, and
``construct_Stot_and_rhstot_linearOperator`` (258-302) applies the interface
system Stot x = x + sum of the couplings.  Here the slab solves run in
libslablu (``slu_slab_maps_apply``: Chebyshev iterations on -A_ii, every
slab and right-hand side at once), for the stencil discretisation of
solver/stencil/stencilSolver.py with c11 = c22 (= c33) = 1 and a zeroth-order
term kappa^2 c(x): the 2-D Laplace slabs of the C1 family and the 3-D
variable-coefficient Helmholtz slabs of C3.

Geometry: [0,1]^d cut into ``nslabs`` slabs of width H = 1/nslabs (upstream's
geometry.geom_2D.square.dSlabs / geometry.geom_3D.cube.dSlabs): double slab s
spans [s H, (s + 2) H] and carries interface s + 1 on its centre plane, so
there are nslabs - 1 interfaces of m = (ny - 2)(nz - 2) points each.
"""
import ctypes

import numpy as np
import torch

from .. import _dev as dv
from .. import _lib as L


class SlabGeometry:
    """Stencil grid of every double slab: ``nx`` points across a double slab
    (odd), ``ny`` (and ``nz``; 0 in 2-D) along the interface."""

    def __init__(self, nslabs, nx, ny, nz=0, kappa=0.0, coef=0):
        if nx % 2 == 0 or nx < 3:
            raise ValueError("nx must be odd and >= 3")
        self.nslabs, self.nx, self.ny, self.nz = int(nslabs), int(nx), int(ny), int(nz)
        self.kappa, self.coef = float(kappa), int(coef)
        self.H = 1.0 / nslabs
        self.width = 2.0 * self.H
        self.m = (ny - 2) * (nz - 2 if nz else 1)
        self.nif = nslabs - 1

    def x0(self, slabs=None):
        idx = np.arange(self.nif) if slabs is None else np.asarray(slabs)
        return (idx * self.H).astype(np.float64)

    def points(self, slab=0):
        """The points of interface ``slab`` (x = (slab + 1) H) in the stMap
        XXI order of upstream (XXi[Ic]: z fastest), one row per point."""
        ys = np.linspace(0.0, 1.0, self.ny)[1:-1]
        xc = (slab + 1) * self.H
        if not self.nz:
            return np.stack([np.full(ys.size, xc), ys], axis=1)
        zs = np.linspace(0.0, 1.0, self.nz)[1:-1]
        Y, Z = np.meshgrid(ys, zs, indexing="ij")
        return np.stack([np.full(Y.size, xc), Y.ravel(), Z.ravel()], axis=1)


class SlabMaps:
    """The maps of a set of double slabs (all interfaces by default)."""

    def __init__(self, geom, slabs=None, tol=1e-14):
        self.g = geom
        self.slabs = np.arange(geom.nif) if slabs is None else np.asarray(slabs)
        self.tol = float(tol)
        self.steps = 0

    def _call(self, XL, XR, YL, YR, ncols, trans):
        g = self.g
        x0 = self.g.x0(self.slabs)
        steps = ctypes.c_int(0)
        ld = ncols
        L.check(L.lib().slu_slab_maps_apply(
            L.handle(), g.nx, g.ny, g.nz, g.width, g.kappa, g.coef, len(self.slabs),
            x0.ctypes.data_as(ctypes.c_void_p), L.ptr(XL), L.ptr(XR), ld, L.ptr(YL), L.ptr(YR),
            ld, ncols, 1 if trans else 0, self.tol, ctypes.byref(steps)))
        self.steps = steps.value

    def apply(self, XL=None, XR=None):
        """Y_s = S_l(s) XL_s + S_r(s) XR_s for every slab of the set: device
        tensors of (len(slabs) * m) x c (XL or XR may be None)."""
        X = XL if XL is not None else XR
        c = X.shape[1]
        Y = torch.empty((len(self.slabs) * self.g.m, c), dtype=torch.float64, device="cuda")
        XL = XL.contiguous() if XL is not None else None
        XR = XR.contiguous() if XR is not None else None
        self._call(XL, XR, Y, None, c, False)
        return Y

    def apply_t(self, X, left=True, right=True):
        """(S_l(s)^T X_s, S_r(s)^T X_s) for every slab of the set."""
        X = X.contiguous()
        c = X.shape[1]
        shape = (len(self.slabs) * self.g.m, c)
        YL = torch.empty(shape, dtype=torch.float64, device="cuda") if left else None
        YR = torch.empty(shape, dtype=torch.float64, device="cuda") if right else None
        self._call(X, None, YL, YR, c, True)
        return YL, YR


class SlabMapOperator:
    """One map S_l or S_r of one double slab as a linear operator (.shape,
    .matmat, .rmatmat, .T, @), the ``stMap.A`` of oms.compute_stmaps
    (multislab/oms.py:117-125); numpy in -> numpy out, CUDA in -> CUDA out."""

    def __init__(self, geom, slab, side, tol=1e-14, transpose=False):
        self.g, self.slab, self.side = geom, int(slab), side
        self.maps = SlabMaps(geom, [slab], tol)
        self.shape = (geom.m, geom.m)
        self.dtype = np.float64
        self._t = transpose

    @property
    def T(self):
        return SlabMapOperator(self.g, self.slab, self.side, self.maps.tol, not self._t)

    def _apply(self, v, trans):
        X, one = dv.prepare_rhs(v)
        if not trans:
            Y = self.maps.apply(X if self.side == "l" else None, X if self.side == "r" else None)
        else:
            YL, YR = self.maps.apply_t(X, self.side == "l", self.side == "r")
            Y = YL if self.side == "l" else YR
        return dv.finish(Y, v, one)

    def matmat(self, v):
        return self._apply(v, self._t)

    def rmatmat(self, v):
        return self._apply(v, not self._t)

    matvec = matmat
    rmatvec = rmatmat

    def __matmul__(self, v):
        return self.matmat(v)


class stMap:
    """solver/solver.py:30-37: an operator with its source / target points."""

    def __init__(self, A, XXI, XXJ, m_large=0, n_large=0):
        self.XXI, self.XXJ, self.A = XXI, XXJ, A
        self.m_large, self.n_large = m_large, n_large


def slab_stmaps(geom, tol=1e-14):
    """Per interface i: (st_l, st_r) of double slab i as stMaps (None where the
    slab's edge is the global boundary), the inputs of the assembler loop of
    construct_Stot_helper (multislab/oms.py:159-240)."""
    out = []
    for i in range(geom.nif):
        pts = geom.points(i)
        st_l = stMap(SlabMapOperator(geom, i, "l", tol), pts, pts) if i > 0 else None
        st_r = stMap(SlabMapOperator(geom, i, "r", tol), pts, pts) if i < geom.nif - 1 else None
        out.append((st_l, st_r))
    return out


class StotOperator:
    """The interface system Stot x = x + S_l(i) x_{i-1} + S_r(i) x_{i+1}
    (construct_Stot_and_rhstot_linearOperator, multislab/oms.py:258-302),
    applied matrix-free through the slab solves in float64: every slab of
    every column in one batched call.  Operates on (nif * m) x c device
    tensors (or numpy, returned as numpy)."""

    def __init__(self, geom, tol=1e-14):
        self.g = geom
        self.maps = SlabMaps(geom, None, tol)
        n = geom.nif * geom.m
        self.shape = (n, n)
        self.dtype = np.float64

    def _shifted(self, X):
        m, n = self.g.m, self.g.nif
        Xv = X.view(n, m, -1)
        XL = torch.zeros_like(Xv)
        XR = torch.zeros_like(Xv)
        XL[1:] = Xv[:-1]
        XR[:-1] = Xv[1:]
        return XL.view(n * m, -1), XR.view(n * m, -1)

    def dev_matmat(self, X):
        XL, XR = self._shifted(X)
        return X + self.maps.apply(XL, XR)

    def dev_rmatmat(self, X):
        m, n = self.g.m, self.g.nif
        YL, YR = self.maps.apply_t(X)
        YL, YR = YL.view(n, m, -1), YR.view(n, m, -1)
        out = X.clone().view(n, m, -1)
        out[:-1] += YL[1:]       # S_l(i)^T acts on interface i - 1
        out[1:] += YR[:-1]       # S_r(i)^T acts on interface i + 1
        return out.view(n * m, -1)

    def matmat(self, v):
        X, one = dv.prepare_rhs(v)
        return dv.finish(self.dev_matmat(X), v, one)

    def rmatmat(self, v):
        X, one = dv.prepare_rhs(v)
        return dv.finish(self.dev_rmatmat(X), v, one)

    matvec = matmat
    rmatvec = rmatmat

    def __matmul__(self, v):
        return self.matmat(v)
