"""ULV factorisation and solve of HBS matrices on the GPU -- drop-in for the
public functions of SslabLU matAssembly/HBS/ULVsparse.py.

    compute_ULV(Umats, Dmats, Vmats, Nbvec) -> Qlist, Wlist, Uulist, Rlist, NNvec
                                                        (ULVsparse.py:231-293)
    solve(Umats, Dmats, Qlist, Wlist, Uulist, Rlist, NNvec, Nbvec, rhs, mode='N')
                                                        (ULVsparse.py:295-358)

Factors are the upstream stacked block lists (level 0 = leaves).  Both run in
libslablu (slu_ulv_factor, slu_hbs_set_ulv_level + slu_ulv_solve); numpy
lists come back as numpy arrays.  The right-hand side is in tree (block)
order, as upstream's solve expects.
"""
import ctypes

import numpy as np

from ... import _dev as dv
from ... import _lib as L
from .HBSnew import HBSMAT


def _levels(Dmats, Umats, Nbvec):
    out = []
    Lv = len(Dmats)
    for t in range(Lv):
        Nb = int(Nbvec[t])
        n = int(Dmats[t].shape[0]) // Nb
        k = int(Umats[t].shape[1]) if t < Lv - 1 else 0
        out.append((Nb, n, k))
    return out


def _fac(Nbvec):
    """Children per box: the ratio of consecutive block counts, as upstream
    derives it (ULVsparse.py:120, 143: NbB // NbA); 2 for a one-level tree."""
    return int(Nbvec[0]) // int(Nbvec[1]) if len(Nbvec) > 1 else 2


def compute_ULV(Umats, Dmats, Vmats, Nbvec):
    """ULV factors of given HBS factors (ULVsparse.py:231-293); binary or
    quad trees."""
    H = HBSMAT().set_mats(Umats, Dmats, Vmats, list(Nbvec), fac=_fac(Nbvec))
    H.compute_ULV()
    Lv = len(Dmats)
    Uulist = [H._export(6, t) for t in range(Lv - 1)]
    return H.Qlist, H.Wlist, Uulist, H.Rlist, H.NNvec.copy()


def solve(Umats, Dmats, Qlist, Wlist, Uulist, Rlist, NNvec, Nbvec, rhs, mode="N"):
    """ULV solve with given factors (ULVsparse.py:295-358)."""
    if mode not in ("N", "T"):
        raise NotImplementedError("mode not recognized")
    Lv = len(Dmats)
    N = int(Dmats[0].shape[0])
    geo = _levels(Dmats, Umats, Nbvec)
    H = HBSMAT()
    H.fac = _fac(Nbvec)
    H.shape = (N, N)
    H.perm = np.arange(N, dtype=np.int64)
    H._new_op(N, Lv, None)
    h = L.handle()
    keep = []
    for t, (Nb, n, k) in enumerate(geo):
        D = dv.to_dev(Dmats[t])
        U = dv.to_dev(Umats[t]) if t < Lv - 1 else None
        keep += [D, U]
        L.check(L.lib().slu_hbs_set_level(h, H._op, t, Nb, n, k, L.ptr(U), None, L.ptr(D)))
    for t, (Nb, n, k) in enumerate(geo):
        Q = dv.to_dev(Qlist[t])
        R = dv.to_dev(Rlist[t])
        W = dv.to_dev(Wlist[t]) if t < Lv - 1 else None
        Uu = dv.to_dev(Uulist[t]) if t < Lv - 1 else None
        keep += [Q, R, W, Uu]
        L.check(L.lib().slu_hbs_set_ulv_level(h, H._op, t, L.ptr(Q), L.ptr(W), L.ptr(R),
                                              L.ptr(Uu)))
    X, one = dv.prepare_rhs(rhs)
    X = X.clone()
    L.check(L.lib().slu_ulv_solve(h, H._op, L.ptr(X), X.shape[1], X.shape[1], int(mode == "T")))
    L.sync()
    return dv.finish(X, rhs, one)
