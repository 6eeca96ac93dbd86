"""Functional HBS Thomas solver on the GPU -- drop-in for SslabLU
multislab/omsdirectsolveHBS.py.

    Sprime_Linop(Sl, Sprime_prev, Sr, id=False)          (omsdirectsolveHBS.py:19-52)
    build_block_tridiagonal_solver(S_rk_list, tree, quad, rk)   (58-101)
    block_tridiagonal_solve(OMS, T, rhs)                 (103-138)

Deliberate difference: upstream's transpose branch of Sprime_Linop
(omsdirectsolveHBS.py:45) applies Sprime_prev.solve without mode='T', so its
transposed sketches are wrong whenever S' is nonsymmetric.  This module uses
the transposed solve, as the direct_solve version of the same operator does
(direct_solve/omsdirectsolveHBS.py:134); for symmetric S' both agree.
"""
import torch

from .. import _dev as dv
from ..direct_solve.omsdirectsolveHBS import Sprime_Linop, id_op  # noqa: F401
from ..matAssembly.HBS import HBSnew


def build_block_tridiagonal_solver(S_rk_list, tree, quad, rk):
    m = int(S_rk_list[0][0].shape[0])
    n = len(S_rk_list) - 1
    I = id_op(m)
    Sl = [S_rk_list[i][0] for i in range(1, n + 1)]
    Sr = [S_rk_list[i][-1] for i in range(n)]
    Sp = [I]
    for i in range(1, n + 1):
        op = (Sprime_Linop(Sl[0], I, Sr[0], id=True) if i == 1
              else Sprime_Linop(Sl[i - 1], Sp[i - 1], Sr[i - 1]))
        h = HBSnew.HBSMAT(op, tree, quad)
        h.construct(rk, compute_ULV=True)
        Sp.append(h)
    return Sl, Sp, Sr


def block_tridiagonal_solve(OMS, T, rhs):
    Sl, Sp, Sr = T
    n = len(Sl)
    idx = [slice(r.start, r.stop) if isinstance(r, range) else r for r in OMS.glob_target_dofs]
    d, one = dv.prepare_rhs(rhs)
    d = d.clone()
    for i in range(1, n + 1):
        if i == 1:
            d[idx[i]] -= dv.dev_apply(Sl[0], d[idx[0]])
        else:
            d[idx[i]] -= dv.dev_apply(Sl[i - 1], dv.dev_solve(Sp[i - 1], d[idx[i - 1]]))
    x = torch.zeros_like(d)
    x[idx[n]] = dv.dev_solve(Sp[n], d[idx[n]])
    for i in range(n - 1, 0, -1):
        x[idx[i]] = dv.dev_solve(Sp[i], d[idx[i]] - dv.dev_apply(Sr[i], x[idx[i + 1]]))
    x[idx[0]] = d[idx[0]] - dv.dev_apply(Sr[0], x[idx[1]])
    return dv.finish(x, rhs, one)
