"""RB-HBS-preconditioned GMRES on the interface operator, all on the GPU:
upstream's iterative interface solve (test/3D/cubeTest.py:158-186 with
multislab/oms.py:258-302): Stot applied matrix-free through the slab solves,
the maps compressed by the rkHBS assembler (matAssembly/matAssembler.py:
104-133) into the preconditioner RedBlackSolverHBS.  The solution must reach
a 1e-10 relative residual and match the dense solve of the system assembled
from the CPU oracle's maps (pinned to upstream) to 1e-9."""
import numpy as np
import pytest

from tests._cases import relerr
from tests._gpu import need_gpu

pytestmark = pytest.mark.gpu


def test_rbhbs_preconditioned_gmres_c1_layout():
    need_gpu()
    import torch
    from oracle.slabmaps import poisson2d_couplings
    from sslablu_gb300.direct_solve.omsdirectsolveHBS import RedBlackSolverHBS
    from sslablu_gb300.matAssembly.matAssembler import rkHMatAssembler
    from sslablu_gb300.multislab.gmres import gmres
    from sslablu_gb300.multislab.slabmaps import SlabGeometry, StotOperator, slab_stmaps
    g = SlabGeometry(9, 17, 66)            # 8 interfaces of 64 points
    m, n = g.m, g.nif
    np.random.seed(3)
    asm = rkHMatAssembler(16, 8)
    S_rk = []
    for i, (st_l, st_r) in enumerate(slab_stmaps(g)):
        row = []
        if st_l is not None:
            row.append(asm.assemble(st_l))
        if st_r is not None:
            row.append(asm.assemble(st_r))
        S_rk.append(row)
    tree = S_rk[0][0].tree
    rb = RedBlackSolverHBS(m, 8, tree, False)
    rb.factorize(S_rk)
    St = StotOperator(g)
    B = np.random.default_rng(5).standard_normal((n * m, 4))
    X, it, rel = gmres(St.dev_matmat, torch.from_numpy(B).cuda(), rb.solve, tol=1e-10)
    X = X.cpu().numpy()
    assert rel <= 1e-10 and 1 <= it <= 60
    C = poisson2d_couplings(m, 9, 17)
    M = np.eye(n * m)
    for i in range(n):
        if i > 0:
            M[i * m:(i + 1) * m, (i - 1) * m:i * m] = C[i][0]
        if i < n - 1:
            M[i * m:(i + 1) * m, (i + 1) * m:(i + 2) * m] = C[i][1]
    res = np.linalg.norm(B - M @ X, axis=0) / np.linalg.norm(B, axis=0)
    assert res.max() <= 2e-10
    assert relerr(X, np.linalg.solve(M, B)) < 1e-9
    # without a preconditioner GMRES needs more steps for the same residual
    X2, it2, rel2 = gmres(St.dev_matmat, torch.from_numpy(B).cuda(), None, tol=1e-10)
    assert rel2 <= 1e-10 and it2 > it
