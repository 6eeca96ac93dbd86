"""sslablu_gb300: GB300-native slab direct-solve path of SslabLU.

Drop-in mirrors of the upstream hot-path modules, running hand-written sm_103a
CUDA through libslablu.so (include/slablu.h):

    sslablu_gb300.matAssembly.HBS.HBSnew      HBSMAT (randomized HBS compression,
                                               apply, ULV solve)
    sslablu_gb300.matAssembly.HBS.ULVsparse   compute_ULV / solve
    sslablu_gb300.direct_solve.omsdirectsolve      RedBlackSolver, BlockTridiagonalSolver
    sslablu_gb300.direct_solve.omsdirectsolveHBS   RedBlackSolverHBS, ThomasSolverHBS, linops
    sslablu_gb300.multislab.omsdirectsolve[HBS]    functional Thomas solvers

numpy inputs give numpy outputs (as upstream); CUDA tensors stay on the device.
"""
__version__ = "0.1.0"
