"""CPU oracle for the slab direct-solve path -- TEST INFRASTRUCTURE ONLY.

This package restates, in vectorised numpy, the algorithms of SslabLU's
HBS compression (matAssembly/HBS/HBSnew.py), ULV factorisation and solve
(matAssembly/HBS/ULVsparse.py) and the block-tridiagonal direct solvers
(direct_solve/omsdirectsolve.py, direct_solve/omsdirectsolveHBS.py,
multislab/omsdirectsolve.py).  Every function cites the upstream file:line it
follows.  Dense kernels (QR, SVD, pinv, LU) call the same LAPACK routines
through numpy/scipy that upstream calls, so the oracle reproduces upstream
results to rounding.

Parity is pinned: tests/golden/*.npz were produced by running the upstream
modules themselves (tests/golden/make_golden.py) and tests/test_oracle_golden.py
checks this restatement against them.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this package.  The product (sslablu_gb300) never does.
"""
