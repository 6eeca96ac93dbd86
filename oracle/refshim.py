"""Import helper for the upstream SslabLU sources (test infrastructure only).

The upstream package imports several optional modules at module top that are
absent here (matplotlib, jax, tensorly) and two empty git submodules.  This
helper installs empty stand-ins in ``sys.modules`` and puts the upstream tree
on ``sys.path`` so that ``matAssembly.HBS.HBSnew``, ``matAssembly.HBS.ULVsparse``
and ``direct_solve.omsdirectsolve[HBS]`` import unmodified.  It is used only by
``tests/golden/make_golden.py`` (to freeze golden vectors) and by CPU tests that
cross-check the oracle when the upstream tree is present; nothing on the GPU
machine reads it.
"""
import os
import sys
import types

REF_ROOT = os.environ.get("SSLABLU_REF_ROOT", "/root/reference")


def available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, "matAssembly", "HBS", "HBSnew.py"))


def _stub(name, **attrs):
    if name in sys.modules:
        return sys.modules[name]
    m = types.ModuleType(name)
    m.__path__ = []  # behave like a package so submodules can be stubbed
    for k, v in attrs.items():
        setattr(m, k, v)
    sys.modules[name] = m
    parent, _, child = name.rpartition(".")
    if parent and parent in sys.modules:
        setattr(sys.modules[parent], child, m)
    return m


def install():
    """Install the stand-ins and return the upstream root (raises if absent)."""
    if not available():
        raise RuntimeError("upstream SslabLU tree not found at %s" % REF_ROOT)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", "")
    for name in ["matplotlib", "matplotlib.pyplot", "matplotlib.tri",
                 "jax", "jax.numpy", "tensorly", "tensorly.tenalg"]:
        _stub(name)
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    return REF_ROOT


def _install_pipeline_stubs():
    """Stand-ins for the two empty HPS submodules (solver.hpsmultidomain,
    solver.spectralmultidomain) and the missing simpleoctree, aliased to the
    upstream modules that provide the same names where one exists."""
    import importlib
    import solver  # noqa: F401  (upstream package, plain directory)
    import matAssembly.HBS  # noqa: F401
    for name in ["solver.hpsmultidomain", "solver.hpsmultidomain.hpsmultidomain",
                 "solver.hpsmultidomain.hpsmultidomain.domain_driver",
                 "solver.hpsmultidomain.hpsmultidomain.geom",
                 "solver.spectralmultidomain", "solver.spectralmultidomain.hps",
                 "solver.spectralmultidomain.hps.cheb_utils",
                 "matAssembly.HBS.simpleoctree", "matAssembly.HBS.simpleoctree.simpletree"]:
        _stub(name)
    pdo_mod = importlib.import_module("pdo.pdo")
    sys.modules["solver.hpsmultidomain.hpsmultidomain.pdo"] = pdo_mod
    sys.modules["solver.hpsmultidomain.hpsmultidomain"].pdo = pdo_mod
    su = importlib.import_module("solver.sparse_utils")
    sys.modules["solver.spectralmultidomain.hps.sparse_utils"] = su
    sys.modules["solver.spectralmultidomain.hps"].sparse_utils = su


def import_pipeline():
    """Return the upstream slab pipeline modules (oms, stencil solver, pdo,
    square and cube geometries, assemblers) as a namespace."""
    install()
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        _install_pipeline_stubs()
        import multislab.oms as oms
        import solver.solver as solver
        import pdo.pdo as pdo
        import geometry.geom_2D.square as square
        import geometry.geom_3D.cube as cube
        import matAssembly.matAssembler as matAssembler
        import matAssembly.HBS.slabTree as slabTree
    return types.SimpleNamespace(oms=oms, solver=solver, pdo=pdo, square=square, cube=cube,
                                 matAssembler=matAssembler, slabTree=slabTree)


def import_hot_path():
    """Return the upstream hot-path modules as a namespace."""
    install()
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        import matAssembly.HBS.ULVsparse as ULVsparse
        import matAssembly.HBS.HBSnew as HBSnew
        import direct_solve.omsdirectsolve as omsdirectsolve
        import direct_solve.omsdirectsolveHBS as omsdirectsolveHBS
    return types.SimpleNamespace(ULVsparse=ULVsparse, HBSnew=HBSnew,
                                 omsdirectsolve=omsdirectsolve,
                                 omsdirectsolveHBS=omsdirectsolveHBS)
