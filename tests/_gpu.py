"""Helpers for the GPU parity tests (skip when no CUDA device)."""
import pytest

torch = pytest.importorskip("torch")


def need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sslablu_gb300 import _lib
    _lib.lib()  # raises if libslablu.so is missing: no silent fallback
