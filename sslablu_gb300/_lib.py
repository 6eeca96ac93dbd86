"""ctypes binding of libslablu.so (the C ABI declared in include/slablu.h).

The library is the only compute path: if it is missing or no CUDA device is
present, `lib()` raises -- there is no CPU fallback.  torch provides device
memory and the stream: the default handle follows torch's current CUDA stream,
so library kernels and torch ops on that stream stay ordered.
"""
import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libslablu.so")

c_int, c_double, c_void_p, c_size_t, c_longlong = (ctypes.c_int, ctypes.c_double,
                                                    ctypes.c_void_p, ctypes.c_size_t,
                                                    ctypes.c_longlong)
P = c_void_p

# name -> argtypes (all return int status)
SIGNATURES = {
    "slu_version": [],
    "slu_last_error": [ctypes.c_char_p, c_size_t],
    "slu_create": [P, ctypes.POINTER(c_void_p)],
    "slu_destroy": [P],
    "slu_set_stream": [P, P],
    "slu_sync": [P],
    "slu_hbs_create": [P, c_int, c_int, c_int, P, ctypes.POINTER(c_void_p)],
    "slu_hbs_destroy": [P],
    "slu_hbs_compress": [P, P, c_int, c_int, c_int, P, P, P, P, c_int],
    "slu_hbs_set_level": [P, P, c_int, c_int, c_int, c_int, P, P, P],
    "slu_ulv_factor": [P, P],
    "slu_hbs_set_ulv_level": [P, P, c_int, P, P, P, P],
    "slu_hbs_apply": [P, P, c_int, P, c_int, P, c_int, c_int],
    "slu_ulv_solve": [P, P, P, c_int, c_int, c_int],
    "slu_ulv_solve_noalloc": [P, P, P, c_int, c_int, c_int],
    "slu_hbs_prepare_f32": [P, P],
    "slu_ulv_solve_f32": [P, P, P, c_int, c_int, c_int],
    "slu_refine": [P, P, P, c_int, P, c_int, c_int, c_double, c_int, P, P],
    "slu_ulv_solve_grouped": [P, c_int, P, P, P, P],
    "slu_hbs_set_null_space": [P, c_int],
    "slu_hbs_prepare_dfloat": [P, P],
    "slu_ulv_solve_dfloat": [P, P, P, c_int, c_int],
    "slu_ulv_solve_into": [P, P, P, c_int, P, c_int, c_int, c_int],
    "slu_ulv_solve_plan_create": [P, P, P, c_int, P, c_int, c_int, c_int, ctypes.POINTER(c_void_p)],
    "slu_ulv_solve_plan_launch": [P, P, c_int],
    "slu_ulv_solve_grouped_plan_create": [P, c_int, P, P, P, P, ctypes.POINTER(c_void_p)],
    "slu_refine_grouped_plan_create": [P, c_int, P, P, P, P, P, P, ctypes.POINTER(c_void_p)],
    "slu_refine_plan_run": [P, P, c_double, c_int, P, P],
    "slu_refine_plan_destroy": [P],
    "slu_ulv_solve_plan_destroy": [P],
    "slu_ulv_autotune": [P, P, c_int, c_int, c_int, P, c_int, P],
    "slu_hbs_set_refine_inner": [P, c_int],
    "slu_ulv_solve_timed": [P, P, P, c_int, c_int, P, P, P, c_int, P],
    "slu_hbs_apply_grouped": [P, c_int, P, P, P, P, P, P, P],
    "slu_refine_grouped": [P, c_int, P, P, P, P, P, P, c_double, c_int, P, P],
    "slu_hbs_info": [P, P, P, P, P, P],
    "slu_hbs_export": [P, P, c_int, c_int, P, c_size_t, P],
    "slu_hbs_nbytes": [P, c_int, P],
    "slu_lu_factor": [P, c_int, P, c_int, c_longlong, P, c_longlong, c_int, P],
    "slu_lu_solve": [P, c_int, c_int, P, c_int, c_longlong, P, c_longlong, P, c_int, c_longlong,
                     c_int, c_int],
    "slu_gemm_batched": [P, c_int, c_int, c_int, c_int, c_int, c_double, P, c_int, c_longlong, P,
                         c_int, c_longlong, c_double, P, c_int, c_longlong, c_int],
    "slu_gemm_split3": [P, c_int, c_int, c_int, c_double, P, c_int, P, c_int, c_double, P, c_int],
    "slu_rb_factor": [P, c_int, c_int, P, P, P, ctypes.POINTER(c_void_p)],
    "slu_rb_solve": [P, P, P, c_int, c_int],
    "slu_rb_factor_mixed": [P, c_int, c_int, P, P, P, ctypes.POINTER(c_void_p)],
    "slu_rb_refine": [P, P, P, c_int, P, c_int, c_int, c_double, c_int, P, P],
    "slu_rb_destroy": [P],
    "slu_thomas_factor": [P, c_int, c_int, P, P, P, ctypes.POINTER(c_void_p)],
    "slu_thomas_solve": [P, P, P, c_int, c_int],
    "slu_fp64_peak": [P, c_int, P, P],
    "slu_rb_factor_cyclic": [P, c_int, c_int, P, P, P, ctypes.POINTER(c_void_p)],
    "slu_rb_solve_tc": [P, P, P, c_int, c_int],
    "slu_slab_maps_apply": [P, c_int, c_int, c_int, c_double, c_double, c_int, c_int, P, P, P,
                            c_int, P, P, c_int, c_int, c_int, c_double, P],
    "slu_grouped_program_create": [P, c_int, P, P, P, P, P, P, P, P, ctypes.POINTER(c_void_p)],
    "slu_strong_create": [P, c_longlong, c_int, c_int, P, ctypes.POINTER(c_void_p)],
    "slu_strong_destroy": [P],
    "slu_strong_compress": [P, P, c_int, c_int, P, P, P, P, c_int, P, P, P],
    "slu_strong_apply": [P, P, c_int, P, c_int, P, c_int, c_int],
    "slu_strong_info": [P, c_int, c_int, ctypes.POINTER(c_longlong)],
    "slu_strong_export": [P, P, c_int, c_int, P],
    "slu_hbs_prepare_ozaki": [P, P],
    "slu_ulv_solve_ozaki": [P, P, P, c_int, P, c_int, c_int, c_int],
    "slu_hbs_apply_ozaki": [P, P, P, c_int, P, c_int, c_int, c_int],
}

ERRORS = {1: "bad argument", 2: "allocation failed", 3: "CUDA error", 4: "numerical failure",
          5: "bad state", 6: "not converged", 7: "device wait timed out"}


class SluError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libslablu error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


_lib = None
_lock = threading.Lock()


def load_cdll(path=LIB_PATH):
    """Load the shared library and attach the signatures (no GPU needed)."""
    if not os.path.exists(path):
        raise ImportError("libslablu.so not found at %s: build it with "
                          "`python -m sslablu_gb300.build` (CUDA toolkit required)" % path)
    dll = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        f = getattr(dll, name)
        f.argtypes = args
        f.restype = c_int
    dll.slu_launch_count.argtypes = []
    dll.slu_launch_count.restype = c_longlong
    dll.slu_set_blocking_waits.argtypes = [c_int]
    dll.slu_set_blocking_waits.restype = None
    return dll


def launch_count():
    return int(lib().slu_launch_count())


def lib():
    """The loaded library; raises if it or a CUDA device is unavailable."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                import torch
                if not torch.cuda.is_available():
                    raise RuntimeError("sslablu_gb300 needs a CUDA device (GB300, sm_103a); "
                                       "no CPU fallback exists")
                _lib = load_cdll()
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().slu_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status):
    if status != 0:
        raise SluError(status, last_error())


class _HandleCache(threading.local):
    def __init__(self):
        self.handles = {}


_handles = _HandleCache()


def handle():
    """Per-thread handle for torch's current device and stream (one handle per
    stream, so work on different streams never shares a scratch arena)."""
    import torch
    dev = torch.cuda.current_device()
    stream = torch.cuda.current_stream(dev).cuda_stream
    key = (dev, stream)
    h = _handles.handles.get(key)
    if h is None:
        out = c_void_p()
        check(lib().slu_create(c_void_p(stream), ctypes.byref(out)))
        h = out
        _handles.handles[key] = h
    return h


def sync():
    check(lib().slu_sync(handle()))


def ptr(t):
    """Device pointer of a torch tensor (None -> NULL)."""
    return c_void_p(0) if t is None else c_void_p(t.data_ptr())


def host_ptr(a):
    return a.ctypes.data_as(c_void_p)


def i64(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.int64))
