"""ctypes binding of libwbgpu.so (the C ABI declared in include/wbgpu.h).

The shared library is the only compute path: if it is missing or cannot be
loaded, every distance call raises ``RuntimeError`` (there is no CPU
fallback).  Build it with ``python -c "import __graft_entry__ as g; g.build()"``
or ``python wildboar_gb300/_build.py``.
"""

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwbgpu.so")

WB_OK = 0
WB_EINVAL = 1
WB_ENOMEM = 2
WB_ECUDA = 3
WB_ETIMEOUT = 4
WB_EUNSUPPORTED = 5

WB_F64 = 0
WB_F32 = 1


class Series(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("n", ctypes.c_int64),
        ("n_dims", ctypes.c_int64),
        ("n_timestep", ctypes.c_int64),
        ("dtype", ctypes.c_int32),
        ("on_device", ctypes.c_int32),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("r", ctypes.c_double),
        ("g", ctypes.c_double),
        ("p", ctypes.c_double),
        ("epsilon", ctypes.c_double),
        ("c", ctypes.c_double),
        ("penalty", ctypes.c_double),
        ("stiffness", ctypes.c_double),
    ]


_lib = None
_lock = threading.Lock()


def _declare(L):
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    i64 = ctypes.c_int64
    i32 = ctypes.c_int32
    L.wb_pairwise_distance.argtypes = [P(Series), P(Series), i64, i32, P(Params), vp, i32, vp]
    L.wb_paired_distance.argtypes = [P(Series), P(Series), i64, i32, P(Params), vp, i32, vp]
    L.wb_argmin_distance.argtypes = [P(Series), P(Series), i64, i32, P(Params), i64, vp, vp,
                                     vp, i32, vp]
    L.wb_pairwise_subsequence_distance.argtypes = [vp, vp, vp, vp, vp, i64, P(Series), i64,
                                                   i32, P(Params), vp, vp, i32, vp]
    L.wb_paired_subsequence_distance.argtypes = [vp, vp, vp, vp, vp, i64, P(Series), i64,
                                                 i32, P(Params), vp, vp, i32, vp]
    L.wb_argmin_subsequence_distance.argtypes = [vp, vp, i64, i64, vp, vp, P(Series), i64,
                                                 i32, P(Params), i32, i64, vp, vp, i32, vp]
    L.wb_subsequence_profile.argtypes = [vp, vp, vp, vp, vp, i64, P(Series), i64, i32,
                                         P(Params), vp, vp, i64, i32, i32, vp]
    L.wb_subsequence_profile_stop.argtypes = [vp, vp, vp, vp, vp, i64, P(Series), i64, vp,
                                              vp, i64, i32, vp]
    L.wb_inject_fault.argtypes = [i32, i64]
    L.wb_last_error.restype = ctypes.c_char_p
    L.wb_version.restype = i32
    L.wb_release_workspace.argtypes = [vp]
    L.wb_launch_count.restype = i64
    L.wb_profile_enable.argtypes = [i32]
    L.wb_profile_last.argtypes = [P(ctypes.c_double)]
    L.wb_alu_probe.argtypes = [i32, i32, P(ctypes.c_double)]
    for name in _OPTIONAL:
        if hasattr(L, name):
            _OPTIONAL[name](L)
    for name, argtypes in _EXTRA_DECLS.items():
        fn = getattr(L, name, None)
        if fn is not None:
            fn.argtypes = argtypes
    for name, restype in _EXTRA_RESTYPES.items():
        fn = getattr(L, name, None)
        if fn is not None:
            fn.restype = restype


# entry points added by later modules register their ctypes signatures here
_OPTIONAL = {}
_EXTRA_DECLS = {}
_EXTRA_RESTYPES = {}


def declare(name, argtypes, restype=None):
    _EXTRA_DECLS[name] = argtypes
    if restype is not None:
        _EXTRA_RESTYPES[name] = restype
    if _lib is not None:
        fn = getattr(_lib, name, None)
        if fn is not None:
            fn.argtypes = argtypes
            if restype is not None:
                fn.restype = restype


def lib():
    """The loaded library; raises RuntimeError when it is unavailable."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise RuntimeError(
                        "libwbgpu.so is not built: run `python wildboar_gb300/_build.py` "
                        "(nvcc, sm_103a); wildboar_gb300 has no CPU fallback"
                    )
                L = ctypes.CDLL(LIB_PATH)
                _declare(L)
                _lib = L
    return _lib


def check(status):
    if status == WB_OK:
        return
    msg = lib().wb_last_error().decode("utf-8", "replace")
    if status == WB_EINVAL:
        raise ValueError(msg)
    if status == WB_ENOMEM:
        raise MemoryError(msg)
    if status == WB_EUNSUPPORTED:
        raise NotImplementedError(msg)
    if status == WB_ETIMEOUT:
        raise TimeoutError(msg)
    raise RuntimeError(msg)


FAULT_NONE, FAULT_RESERVE, FAULT_LAUNCH, FAULT_WAIT = 0, 1, 2, 3


def inject_fault(site, skip=0):
    """Arm a host-side fault that fires once (wb_inject_fault); site 0 disarms."""
    check(lib().wb_inject_fault(int(site), int(skip)))


def launch_count():
    return int(lib().wb_launch_count())


def profile_enable(on=True):
    check(lib().wb_profile_enable(1 if on else 0))


def profile_last_ms():
    v = ctypes.c_double()
    check(lib().wb_profile_last(ctypes.byref(v)))
    return v.value


def alu_probe(dtype=WB_F64, iters=4096):
    v = ctypes.c_double()
    check(lib().wb_alu_probe(dtype, iters, ctypes.byref(v)))
    return v.value


# --------------------------------------------------------------------------
# arrays: numpy (host) or torch CUDA tensors (device)

def is_torch_cuda(a):
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(a, torch.Tensor) and a.is_cuda


def current_stream_handle():
    """cudaStream_t of torch's current stream, or NULL (legacy default)."""
    try:
        import torch

        if torch.cuda.is_available() and torch.cuda.is_initialized():
            return torch.cuda.current_stream().cuda_stream
    except Exception:  # pragma: no cover
        pass
    return None


def series_from_numpy(a, dtype=WB_F64):
    """Series view of a C-contiguous (n, d, L) numpy array (kept alive by caller)."""
    assert a.ndim == 3 and a.flags["C_CONTIGUOUS"]
    s = Series()
    s.data = a.ctypes.data if a.size else None
    s.n, s.n_dims, s.n_timestep = a.shape
    s.dtype = dtype
    s.on_device = 0
    return s


def series_from_torch(t):
    import torch

    assert t.dim() == 3 and t.is_contiguous() and t.is_cuda
    s = Series()
    s.data = t.data_ptr() if t.numel() else None
    s.n, s.n_dims, s.n_timestep = t.shape
    s.dtype = WB_F64 if t.dtype == torch.float64 else WB_F32
    s.on_device = 1
    return s


def ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()
