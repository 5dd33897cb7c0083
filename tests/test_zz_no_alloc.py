"""wb_pairwise_distance_noalloc against wb_pairwise_distance, through the C ABI.

The no-allocation entry point exists for callers that cannot let a library
allocate device memory (memory reserved and accounted up front, or a loop in
which a device-synchronising cudaMalloc/cudaFree is not allowed).  Bands that
fit in shared memory need no scratch; wider ones use a static device array,
so this file checks that two calls in a row -- the second reusing the array
the first one left behind -- give bit for bit the results of the allocating
entry point, on narrow and wide bands, univariate and multivariate input, and
that oversize problems and unsupported metrics are rejected.
It runs last (file name) and does not depend on any other test.
"""

import ctypes
import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from wildboar_gb300 import _build, _lib  # noqa: E402


_build.build()
L = _lib.lib()
L.wb_pairwise_distance_noalloc.argtypes = [
    ctypes.POINTER(_lib.Series), ctypes.POINTER(_lib.Series), ctypes.c_int64,
    ctypes.c_int32, ctypes.POINTER(_lib.Params), ctypes.c_void_p, ctypes.c_void_p,
]
L.wb_noalloc_scratch_bytes.restype = ctypes.c_int64

IDS = {"euclidean": 0, "dtw": 1, "wdtw": 2, "adtw": 5, "lcss": 6, "wlcss": 7, "edr": 8,
       "erp": 9, "msm": 10, "twe": 11}


def _params(**kw):
    p = _lib.Params()
    p.r = kw.get("r", 1.0)
    p.g = kw.get("g", 0.05)
    p.p = kw.get("p", 1.0)
    p.epsilon = kw.get("epsilon", float("nan"))
    p.c = kw.get("c", 1.0)
    p.penalty = kw.get("penalty", 1.0)
    p.stiffness = kw.get("stiffness", 0.001)
    return p


def _series(t):
    t = t.reshape(t.shape[0], 1, t.shape[-1]) if t.dim() == 2 else t
    return _lib.series_from_torch(t.contiguous()), t


def _both(X, Y, metric, dim=0, **kw):
    sx, X3 = _series(X)
    sy, Y3 = (None, None) if Y is None else _series(Y)
    ny = X.shape[0] if Y is None else Y.shape[0]
    p = _params(**kw)
    stream = torch.cuda.current_stream().cuda_stream
    ref = torch.zeros((X.shape[0], ny), dtype=torch.float64, device="cuda")
    st = L.wb_pairwise_distance(ctypes.byref(sx), None if sy is None else ctypes.byref(sy),
                                dim, IDS[metric], ctypes.byref(p), ref.data_ptr(), 1, stream)
    _lib.check(st)
    outs = []
    for _ in range(2):
        out = torch.full((X.shape[0], ny), -1.0, dtype=torch.float64, device="cuda")
        st = L.wb_pairwise_distance_noalloc(
            ctypes.byref(sx), None if sy is None else ctypes.byref(sy), dim, IDS[metric],
            ctypes.byref(p), out.data_ptr(), stream)
        _lib.check(st)
        outs.append(out)
    torch.cuda.synchronize()
    return ref.cpu().numpy(), [o.cpu().numpy() for o in outs]


CASES = [
    ("dtw", (40, 33, 128, 128), {"r": 0.1}),
    ("dtw", (12, 9, 300, 300), {"r": 1.0}),
    ("dtw", (20, 17, 90, 61), {"r": 0.2}),
    ("wdtw", (25, 30, 100, 100), {"r": 0.3, "g": 0.2}),
    ("adtw", (16, 16, 80, 80), {"r": 0.5, "p": 0.4}),
    ("lcss", (18, 21, 70, 95), {"r": 0.3, "epsilon": 0.7}),
    ("wlcss", (10, 10, 60, 60), {"r": 1.0, "epsilon": 0.5}),
    ("edr", (14, 15, 88, 88), {"r": 0.2, "epsilon": 0.4}),
    ("msm", (22, 19, 77, 77), {"r": 0.15, "c": 0.5}),
    ("euclidean", (31, 29, 64, 64), {}),
    # a band ring too wide for shared memory: the static array
    ("dtw", (7, 5, 3000, 3000), {"r": 1.0}),
    ("wdtw", (6, 4, 2600, 2600), {"r": 1.0, "g": 0.01}),
]


@pytest.mark.parametrize("metric,shape,params", CASES)
def test_noalloc_matches_allocating_entry(metric, shape, params):
    nx, ny, lx, ly = shape
    rng = np.random.default_rng(zlib.crc32(repr((metric, shape)).encode()))
    X = torch.as_tensor(np.cumsum(rng.standard_normal((nx, lx)), axis=1), device="cuda")
    Y = torch.as_tensor(np.cumsum(rng.standard_normal((ny, ly)), axis=1), device="cuda")
    ref, outs = _both(X, Y, metric, **params)
    for out in outs:
        np.testing.assert_array_equal(out, ref)


def test_noalloc_singleton_path():
    rng = np.random.default_rng(5)
    X = torch.as_tensor(np.cumsum(rng.standard_normal((37, 70)), axis=1), device="cuda")
    ref, outs = _both(X, None, "dtw", r=0.2)
    for out in outs:
        np.testing.assert_array_equal(out, ref)
        assert np.all(np.diag(out) == 0.0)


def test_noalloc_multivariate_dim():
    # (n, 3, L) input, dim 2: series start at dim * L with stride 3 L
    rng = np.random.default_rng(6)
    X = torch.as_tensor(np.cumsum(rng.standard_normal((19, 3, 80)), axis=-1), device="cuda")
    Y = torch.as_tensor(np.cumsum(rng.standard_normal((11, 3, 80)), axis=-1), device="cuda")
    for metric, params in (("dtw", {"r": 0.1}), ("msm", {"r": 0.3})):
        ref, outs = _both(X, Y, metric, dim=2, **params)
        for out in outs:
            np.testing.assert_array_equal(out, ref)
    # dim 2 of the input is not dim 0
    ref0, _ = _both(X, Y, "dtw", dim=0, r=0.1)
    assert not np.array_equal(ref0, ref)


@pytest.mark.parametrize("metric,params,status,text", [
    ("erp", {"g": 0.1}, "WB_EUNSUPPORTED", b"not provided without allocation"),
    ("twe", {}, "WB_EUNSUPPORTED", b"not provided without allocation"),
    ("edr", {}, "WB_EINVAL", b"explicit edr epsilon"),
])
def test_noalloc_rejects_metrics_that_need_tables(metric, params, status, text):
    X = torch.zeros((3, 1, 16), dtype=torch.float64, device="cuda")
    sx, _ = _series(X)
    out = torch.empty((3, 3), dtype=torch.float64, device="cuda")
    p = _params(**params)
    st = L.wb_pairwise_distance_noalloc(ctypes.byref(sx), ctypes.byref(sx), 0, IDS[metric],
                                        ctypes.byref(p), out.data_ptr(), None)
    assert st == getattr(_lib, status)
    assert text in L.wb_last_error()


def test_noalloc_rejects_oversize_and_host_inputs():
    cap = L.wb_noalloc_scratch_bytes()
    # a full band of length Lx needs (Lx + 1) doubles per thread, 128 threads per block
    lx = cap // (128 * 8) + 8
    X = torch.zeros((1, lx), dtype=torch.float64, device="cuda")
    sx, _ = _series(X)
    out = torch.empty((1, 1), dtype=torch.float64, device="cuda")
    p = _params(r=1.0)
    st = L.wb_pairwise_distance_noalloc(ctypes.byref(sx), ctypes.byref(sx), 0, IDS["dtw"],
                                        ctypes.byref(p), out.data_ptr(), None)
    assert st == _lib.WB_EINVAL
    assert b"static scratch" in L.wb_last_error()
    host = np.zeros((2, 1, 8))
    sh = _lib.series_from_numpy(host)
    st = L.wb_pairwise_distance_noalloc(ctypes.byref(sh), ctypes.byref(sh), 0, IDS["dtw"],
                                        ctypes.byref(p), out.data_ptr(), None)
    assert st == _lib.WB_EINVAL
    assert b"device memory" in L.wb_last_error()
