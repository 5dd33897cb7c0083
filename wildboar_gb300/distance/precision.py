"""Precision forms of the distance path (no counterpart in the reference).

* ``pairwise_euclidean_tc(x, y)`` -- the full-series euclidean matrix as
  |x|^2 + |y|^2 - 2 X Y^T with the dot products on the tensor cores (tcgen05,
  kind::tf32, 3xTF32 split, FP32 accumulation), see ``wb_euclidean_tc``.
* ``pairwise_dtw_fp32(x, y, r)`` -- dtw / wdtw with FP32 costs and compensated
  (TwoSum) accumulation, FP64 only for the final square root
  (``wb_dtw32_distance``).
* ``pairwise_distance_fp32(x, y, metric=..., metric_params=...)`` -- every
  elastic metric in FP32 with compensated accumulation, with the arguments,
  validation and output layout of ``pairwise_distance``
  (``wb_pairwise_distance_fp32``).

The first two take and return CUDA torch tensors; the third takes what
``pairwise_distance`` takes.
"""

import ctypes

import torch

from .. import _lib
from . import _distance
from . import batched as _b

_lib.declare("wb_euclidean_tc", [ctypes.POINTER(_lib.Series), ctypes.POINTER(_lib.Series),
                                 ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32,
                                 ctypes.c_void_p])


_lib.declare("wb_pairwise_distance_fp32",
             [ctypes.POINTER(_lib.Series), ctypes.POINTER(_lib.Series), ctypes.c_int64,
              ctypes.c_int32, ctypes.POINTER(_lib.Params), ctypes.c_void_p, ctypes.c_int32,
              ctypes.c_void_p])

ELASTIC = ("dtw", "wdtw", "ddtw", "wddtw", "adtw", "lcss", "wlcss", "edr", "erp", "msm",
           "twe")


def pairwise_distance_fp32(x, y=None, *, dim="mean", metric="dtw", metric_params=None):
    """``pairwise_distance`` of an elastic metric in FP32.

    Same arguments, validation and output (float64 values, shapes, squeezing)
    as ``pairwise_distance``; the recurrence runs on float32-rounded series
    with compensated (hi, lo) accumulation.  Relative error against the FP64
    distance is a few float32 ulps of the inputs' rounding (about 1e-7 to
    1e-6 for dtw-like metrics; lcss / edr counts are exact unless rounding
    moves a difference across epsilon).
    """
    if not isinstance(metric, str) or metric not in ELASTIC:
        raise ValueError("pairwise_distance_fp32 supports the elastic metrics %s, got %r"
                         % (", ".join(ELASTIC), metric))
    return _distance._pairwise(x, y, dim, metric, metric_params, "wb_pairwise_distance_fp32")


def _as3(t):
    if t.dim() == 1:
        t = t.reshape(1, 1, -1)
    elif t.dim() == 2:
        t = t.reshape(t.shape[0], 1, t.shape[1])
    # conversions only when needed (each costs a dispatch even as a no-op)
    if t.dtype != torch.float64:
        t = t.to(torch.float64)
    return t if t.is_contiguous() else t.contiguous()


def pairwise_euclidean_tc(x, y, *, dim=0):
    """(n_x, n_y) float64 euclidean distances of CUDA float64 series."""
    X = _as3(x)
    Y = _as3(y)
    out = torch.empty((X.shape[0], Y.shape[0]), dtype=torch.float64, device=X.device)
    sx = _lib.series_from_torch(X)
    sy = _lib.series_from_torch(Y)
    _lib.check(_lib.lib().wb_euclidean_tc(ctypes.byref(sx), ctypes.byref(sy), dim,
                                          out.data_ptr(), 1,
                                          torch.cuda.current_stream().cuda_stream))
    return out


def pairwise_dtw_fp32(x, y, r=1.0, *, g=None, strip=16):
    """(n_x, n_y) float64 dtw (or wdtw with weight steepness g) distances.

    x, y: (n, L) CUDA tensors (cast to float32).
    """
    xf = x.to(torch.float32).contiguous()
    yf = y.to(torch.float32).contiguous()
    w = None
    if g is not None:
        w = _b.logistic_weights(max(xf.shape[1], yf.shape[1]), g, xf.device)
    out = _b.dtw32(xf, yf, r=r, weights=w, strip=strip)
    return out.view(yf.shape[0], xf.shape[0]).t()
