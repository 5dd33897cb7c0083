"""Batched calls for the reference's compiled callers of the distance path.

The proximity trees (tree/_cptree.pyx) and the shapelet transforms
(transform/_cshapelet.pyx) call one metric on one pair at a time from Cython.
``include/wbgpu.h`` gives them two batched C entry points
(``wb_nearest_pivot``, ``wb_subsequence_distance_views``, csrc/batch.cu) that a
``cdef extern`` block can call; these Python functions are the same calls
for Python code and for the tests.
"""

import ctypes

import numpy as np

from .. import _lib
from ._distance import _as_input, check_metric, check_subsequence_metric
from ._subsequence import _transient_stats_rows

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_lib.declare("wb_nearest_pivot", [ctypes.POINTER(_lib.Series), _i64, _i64, _vp, _vp, _vp, _vp,
                                  _vp, _vp, _vp, _i32, _vp, _vp, _vp])
_lib.declare("wb_subsequence_distance_views",
             [ctypes.POINTER(_lib.Series), _vp, _vp, _vp, _vp, _vp, _vp, _i64,
              ctypes.POINTER(_lib.Series), _i64, _i32, ctypes.POINTER(_lib.Params), _vp, _vp,
              _vp])


def _csr(lists):
    ptr = np.zeros(len(lists) + 1, dtype=np.int64)
    ptr[1:] = np.cumsum([len(a) for a in lists])
    flat = (np.concatenate([np.asarray(a, dtype=np.int64) for a in lists])
            if lists else np.zeros(0, np.int64))
    return ptr, np.ascontiguousarray(flat, dtype=np.int64)


def nearest_pivot(x, groups, metrics, *, dim=0):
    """Nearest pivot of every sample of every group, as a proximity-tree node
    partitions its samples (tree/_cptree.pyx:869-894; find_min_branch, :273-290).

    ``groups`` is a list of (samples, pivots, slot): row indices of ``x`` and
    an index into ``metrics``, a list of (metric name, metric_params).
    Returns (branch, distance) arrays aligned with the concatenated samples:
    the position, within its group's pivots, of the first pivot at the
    strictly smallest distance (the metric's full distance, as the tree calls
    it), and that distance.
    """
    X = _as_input(x)
    mids = np.array([check_metric(m).metric_id if isinstance(m, str) else -1
                     for m, _ in metrics], dtype=np.int32)
    params = (_lib.Params * len(metrics))()
    for k, (m, p) in enumerate(metrics):
        params[k] = check_metric(m)(**(p or {})).params()
    s_ptr, s_flat = _csr([g[0] for g in groups])
    p_ptr, p_flat = _csr([g[1] for g in groups])
    slots = np.array([g[2] for g in groups], dtype=np.int32)
    branch = np.empty(s_flat.shape[0], dtype=np.int64)
    dist = np.empty(s_flat.shape[0])
    sx = X.series()
    st = _lib.lib().wb_nearest_pivot(
        ctypes.byref(sx), dim, len(groups), _lib.ptr(s_ptr), _lib.ptr(s_flat), _lib.ptr(p_ptr),
        _lib.ptr(p_flat), _lib.ptr(slots), _lib.ptr(mids), ctypes.cast(params, _vp),
        len(metrics), _lib.ptr(branch), _lib.ptr(dist), _lib.current_stream_handle())
    _lib.check(st)
    return branch.astype(np.intp), dist


def subsequence_distance_views(x, views, target=None, *, dim=0, metric="euclidean",
                               metric_params=None):
    """Minimum distance and first argmin window of subsequence views of ``x``
    (rows (sample, dim, start, length)) in every series of ``target``
    (default: ``x``), with the view statistics of _ts_view_update_statistics
    (distance/_cdistance.pyx:167-185), as the shapelet transform evaluates its
    attributes (transient_distance, :265-282).  Returns (dist, idx), each
    (n_target, n_views).
    """
    X = _as_input(x)
    T = X if target is None else _as_input(target)
    views = np.ascontiguousarray(np.atleast_2d(np.asarray(views, dtype=np.int64)))
    if views.shape[1] != 4:
        raise ValueError("views must be rows of (sample, dim, start, length)")
    Metric_ = check_subsequence_metric(metric)
    m = Metric_(**(metric_params or {}))
    host = X.arr.detach().cpu().numpy() if X.device else X.arr
    pad = np.zeros((views.shape[0], int(views[:, 3].max()) if views.shape[0] else 1))
    for i, v in enumerate(views):
        pad[i, :v[3]] = host[v[0], v[1], v[2]:v[2] + v[3]]
    means, stds = _transient_stats_rows(pad, views[:, 3])
    vs = [np.ascontiguousarray(views[:, k]) for k in range(4)]
    dev = T.device
    if dev:
        import torch

        dist = torch.empty((T.shape[0], views.shape[0]), dtype=torch.float64,
                           device=T.arr.device)
        idx = torch.empty((T.shape[0], views.shape[0]), dtype=torch.int64, device=T.arr.device)
    else:
        dist = np.empty((T.shape[0], views.shape[0]))
        idx = np.empty((T.shape[0], views.shape[0]), dtype=np.int64)
    sx, st_ = X.series(), T.series()
    p = m.params() if hasattr(m, "params") else _lib.Params()
    st = _lib.lib().wb_subsequence_distance_views(
        ctypes.byref(sx), _lib.ptr(vs[0]), _lib.ptr(vs[1]), _lib.ptr(vs[2]), _lib.ptr(vs[3]),
        _lib.ptr(means), _lib.ptr(stds), views.shape[0], ctypes.byref(st_), dim, m.metric_id,
        ctypes.byref(p), _lib.ptr(dist), _lib.ptr(idx), _lib.current_stream_handle())
    _lib.check(st)
    if not dev:
        idx = idx.astype(np.intp)
    return dist, idx


__all__ = ["nearest_pivot", "subsequence_distance_views"]
