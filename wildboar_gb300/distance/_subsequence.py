"""Subsequence search on the GPU: distance profiles and threshold matches.

Mirrors ``distance_profile`` (dilation 1, no padding), ``subsequence_match``
and ``paired_subsequence_match`` of the reference
(distance/_distance.py:732-1080, 1477-1620).  One device call,
``wb_subsequence_profile``, returns for every window of every (subsequence,
series) pair the final value of the metric's recurrence and its abandon key
(the largest per-row minimum the reference's early abandoning compares with
its threshold); the distances and the match sets of
``SubsequenceMetric._matches`` (distance/_cdistance.pyx:301-432) follow from
those two numbers on the host for any threshold.  The post-filters
(``_filter_by_max_dist``, ``_exclude_trivial_matches``,
``_filter_by_max_matches``, distance/_distance.py:400-512) are restated here.
"""

import ctypes
import math
import numbers
import warnings

import numpy as np

from .. import _lib
from ._distance import (
    InvalidParameterError,
    _as_input,
    _device_of,
    _empty,
    _stream,
    _format_return,
    _pack_shapelets,
    _validate_subsequence,
    check_metric,
    check_subsequence_metric,
)

_P = ctypes.POINTER
_lib.declare("wb_dilated_profile", [_P(_lib.Series), _P(_lib.Series), ctypes.c_int64,
                                    ctypes.c_int32, _P(_lib.Params), ctypes.c_int64,
                                    ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                    ctypes.c_int32, ctypes.c_void_p])
_lib.declare("wb_mass_profile", [_P(_lib.Series), _P(_lib.Series), ctypes.c_void_p,
                                 ctypes.c_int32, ctypes.c_void_p])
from ._metrics import check_scalar

_SQRT = {0, 1, 2, 3, 4, 5, 32, 33}      # euclidean, dtw family, scaled_euclidean / dtw
_SCALED_DTW = 33
_EUCLID = {0, 32}
_LCSS, _EDR = 6, 8


def _std_below_mean(s):
    # distance/_distance.py:310-330
    def f(x):
        return max(np.mean(x) - s * np.std(x), np.min(x))

    return f


_THRESHOLD = {"auto": _std_below_mean(2.0)}


def _check_type(x, name, target_type, required=True):
    """utils/validation.py:65-108."""

    def type_name(t):
        if t.__module__ == "builtins":
            return t.__qualname__
        if t == numbers.Real:
            return "float"
        if t == numbers.Integral:
            return "int"
        return f"{t.__module__}.{t.__qualname__}"

    if isinstance(target_type, tuple):
        target = "{" + ", ".join(type_name(t) for t in target_type) + "}"
    else:
        target = type_name(target_type)
    if x is None:
        if required:
            raise TypeError(f"{name} must be an instance of {target}, not None")
        return
    if not isinstance(x, target_type):
        raise TypeError(f"{name} must be an instance of {target}, not "
                        f"{type(x).__qualname__}")


def _check_option(options, key, name):
    """utils/validation.py:111-143."""
    if key in options:
        return options[key]
    keys = ["'%s'" % k for k in sorted(options.keys())]
    if len(keys) == 1:
        msg = f"{name} must be {keys[0]}, got {key}"
    else:
        msg = f"{name} must be {', '.join(keys[:-1])} or {keys[-1]}, got {key}"
    raise ValueError(msg)


def _transient_stats_rows(S, lens):
    """Mean and std of the rows S[i, :lens[i]] as _ts_view_update_statistics
    computes them (distance/_cdistance.pyx:167-185): sequential sums (np.cumsum
    adds left to right like the reference's loop), std 0 when the variance is
    <= 1e-13.  The square is v * v: ``current_value ** 2`` is Cython's
    pow(v, 2.0), which the C compiler folds to v * v (a libm pow may round
    differently for large values)."""
    S = np.ascontiguousarray(S, dtype=np.float64)
    lens = np.asarray(lens, dtype=np.int64)
    rows = np.arange(S.shape[0])
    ex = np.cumsum(S, axis=1)[rows, lens - 1]
    ex2 = np.cumsum(S * S, axis=1)[rows, lens - 1]
    mean = ex / lens
    var = ex2 / lens - mean * mean
    std = np.where(var > 1e-13, np.sqrt(np.where(var > 1e-13, var, 0.0)), 0.0)
    return mean, std


def _transient_stats(s):
    """_transient_stats_rows of one subsequence: (mean, std) as floats."""
    s = np.asarray(s, dtype=np.float64).ravel()
    mean, std = _transient_stats_rows(s[None, :], [s.shape[0]])
    return float(mean[0]), float(std[0])


def _profile_raw(shapelets, X, dim, metric, transient=False, stop_sq=None):
    """(raw, key, lengths) of every window, pair i = (shapelets[i], x[i]).

    raw / key are (n, ld) float64 numpy arrays, NaN past a pair's windows.
    transient: the distance profile's shapelet statistics, zero std kept.
    stop_sq (scaled_euclidean): each window's sum stops once it reaches
    stop_sq, as the reference's matching scan does (wb_subsequence_profile_stop).
    """
    packed, offs, lens, means, stds = _pack_shapelets(
        shapelets, metric.scaled or getattr(metric, "needs_std", False))
    if transient and means is not None:
        pad = np.zeros((len(shapelets), int(max(len(s) for s in shapelets))))
        for i, sh in enumerate(shapelets):
            pad[i, :len(sh)] = sh
        means, stds = _transient_stats_rows(pad, [len(sh) for sh in shapelets])
    n = len(shapelets)
    T = X.shape[-1]
    ld = int(T - lens.min() + 1)
    raw = np.empty((n, ld))
    key = np.empty((n, ld))
    arr = X.arr
    if X.device:
        arr = X.arr.detach().cpu().numpy()
    arr = np.ascontiguousarray(arr, dtype=np.float64)
    sx = _lib.series_from_numpy(arr)
    p = metric.params() if hasattr(metric, "params") else _lib.Params()
    if stop_sq is not None:
        stop = np.full(n, float(stop_sq))
        st = _lib.lib().wb_subsequence_profile_stop(
            _lib.ptr(packed), _lib.ptr(offs), _lib.ptr(lens), _lib.ptr(means),
            _lib.ptr(stds), n, ctypes.byref(sx), dim, _lib.ptr(stop), _lib.ptr(raw), ld, 0,
            None)
        key[:] = np.nan
    else:
        st = _lib.lib().wb_subsequence_profile(
            _lib.ptr(packed), _lib.ptr(offs), _lib.ptr(lens), _lib.ptr(means), _lib.ptr(stds),
            n, ctypes.byref(sx), dim, metric.metric_id, ctypes.byref(p), _lib.ptr(raw),
            _lib.ptr(key), ld, 1 if transient else 0, 0, None)
    _lib.check(st)
    return raw, key, lens


def _distances(metric_id, raw, L):
    if metric_id in _SQRT:
        with np.errstate(invalid="ignore"):  # negative adtw costs: NaN, as C's sqrt
            return np.sqrt(raw)
    if metric_id == _LCSS:
        return 1 - raw / L
    if metric_id == _EDR:
        return raw / L
    return raw


def _match_mask(metric_id, raw, key, dist, L, T, t):
    """Windows SubsequenceMetric._matches keeps for threshold t."""
    with np.errstate(invalid="ignore"):
        if metric_id in _EUCLID:
            return raw <= t * t
        if metric_id == _SCALED_DTW:
            # scaled_dtw_matches: every bound and the abandoning test fail on
            # ">= t^2" (distance/_elastic.pyx:520-600)
            t2 = t * t
            return (key < t2) & (raw <= t2)
        if metric_id in (1, 2, 3, 4, 5):  # dtw, wdtw, ddtw, wddtw, adtw
            t2 = t * t
            return ~(key > t2) & (raw <= t2)
        if metric_id == _LCSS:
            thr = L - t * L if not math.isinf(t) else t
            return ~(key > thr) & (dist <= t)
        if metric_id == _EDR:
            return ~(key > t * max(L, T)) & (dist <= t)
        return ~(key > t) & (raw <= t)


def _matches_from_profile(mid, raw, key, lens, T, threshold):
    """Per pair: (indices, distances) arrays or None, from every window's raw
    value and abandon key; all pairs at once (a pair's windows past its last
    one are excluded explicitly)."""
    n, ld = raw.shape
    lens = np.asarray(lens, dtype=np.int64)
    Lc = lens.astype(np.float64)[:, None]
    d = _distances(mid, raw, Lc)
    if mid == _EDR:
        keep = _match_mask_edr(raw, key, d, Lc, T, threshold)
    else:
        keep = _match_mask(mid, raw, key, d, Lc, T, threshold)
    keep &= np.arange(ld)[None, :] < (T - lens + 1)[:, None]
    rows, cols = np.nonzero(keep)
    vals = d[rows, cols]
    bounds = np.searchsorted(rows, np.arange(n + 1))
    out_i, out_d = [], []
    for i in range(n):
        a, b = bounds[i], bounds[i + 1]
        if a == b:
            out_i.append(None)
            out_d.append(None)
        else:
            out_i.append(cols[a:b].astype(np.intp))
            out_d.append(np.asarray(vals[a:b], dtype=np.double))
    return out_i, out_d


def _match_mask_edr(raw, key, dist, L, T, t):
    """_match_mask for edr with per-row lengths L (an (n, 1) array)."""
    with np.errstate(invalid="ignore"):
        return ~(key > t * np.maximum(L, T)) & (dist <= t)


def _matches(shapelets, X, dim, metric, threshold):
    """Per pair: (indices, distances) arrays or None, as _subsequence_match."""
    stop = None
    if metric.metric_id == 32 and math.isfinite(threshold):
        # scaled_euclidean_distance_matches stops a window's sum at the first
        # term where it is >= t^2 and keeps it if that partial sum is <= t^2
        stop = threshold * threshold
    raw, key, lens = _profile_raw(shapelets, X, dim, metric, stop_sq=stop)
    return _matches_from_profile(metric.metric_id, raw, key, lens, X.shape[-1], threshold)


def _any_in_exclude(lst, i, exclude):
    for e in lst:
        if i - exclude < e < i + exclude:
            return True
    return False


def _exclude_trivial_matches(indicies, distances, exclude):
    ind_out, dist_out = [], []
    for index, distance in zip(indicies, distances):
        if index is None:
            ind_out.append(None)
            dist_out.append(None)
            continue
        sort = np.argsort(distance)
        keep = np.zeros(sort.size, dtype=bool)
        excluded = []
        for i in range(index.size):
            if not _any_in_exclude(excluded, index[sort[i]], exclude):
                excluded.append(index[sort[i]])
                keep[sort[i]] = True
        ind_out.append(index[keep])
        dist_out.append(distance[keep])
    return ind_out, dist_out


def _filter_by_max_matches(indicies, distances, max_matches):
    ind_out, dist_out = [], []
    for index, distance in zip(indicies, distances):
        if index is None:
            ind_out.append(None)
            dist_out.append(None)
        else:
            idx = np.argsort(distance)[:max_matches]
            ind_out.append(index[idx])
            dist_out.append(distance[idx])
    return ind_out, dist_out


def _filter_by_max_dist(indicies, distances, max_dist):
    ind_out, dist_out = [], []
    for sample, (index, distance) in enumerate(zip(indicies, distances)):
        if index is None:
            ind_out.append(None)
            dist_out.append(None)
        else:
            mask = max_dist(sample, distance)
            ind_out.append(index[mask])
            dist_out.append(distance[mask])
    return ind_out, dist_out


def _jagged(lst):
    arr = np.empty(len(lst), dtype=object)
    arr[:] = lst
    return arr


# the metric names distance_profile accepts (the reference's
# _SUBSEQUENCE_METRICS keys, distance/_distance.py:149-183); the pointwise
# metrics among them (normalized_euclidean, manhattan, minkowski, chebyshev,
# cosine, angular and their scaled_ forms) are not provided here
_PROFILE_METRIC_NAMES = (
    "euclidean", "scaled_euclidean", "normalized_euclidean", "adtw", "scaled_adtw", "wdtw",
    "scaled_wdtw", "ddtw", "scaled_ddtw", "wddtw", "scaled_wddtw", "dtw", "scaled_dtw",
    "lcss", "scaled_lcss", "edr", "scaled_edr", "twe", "scaled_twe", "msm", "scaled_msm",
    "erp", "scaled_erp", "mass", "manhattan", "scaled_manhattan", "minkowski",
    "scaled_minkowski", "chebyshev", "scaled_chebyshev", "cosine", "scaled_cosine",
    "angular", "scaled_angular")


def _validate_profile_params(dilation, padding, dim, metric):
    # @validate_params of distance/_distance.py:1460-1476
    if not (callable(metric) or (isinstance(metric, str) and metric in _PROFILE_METRIC_NAMES)):
        opts = ", ".join(repr(m) for m in _PROFILE_METRIC_NAMES)
        raise InvalidParameterError(
            "The 'metric' parameter of distance_profile must be a callable or a str among "
            f"{{{opts}}}. Got {metric!r} instead.")
    if not (isinstance(dilation, numbers.Integral) and not isinstance(dilation, bool)) or \
            dilation < 1:
        raise InvalidParameterError(
            "The 'dilation' parameter of distance_profile must be an int in the range "
            f"[1, inf). Got {dilation!r} instead.")
    if not ((isinstance(padding, numbers.Integral) and not isinstance(padding, bool)
             and padding >= 0) or padding == "same"):
        raise InvalidParameterError(
            "The 'padding' parameter of distance_profile must be an int in the range "
            f"[0, inf) or a str among {{'same'}}. Got {padding!r} instead.")
    if not (isinstance(dim, numbers.Integral) and not isinstance(dim, bool)) or dim < 0:
        raise InvalidParameterError(
            "The 'dim' parameter of distance_profile must be an int in the range [0, inf). "
            f"Got {dim!r} instead.")


def _profile_device_call(entry, Y, X, out_shape, *args):
    """One profile entry point; the result is a host array like the other
    profile paths."""
    dev = _device_of(X, Y)
    out = _empty(dev, out_shape)
    sy, sx = Y.series(), X.series()
    st = getattr(_lib.lib(), entry)(ctypes.byref(sy), ctypes.byref(sx), *args,
                                    _lib.ptr(out), 1 if dev is not None else 0,
                                    _stream(X, Y))
    _lib.check(st)
    return out.cpu().numpy() if dev is not None else out


def distance_profile(y, x, *, dilation=1, padding=0, dim=0, metric="mass",
                     metric_params=None, scale=False, n_jobs=None):
    """Distance of the subsequence(s) y at every time point of x.

    Mirrors distance/_distance.py:1477-1620.  Dilation 1 without padding runs
    the SubsequenceMetric profile; the default metric "mass" is the
    z-normalised euclidean profile of the MASS formula, evaluated with exact
    dot products where the reference uses a pocketfft cross-correlation
    (wb_mass_profile: equal up to the FFT's rounding).  Dilation or padding
    runs _dilated_distance_profile (distance/_cdistance.pyx:1809-1841) with the
    pairwise metric ("mass" and "scaled_*" metrics become their unscaled
    pairwise metric on z-normalised windows; wb_dilated_profile).
    """
    _validate_profile_params(dilation, padding, dim, metric)
    y = np.asarray(y, dtype=float).squeeze()
    xa = x
    if not _lib.is_torch_cuda(x):
        xa = np.asarray(x, dtype=float).squeeze()
    xdim = xa.dim() if hasattr(xa, "dim") else xa.ndim
    if xdim == 1 and y.ndim != 1:
        xa = np.broadcast_to(xa, shape=(y.shape[0], xa.shape[0]))
        xdim = 2
    if y.ndim == 1 and xdim != 1:
        y = np.broadcast_to(y, shape=(xa.shape[0], y.shape[0]))
    X = _as_input(xa)
    y2 = np.ascontiguousarray(np.atleast_2d(y))
    L = y2.shape[1]
    shapelet_size = (L - 1) * dilation + 1
    if padding == "same":
        if L % 2 == 0:
            raise ValueError("padding='same' is only supported for odd subsequence length")
        padding = shapelet_size // 2
    if shapelet_size > X.shape[-1] + 2 * padding:
        raise ValueError("subsequence in y is larger than input in x.")
    if y2.shape[0] != X.shape[0]:
        raise ValueError("y and x must have the same number of samples.")
    if dim >= X.shape[1]:
        raise ValueError(f"The parameter dim must be dim ({dim}) < n_dims ({X.shape[1]})")
    metric_params = metric_params if metric_params is not None else {}
    base = metric[7:] if isinstance(metric, str) and metric.startswith("scaled_") else metric
    if base in ("normalized_euclidean", "manhattan", "minkowski", "chebyshev", "cosine",
                "angular"):
        raise NotImplementedError(
            f"the pointwise metric {metric!r} is not provided by wildboar_gb300")
    if dilation == 1 and padding == 0:
        if metric == "mass":
            Y = _as_input(y2)
            dp = _profile_device_call("wb_mass_profile", Y, X,
                                      (X.shape[0], X.shape[-1] - L + 1))
            return np.squeeze(dp)
        Metric_ = check_subsequence_metric(metric, scale=scale)
        m = Metric_(**metric_params)
        shapelets = [np.ascontiguousarray(r, dtype=float) for r in y2]
        # _DistanceProfile reads y[i, 0] and x[i, 0] whatever dim is
        # (distance/_cdistance.pyx:1680-1699)
        raw, key, lens = _profile_raw(shapelets, X, 0, m, transient=True)
        nwin = X.shape[-1] - L + 1
        dp = _distances(m.metric_id, raw[:, :nwin], float(L))
        if m.metric_id == _SCALED_DTW:
            # the profile is scaled_dtw_matches with an infinite threshold over
            # a profile of ones: windows it does not keep stay 1
            keep = _match_mask(m.metric_id, raw[:, :nwin], key[:, :nwin], dp, float(L),
                               X.shape[-1], math.inf)
            dp = np.where(keep, dp, 1.0)
        return np.squeeze(dp)
    # distance/_distance.py:1590-1616
    if metric == "mass":
        metric = "scaled_euclidean"
    scale = (isinstance(metric, str) and metric.startswith("scaled_")) or scale
    if isinstance(metric, str) and metric.startswith("scaled_"):
        metric = metric[7:]
    Metric_ = check_metric(metric)
    m = Metric_(**metric_params)
    if scale:
        std = np.std(y2, axis=-1, keepdims=True)
        mean = np.mean(y2, axis=-1, keepdims=True)
        std[std < 1e-13] = 1  # EPSILON of distance/_cdistance.pxd
        y2 = (y2 - mean) / std
    Y = _as_input(np.ascontiguousarray(y2))
    out_size = X.shape[-1] + 2 * padding - shapelet_size + 1
    p = m.params()
    dp = _profile_device_call("wb_dilated_profile", Y, X, (X.shape[0], out_size), dim,
                              m.metric_id, ctypes.byref(p), dilation, padding,
                              1 if scale else 0)
    return np.squeeze(dp)


def subsequence_match(y, x, threshold=None, *, dim=0, metric="euclidean", metric_params=None,
                      scale=False, max_matches=None, exclude=None, return_distance=False,
                      n_jobs=None):
    """Positions where y is within `threshold` of the series in x.

    Mirrors distance/_distance.py:732-924 (thresholds: float, callable,
    'auto' or one per sample; max_matches; exclude; jagged outputs with None
    for samples without a match).
    """
    y = _validate_subsequence(y)
    if len(y) > 1:
        raise ValueError("A single subsequence expected, got %d" % len(y))
    y = y[0]
    X = _as_input(x)
    if y.shape[0] > X.shape[-1]:
        raise ValueError("Invalid subsequnce shape (%d > %d)" % (y.shape[0], X.shape[-1]))
    n_dims = X.shape[1]
    if not 0 >= dim < n_dims:
        raise ValueError("The parameter dim must be 0 <= dim < n_dims")
    Metric_ = check_subsequence_metric(metric, scale=scale)
    metric_params = metric_params if metric_params is not None else {}
    if n_jobs is not None:
        warnings.warn("n_jobs is not yet supported.", UserWarning)
    if threshold is None:
        threshold = np.inf
        if max_matches is None:
            max_matches = 10
    if callable(threshold):
        threshold_fn = threshold

        def max_dist(_, d):
            return d <= threshold_fn(d)

        threshold = np.inf
    elif isinstance(threshold, str):
        threshold_fn = _check_option(_THRESHOLD, threshold, "threshold")

        def max_dist(_, d):
            return d <= threshold_fn(d)

        threshold = np.inf
    elif hasattr(threshold, "__len__") or hasattr(threshold, "__array__"):
        threshold_array = np.asarray(threshold)
        n_samples = X.shape[0] if X.ndim > 1 else 1
        if len(threshold_array) != n_samples:
            raise ValueError(
                f"threshold array length ({len(threshold_array)}) must match "
                f"the number of samples ({n_samples})"
            )

        def max_dist(i, d):
            return d <= threshold_array[i]

        threshold = np.inf
    elif not isinstance(threshold, numbers.Real):
        raise TypeError("threshold must be str, callable, array-like or float, not %s"
                        % type(threshold).__qualname__)
    else:
        max_dist = None

    _check_type(exclude, "exclude", (numbers.Integral, numbers.Real), required=False)
    if isinstance(exclude, numbers.Integral):
        check_scalar(exclude, "exclude", numbers.Integral, min_val=0)
    elif isinstance(exclude, numbers.Real):
        check_scalar(exclude, "exclude", numbers.Real, min_val=0)
        exclude = math.ceil(y.size * exclude)

    m = Metric_(**metric_params)
    shapelets = [y] * X.shape[0]
    indices, distances = _matches(shapelets, X, dim, m, float(threshold))
    if max_dist is not None:
        indices, distances = _filter_by_max_dist(indices, distances, max_dist)
    if exclude:
        indices, distances = _exclude_trivial_matches(indices, distances, exclude)
    if max_matches:
        indices, distances = _filter_by_max_matches(indices, distances, max_matches)
    # the reference formats with len(y), y being the subsequence itself here
    indices = _format_return(_jagged(indices), len(y), X.ndim)
    if indices.size == 1:
        indices = indices.item()
    if return_distance:
        distances = _format_return(_jagged(distances), len(y), X.ndim)
        if distances.size == 1:
            distances = distances.item()
        return indices, distances
    return indices


def paired_subsequence_match(y, x, threshold=None, *, dim=0, metric="euclidean",
                             metric_params=None, scale=False, max_matches=None,
                             return_distance=False, n_jobs=None):
    """Positions where the i:th subsequence is within `threshold` of the i:th
    series.  Mirrors distance/_distance.py:927-1079."""
    y = _validate_subsequence(y)
    X = _as_input(x)
    if X.ndim == 1:
        raise ValueError("Expected 2D array, got 1D array instead")
    if len(y) != X.shape[0]:
        raise ValueError("x and y must have the same number of samples")
    n_dims = X.shape[1]
    if not 0 >= dim < n_dims:
        raise ValueError("The parameter dim must be 0 <= dim < n_dims")
    for s in y:
        if s.shape[0] > X.shape[-1]:
            raise ValueError("invalid subsequnce shape (%d > %d)" % (s.shape[0], X.shape[-1]))
    Metric_ = check_subsequence_metric(metric, scale=scale)
    metric_params = metric_params if metric_params is not None else {}
    if n_jobs is not None:
        warnings.warn("n_jobs is not yet supported.", UserWarning)
    if threshold is None:
        threshold = np.inf
        if max_matches is None:
            max_matches = 10
    # the reference's one-argument max_dist here is later called with
    # (sample, distances) by _filter_by_max_dist; kept as it is
    if callable(threshold):
        threshold_fn = threshold

        def max_dist(d):
            return d <= threshold_fn(d)

        threshold = np.inf
    elif isinstance(threshold, str):
        threshold_fn = _check_option(_THRESHOLD, threshold, "threshold")

        def max_dist(d):
            return d <= threshold_fn(d)

        threshold = np.inf
    elif not isinstance(threshold, numbers.Real):
        raise TypeError("threshold must be str, callable or float, not %s"
                        % type(threshold).__qualname__)
    else:
        max_dist = None
    m = Metric_(**metric_params)
    indices, distances = _matches(y, X, dim, m, float(threshold))
    if max_dist is not None:
        indices, distances = _filter_by_max_dist(indices, distances, max_dist)
    if max_matches:
        indices, distances = _filter_by_max_matches(indices, distances, max_matches)
    indices = _format_return(_jagged(indices), len(y), X.ndim)
    if indices.size == 1:
        indices = indices.reshape(1)
    if return_distance:
        distances = _format_return(_jagged(distances), len(y), X.ndim)
        if distances.size == 1:
            distances = distances.reshape(1)
        return indices, distances
    return indices


def argmin_subsequence_distance(y, x, *, dim=0, k=1, metric="euclidean", metric_params=None,
                                scale=False, return_distance=False, n_jobs=None):
    """The k closest windows of the i:th subsequence in the i:th series.

    Mirrors distance/_distance.py:1636-1761: y is an (n, m_timestep) float
    array or a list of 1-D arrays (zero padded to the longest); a 1-D x is
    broadcast to n rows; ``scaled_*`` metric names (or scale=True) z-normalise
    the subsequence and every window.  Indices (n, k) come in the reference's
    heap order.  The reference reads y[i] at ``dim`` too, which only exists for
    dim 0; here y[i] is always the subsequence.
    """
    from ._distance import check_metric

    if isinstance(y, np.ndarray) and y.dtype == float:
        if y.ndim != 2:
            raise ValueError("Expected 2D array, got %dD array instead" % y.ndim)
        S = np.ascontiguousarray(y, dtype=np.float64)
        y_len = np.full(S.shape[0], S.shape[1], dtype=np.int64)
    else:
        y_len = np.empty(len(y), dtype=np.int64)
        for i, shapelet in enumerate(y):
            if np.ndim(shapelet) > 1:
                raise ValueError("shapelet must be 1d-array")
            y_len[i] = np.shape(shapelet)[0]
        S = np.zeros((len(y), int(np.max(y_len))), dtype=float)
        for i, shapelet in enumerate(y):
            S[i, : y_len[i]] = shapelet
    if _lib.is_torch_cuda(x):
        x = x.detach().cpu().numpy()
    x = np.asarray(x, dtype=float)
    if x.ndim == 1:
        x = np.broadcast_to(x, shape=(S.shape[0], x.shape[0]))
    X = _as_input(np.ascontiguousarray(x))
    if not S.shape[1] <= X.shape[-1]:
        raise ValueError("the longest subsequence must be shorter than samples.")
    if S.shape[0] != X.shape[0]:
        raise ValueError("both arrays must have the same number of samples.")
    if dim >= X.shape[1]:
        raise ValueError(f"The parameter dim must be dim ({dim}) < n_dims ({X.shape[1]})")
    if not k <= (X.shape[-1] - S.shape[1] + 1):
        raise ValueError("k must be less x.shape[-1] - y.shape[-1] + 1.")
    scale = (isinstance(metric, str) and metric.startswith("scaled_")) or scale
    if isinstance(metric, str) and metric.startswith("scaled_"):
        metric = metric[7:]
    Metric_ = check_metric(metric)
    metric_params = metric_params if metric_params is not None else {}
    m = Metric_(**metric_params)
    n = S.shape[0]
    means = stds = None
    if scale:
        means, stds = _transient_stats_rows(S, y_len)
    indices = np.zeros((n, k), dtype=np.int64)
    distances = np.zeros((n, k))
    sx = X.series()
    p = m.params()
    st_ = _lib.lib().wb_argmin_subsequence_distance(
        _lib.ptr(S), _lib.ptr(y_len), S.shape[1], n, _lib.ptr(means), _lib.ptr(stds),
        ctypes.byref(sx), dim, m.metric_id, ctypes.byref(p), 1 if scale else 0, k,
        _lib.ptr(indices), _lib.ptr(distances), 0, None)
    _lib.check(st_)
    indices = indices.astype(np.intp, copy=False)
    if return_distance:
        return indices, distances
    return indices
