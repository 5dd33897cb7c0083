"""Drop-in distance API computed on the GPU.

Same signatures, argument checks, dim handling and return shapes as the
reference's public functions (wildboar src/wildboar/distance/_distance.py):
``pairwise_distance`` (:1178-1304), ``paired_distance`` (:1082-1175),
``argmin_distance`` (:1307-1457) and ``pairwise_subsequence_distance``
(:543-636).  numpy inputs are validated like the reference and staged to the
device by the library; CUDA torch tensors (float64) are used in place and the
results come back as CUDA tensors.  All distances are computed by libwbgpu.so;
``n_jobs`` is accepted and ignored.
"""

import ctypes
import numbers
import warnings

import numpy as np

from .. import _lib
from ._metrics import _METRICS, _SUBSEQUENCE_METRICS, Metric
from ._validation import check_array, check_ts_array

__all__ = [
    "pairwise_distance",
    "paired_distance",
    "argmin_distance",
    "pairwise_subsequence_distance",
    "check_metric",
    "check_subsequence_metric",
]


class InvalidParameterError(ValueError, TypeError):
    """Raised like sklearn's @validate_params (subclass of ValueError and TypeError)."""


def check_metric(metric):
    """distance/_distance.py:231-260 (string metrics)."""
    if isinstance(metric, str) and metric in _METRICS:
        return _METRICS[metric]
    if callable(metric):
        raise NotImplementedError(
            "callable metrics are evaluated by Python in the reference; wildboar_gb300 "
            "computes the built-in metrics only"
        )
    raise ValueError(
        "unsupported metric {}, 'metric' must be callable or a str among {}".format(
            metric, set(_METRICS.keys())
        )
    )


def check_subsequence_metric(metric, scale=False):
    """distance/_distance.py:263-307."""
    if callable(metric):
        raise NotImplementedError("callable subsequence metrics are not provided")
    if scale and not metric.startswith("scaled_"):
        metric = "scaled_" + metric
    if metric in _SUBSEQUENCE_METRICS:
        return _SUBSEQUENCE_METRICS[metric]
    raise ValueError(
        ("unsupported metric '{}', 'metric' must be callable or a str among {}").format(
            metric, set(_SUBSEQUENCE_METRICS.keys())
        )
    )


def _format_return(x, y_dims, x_dims):
    """distance/_distance.py:514-540."""
    if x_dims == 1 and y_dims == 1 and _size(x) == 1:
        return x.item()
    elif x_dims == 1 or y_dims == 1:
        return _squeeze(x)
    return x


def _size(x):
    return x.size if isinstance(x, np.ndarray) else x.numel()


def _squeeze(x):
    return np.squeeze(x) if isinstance(x, np.ndarray) else x.squeeze()


# --------------------------------------------------------------------------
# array plumbing: host numpy (validated like the reference) or CUDA tensors


class _Input:
    """One validated input: ``arr`` is (n, d, L) float64, numpy or CUDA tensor."""

    def __init__(self, a, ndim, arr, device):
        self.orig = a
        self.ndim = ndim
        self.arr = arr
        self.device = device

    @property
    def shape(self):
        return tuple(self.arr.shape)

    def series(self):
        if self.device:
            return _lib.series_from_torch(self.arr)
        return _lib.series_from_numpy(self.arr)


def _check_torch(t, name=""):
    import torch

    if t.dim() == 0 or t.dim() > 3:
        raise ValueError("Found array with dim %d. None expected <= 3." % t.dim())
    if t.shape[0] < 1 or t.shape[-1] < 1:
        raise ValueError(f"Found array with shape {tuple(t.shape)}; need samples and timesteps")
    t = t.to(torch.float64)
    if torch.isnan(t).any().item():
        raise ValueError(f"Input {name + ' ' if name else ''}contains NaN.")
    if torch.isinf(t).any().item():
        raise ValueError(f"Input {name + ' ' if name else ''}contains infinity.")
    return t


def _as_input(a):
    if _lib.is_torch_cuda(a):
        t = _check_torch(a)
        ndim = t.dim()
        if ndim == 1:
            t = t.reshape(1, 1, -1)
        elif ndim == 2:
            t = t.reshape(t.shape[0], 1, t.shape[1])
        return _Input(a, ndim, t.contiguous(), True)
    x = check_array(a, allow_3d=True, ensure_2d=False, dtype=float)
    return _Input(a, x.ndim, check_ts_array(x), False)


def _empty(device_like, shape, dtype=np.float64):
    if device_like is not None:
        import torch

        tdt = torch.float64 if dtype == np.float64 else torch.int64
        return torch.empty(shape, dtype=tdt, device=device_like.arr.device)
    return np.empty(shape, dtype=dtype)


def _zeros(device_like, shape):
    if device_like is not None:
        import torch

        return torch.zeros(shape, dtype=torch.float64, device=device_like.arr.device)
    return np.zeros(shape)


def _stream(*inputs):
    if any(i is not None and i.device for i in inputs):
        return _lib.current_stream_handle()
    return None


def _mean_dims(ds):
    """np.mean(list, axis=0): sequential sum over dims, then / n_dims."""
    if isinstance(ds[0], np.ndarray):
        return np.mean(ds, axis=0)
    acc = ds[0].clone()
    for d in ds[1:]:
        acc += d
    return acc / len(ds)


def _stack_dims(ds):
    if isinstance(ds[0], np.ndarray):
        return np.stack(ds, axis=0)
    import torch

    return torch.stack(ds, dim=0)


def _dims(fn, n_dims, dim):
    if n_dims == 1 and dim == "mean":
        dim = 0
    if isinstance(dim, str) and dim in ("mean", "full"):
        ds = [fn(d) for d in range(n_dims)]
        return _mean_dims(ds) if dim == "mean" else _stack_dims(ds)
    if isinstance(dim, numbers.Integral) and not isinstance(dim, bool) and 0 <= dim < n_dims:
        return fn(int(dim))
    raise ValueError("The parameter dim must be 0 <= dim < n_dims")


def _device_of(*inputs):
    for i in inputs:
        if i is not None and i.device:
            return i
    return None


def _pairwise_one(X, Y, dim, metric, entry="wb_pairwise_distance"):
    dev = _device_of(X, Y)
    ny = X.shape[0] if Y is None else Y.shape[0]
    out = _zeros(dev, (X.shape[0], ny)) if Y is None else _empty(dev, (X.shape[0], ny))
    sx = X.series()
    sy = None if Y is None else Y.series()
    p = metric.params()
    st = getattr(_lib.lib(), entry)(
        ctypes.byref(sx), None if sy is None else ctypes.byref(sy), dim,
        metric.metric_id, ctypes.byref(p), _lib.ptr(out), 1 if dev else 0, _stream(X, Y))
    _lib.check(st)
    return out


def _paired_one(X, Y, dim, metric):
    dev = _device_of(X, Y)
    out = _empty(dev, (X.shape[0],))
    sx, sy = X.series(), Y.series()
    p = metric.params()
    st = _lib.lib().wb_paired_distance(
        ctypes.byref(sx), ctypes.byref(sy), dim, metric.metric_id, ctypes.byref(p),
        _lib.ptr(out), 1 if dev else 0, _stream(X, Y))
    _lib.check(st)
    return out


# --------------------------------------------------------------------------
# public API


def pairwise_distance(x, y=None, *, dim="mean", metric="euclidean", metric_params=None,
                      n_jobs=None):
    """Compute the distance between every time series in X and Y.

    Mirrors distance/_distance.py:1178-1304: ``y=None`` (or ``y is x``) takes
    the singleton path (upper triangle, mirrored, zero diagonal, no squeeze);
    otherwise the result is squeezed like the reference's ``_format_return``.
    """
    return _pairwise(x, y, dim, metric, metric_params, "wb_pairwise_distance")


def _pairwise(x, y, dim, metric, metric_params, entry):
    Metric_ = check_metric(metric)
    metric_params = metric_params if metric_params is not None else {}
    metric = Metric_(**metric_params)
    if y is None:
        y = x
    if x is y:
        X = _as_input(x)
        if X.ndim == 1:
            return 0.0
        n_dims = X.shape[1]
        return _dims(lambda d: _pairwise_one(X, None, d, metric, entry), n_dims, dim)
    X = _as_input(x)
    Y = _as_input(y)
    if X.ndim != 1 and Y.ndim != 1 and X.ndim != Y.ndim:
        raise ValueError(
            "x (%dD-array) and y (%dD-array) are not compatible" % (X.ndim, Y.ndim)
        )
    if X.ndim == 3 and X.shape[1] != Y.shape[1]:
        raise ValueError("x and y must have the same number of dimensions.")
    if X.shape[-1] != Y.shape[-1] and not metric.is_elastic:
        raise ValueError(
            "Illegal n_timestep (%r != %r) for non-elastic distance measure"
            % (X.shape[-1], Y.shape[-1])
        )
    n_dims = X.shape[1]
    if Y.shape[1] != n_dims:
        raise ValueError("x and y must have the same number of dimensions.")
    d = _dims(lambda k: _pairwise_one(X, Y, k, metric, entry), n_dims, dim)
    return _format_return(d, Y.ndim, X.ndim)


def paired_distance(x, y, *, dim="mean", metric="euclidean", metric_params=None,
                    n_jobs=None):
    """Compute the distance between the i:th time series (distance/_distance.py:1082-1175)."""
    if _lib.is_torch_cuda(x) or _lib.is_torch_cuda(y):
        X, Y = _as_input(x), _as_input(y)
        if X.ndim != Y.ndim:
            raise ValueError(
                "x (%dD-array) and y (%dD-array) are not compatible." % (X.ndim, Y.ndim)
            )
        if tuple(X.shape) != tuple(Y.shape):
            raise ValueError("x and y must have the same shape")
        x_ndim, y_ndim = X.ndim, Y.ndim
    else:
        xa = check_array(x, allow_3d=True, ensure_2d=False, dtype=float)
        ya = check_array(y, allow_3d=True, ensure_2d=False, dtype=float)
        xa, ya = np.broadcast_arrays(xa, ya)
        if xa.ndim != ya.ndim:
            raise ValueError(
                "x (%dD-array) and y (%dD-array) are not compatible." % (xa.ndim, ya.ndim)
            )
        if xa.ndim == 3 and xa.shape[1] != ya.shape[1]:
            raise ValueError("x and y must have the same number of dimensions.")
        if xa.ndim > 1 and ya.ndim > 1 and xa.shape[0] != ya.shape[0]:
            raise ValueError("x and y must have the same number of samples.")
        x_ndim, y_ndim = xa.ndim, ya.ndim
        X = _Input(x, xa.ndim, check_ts_array(xa), False)
        Y = _Input(y, ya.ndim, check_ts_array(ya), False)
    if n_jobs is not None:
        warnings.warn("n_jobs is not yet supported.", UserWarning)
    Metric_ = check_metric(metric)
    metric_params = metric_params if metric_params is not None else {}
    metric = Metric_(**metric_params)
    n_dims = X.shape[1]
    d = _dims(lambda k: _paired_one(X, Y, k, metric), n_dims, dim)
    return _format_return(d, y_ndim, x_ndim)


def _validate_argmin_params(k, metric, metric_params, return_distance, sorted_, n_jobs):
    # @validate_params of distance/_distance.py:1307-1319
    if not (isinstance(k, numbers.Integral) and not isinstance(k, bool)) or k < 1:
        raise InvalidParameterError(
            "The 'k' parameter of argmin_distance must be an int in the range [1, inf). "
            f"Got {k!r} instead."
        )
    if not (callable(metric) or (isinstance(metric, str) and metric in _METRICS)):
        opts = ", ".join(repr(m) for m in sorted(_METRICS))
        raise InvalidParameterError(
            "The 'metric' parameter of argmin_distance must be a callable or a str among "
            f"{{{opts}}}. Got {metric!r} instead."
        )
    if metric_params is not None and not isinstance(metric_params, dict):
        raise InvalidParameterError(
            "The 'metric_params' parameter of argmin_distance must be None or an instance "
            f"of 'dict'. Got {metric_params!r} instead."
        )
    for name, v in (("return_distance", return_distance), ("sorted", sorted_)):
        if not isinstance(v, bool):
            raise InvalidParameterError(
                f"The '{name}' parameter of argmin_distance must be an instance of 'bool'. "
                f"Got {v!r} instead."
            )
    if n_jobs is not None and not isinstance(n_jobs, numbers.Integral):
        raise InvalidParameterError(
            "The 'n_jobs' parameter of argmin_distance must be an instance of 'int' or "
            f"None. Got {n_jobs!r} instead."
        )


def argmin_distance(x, y=None, *, dim=0, k=1, metric="euclidean", metric_params=None,
                    lower_bound=None, sorted=False, return_distance=False, n_jobs=None):
    """Find the indices of the samples with the lowest distance in ``y``.

    Mirrors distance/_distance.py:1307-1457: without ``sorted`` the rows are in
    the order of the reference's k-max-heap (utils/_misc.pyx:18-107),
    including the effect of its early abandoning.
    """
    _validate_argmin_params(k, metric, metric_params, return_distance, sorted, n_jobs)
    metric_params = metric_params if metric_params is not None else {}
    metric = check_metric(metric)(**metric_params)
    X = _as_input(x)
    Y = X if y is None else _as_input(y)
    if X.shape[-1] != Y.shape[-1] and not metric.is_elastic:
        raise ValueError(
            "Illegal n_timestep (%d != %d) for non-elastic distance measure."
            % (X.shape[-1], Y.shape[-1])
        )
    if X.shape[1] != Y.shape[1]:
        raise ValueError("x and y must have the same number of dimensions.")
    dev = _device_of(X, Y)
    lb = None
    if lower_bound is not None:
        if dev is not None and _lib.is_torch_cuda(lower_bound):
            lb = lower_bound.to(dtype=X.arr.dtype)
            if lb.dim() == 1:
                lb = lb.reshape(1, -1)
            lb = lb.contiguous()
            lb_shape = tuple(lb.shape)
        else:
            lb = check_array(lower_bound, ensure_2d=False)
            lb = np.atleast_2d(lb)
            lb_shape = lb.shape
            if dev is not None:
                import torch

                lb = torch.as_tensor(np.ascontiguousarray(lb), device=dev.arr.device)
            else:
                lb = np.ascontiguousarray(lb, dtype=np.float64)
        if X.shape[0] != lb_shape[0] or Y.shape[0] != lb_shape[1]:
            raise ValueError(
                "The lower bound must be of shape (x.shape[0], y.shape[0]), got ({}, {})".format(
                    *lb_shape
                )
            )
    n_dims = X.shape[1]
    k = min(k, Y.shape[0])
    if not (0 <= dim < 1):
        raise ValueError(f"The parameter dim must be dim ({dim}) < n_dims ({n_dims})")
    indices = _empty(dev, (X.shape[0], k), dtype=np.int64)
    distances = _empty(dev, (X.shape[0], k))
    sx = X.series()
    sy = Y.series()
    p = metric.params()
    st = _lib.lib().wb_argmin_distance(
        ctypes.byref(sx), ctypes.byref(sy), dim, metric.metric_id, ctypes.byref(p), k,
        _lib.ptr(lb), _lib.ptr(indices), _lib.ptr(distances), 1 if dev else 0,
        _stream(X, Y))
    _lib.check(st)
    if dev is None:
        indices = indices.astype(np.intp, copy=False)
    if sorted:
        if dev is None:
            order = np.argsort(distances, axis=1, kind="stable")
            indices = np.take_along_axis(indices, order, axis=1)
            if return_distance:
                distances = np.take_along_axis(distances, order, axis=1)
        else:
            import torch

            order = torch.sort(distances, dim=1, stable=True).indices
            indices = torch.take_along_dim(indices, order, dim=1)
            if return_distance:
                distances = torch.take_along_dim(distances, order, dim=1)
    if return_distance:
        return indices, distances
    return indices


def _validate_subsequence(y):
    """distance/_distance.py:336-373."""
    if len(y) == 0:
        raise ValueError("Subsequence y cannot be empty.")
    if isinstance(y, np.ndarray) and y.dtype != object:
        if y.ndim == 1:
            return [y.astype(float)]
        elif y.ndim == 2:
            y = list(y.astype(float))
        else:
            raise ValueError(
                "Expected 2D array, got {}D array instead:\narray={}.\n".format(y.ndim, y)
            )
    elif any(_is_arraylike(e) for e in y):
        y = [np.array(e, dtype=np.double) for e in y]
    else:
        y = [np.array(y, dtype=np.double)]
    return y


def _is_arraylike(x):
    return hasattr(x, "__len__") or hasattr(x, "shape") or hasattr(x, "__array__")


_GROUPED_STATS_OK = None


def _grouped_stats_ok():
    """Whether np.mean / np.std over the rows of a stacked (count, L) array
    give, bit for bit, the values of one call per row (numpy reduces every
    contiguous row with the same pairwise sum); checked once per process."""
    global _GROUPED_STATS_OK
    if _GROUPED_STATS_OK is None:
        rng = np.random.default_rng(12345)
        ok = True
        for L in (1, 7, 8, 9, 16, 33, 100, 128, 129, 300, 513, 1024, 4097):
            A = rng.standard_normal((5, L)) * 1e3 + 7.0
            m, sd = np.mean(A, axis=1), np.std(A, axis=1)
            for i in range(5):
                ok &= bool(np.mean(A[i]).view(np.uint64) == m[i].view(np.uint64))
                ok &= bool(np.std(A[i]).view(np.uint64) == sd[i].view(np.uint64))
        _GROUPED_STATS_OK = ok
    return _GROUPED_STATS_OK


def _shapelet_stats(shapelets, lens, packed=None, offs=None):
    """np.mean / np.std of every shapelet (ScaledSubsequenceMetric.from_array,
    distance/_cdistance.pyx:453-467), one reduction per distinct length (rows
    gathered from the packed float64 copy when it is given)."""
    n = len(shapelets)
    # other dtypes reduce in their own precision: keep one call per shapelet
    all_f64 = all(getattr(s, "dtype", None) == np.float64 for s in shapelets)
    if n < 64 or not all_f64 or not _grouped_stats_ok():
        means = np.array([np.mean(s) for s in shapelets], dtype=np.float64)
        stds = np.array([np.std(s) for s in shapelets], dtype=np.float64)
        return means, stds
    means = np.empty(n)
    stds = np.empty(n)
    for L in np.unique(lens):
        rows = np.flatnonzero(lens == L)
        if packed is not None:
            A = packed[offs[rows][:, None] + np.arange(L)[None, :]]
        else:
            A = np.stack([np.ravel(shapelets[i]) for i in rows])
        means[rows] = np.mean(A, axis=1)
        stds[rows] = np.std(A, axis=1)
    return means, stds


def _pack_shapelets(shapelets, scaled):
    lens = np.array([s.shape[0] for s in shapelets], dtype=np.int64)
    offs = np.zeros(len(shapelets), dtype=np.int64)
    if len(shapelets) > 1:
        offs[1:] = np.cumsum(lens)[:-1]
    packed = np.ascontiguousarray(np.concatenate([np.ravel(s) for s in shapelets]),
                                  dtype=np.float64)
    if scaled:
        # ScaledSubsequenceMetric.from_array: distance/_cdistance.pyx:453-467
        means, stds = _shapelet_stats(shapelets, lens, packed, offs)
        stds[stds <= 1e-13] = 0.0
    else:
        means = stds = None
    return packed, offs, lens, means, stds


def _subsequence_call(y, X, dim, metric, paired):
    """Run the pairwise ((n_x, m) outputs) or paired ((m,) outputs) subsequence
    entry for validated shapelets y and input X."""
    packed, offs, lens, means, stds = _pack_shapelets(
        y, metric.scaled or getattr(metric, "needs_std", False))
    dev = _device_of(X)
    m = len(y)
    if dev is not None:
        import torch

        devc = X.arr.device
        packed = torch.as_tensor(packed, device=devc)
        offs = torch.as_tensor(offs, device=devc)
        lens = torch.as_tensor(lens, device=devc)
        if means is not None:
            means = torch.as_tensor(means, device=devc)
            stds = torch.as_tensor(stds, device=devc)
    shape = (m,) if paired else (X.shape[0], m)
    dist = _empty(dev, shape)
    idx = _empty(dev, shape, dtype=np.int64)
    sx = X.series()
    p = metric.params() if hasattr(metric, "params") else _lib.Params()
    entry = (_lib.lib().wb_paired_subsequence_distance if paired
             else _lib.lib().wb_pairwise_subsequence_distance)
    st = entry(
        _lib.ptr(packed), _lib.ptr(offs), _lib.ptr(lens), _lib.ptr(means), _lib.ptr(stds),
        m, ctypes.byref(sx), dim, metric.metric_id, ctypes.byref(p), _lib.ptr(dist),
        _lib.ptr(idx), 1 if dev else 0, _stream(X))
    _lib.check(st)
    if dev is None:
        idx = idx.astype(np.intp, copy=False)
    return dist, idx


def pairwise_subsequence_distance(y, x, *, dim=0, metric="euclidean", metric_params=None,
                                  scale=False, return_index=False, n_jobs=None):
    """Minimum subsequence distance between subsequences and time series.

    Mirrors distance/_distance.py:543-636: every subsequence in y against
    every series in x, (n_samples, n_subsequences) outputs.
    """
    y = _validate_subsequence(y)
    X = _as_input(x)
    for s in y:
        if s.shape[0] > X.shape[-1]:
            raise ValueError(
                "Invalid subsequnce shape (%d > %d)" % (s.shape[0], X.shape[-1])
            )
    Metric_ = check_subsequence_metric(metric, scale=scale)
    metric_params = metric_params or {}
    metric = Metric_(**metric_params)
    if not (0 <= dim < X.shape[1]):
        raise ValueError("The parameter dim must be 0 <= dim < n_dims")
    dist, idx = _subsequence_call(y, X, dim, metric, paired=False)
    if return_index:
        return _format_return(dist, len(y), X.ndim), _format_return(idx, len(y), X.ndim)
    return _format_return(dist, len(y), X.ndim)


def paired_subsequence_distance(y, x, *, dim=0, metric="euclidean", metric_params=None,
                                scale=False, return_index=False, n_jobs=None):
    """Minimum subsequence distance between the i:th subsequence and the i:th
    time series.

    Mirrors distance/_distance.py:639-729 (including its dim check, which
    accepts dim 0 only, and its messages); outputs have shape (n_samples,).
    """
    y = _validate_subsequence(y)
    X = _as_input(x)
    n_dims = X.shape[1]
    if not 0 >= dim < n_dims:
        raise ValueError("The parameter dim must be 0 <= dim < n_dims")
    for s in y:
        if s.shape[0] > X.shape[-1]:
            raise ValueError(
                "Invalid subsequnce shape (%d > %d)" % (s.shape[0], X.shape[-1])
            )
    Metric_ = check_subsequence_metric(metric, scale=scale)
    n_samples = X.shape[0] if X.ndim > 1 else 1
    if len(y) != n_samples:
        raise ValueError(
            "The number of subsequences and samples must be the same, got %d "
            "subsequences and %d samples." % (len(y), n_samples)
        )
    metric_params = metric_params if metric_params is not None else {}
    metric = Metric_(**metric_params)
    dist, idx = _subsequence_call(y, X, dim, metric, paired=True)
    if return_index:
        return _format_return(dist, len(y), X.ndim), _format_return(idx, len(y), X.ndim)
    return _format_return(dist, len(y), X.ndim)
