"""ctypes front end of the CPU oracle (test infrastructure only).

Loaded by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs; the
product package never imports this module.  The functions mirror the
reference's Cython entry points (``_pairwise_distance``,
``_singleton_pairwise_distance``, ``_paired_distance``, ``_argmin_distance``,
``_pairwise_subsequence_distance`` in wildboar's distance/_cdistance.pyx) on
(n_samples, n_dims, n_timestep) float64 arrays.
"""

import ctypes
import math
import os

import numpy as np

from . import build as _build

METRIC_IDS = {
    "euclidean": 0,
    "dtw": 1,
    "wdtw": 2,
    "ddtw": 3,
    "wddtw": 4,
    "adtw": 5,
    "lcss": 6,
    "wlcss": 7,
    "edr": 8,
    "erp": 9,
    "msm": 10,
    "twe": 11,
    "scaled_euclidean": 32,
}

# Constructor defaults of the reference metric classes
# (distance/_elastic.pyx:3133, 3231, 3325, 3407, 3347, 3440, 3545, 3574, 3681,
# 3895, 3995).
DEFAULTS = {
    "euclidean": {},
    "dtw": {"r": 1.0},
    "ddtw": {"r": 1.0},
    "wdtw": {"r": 1.0, "g": 0.05},
    "wddtw": {"r": 1.0, "g": 0.05},
    "adtw": {"r": 1.0, "p": 1.0},
    "lcss": {"r": 1.0, "epsilon": 1.0},
    "wlcss": {"r": 1.0, "epsilon": 1.0, "g": 0.05},
    "erp": {"r": 1.0, "g": 0.0},
    "edr": {"r": 1.0, "epsilon": math.nan},
    "msm": {"r": 1.0, "c": 1.0},
    "twe": {"r": 1.0, "penalty": 1.0, "stiffness": 0.001},
    "scaled_euclidean": {},
}


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


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int64)
        i64 = ctypes.c_int64
        pp = ctypes.POINTER(Params)
        L.wbo_pairwise.argtypes = [dp, i64, i64, i64, dp, i64, i64, i64, i64,
                                   ctypes.c_int, pp, dp, ctypes.c_int]
        L.wbo_paired.argtypes = [dp, dp, i64, i64, i64, i64, i64, ctypes.c_int, pp,
                                 dp, ctypes.c_int]
        L.wbo_argmin.argtypes = [dp, i64, i64, i64, dp, i64, i64, i64, i64,
                                 ctypes.c_int, pp, i64, dp, ip, dp, ctypes.c_int]
        L.wbo_subsequence.argtypes = [dp, ip, ip, dp, dp, i64, dp, i64, i64, i64, i64,
                                      ctypes.c_int, pp, dp, ip, ctypes.c_int]
        L.wbo_dilated_profile.argtypes = [dp, i64, dp, i64, i64, i64, i64, ctypes.c_int, pp,
                                          i64, i64, ctypes.c_int, dp]
        L.wbo_cumulative_mean_std.argtypes = [dp, i64, i64, dp, dp]
        L.wbo_distance_1d.argtypes = [dp, i64, dp, i64, ctypes.c_int, pp]
        L.wbo_distance_1d.restype = ctypes.c_double
        L.wbo_fast_mean_std.argtypes = [dp, i64, dp, dp]
        L.wbo_dtw_alignment.argtypes = [dp, i64, dp, i64, i64, dp, dp]
        L.wbo_mm_epoch.argtypes = [dp, i64, i64, dp, i64, i64, dp, dp, dp, dp, ip, dp]
        L.wbo_dtw_envelope.argtypes = [dp, i64, i64, i64, dp, dp]
        L.wbo_lb_keogh.argtypes = [dp, i64, dp, i64, i64, i64, ctypes.c_int, dp]
        L.wbo_scaled_dtw_subsequence.argtypes = [dp, ip, ip, dp, dp, i64, dp, i64, i64, i64,
                                                 i64, ctypes.c_double, ctypes.c_int,
                                                 ctypes.c_double, ctypes.c_int, dp, ip, dp, i64]
        L.wbo_subsequence_matches.argtypes = [dp, ip, ip, dp, dp, i64, dp, i64, i64, i64,
                                              ctypes.c_int, pp, ctypes.c_double, dp, dp, i64,
                                              ctypes.c_int, ctypes.c_int]
        L.wbo_argmin_subsequence.argtypes = [dp, ip, i64, i64, dp, i64, i64, i64,
                                             ctypes.c_int, pp, ctypes.c_int, i64, ip, dp,
                                             ctypes.c_int]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def make_params(metric, metric_params=None):
    p = dict(DEFAULTS[metric])
    p.update(metric_params or {})
    s = Params()
    s.r = p.get("r", 1.0)
    s.g = p.get("g", 0.0)
    s.p = p.get("p", 1.0)
    s.epsilon = p.get("epsilon", math.nan)
    s.c = p.get("c", 1.0)
    s.penalty = p.get("penalty", 1.0)
    s.stiffness = p.get("stiffness", 0.001)
    return s


def _ts(x):
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x.reshape(1, 1, -1)
    elif x.ndim == 2:
        x = x.reshape(x.shape[0], 1, x.shape[1])
    return np.ascontiguousarray(x)


def n_threads_default():
    return os.cpu_count() or 1


def pairwise(x, y=None, *, dim=0, metric="dtw", metric_params=None, n_threads=1):
    """One-dim pairwise distance matrix; y=None is the singleton (x is y) path."""
    X = _ts(x)
    p = make_params(metric, metric_params)
    if y is None:
        out = np.zeros((X.shape[0], X.shape[0]))
        lib().wbo_pairwise(_dp(X), X.shape[0], X.shape[1], X.shape[2], None, 0, 0, 0,
                           dim, METRIC_IDS[metric], ctypes.byref(p), _dp(out), n_threads)
        return out
    Y = _ts(y)
    out = np.empty((X.shape[0], Y.shape[0]))
    lib().wbo_pairwise(_dp(X), X.shape[0], X.shape[1], X.shape[2], _dp(Y), Y.shape[0],
                       Y.shape[1], Y.shape[2], dim, METRIC_IDS[metric], ctypes.byref(p),
                       _dp(out), n_threads)
    return out


def paired(x, y, *, dim=0, metric="dtw", metric_params=None, n_threads=1):
    A = _ts(x)
    B = _ts(y)
    p = make_params(metric, metric_params)
    out = np.empty(A.shape[0])
    lib().wbo_paired(_dp(A), _dp(B), A.shape[0], A.shape[1], A.shape[2], B.shape[2], dim,
                     METRIC_IDS[metric], ctypes.byref(p), _dp(out), n_threads)
    return out


def argmin(x, y, *, k=1, dim=0, metric="dtw", metric_params=None, lower_bound=None,
           n_threads=1):
    X = _ts(x)
    Y = _ts(y)
    k = min(k, Y.shape[0])
    p = make_params(metric, metric_params)
    idx = np.zeros((X.shape[0], k), dtype=np.int64)
    dist = np.zeros((X.shape[0], k))
    lb = None
    if lower_bound is not None:
        lb = np.ascontiguousarray(lower_bound, dtype=np.float64)
    lib().wbo_argmin(_dp(X), X.shape[0], X.shape[1], X.shape[2], _dp(Y), Y.shape[0],
                     Y.shape[1], Y.shape[2], dim, METRIC_IDS[metric], ctypes.byref(p), k,
                     _dp(lb), _ip(idx), _dp(dist), n_threads)
    return idx, dist


# Constructor defaults of the elastic subsequence metric classes
# (distance/_elastic.pyx:2206-3124)
SUBSEQ_DEFAULTS = {
    "dtw": {"r": 1.0},
    "wdtw": {"r": 1.0, "g": 0.05},
    "ddtw": {"r": 1.0},
    "wddtw": {"r": 1.0, "g": 0.05},
    "adtw": {"r": 1.0, "p": 1.0},
    "lcss": {"r": 1.0, "epsilon": 1.0},
    "edr": {"r": 1.0, "epsilon": math.nan},
    "erp": {"r": 1.0, "g": 0.0},
    "msm": {"r": 1.0, "c": 1.0},
    "twe": {"r": 1.0, "penalty": 1.0, "stiffness": 0.001},
}


def subsequence(shapelets, x, *, dim=0, metric="euclidean", metric_params=None,
                n_threads=1, stats=None):
    """(n_samples, n_shapelets) min distance and first argmin index.

    stats: (means, stds) of the shapelets as the caller holds them (e.g. a
    SubsequenceView's _ts_view_update_statistics) instead of np.mean / np.std.
    """
    if metric == "scaled_dtw":
        return scaled_dtw_subsequence(shapelets, x, r=(metric_params or {}).get("r", 1.0),
                                      dim=dim, stats=stats)
    X = _ts(x)
    shp = [np.asarray(s, dtype=np.float64).ravel() for s in shapelets]
    lens = np.array([s.shape[0] for s in shp], dtype=np.int64)
    offs = np.zeros(len(shp), dtype=np.int64)
    offs[1:] = np.cumsum(lens)[:-1]
    packed = np.ascontiguousarray(np.concatenate(shp))
    # ScaledSubsequenceMetric.from_array: distance/_cdistance.pyx:453-467
    smean = np.array([np.mean(s) for s in shp])
    sstd = np.array([np.std(s) for s in shp])
    sstd[sstd <= 1e-13] = 0.0
    if stats is not None:
        smean = np.ascontiguousarray(stats[0], dtype=np.float64)
        sstd = np.ascontiguousarray(stats[1], dtype=np.float64)
    dist = np.empty((X.shape[0], len(shp)))
    idx = np.zeros((X.shape[0], len(shp)), dtype=np.int64)
    pd = dict(SUBSEQ_DEFAULTS.get(metric, {}))
    pd.update(metric_params or {})
    p = Params()
    p.r = pd.get("r", 1.0)
    p.g = pd.get("g", 0.0)
    p.p = pd.get("p", 1.0)
    p.epsilon = pd.get("epsilon", math.nan)
    p.c = pd.get("c", 1.0)
    p.penalty = pd.get("penalty", 1.0)
    p.stiffness = pd.get("stiffness", 0.001)
    lib().wbo_subsequence(_dp(packed), _ip(offs), _ip(lens), _dp(smean), _dp(sstd),
                          len(shp), _dp(X), X.shape[0], X.shape[1], X.shape[2], dim,
                          METRIC_IDS[metric], ctypes.byref(p), _dp(dist), _ip(idx),
                          n_threads)
    return dist, idx


def _subseq_params(metric, metric_params):
    pd = dict(SUBSEQ_DEFAULTS.get(metric, {}))
    pd.update(metric_params or {})
    p = Params()
    p.r = pd.get("r", 1.0)
    p.g = pd.get("g", 0.0)
    p.p = pd.get("p", 1.0)
    p.epsilon = pd.get("epsilon", math.nan)
    p.c = pd.get("c", 1.0)
    p.penalty = pd.get("penalty", 1.0)
    p.stiffness = pd.get("stiffness", 0.001)
    return p


def subsequence_matches(shapelets, x, threshold, *, dim=0, metric="euclidean",
                        metric_params=None, transient=False, n_threads=1):
    """SubsequenceMetric._matches for pairs (shapelets[i], x[i]).

    Returns (dist, keep), each (n, ld) with ld = n_timestep - min length + 1:
    every window's distance as the reference computes it and 1.0 where the
    reference keeps the window for `threshold` (NaN / 0 past a pair's last
    window).  threshold=inf gives the distance profile.  transient: the
    shapelet statistics of _DistanceProfile (fast_mean_std, a zero std kept,
    distance/_cdistance.pyx:1680-1699) instead of from_array's np.mean/np.std.
    """
    X = _ts(x)
    shp = [np.asarray(s, dtype=np.float64).ravel() for s in shapelets]
    lens = np.array([s.shape[0] for s in shp], dtype=np.int64)
    if metric == "scaled_dtw":
        r = (metric_params or {}).get("r", 1.0)
        ld = int(X.shape[2] - lens.min() + 1)
        dist, keep = scaled_dtw_matches(shp, X, threshold, r=r, dim=dim, transient=transient)
        return dist[:, :ld], keep[:, :ld]
    offs = np.zeros(len(shp), dtype=np.int64)
    offs[1:] = np.cumsum(lens)[:-1]
    packed = np.ascontiguousarray(np.concatenate(shp))
    smean = np.array([np.mean(s) for s in shp])
    sstd = np.array([np.std(s) for s in shp])
    sstd[sstd <= 1e-13] = 0.0
    if transient:
        st = [fast_mean_std(s) for s in shp]
        smean = np.array([a for a, _ in st])
        sstd = np.array([b for _, b in st])
    ld = int(X.shape[2] - lens.min() + 1)
    dist = np.full((len(shp), ld), np.nan)
    keep = np.zeros((len(shp), ld))
    p = _subseq_params(metric, metric_params)
    lib().wbo_subsequence_matches(_dp(packed), _ip(offs), _ip(lens), _dp(smean), _dp(sstd),
                                  len(shp), _dp(X), X.shape[1], X.shape[2], dim,
                                  METRIC_IDS[metric], ctypes.byref(p), float(threshold),
                                  _dp(dist), _dp(keep), ld, 1 if transient else 0,
                                  n_threads)
    return dist, keep


def argmin_subsequence(y, x, *, k=1, dim=0, metric="euclidean", metric_params=None,
                       scale=False, n_threads=1):
    """_argmin_subsequence_distance: (n, k) indices and distances in heap order.

    y: (n, L) array or a list of n 1-D arrays (zero padded to the longest, as
    argmin_subsequence_distance does); pair i = (y[i], x[i]).
    """
    X = _ts(x)
    if isinstance(y, np.ndarray) and y.ndim == 2:
        S = np.ascontiguousarray(y, dtype=np.float64)
        lens = np.full(S.shape[0], S.shape[1], dtype=np.int64)
    else:
        lens = np.array([len(s) for s in y], dtype=np.int64)
        S = np.zeros((len(y), int(lens.max())))
        for i, s in enumerate(y):
            S[i, :len(s)] = s
    if metric.startswith("scaled_"):
        metric = metric[7:]
        scale = True
    idx = np.zeros((S.shape[0], k), dtype=np.int64)
    dist = np.zeros((S.shape[0], k))
    p = make_params(metric, metric_params)
    lib().wbo_argmin_subsequence(_dp(S), _ip(lens), S.shape[1], S.shape[0], _dp(X),
                                 X.shape[1], X.shape[2], dim, METRIC_IDS[metric],
                                 ctypes.byref(p), 1 if scale else 0, k, _ip(idx),
                                 _dp(dist), n_threads)
    return idx, dist


def distance_1d(x, y, *, metric="dtw", metric_params=None):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    p = make_params(metric, metric_params)
    return lib().wbo_distance_1d(_dp(x), x.shape[0], _dp(y), y.shape[0],
                                 METRIC_IDS[metric], ctypes.byref(p))


def fast_mean_std(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    m = ctypes.c_double()
    s = ctypes.c_double()
    lib().wbo_fast_mean_std(_dp(x), x.shape[0], ctypes.byref(m), ctypes.byref(s))
    return m.value, s.value


def dtw_alignment(x, y, *, r=1.0, weights=None):
    """distance/dtw.py:246-290 followed by _dtw_alignment (_elastic.pyx:1011-1073).

    Cells outside the band are NaN here (the reference leaves np.empty garbage).
    """
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    n, m = x.shape[0], y.shape[0]
    warp = max(int(math.floor(max(n, m) * r)), 1)
    out = np.full((n, m), np.nan)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    rc = lib().wbo_dtw_alignment(_dp(x), n, _dp(y), m, warp, _dp(w), _dp(out))
    if rc != 0:
        raise ValueError("invalid r")
    return out


def dtw_mapping(alignment):
    """Traceback of distance/dtw.py:362-426: ties prefer diag, then up, then left."""
    a = alignment
    n, m = a.shape
    i, j = n - 1, m - 1
    path = [(i, j)]
    while i > 0 or j > 0:
        if i == 0:
            j -= 1
        elif j == 0:
            i -= 1
        else:
            cand = [a[i - 1, j - 1], a[i - 1, j], a[i, j - 1]]
            c = int(np.argmin(cand))
            if c == 0:
                i -= 1
                j -= 1
            elif c == 1:
                i -= 1
            else:
                j -= 1
        path.append((i, j))
    return path[::-1]


# --------------------------------------------------------------------------
# dtw_average (method="mm") and the estimators that use the distance path


def jeong_weight(n, g=0.05):
    """distance/dtw.py:330-359."""
    return 1.0 / (1.0 + np.exp(-g * (np.arange(n, dtype=float) - n / 2.0)))


def mm_epoch(X, mean, *, r=1.0, weights=None, sample_weight=None, return_last=False):
    """One epoch of _mm_dtw_average (distance/dtw.py:668-682) in C: new mean."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    mean = np.ascontiguousarray(mean, dtype=np.float64)
    N, T = X.shape
    nm = mean.shape[0]
    warp = max(int(math.floor(max(nm, T) * r)), 1)
    out = np.empty(nm)
    work = np.empty(nm * T)
    path = np.empty(2 * (nm + T), dtype=np.int64)
    last = np.empty(N) if return_last else None
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    sw = None if sample_weight is None else np.ascontiguousarray(sample_weight,
                                                                  dtype=np.float64)
    rc = lib().wbo_mm_epoch(_dp(X), N, T, _dp(mean), nm, warp, _dp(w), _dp(sw), _dp(out),
                            _dp(work), _ip(path), _dp(last))
    if rc != 0:
        raise ValueError("invalid r")
    return (out, last) if return_last else out


def dtw_average_mm(X, *, r=1.0, g=None, init, sample_weight=None, tol=1e-5, max_epoch=50):
    """dtw_average(method="mm") with an array init (distance/dtw.py:429-594,
    661-690): returns (mean, cost)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    mean = np.array(init, dtype=np.float64, copy=True)
    if g is None:
        metric, params, weights = "dtw", {"r": r}, None
    else:
        metric, params = "wdtw", {"r": r, "g": g}
        weights = jeong_weight(max(mean.shape[0], X.shape[1]), g)

    def costfn(m):
        d = pairwise(m, X, metric=metric, metric_params=params)[0]
        if sample_weight is None:
            return np.mean(d)
        return np.average(d, weights=sample_weight)

    cost = costfn(mean)
    for _ in range(max_epoch):
        mean = mm_epoch(X, mean, r=r, weights=weights, sample_weight=sample_weight)
        prev_cost = cost
        cost = costfn(mean)
        if abs(prev_cost - cost) < tol:
            break
    return mean, cost


def kmeans(x, n_clusters, *, metric="euclidean", r=1.0, g=None, n_init="auto",
           max_iter=300, tol=1e-3, random_state=None):
    """KMeans.fit (distance/_neighbors.py:309-548): returns (labels, centers,
    inertia, n_iter)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    rs = random_state if isinstance(random_state, np.random.RandomState) \
        else np.random.RandomState(random_state)
    if metric == "euclidean":
        dmetric, dparams = "euclidean", {}
    elif g is None:
        dmetric, dparams = "dtw", {"r": r}
    else:
        dmetric, dparams = "wdtw", {"r": r, "g": g}

    def assign(c):
        idx, dist = argmin(x, c, k=1, metric=dmetric, metric_params=dparams)
        return np.ravel(idx).astype(np.intp), dist

    def fit_one():
        cent = x[rs.choice(x.shape[0], size=n_clusters, replace=False)]
        prev_cost, cost, reassign, it = np.inf, -np.inf, True, 0
        assigned = dist = None
        for it in range(max_iter):
            assigned, dist = assign(cent)
            prev_cost, cost = cost, paired(x, cent[assigned], metric=dmetric,
                                           metric_params=dparams).sum() / x.shape[0]
            if math.isclose(cost, prev_cost, rel_tol=tol):
                reassign = False
                break
            for c in range(n_clusters):
                grp = x[assigned == c]
                if grp.shape[0] == 0:
                    far = dist.min(axis=1).argmax()
                    assigned[far] = c
                    cent[c] = x[far]
                elif grp.shape[0] == 1:
                    cent[c] = grp
                elif metric == "euclidean":
                    cent[c] = grp.mean(axis=0)
                else:
                    rs.randint(np.iinfo(np.int32).max)
                    cent[c] = dtw_average_mm(grp, r=r, g=g, init=cent[c])[0]
        return it, cost, cent, assigned, reassign

    best = None
    for _ in range(1 if n_init == "auto" else n_init):
        res = fit_one()
        if best is None or res[1] < best[1]:
            best = res
    it, cost, cent, assigned, reassign = best
    if reassign:
        assigned, _ = assign(cent)
    return assigned, cent, cost, it


def knn_predict_proba(x_train, y_train, x, *, n_neighbors=5, metric="euclidean",
                      metric_params=None):
    """KNeighborsClassifier.predict_proba (distance/_neighbors.py:237-287), 2-D x."""
    classes, yi = np.unique(y_train, return_inverse=True)
    closest, _ = argmin(x, x_train, k=n_neighbors, metric=metric, metric_params=metric_params)
    preds = yi[closest]
    probs = np.empty((np.asarray(x).shape[0], len(classes)))
    for i in range(len(classes)):
        probs[:, i] = np.sum(preds == i, axis=1) / n_neighbors
    return probs


# --------------------------------------------------------------------------
# scaled_dtw subsequence metric (UCR-suite scan)


def _packed(shapelets):
    shp = [np.asarray(s, dtype=np.float64).ravel() for s in shapelets]
    lens = np.array([s.shape[0] for s in shp], dtype=np.int64)
    offs = np.zeros(len(shp), dtype=np.int64)
    offs[1:] = np.cumsum(lens)[:-1]
    return shp, np.ascontiguousarray(np.concatenate(shp)), offs, lens


def scaled_dtw_subsequence(shapelets, x, *, r=1.0, dim=0, paired=False, stats=None):
    """pairwise / paired_subsequence_distance with metric="scaled_dtw"
    (ScaledDtwSubsequenceMetric, distance/_elastic.pyx:1928-2204, scan
    :353-465): (min distance, first argmin window); (n_samples, m) or (m,)."""
    X = _ts(x)
    shp, packed, offs, lens = _packed(shapelets)
    smean = np.array([np.mean(s) for s in shp])
    sstd = np.array([np.std(s) for s in shp])
    sstd[sstd <= 1e-13] = 0.0
    if stats is not None:
        smean = np.ascontiguousarray(stats[0], dtype=np.float64)
        sstd = np.ascontiguousarray(stats[1], dtype=np.float64)
    shape = (len(shp),) if paired else (X.shape[0], len(shp))
    dist = np.empty(shape)
    idx = np.zeros(shape, dtype=np.int64)
    lib().wbo_scaled_dtw_subsequence(_dp(packed), _ip(offs), _ip(lens), _dp(smean), _dp(sstd),
                                     len(shp), _dp(X), X.shape[0], X.shape[1], X.shape[2], dim,
                                     float(r), 1 if paired else 0, -1.0, 0, _dp(dist),
                                     _ip(idx), None, 0)
    return dist, idx


def scaled_dtw_matches(shapelets, x, threshold, *, r=1.0, dim=0, transient=False):
    """scaled_dtw_matches (distance/_elastic.pyx:468-620) of shapelet i in
    x[i, dim]: (distance per window, keep flags), (n, n_timestep).
    threshold=inf with transient=True is the distance profile
    (_DistanceProfile: fast transient statistics, a zero std kept)."""
    X = _ts(x)
    shp, packed, offs, lens = _packed(shapelets)
    if transient:
        stats = [fast_mean_std(s) for s in shp]
        smean = np.array([a for a, _ in stats])
        sstd = np.array([b for _, b in stats])
    else:
        smean = np.array([np.mean(s) for s in shp])
        sstd = np.array([np.std(s) for s in shp])
        sstd[sstd <= 1e-13] = 0.0
    ld = X.shape[2]
    dist = np.ones((len(shp), ld)) if transient else np.full((len(shp), ld), np.nan)
    keep = np.zeros((len(shp), ld))
    lib().wbo_scaled_dtw_subsequence(_dp(packed), _ip(offs), _ip(lens), _dp(smean), _dp(sstd),
                                     len(shp), _dp(X), X.shape[0], X.shape[1], X.shape[2], dim,
                                     float(r), 1, float(threshold), 1 if transient else 0,
                                     _dp(dist), None, _dp(keep), ld)
    return dist, keep


# --------------------------------------------------------------------------
# lower bounds (distance/lb.py)


def _warp_size(n, r):
    w = max(math.floor(n * r), 1)
    return w - 1 if w == n else w


def dtw_envelope(X, warp):
    """_dtw_envelop (distance/_elastic.pyx:1076-1092) of every row."""
    X = np.ascontiguousarray(np.atleast_2d(X), dtype=np.float64)
    lo = np.empty_like(X)
    up = np.empty_like(X)
    if lib().wbo_dtw_envelope(_dp(X), X.shape[0], X.shape[1], int(warp), _dp(lo), _dp(up)):
        raise ValueError("invalid r")
    return lo, up


def lb_keogh(Q, X, *, r=1.0, kind="both"):
    """DtwKeoghLowerBound(r, kind).fit(X).transform(Q) (distance/lb.py:314-432)."""
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    X = np.ascontiguousarray(X, dtype=np.float64)
    out = np.empty((Q.shape[0], X.shape[0]))
    lib().wbo_lb_keogh(_dp(Q), Q.shape[0], _dp(X), X.shape[0], X.shape[1],
                       _warp_size(X.shape[1], r), {"both": 0, "left": 1, "right": 2}[kind],
                       _dp(out))
    return out


def lb_kim(Q, X):
    """DtwKimLowerBound().fit(X).transform(Q) (distance/lb.py:198-311),
    restated with numpy: per query, vectorised over the fitted series."""
    X = np.asarray(X, dtype=np.float64)
    Q = np.asarray(Q, dtype=np.float64)
    n = X.shape[-1]

    def sq(a, b):
        v = a - b
        return v * v

    out = np.empty((Q.shape[0], X.shape[0]))
    for i in range(Q.shape[0]):
        a0, a0e, b0, b0e = X[:, 0], X[:, -1], Q[i, 0], Q[i, -1]
        d = sq(a0, b0) + sq(a0e, b0e)
        if n > 1:
            a1, a1e, b1, b1e = X[:, 1], X[:, -2], Q[i, 1], Q[i, -2]
            d += np.minimum(sq(a1, b0), np.minimum(sq(a0, b1), sq(a1, b1)))
            d += np.minimum(sq(a1e, b1), np.minimum(sq(a0e, b1e), sq(a1e, b1e)))
            if n > 2:
                a2, a2e, b2, b2e = X[:, 2], X[:, -3], Q[i, 2], Q[i, -3]
                d += np.minimum(sq(a0, b2), np.minimum(sq(a1, b2), np.minimum(
                    sq(a2, b2), np.minimum(sq(a2, b1), sq(a2, b0)))))
                d += np.minimum(sq(a0e, b2e), np.minimum(sq(a1e, b2e), np.minimum(
                    sq(a2e, b2e), np.minimum(sq(a2e, b1e), sq(a2e, b0e)))))
        out[i] = d
    return out


def dtw_average_ssg(X, *, r=1.0, g=None, init, sample_weight=None, max_epoch=50,
                    learning_rate=0.1, decay=0.9, max_stable=5, random_state):
    """_ssg_dtw_average (distance/dtw.py:597-658) with the oracle's alignment
    and traceback; random_state is the RandomState the reference passes on."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    mean = np.array(init, dtype=np.float64, copy=True)
    if g is None:
        metric, params, weights = "dtw", {"r": r}, None
    else:
        metric, params = "wdtw", {"r": r, "g": g}
        weights = jeong_weight(max(mean.shape[0], X.shape[1]), g)

    def costfn(m):
        d = pairwise(m, X, metric=metric, metric_params=params)[0]
        if sample_weight is None:
            return np.mean(d)
        return np.average(d, weights=sample_weight)

    best_mean = None
    order = np.arange(X.shape[0])
    min_cost = np.inf
    n_stable = 0
    z = np.empty(mean.shape[0])
    for epoch in range(max_epoch):
        if n_stable > max_stable:
            break
        random_state.shuffle(order)
        for i, o in enumerate(order):
            z.fill(0)
            path = dtw_mapping(dtw_alignment(mean, X[o], r=r, weights=weights))
            w = 1.0 if sample_weight is None else sample_weight[o]
            for m_, x_ in path:
                z[m_] += mean[m_] - X[o, x_] * w
            mean -= learning_rate * z
            if epoch == 0:
                learning_rate = decay**i * learning_rate
        cost = costfn(mean)
        if cost < min_cost:
            min_cost = cost
            n_stable = 0
            best_mean = mean.copy()
        else:
            n_stable += 1
    return best_mean, min_cost


def dilated_profile(y, x, *, dilation=1, padding=0, dim=0, metric="euclidean",
                    metric_params=None, scale=False):
    """distance_profile with dilation / padding (distance/_distance.py:1560-1619,
    _cdistance.pyx:804-933, 1809-1841): y (n, L) one subsequence per sample,
    x (n, d, T) or (n, T).  "mass" and "scaled_*" metrics run their unscaled
    pairwise metric on z-normalised windows.  Positions the reference leaves
    unwritten (an infinite distance) are NaN."""
    Y = np.ascontiguousarray(np.atleast_2d(np.asarray(y, dtype=np.float64)))
    X = np.asarray(x, dtype=np.float64)
    if X.ndim == 2:
        X = X[:, None, :]
    X = np.ascontiguousarray(X)
    L = Y.shape[1]
    if padding == "same":
        padding = ((L - 1) * dilation + 1) // 2
    if metric == "mass":
        metric = "scaled_euclidean"
    scale = metric.startswith("scaled_") or scale
    if metric.startswith("scaled_"):
        metric = metric[7:]
    if scale:
        std = np.std(Y, axis=-1, keepdims=True)
        mean = np.mean(Y, axis=-1, keepdims=True)
        std[std < 1e-13] = 1
        Y = np.ascontiguousarray((Y - mean) / std)
    n, d, T = X.shape
    out = np.empty((n, T + 2 * padding - ((L - 1) * dilation + 1) + 1))
    p = make_params(metric, metric_params)
    rc = lib().wbo_dilated_profile(_dp(Y), L, _dp(X), n, d, T, dim, METRIC_IDS[metric],
                                   ctypes.byref(p), dilation, padding, 1 if scale else 0,
                                   _dp(out))
    if rc != 0:
        raise ValueError("invalid dilation / padding")
    return out


def mass_profile(y, x):
    """The "mass" distance profile (ScaledMassSubsequenceMetric,
    distance/_mass.pyx:35-240 with cumulative_mean_std, utils/_stats.pyx:95-111,
    and the transient statistics of _cdistance.pyx:167-185): y (n, L), x
    (n, T) (dim 0).  The cross-correlation is numpy's FFT of the zero-padded
    reversed subsequence times the series, as the reference does with its
    vendored pocketfft."""
    Y = np.atleast_2d(np.asarray(y, dtype=np.float64))
    X = np.asarray(x, dtype=np.float64)
    if X.ndim == 3:
        X = X[:, 0, :]
    X = np.atleast_2d(X)
    n, T = X.shape
    L = Y.shape[1]
    nw = T - L + 1
    out = np.empty((n, nw))
    eps = 1e-10
    for i in range(n):
        yi = np.ascontiguousarray(Y[i])
        ex = np.cumsum(yi)[-1]
        ex2 = np.cumsum(yi * yi)[-1]
        mu = ex / L
        var = ex2 / L - mu * mu
        sd = math.sqrt(var) if var > 1e-13 else 0.0
        mt = np.empty(nw)
        st = np.empty(nw)
        xi = np.ascontiguousarray(X[i])
        lib().wbo_cumulative_mean_std(_dp(xi), T, L, _dp(mt), _dp(st))
        yb = np.zeros(T, dtype=complex)
        yb[:L] = yi[::-1]
        qt = np.fft.ifft(np.fft.fft(xi.astype(complex)) * np.fft.fft(yb)).real[L - 1:]
        for w in range(nw):
            zx, zy = st[w] <= eps, sd <= eps
            if zx != zy:
                out[i, w] = math.sqrt(L)
            elif zx:
                out[i, w] = 0.0
            else:
                z = 2 * (L - (qt[w] - L * mt[w] * mu) / (st[w] * sd))
                out[i, w] = 0.0 if z < eps else math.sqrt(z)
    return out
