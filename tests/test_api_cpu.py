"""CPU-only checks: C ABI symbols, metric registry and validation, failure
without a GPU (no silent CPU fallback)."""

import ctypes
import os
import pickle
import re

import numpy as np
import pytest

from wildboar_gb300 import _build, _lib
from wildboar_gb300.distance import (
    _METRICS,
    argmin_distance,
    pairwise_distance,
    pairwise_subsequence_distance,
)
from wildboar_gb300.distance._validation import is_end_of_series

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            with open(os.path.join(inc, f)) as fh:
                text = fh.read()
            syms |= set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(wb_\w+)\s*\(", text, re.M))
    return syms


@pytest.fixture(scope="module")
def libpath():
    return _build.build()


def test_library_exports_every_declared_symbol(libpath):
    syms = _header_symbols()
    assert {"wb_pairwise_distance", "wb_paired_distance", "wb_argmin_distance",
            "wb_pairwise_subsequence_distance", "wb_last_error"} <= syms
    L = ctypes.CDLL(libpath)
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing


def test_no_gpu_raises_instead_of_falling_back():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        pairwise_distance(np.ones((2, 4)), np.zeros((2, 4)), metric="dtw")


@pytest.mark.parametrize("metric", sorted(_METRICS))
def test_pickle(metric):
    m = _METRICS[metric]()
    m2 = pickle.loads(pickle.dumps(m))
    assert m == m2 and type(m2) is type(m)


@pytest.mark.parametrize("metric", sorted(_METRICS))
def test_metric_raises_bad_argument(metric):
    # test_distance.py:809-813
    with pytest.raises(TypeError):
        _METRICS[metric](not_an_argument=10)


@pytest.mark.parametrize("metric", ["dtw", "ddtw", "wdtw", "wddtw", "adtw", "lcss", "wlcss",
                                    "erp", "edr", "msm", "twe"])
@pytest.mark.parametrize("r", [-0.1, 1.1])
def test_raises_bad_r_argument_value(metric, r):
    # test_distance.py:816-826
    with pytest.raises(ValueError, match="r =="):
        _METRICS[metric](r=r)


@pytest.mark.parametrize("metric,params,match", [
    ("lcss", {"epsilon": 0}, "epsilon == 0.0, must be > 0"),
    ("lcss", {"epsilon": -1}, "epsilon"),
    ("edr", {"epsilon": 0}, "epsilon == 0.0, must be > 0"),
    ("msm", {"c": -1}, "c == -1.0, must be >= 0"),
    ("twe", {"penalty": -1}, "penalty == -1.0, must be >= 0.0"),
    ("twe", {"stiffness": 0}, "stiffness == 0.0, must be > 0.0"),
    ("erp", {"g": -1}, "g == -1.0, must be >= 0"),
    ("wdtw", {"g": -1}, "g == -1.0, must be >= 0.0"),
])
def test_raises_bad_argument_value(metric, params, match):
    # test_distance.py:829-848
    with pytest.raises(ValueError, match=match):
        _METRICS[metric](**params)


def test_lcss_threshold_is_deprecated():
    with pytest.warns(FutureWarning):
        m = _METRICS["lcss"](threshold=0.5)
    assert m.epsilon == 0.5


def test_unknown_metric():
    with pytest.raises(ValueError, match="unsupported metric"):
        pairwise_distance(np.ones((2, 3)), metric="nope")


def test_nan_and_eos_are_rejected():
    x = np.ones((3, 5))
    x[1, 2] = np.nan
    with pytest.raises(ValueError, match="Input contains NaN."):
        pairwise_distance(x, np.ones((2, 5)), metric="dtw")
    eos = np.array(0x7F800009, dtype="I").view("f").item()
    x = np.ones((3, 5))
    x[0, 4] = eos
    assert is_end_of_series(x).sum() == 1
    with pytest.raises(ValueError, match="expected time series of equal length"):
        pairwise_distance(x, np.ones((2, 5)), metric="dtw")
    x = np.ones((3, 5))
    x[0, 0] = np.inf
    with pytest.raises(ValueError, match="infinity"):
        pairwise_distance(x, np.ones((2, 5)), metric="dtw")


def test_shape_errors():
    with pytest.raises(ValueError, match="not compatible"):
        pairwise_distance(np.ones((2, 3, 4)), np.ones((2, 4)), metric="dtw")
    with pytest.raises(ValueError, match="same number of dimensions"):
        pairwise_distance(np.ones((2, 3, 4)), np.ones((2, 2, 4)), metric="dtw")
    with pytest.raises(ValueError, match="Illegal n_timestep"):
        pairwise_distance(np.ones((2, 4)), np.ones((2, 5)), metric="euclidean")
    with pytest.raises(ValueError, match="dim"):
        pairwise_distance(np.ones((2, 3, 4)), np.ones((2, 3, 4)), dim=3, metric="dtw")


def test_singleton_1d_is_zero():
    assert pairwise_distance(np.ones(5), metric="dtw") == 0.0


def test_argmin_parameter_validation():
    with pytest.raises(ValueError, match="'k' parameter"):
        argmin_distance(np.ones((2, 4)), np.ones((3, 4)), k=0)
    with pytest.raises(TypeError, match="'metric' parameter"):
        argmin_distance(np.ones((2, 4)), np.ones((3, 4)), metric="nope")
    with pytest.raises(ValueError, match="lower bound must be of shape"):
        argmin_distance(np.ones((2, 4)), np.ones((3, 4)), metric="dtw",
                        lower_bound=np.ones((2, 2)))
    with pytest.raises(ValueError, match="dim"):
        argmin_distance(np.ones((2, 4)), np.ones((3, 4)), metric="dtw", dim=1)


def test_subsequence_validation():
    with pytest.raises(ValueError, match="cannot be empty"):
        pairwise_subsequence_distance([], np.ones((2, 10)))
    with pytest.raises(ValueError, match="Invalid subsequnce shape"):
        pairwise_subsequence_distance(np.ones(11), np.ones((2, 10)))
    with pytest.raises(ValueError, match="unsupported metric"):
        pairwise_subsequence_distance(np.ones(3), np.ones((2, 10)), metric="manhattan")


def test_params_struct_matches_header():
    # wb_params is seven doubles in declaration order
    assert ctypes.sizeof(_lib.Params) == 7 * 8
    assert ctypes.sizeof(_lib.Series) == 8 + 3 * 8 + 2 * 4


def test_subsequence_search_validation():
    # the checks of distance/_distance.py:639-1761 run before any device call
    from wildboar_gb300.distance import (
        argmin_subsequence_distance,
        distance_profile,
        paired_subsequence_distance,
        paired_subsequence_match,
        subsequence_match,
    )

    X = np.cumsum(np.random.default_rng(0).standard_normal((4, 30)), axis=1)
    with pytest.raises(ValueError, match="same"):
        paired_subsequence_distance([X[0, :5], X[1, :5]], X)
    with pytest.raises(ValueError, match="Invalid subsequnce shape"):
        paired_subsequence_distance([np.zeros(40)] * 4, X)
    with pytest.raises(ValueError, match="dim"):
        paired_subsequence_distance([X[i, :5] for i in range(4)], X.reshape(4, 1, 30), dim=1)
    with pytest.raises(ValueError, match="single subsequence"):
        subsequence_match([X[0, :5], X[1, :5]], X)
    with pytest.raises(TypeError, match="threshold"):
        subsequence_match(X[0, :5], X, threshold=object())
    with pytest.raises(ValueError, match="threshold array length"):
        subsequence_match(X[0, :5], X, threshold=[1.0, 2.0])
    with pytest.raises(ValueError, match="threshold must be"):
        subsequence_match(X[0, :5], X, threshold="median")
    with pytest.raises(ValueError, match="exclude"):
        subsequence_match(X[0, :5], X, threshold=1.0, exclude=-1)
    with pytest.raises(ValueError, match="same number of samples"):
        paired_subsequence_match([X[0, :5]], X)
    with pytest.raises(ValueError, match="k must be less"):
        argmin_subsequence_distance(X[:, :10], X, k=30)
    with pytest.raises(ValueError, match="same number of samples"):
        argmin_subsequence_distance(X[:2, :10], X)
    with pytest.raises(ValueError, match="shorter than samples"):
        argmin_subsequence_distance(np.zeros((4, 40)), X)
    with pytest.raises(ValueError, match="same number of samples"):
        distance_profile(X[:2, :10], X)
    with pytest.raises(ValueError, match="larger than input"):
        distance_profile(np.zeros(40), X, metric="euclidean")


def test_sharded_requires_process_group():
    from wildboar_gb300.distance import sharded

    with pytest.raises(ValueError):
        sharded.shard_bounds(3, -1, 2)


def test_transient_statistics_match_the_oracle_bitwise():
    # the host helper of the subsequence searches against the oracle's C
    # fast_mean_std (gcc -O2: pow(v, 2.0) folded into v * v, as in the
    # reference's build), on ragged rows with large values and constant rows
    from oracle import oracle as O
    from wildboar_gb300.distance._subsequence import _transient_stats_rows

    rng = np.random.default_rng(5)
    n, width = 400, 90
    lens = rng.integers(1, width + 1, size=n)
    S = np.zeros((n, width))
    for i in range(n):
        S[i, :lens[i]] = rng.standard_normal(lens[i]) * rng.choice([1e-9, 1.0, 1e6, 3e12])
    S[5, :lens[5]] = 2.5          # constant: std 0
    S[6, :lens[6]] = 0.0
    mean, std = _transient_stats_rows(S, lens)
    for i in range(n):
        om, os_ = O.fast_mean_std(S[i, :lens[i]])
        assert np.float64(om).view(np.uint64) == mean[i].view(np.uint64), i
        assert np.float64(os_).view(np.uint64) == std[i].view(np.uint64), i


@pytest.mark.parametrize("mid", [0, 1, 2, 5, 6, 7, 8, 9, 10, 11, 33])
@pytest.mark.parametrize("threshold", [0.5, 3.0, float("inf")])
def test_subsequence_match_filter_all_pairs_at_once(mid, threshold):
    # the vectorised post-filter of subsequence_match against the per-pair
    # filter it replaces, on synthetic (raw, key) profiles with ragged lengths
    from wildboar_gb300.distance import _subsequence as S

    rng = np.random.default_rng(mid + int(threshold) if threshold < 1e9 else mid + 99)
    T, n = 60, 9
    lens = rng.integers(3, 20, size=n)
    ld = int(T - lens.min() + 1)
    raw = np.abs(rng.standard_normal((n, ld))) * 4
    key = raw * rng.uniform(0.2, 1.5, size=raw.shape)
    if mid == 5:
        raw -= 1.0  # adtw may go negative
    for i in range(n):
        raw[i, T - lens[i] + 1:] = np.nan
        key[i, T - lens[i] + 1:] = np.nan
    got_i, got_d = S._matches_from_profile(mid, raw, key, lens, T, threshold)
    for i in range(n):
        L = int(lens[i])
        nwin = T - L + 1
        r, k = raw[i, :nwin], key[i, :nwin]
        d = S._distances(mid, r, L)
        keep = S._match_mask(mid, r, k, d, L, T, threshold)
        idx = np.flatnonzero(keep)
        if idx.size == 0:
            assert got_i[i] is None and got_d[i] is None
        else:
            np.testing.assert_array_equal(got_i[i], idx)
            assert np.array_equal(got_d[i].view(np.uint64),
                                  np.asarray(d[keep], dtype=np.double).view(np.uint64))


def test_shapelet_statistics_grouped_by_length_bitwise():
    # ScaledSubsequenceMetric.from_array takes np.mean / np.std per shapelet;
    # the host computes them once per distinct length over stacked rows
    from wildboar_gb300.distance._distance import _shapelet_stats

    rng = np.random.default_rng(8)
    shp = [np.cumsum(rng.standard_normal(int(L))) * rng.choice([1e-6, 1.0, 1e7])
           for L in rng.integers(1, 300, size=700)]
    lens = np.array([len(s) for s in shp])
    mean, std = _shapelet_stats(shp, lens)
    for i, s in enumerate(shp):
        assert np.mean(s).view(np.uint64) == mean[i].view(np.uint64), i
        assert np.std(s).view(np.uint64) == std[i].view(np.uint64), i


def test_distance_profile_parameter_validation():
    # @validate_params of distance_profile (distance/_distance.py:1460-1476) and
    # the checks of its body (:1561-1581); all raise before any device call
    from wildboar_gb300.distance import InvalidParameterError, distance_profile

    y, x = np.arange(5.0), np.cumsum(np.ones((2, 30)), axis=1)
    with pytest.raises(InvalidParameterError, match="'dilation' parameter"):
        distance_profile(y, x, dilation=0)
    with pytest.raises(InvalidParameterError, match="'padding' parameter"):
        distance_profile(y, x, padding=-1)
    with pytest.raises(InvalidParameterError, match="'padding' parameter"):
        distance_profile(y, x, padding="valid")
    with pytest.raises(InvalidParameterError, match="'metric' parameter"):
        distance_profile(y, x, metric="wlcss")
    with pytest.raises(ValueError, match="only supported for odd"):
        distance_profile(np.arange(4.0), x, padding="same")
    with pytest.raises(ValueError, match="larger than input"):
        distance_profile(np.arange(9.0), x[:, :5], dilation=2, padding=1)
    with pytest.raises(NotImplementedError, match="pointwise"):
        distance_profile(y, x, metric="scaled_manhattan", dilation=2)


def test_kept_direction_bytes_on_the_host():
    # wb_dtw32_keep_bytes is host arithmetic (no device call): per batch of 32
    # items the two strip tables (256-byte aligned) and 32 lanes x cap words,
    # cap = strips of the shorter (dtw) or x (wdtw) length x the longer length,
    # rounded to whole groups of 8
    import ctypes

    from wildboar_gb300 import _lib
    from wildboar_gb300.distance import batched as B

    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libwbgpu.so is not built")
    fn = _lib.lib().wb_dtw32_keep_bytes

    def job(x_len, y_len, n_items, weighted=False):
        j = B.Dtw32()
        j.x_len, j.y_len, j.nx, j.ny = x_len, y_len, 1, n_items
        j.n_items, j.r = n_items, 0.2
        j.weights = 8 if weighted else None  # only whether it is set matters here
        return j

    def want(x_len, y_len, n_items, weighted=False):
        rows = x_len if weighted else min(x_len, y_len)
        strips = (rows - 2) // 16 + 1 if rows > 1 else 0
        cap = (max(strips * max(x_len, y_len), 8) + 7) // 8 * 8
        tab = (2 * max(strips, 1) * 4 + 255) // 256 * 256
        return (n_items + 31) // 32 * (tab + 32 * cap * 4)

    for args in ((256, 256, 131072), (300, 180, 360), (140, 260, 360, True), (1, 1, 5),
                 (2048, 32, 33), (17, 17, 0)):
        assert fn(ctypes.byref(job(*args))) == want(*args), args
    # C5: 4096 x 32 pairs of length 256 keep 2.1 GB of directions
    assert abs(fn(ctypes.byref(job(256, 256, 131072))) / 1e9 - 2.15) < 0.01
    assert fn(ctypes.byref(job(0, 5, 3))) == -1
    assert fn(None) == -1
