"""paired_subsequence_distance, argmin_subsequence_distance, distance_profile,
subsequence_match and paired_subsequence_match on the GPU.

Parity: the reference's own outputs (golden fixtures made by running it,
tests/golden/make_golden.py) through the public API, and the CPU oracle on
larger seeded cases.  Distances within 1e-12 relative (the kernels perform
the reference's operations; 1e-12 absorbs libm differences between
machines), indices and match sets exact.
"""

import math
import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from tests import _golden  # noqa: E402
from wildboar_gb300.distance import (  # noqa: E402
    argmin_subsequence_distance,
    distance_profile,
    paired_subsequence_distance,
    paired_subsequence_match,
    subsequence_match,
)

RTOL = 1e-12


def _flat(res):
    idx, dist = res
    idx = np.atleast_1d(np.asarray(idx, dtype=object)) if not isinstance(idx, np.ndarray) \
        else idx
    if idx.dtype != object:  # a single sample's matches come back as one array
        idx, dist = [idx], [dist]
    counts = np.array([0 if a is None else len(a) for a in idx], dtype=np.int64)
    fi = [np.asarray(a, dtype=np.int64) for a in idx if a is not None]
    fd = [np.asarray(a, dtype=float) for a in dist if a is not None]
    return (counts, np.concatenate(fi) if fi else np.zeros(0, np.int64),
            np.concatenate(fd) if fd else np.zeros(0))


def _cases(kind):
    cs = _golden.cases(kind)
    return pytest.mark.parametrize("case", cs, ids=[c["name"] for c in cs])


@_cases("paired_subsequence")
def test_paired_subsequence_golden(case):
    a = case["args"]
    shp = _golden.unpack_shapelets(case)
    d, i = paired_subsequence_distance(shp, case["inputs"]["x"], metric=a["metric"],
                                       metric_params=a.get("metric_params"),
                                       return_index=True)
    np.testing.assert_allclose(d, case["outputs"]["d"], rtol=RTOL, atol=0)
    np.testing.assert_array_equal(i, case["outputs"]["idx"])


@_cases("argmin_subsequence")
def test_argmin_subsequence_golden(case):
    a = case["args"]
    inp = case["inputs"]
    idx, dist = argmin_subsequence_distance(inp["y"], inp["x"], k=a["k"], metric=a["metric"],
                                            metric_params=a.get("metric_params"),
                                            scale=a["scale"], return_distance=True)
    np.testing.assert_array_equal(idx, case["outputs"]["idx"])
    np.testing.assert_allclose(dist, case["outputs"]["dist"], rtol=RTOL, atol=0)


@_cases("dilated_profile")
def test_dilated_profile_golden(case):
    a = case["args"]
    inp = case["inputs"]
    dp = distance_profile(inp["y"], inp["x"], metric=a["metric"],
                          metric_params=a.get("metric_params"), dilation=a["dilation"],
                          padding=a["padding"], dim=a.get("dim", 0),
                          scale=a.get("scale", False))
    want = case["outputs"]["d"]
    assert dp.shape == want.shape
    np.testing.assert_allclose(dp, want, rtol=RTOL, atol=0)


# the reference's MASS cross-correlation is a pocketfft product, the kernel's
# an exact dot product: the profiles agree to the FFT's rounding
MASS_ATOL = 1e-8


@_cases("mass_profile")
def test_mass_profile_golden(case):
    inp = case["inputs"]
    dp = distance_profile(inp["y"], inp["x"])
    want = case["outputs"]["d"]
    assert dp.shape == want.shape
    np.testing.assert_allclose(dp, want, rtol=0, atol=MASS_ATOL)


@pytest.mark.parametrize("metric,params", [("euclidean", {}), ("mass", {}), ("dtw", {"r": 0.2}),
                                           ("scaled_msm", {}), ("wdtw", {"g": 0.1}),
                                           ("edr", {}), ("twe", {})])
@pytest.mark.parametrize("dilation,padding", [(1, 4), (3, 0), (2, "same"), (5, 17)])
def test_dilated_profile_vs_oracle(metric, params, dilation, padding):
    rng = np.random.default_rng(zlib.crc32(repr((metric, dilation, padding)).encode()))
    X = np.cumsum(rng.standard_normal((6, 2, 300)), axis=-1)
    Y = np.cumsum(rng.standard_normal((6, 11)), axis=-1)
    want = O.dilated_profile(Y, X, dilation=dilation, padding=padding, dim=1, metric=metric,
                             metric_params=params)
    got = distance_profile(Y, X, dilation=dilation, padding=padding, dim=1, metric=metric,
                           metric_params=params)
    np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)
    # device inputs give the same host profile
    got_d = distance_profile(Y, torch.as_tensor(X, device="cuda"), dilation=dilation,
                             padding=padding, dim=1, metric=metric, metric_params=params)
    np.testing.assert_array_equal(got_d, got)


def test_mass_profile_vs_oracle():
    rng = np.random.default_rng(31)
    X = np.cumsum(rng.standard_normal((5, 500)), axis=-1)
    Y = np.cumsum(rng.standard_normal((5, 37)), axis=-1)
    X[3, 100:200] = -2.0
    np.testing.assert_allclose(distance_profile(Y, X), O.mass_profile(Y, X), rtol=0,
                               atol=MASS_ATOL)


@_cases("distance_profile")
def test_distance_profile_golden(case):
    a = case["args"]
    inp = case["inputs"]
    dp = distance_profile(inp["y"], inp["x"], metric=a["metric"],
                          metric_params=a.get("metric_params"))
    np.testing.assert_allclose(dp, case["outputs"]["d"], rtol=RTOL, atol=0)


@_cases("subsequence_match")
def test_subsequence_match_golden(case):
    a = case["args"]
    inp = case["inputs"]
    res = subsequence_match(inp["y"], inp["x"], metric=a["metric"],
                            metric_params=a.get("metric_params"), return_distance=True,
                            **a["kw"])
    counts, idx, dist = _flat(res)
    np.testing.assert_array_equal(counts, case["outputs"]["counts"])
    np.testing.assert_array_equal(idx, case["outputs"]["idx"])
    np.testing.assert_allclose(dist, case["outputs"]["dist"], rtol=RTOL, atol=0)


@_cases("paired_subsequence_match")
def test_paired_subsequence_match_golden(case):
    a = case["args"]
    shp = _golden.unpack_shapelets(case)
    res = paired_subsequence_match(shp, case["inputs"]["x"], metric=a["metric"],
                                   metric_params=a.get("metric_params"),
                                   return_distance=True, **a["kw"])
    counts, idx, dist = _flat(res)
    np.testing.assert_array_equal(counts, case["outputs"]["counts"])
    np.testing.assert_array_equal(idx, case["outputs"]["idx"])
    np.testing.assert_allclose(dist, case["outputs"]["dist"], rtol=RTOL, atol=0)


ARGMIN_METRICS = [
    ("euclidean", {}, False), ("euclidean", {}, True), ("dtw", {"r": 0.2}, False),
    ("dtw", {"r": 0.5}, True), ("wdtw", {"g": 0.1}, False), ("ddtw", {"r": 0.3}, False),
    ("ddtw", {}, True), ("adtw", {"p": 0.4}, False), ("adtw", {"p": -0.1}, True),
    ("lcss", {"epsilon": 0.4}, False), ("edr", {"epsilon": 0.3}, True),
    ("erp", {"g": 0.1}, False), ("erp", {}, True), ("msm", {"c": 0.7}, False),
    ("twe", {"penalty": 0.5}, True),
]


@pytest.mark.parametrize("metric,params,scale", ARGMIN_METRICS,
                         ids=[f"{m}-{s}-{i}" for i, (m, _, s) in enumerate(ARGMIN_METRICS)])
def test_argmin_subsequence_vs_oracle(metric, params, scale):
    rng = np.random.default_rng(41)
    X = np.cumsum(rng.standard_normal((17, 150)), axis=1)
    lens = rng.integers(8, 40, size=17)
    Y = [np.cumsum(rng.standard_normal(int(L))) for L in lens]
    Y[3] = X[3, 50:50 + len(Y[3])].copy()
    k = 5
    idx, dist = argmin_subsequence_distance(Y, X, k=k, metric=metric, metric_params=params,
                                            scale=scale, return_distance=True)
    oi, od = O.argmin_subsequence(Y, X, k=k, metric=metric, metric_params=params,
                                  scale=scale)
    np.testing.assert_array_equal(idx, oi)
    np.testing.assert_allclose(dist, od, rtol=RTOL, atol=0)


PROFILE_METRICS = [("euclidean", {}), ("scaled_euclidean", {}), ("dtw", {"r": 0.3}),
                   ("wdtw", {"g": 0.2}), ("ddtw", {}), ("adtw", {"p": -0.2}),
                   ("lcss", {"epsilon": 0.5}), ("edr", {}), ("erp", {"g": 0.3}),
                   ("msm", {}), ("twe", {"stiffness": 0.01})]


@pytest.mark.parametrize("metric,params", PROFILE_METRICS, ids=[m for m, _ in PROFILE_METRICS])
def test_profile_and_matches_vs_oracle(metric, params):
    rng = np.random.default_rng(43)
    X = np.cumsum(rng.standard_normal((9, 120)), axis=1)
    q = X[4, 30:52].copy() + rng.standard_normal(22) * 0.05
    dp = distance_profile(q, X, metric=metric, metric_params=params)
    od, _ = O.subsequence_matches([q] * 9, X, math.inf, metric=metric, metric_params=params,
                                  transient=True)
    np.testing.assert_allclose(dp, od, rtol=RTOL, atol=0)
    # matches at a threshold near the 20th percentile of the profile
    thr = float(np.nanpercentile(dp, 20))
    res = subsequence_match(q, X, thr, metric=metric, metric_params=params,
                            return_distance=True)
    counts, idx, dist = _flat(res)
    d2, keep = O.subsequence_matches([q] * 9, X, thr, metric=metric, metric_params=params)
    want_counts = (keep > 0).sum(axis=1)
    np.testing.assert_array_equal(counts, want_counts)
    np.testing.assert_array_equal(idx, np.concatenate(
        [np.flatnonzero(keep[i] > 0) for i in range(9)]))
    np.testing.assert_allclose(dist, d2[keep > 0], rtol=RTOL, atol=0)


@pytest.mark.parametrize("metric", ["euclidean", "scaled_euclidean"])
def test_min_scan_near_ties_vs_oracle(metric):
    # periodic series: many windows tie or nearly tie with the best one, so the
    # FP32 pre-filter must keep every window that can still be the first minimum
    from wildboar_gb300.distance import pairwise_subsequence_distance

    rng = np.random.default_rng(44)
    t = np.arange(600)
    base = np.sin(t * 2 * np.pi / 37.0) * 3.0 + 50.0
    X = np.stack([base + rng.standard_normal(600) * s for s in (0.0, 1e-9, 1e-6, 1e-3, 0.1)])
    shp = [base[k:k + L].copy() for k, L in ((0, 37), (5, 74), (11, 20), (3, 111))]
    shp += [base[0:50] + 1e-7, np.full(16, 50.0), rng.standard_normal(40)]
    d, i = pairwise_subsequence_distance(shp, X, metric=metric, return_index=True)
    od, oi = O.subsequence(shp, X, metric=metric)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


@pytest.mark.parametrize("r", [0.0, 0.05, 0.2, 1.0])
def test_scaled_dtw_scan_vs_oracle(r):
    # the UCR scan: lower bounds prune windows against the running best; the
    # GPU's 32-window replay must take the reference's decisions
    from wildboar_gb300.distance import (paired_subsequence_distance,
                                         pairwise_subsequence_distance)

    rng = np.random.default_rng(45)
    X = np.cumsum(rng.standard_normal((12, 300)), axis=1)
    X[5, 100:140] = X[5, 100]
    shp = [X[k % 12, 20 + 7 * k:20 + 7 * k + L].copy() + 0.02 * rng.standard_normal(L)
           for k, L in enumerate((8, 16, 16, 33, 64, 5, 100, 23))]
    shp.append(rng.standard_normal(40))
    d, i = pairwise_subsequence_distance(shp, X, metric="scaled_dtw", metric_params={"r": r},
                                         return_index=True)
    od, oi = O.scaled_dtw_subsequence(shp, X, r=r)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_allclose(d, od, rtol=RTOL, atol=0)
    d, i = paired_subsequence_distance(shp[:9] + shp[:3], X, metric="scaled_dtw",
                                       metric_params={"r": r}, return_index=True)
    od, oi = O.scaled_dtw_subsequence(shp[:9] + shp[:3], X, r=r, paired=True)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_allclose(d, od, rtol=RTOL, atol=0)


@pytest.mark.parametrize("r", [0.1, 1.0])
def test_scaled_dtw_profile_and_matches_vs_oracle(r):
    rng = np.random.default_rng(46)
    X = np.cumsum(rng.standard_normal((7, 200)), axis=1)
    q = X[3, 50:80].copy() + rng.standard_normal(30) * 0.05
    dp = distance_profile(q, X, metric="scaled_dtw", metric_params={"r": r})
    od, _ = O.scaled_dtw_matches([q] * 7, X, np.inf, r=r, transient=True)
    np.testing.assert_allclose(dp, od[:, :171], rtol=RTOL, atol=0)
    thr = float(np.nanpercentile(dp, 15))
    res = subsequence_match(q, X, thr, metric="scaled_dtw", metric_params={"r": r},
                            return_distance=True)
    counts, idx, dist = _flat(res)
    d2, keep = O.scaled_dtw_matches([q] * 7, X, thr, r=r)
    keep = keep[:, :171]
    np.testing.assert_array_equal(counts, (keep > 0).sum(axis=1))
    np.testing.assert_array_equal(idx, np.concatenate(
        [np.flatnonzero(keep[i] > 0) for i in range(7)]))
    np.testing.assert_allclose(dist, d2[:, :171][keep > 0], rtol=RTOL, atol=0)


@pytest.mark.parametrize("left,right", [("euclidean", "dtw"),
                                        ("scaled_euclidean", "scaled_dtw")])
def test_subsequence_match_equivalent(left, right):
    # the reference's test_subsequence_match_equivalent
    # (tests/wildboar/distance/test_distance.py:1440-1477) on random walks:
    # a warp window of 0 makes dtw the euclidean distance
    rng = np.random.default_rng(47)
    x = np.cumsum(rng.standard_normal((10, 150)), axis=1)
    q = x[9, 40:60].copy()

    def run(metric):
        return subsequence_match(q, x[0:9], return_distance=True, max_matches=20, exclude=4,
                                 metric=metric,
                                 metric_params={"r": 0.0} if "dtw" in metric else {})

    li, ld = run(left)
    ri, rd = run(right)
    for a, b in zip(ld, rd):
        np.testing.assert_almost_equal(a, b)
    for a, b in zip(li, ri):
        np.testing.assert_array_equal(a, b)


LONG_SCAN = [("dtw", {"r": 0.1}), ("dtw", {"r": 1.0}), ("wdtw", {"g": 0.1}), ("ddtw", {"r": 0.3}),
             ("adtw", {"p": 0.5}), ("adtw", {"p": -0.2}), ("edr", {}), ("edr", {"epsilon": 0.4}),
             ("erp", {"g": 0.1}), ("msm", {"c": 0.5}), ("twe", {"penalty": 0.5,
                                                               "stiffness": 0.01}),
             ("lcss", {"epsilon": 0.5})]


@pytest.mark.parametrize("metric,params", LONG_SCAN,
                         ids=[f"{m}-{i}" for i, (m, _) in enumerate(LONG_SCAN)])
def test_elastic_subsequence_long_scan_vs_oracle(metric, params):
    # several rounds of 32 windows per (series, shapelet), near matches planted
    # late in some series: the rounds abandon at the best earlier window
    from wildboar_gb300.distance import pairwise_subsequence_distance

    rng = np.random.default_rng(55)
    X = np.cumsum(rng.standard_normal((6, 300)), axis=1)
    shp = [np.cumsum(rng.standard_normal(int(n))) for n in rng.integers(8, 41, size=24)]
    for k in range(0, 24, 5):
        s = k % 6
        pos = 200 + 3 * k
        X[s, pos:pos + len(shp[k])] = shp[k] + 0.05 * rng.standard_normal(len(shp[k]))
    d, i = pairwise_subsequence_distance(shp, X, metric=metric, metric_params=params,
                                         return_index=True)
    od, oi = O.subsequence(shp, X, metric=metric, metric_params=params)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_allclose(d, od, rtol=RTOL, atol=0)


@pytest.mark.parametrize("metric,params", LONG_SCAN,
                         ids=[f"{m}-{i}" for i, (m, _) in enumerate(LONG_SCAN)])
@pytest.mark.parametrize("scale", [False, True])
def test_argmin_subsequence_long_scan_vs_oracle(monkeypatch, metric, params, scale):
    # many rounds of windows with near matches early and late: the rounds
    # abandon at the heap threshold of the earlier rounds
    rng = np.random.default_rng(57)
    X = np.cumsum(rng.standard_normal((9, 400)), axis=1)
    lens = rng.integers(10, 45, size=9)
    Y = [np.cumsum(rng.standard_normal(int(L))) for L in lens]
    for s in range(9):
        L = len(Y[s])
        for pos in (20 + 7 * s, 300 + 5 * s):
            X[s, pos:pos + L] = Y[s] + 0.05 * rng.standard_normal(L)
    idx, dist = argmin_subsequence_distance(Y, X, k=3, metric=metric, metric_params=params,
                                            scale=scale, return_distance=True)
    oi, od = O.argmin_subsequence(Y, X, k=3, metric=metric, metric_params=params, scale=scale)
    np.testing.assert_array_equal(idx, oi)
    np.testing.assert_allclose(dist, od, rtol=RTOL, atol=0)
    # every window in full: the same heaps bit for bit
    monkeypatch.setenv("WB_GPU_ARGMIN", "all")
    fidx, fdist = argmin_subsequence_distance(Y, X, k=3, metric=metric, metric_params=params,
                                              scale=scale, return_distance=True)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(np.asarray(dist).view(np.uint64), np.asarray(fdist).view(np.uint64))


def test_transient_statistics_square_like_the_compiled_reference():
    # _ts_view_update_statistics squares with `v ** 2`, which the C compiler
    # folds to v * v; a libm pow may round differently for large values.  The
    # scaled searches must match the oracle (gcc -O2, the same folding) bit
    # for bit on such data.
    rng = np.random.default_rng(71)
    X = np.cumsum(rng.standard_normal((200, 260)), axis=1) * 1e6
    Y = [rng.standard_normal(int(L)) * 1e6 for L in rng.integers(10, 60, size=200)]
    idx, dist = argmin_subsequence_distance(Y, X, k=3, metric="scaled_euclidean",
                                            return_distance=True)
    oi, od = O.argmin_subsequence(Y, X, k=3, metric="scaled_euclidean")
    np.testing.assert_array_equal(idx, oi)
    assert np.array_equal(np.asarray(dist).view(np.uint64), od.view(np.uint64))
    y = Y[0]
    dp = distance_profile(y, X[:20], metric="scaled_euclidean")
    od2, _ = O.subsequence_matches([y] * 20, X[:20], np.inf, metric="scaled_euclidean",
                                   transient=True)
    got = np.asarray(dp)
    np.testing.assert_allclose(got, od2[:, :got.shape[1]], rtol=RTOL, atol=0)
