"""GPU parity: the CUDA path (through the public API and the C ABI) against the
reference's golden outputs and against the CPU oracle on seeded inputs.

FP64 drop-in bar: distances within 1e-12 relative (the kernels perform the
reference's IEEE operations in its order, so they are expected bit-exact),
argmin indices and subsequence argmin indices bit-exact.
"""

import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from tests import _golden  # noqa: E402
from wildboar_gb300 import _lib  # noqa: E402
from wildboar_gb300.distance import (  # noqa: E402
    argmin_distance,
    paired_distance,
    pairwise_distance,
    pairwise_subsequence_distance,
)

RTOL = 1e-12


def _walk(rng, shape):
    return np.cumsum(rng.standard_normal(shape), axis=-1)


def run_api(case):
    a = case["args"]
    metric, params = a.get("metric"), a.get("metric_params", {})
    dim = a.get("dim", "mean")
    inp = case["inputs"]
    kind = case["kind"]
    if kind == "pairwise":
        return {"d": pairwise_distance(inp["x"], inp["y"], dim=dim, metric=metric,
                                       metric_params=params)}
    if kind == "singleton":
        return {"d": pairwise_distance(inp["x"], dim=dim, metric=metric,
                                       metric_params=params)}
    if kind == "paired":
        return {"d": paired_distance(inp["x"], inp["y"], dim=dim, metric=metric,
                                     metric_params=params)}
    if kind == "argmin":
        idx, dist = argmin_distance(inp["x"], inp["y"], k=a["k"], metric=metric,
                                    metric_params=params,
                                    lower_bound=inp.get("lower_bound"),
                                    return_distance=True)
        return {"idx": idx, "dist": dist}
    if kind == "subsequence":
        shp = _golden.unpack_shapelets(case)
        d, i = pairwise_subsequence_distance(shp, inp["x"], metric=metric,
                                             metric_params=params, return_index=True)
        return {"d": d, "idx": i}
    return None


# the subsequence search kinds (paired, argmin, profile, matches) are run by
# tests/test_gpu_subseq_more.py
GOLDEN = [c for c in _golden.cases()
          if c["kind"] in ("pairwise", "singleton", "paired", "argmin", "subsequence")]


@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_golden(case):
    got = run_api(case)
    for key, want in case["outputs"].items():
        g = np.asarray(got[key])
        want = np.asarray(want)
        assert g.shape == want.shape
        if want.dtype.kind in "iu":
            keep = want >= 0  # -1: the reference leaves the index unset
            np.testing.assert_array_equal(g[keep], want[keep])
        else:
            np.testing.assert_allclose(g, want, rtol=RTOL, atol=0)


METRICS = [
    ("dtw", {"r": 0.1}),
    ("dtw", {"r": 1.0}),
    ("dtw", {"r": 0.0}),
    ("wdtw", {"r": 0.3, "g": 0.1}),
    ("ddtw", {"r": 0.2}),
    ("wddtw", {"r": 1.0}),
    ("adtw", {"r": 0.5, "p": 0.5}),
    ("adtw", {"r": 0.5, "p": -0.3}),
    ("lcss", {"r": 0.25, "epsilon": 0.6}),
    ("wlcss", {"r": 1.0, "epsilon": 0.6}),
    ("edr", {"r": 0.4}),
    ("edr", {"r": 1.0, "epsilon": 0.3}),
    ("erp", {"r": 0.3, "g": 0.2}),
    ("msm", {"r": 0.1}),
    ("msm", {"r": 1.0, "c": 0.25}),
    ("twe", {"r": 0.3}),
    ("twe", {"r": 1.0, "penalty": 0.2, "stiffness": 0.05}),
    ("euclidean", {}),
]


@pytest.mark.parametrize("metric,params", METRICS)
@pytest.mark.parametrize("shape", [(23, 17, 64, 64), (9, 12, 90, 57), (11, 7, 40, 131),
                                   (5, 6, 300, 300)])
def test_pairwise_vs_oracle(metric, params, shape):
    nx, ny, lx, ly = shape
    if metric == "euclidean" and lx != ly:
        pytest.skip("euclidean needs equal lengths")
    rng = np.random.default_rng(zlib.crc32(repr((metric, shape)).encode()))
    X = _walk(rng, (nx, lx))
    Y = _walk(rng, (ny, ly))
    got = pairwise_distance(X, Y, metric=metric, metric_params=params)
    want = O.pairwise(X, Y, metric=metric, metric_params=params)
    np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)
    if lx == ly:
        got = pairwise_distance(X, metric=metric, metric_params=params)
        want = O.pairwise(X, None, metric=metric, metric_params=params)
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)
        got = paired_distance(X[: min(nx, ny)], Y[: min(nx, ny)], metric=metric,
                              metric_params=params)
        want = O.paired(X[: min(nx, ny)], Y[: min(nx, ny)], metric=metric,
                        metric_params=params)
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)


@pytest.mark.parametrize("metric,params", METRICS)
@pytest.mark.parametrize("k", [1, 4])
def test_argmin_vs_oracle(metric, params, k):
    rng = np.random.default_rng(7 + k)
    X = _walk(rng, (17, 50))
    Y = _walk(rng, (40, 50 if metric == "euclidean" else 44))
    idx, dist = argmin_distance(X, Y, k=k, metric=metric, metric_params=params,
                                return_distance=True)
    oidx, odist = O.argmin(X, Y, k=k, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)


def test_argmin_lower_bound_vs_oracle():
    rng = np.random.default_rng(3)
    X = _walk(rng, (13, 64))
    Y = _walk(rng, (50, 64))
    full = O.pairwise(X, Y, metric="dtw", metric_params={"r": 0.2})
    lb = full * rng.uniform(0.2, 1.05, size=full.shape)
    idx, dist = argmin_distance(X, Y, k=5, metric="dtw", metric_params={"r": 0.2},
                                lower_bound=lb, return_distance=True)
    oidx, odist = O.argmin(X, Y, k=5, metric="dtw", metric_params={"r": 0.2},
                           lower_bound=lb)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)


def test_argmin_sorted_equals_pairwise_sort():
    # test_argmin_equals_pairwise_distance_argpartition (tests/wildboar/distance/
    # test_distance.py:1543-1560)
    rng = np.random.default_rng(11)
    X = _walk(rng, (20, 70))
    Y = _walk(rng, (60, 70))
    for metric, params in (("dtw", {"r": 0.2}), ("msm", {}), ("euclidean", {})):
        full = pairwise_distance(X, Y, metric=metric, metric_params=params)
        _, dist = argmin_distance(X, Y, k=6, metric=metric, metric_params=params,
                                  sorted=True, return_distance=True)
        np.testing.assert_allclose(dist, np.sort(full, axis=1)[:, :6], rtol=RTOL, atol=0)


@pytest.mark.parametrize("metric", ["euclidean", "scaled_euclidean"])
def test_subsequence_vs_oracle(metric):
    rng = np.random.default_rng(21)
    T = _walk(rng, (14, 300))
    shp = [_walk(rng, (int(n),)) for n in rng.integers(3, 80, size=37)]
    shp.append(T[5, 100:140].copy())
    shp.append(np.full(12, 2.0))
    d, i = pairwise_subsequence_distance(shp, T, metric=metric, return_index=True)
    od, oi = O.subsequence(shp, T, metric=metric)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_allclose(d, od, rtol=RTOL, atol=0)


SUBSEQ_ELASTIC = [
    ("dtw", {"r": 0.2}), ("dtw", {"r": 1.0}), ("wdtw", {"r": 0.5, "g": 0.1}),
    ("ddtw", {"r": 0.3}), ("wddtw", {}), ("adtw", {"p": 0.3}), ("adtw", {"p": -0.1}),
    ("lcss", {"r": 0.3, "epsilon": 0.7}), ("edr", {}), ("edr", {"epsilon": 0.3}),
    ("erp", {"g": 0.2}), ("msm", {"r": 0.2}), ("twe", {"r": 0.4}),
]


@pytest.mark.parametrize("metric,params", SUBSEQ_ELASTIC)
def test_elastic_subsequence_vs_oracle(metric, params):
    rng = np.random.default_rng(zlib.crc32(repr((metric, params)).encode()))
    T = _walk(rng, (6, 120))
    shp = [_walk(rng, (int(n),)) for n in (2, 3, 5, 11, 24, 47, 64)]
    shp.append(T[3, 40:70].copy())
    d, i = pairwise_subsequence_distance(shp, T, metric=metric, metric_params=params,
                                         return_index=True)
    od, oi = O.subsequence(shp, T, metric=metric, metric_params=params)
    lens = np.array([len(s) for s in shp])
    keep = np.ones_like(oi, dtype=bool)
    if metric in ("ddtw", "wddtw"):
        keep[:, lens < 3] = False  # the reference leaves the index unset
    np.testing.assert_array_equal(i[keep], oi[keep])
    np.testing.assert_allclose(d, od, rtol=RTOL, atol=0, equal_nan=True)


def test_subsequence_full_length_equals_pairwise():
    # test_pairwise_subsequence_pairwise_equal (test_distance.py:949-958)
    rng = np.random.default_rng(4)
    X = _walk(rng, (8, 50))
    d = pairwise_subsequence_distance(X[:3], X, metric="euclidean")
    p = pairwise_distance(X, X[:3], metric="euclidean")
    np.testing.assert_allclose(d, p, rtol=RTOL, atol=0)


def test_multivariate_dims():
    rng = np.random.default_rng(8)
    X = _walk(rng, (6, 3, 40))
    Y = _walk(rng, (5, 3, 40))
    for dim in ("mean", "full", 0, 2):
        got = pairwise_distance(X, Y, dim=dim, metric="dtw", metric_params={"r": 0.3})
        ds = [O.pairwise(X, Y, dim=d, metric="dtw", metric_params={"r": 0.3})
              for d in range(3)]
        want = {"mean": np.mean(ds, axis=0), "full": np.stack(ds)}.get(dim)
        if want is None:
            want = ds[dim]
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)


def test_torch_device_inputs_stay_on_device():
    rng = np.random.default_rng(9)
    X = _walk(rng, (30, 77))
    Y = _walk(rng, (20, 77))
    Xt = torch.as_tensor(X, device="cuda")
    Yt = torch.as_tensor(Y, device="cuda")
    got = pairwise_distance(Xt, Yt, metric="twe", metric_params={"r": 0.2})
    assert got.is_cuda and got.dtype == torch.float64
    want = O.pairwise(X, Y, metric="twe", metric_params={"r": 0.2})
    np.testing.assert_allclose(got.cpu().numpy(), want, rtol=RTOL, atol=0)
    idx = argmin_distance(Xt, Yt, k=2, metric="lcss", metric_params={"epsilon": 0.5})
    oidx, _ = O.argmin(X, Y, k=2, metric="lcss", metric_params={"epsilon": 0.5})
    np.testing.assert_array_equal(idx.cpu().numpy(), oidx)


def test_deterministic_bitwise():
    rng = np.random.default_rng(10)
    X = _walk(rng, (64, 128))
    Y = _walk(rng, (64, 128))
    a = pairwise_distance(X, Y, metric="erp", metric_params={"r": 0.2})
    b = pairwise_distance(X, Y, metric="erp", metric_params={"r": 0.2})
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_native_library_runs():
    before = _lib.launch_count()
    pairwise_distance(np.ones((2, 5)), np.zeros((3, 5)), metric="dtw")
    assert _lib.launch_count() > before


ARGMIN_LONG = [("dtw", {"r": 0.1}), ("dtw", {"r": 1.0}), ("wdtw", {"g": 0.1}), ("ddtw", {"r": 0.3}),
              ("adtw", {"p": 0.5}), ("edr", {"epsilon": 0.5}), ("edr", {}), ("erp", {"g": 0.2}),
              ("msm", {"c": 0.5}), ("twe", {"penalty": 0.5, "stiffness": 0.01}),
              ("lcss", {"epsilon": 0.5}), ("adtw", {"p": -0.2})]


@pytest.mark.parametrize("metric,params", ARGMIN_LONG,
                         ids=[f"{m}-{i}" for i, (m, _) in enumerate(ARGMIN_LONG)])
@pytest.mark.parametrize("k", [1, 3, 10])
def test_argmin_many_candidates_vs_oracle(metric, params, k):
    # 300 candidates, a close one late in the scan: the heap replay of the
    # reference's early abandoning over a long candidate list
    rng = np.random.default_rng(70 + k)
    X = _walk(rng, (21, 60))
    Y = _walk(rng, (300, 60))
    Y[250] = X[3] + 0.01 * rng.standard_normal(60)  # a close candidate late in the scan
    idx, dist = argmin_distance(X, Y, k=k, metric=metric, metric_params=params,
                                return_distance=True)
    oidx, odist = O.argmin(X, Y, k=k, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)


def test_argmin_many_candidates_lower_bound_vs_oracle():
    rng = np.random.default_rng(4)
    X = _walk(rng, (13, 64))
    Y = _walk(rng, (200, 64))
    full = O.pairwise(X, Y, metric="dtw", metric_params={"r": 0.2})
    lb = full * rng.uniform(0.2, 1.05, size=full.shape)
    idx, dist = argmin_distance(X, Y, k=5, metric="dtw", metric_params={"r": 0.2},
                                lower_bound=lb, return_distance=True)
    oidx, odist = O.argmin(X, Y, k=5, metric="dtw", metric_params={"r": 0.2},
                           lower_bound=lb)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
