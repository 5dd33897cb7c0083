"""FP32 precision form of every elastic metric (wb_pairwise_distance_fp32).

The recurrences run on float32-rounded series with compensated (hi, lo)
accumulation; the bar is the FP64 oracle on the same float64 inputs:
- dtw, wdtw, ddtw, wddtw, adtw, erp, msm, twe: relative error <= 1e-5;
- adtw with a negative penalty p: the distance is a difference of the path's
  squared costs and its penalties, so the bar is on the squared distance,
  |d32^2 - d64^2| <= 1e-5 (d64^2 + |p| (n + m)), the path having at most n + m
  steps;
- lcss, wlcss, edr: the match counts are exact in FP32 (wlcss sums float32
  weights, within 1e-6), so the distances agree except where float32 rounding
  moves |x_i - y_j| across epsilon; such a cell changes a count by one, so at
  most 1 % of the entries may differ by more than 1e-6, each by at most
  2 / min(n, m) (lcss) or 2 / max(n, m) (edr).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from wildboar_gb300.distance import pairwise_distance  # noqa: E402
from wildboar_gb300.distance.precision import pairwise_distance_fp32  # noqa: E402

RTOL = 1e-5
COUNTS = ("lcss", "wlcss", "edr")

CASES = [
    ("dtw", {"r": 0.1}), ("dtw", {"r": 1.0}), ("dtw", {"r": 0.0}),
    ("wdtw", {"r": 0.3, "g": 0.1}), ("ddtw", {"r": 0.2}), ("wddtw", {"r": 0.5, "g": 0.05}),
    ("adtw", {"r": 0.5, "p": 0.5}), ("adtw", {"r": 1.0, "p": -0.3}),
    ("lcss", {"r": 0.5, "epsilon": 0.7}), ("wlcss", {"r": 1.0, "epsilon": 1.0, "g": 0.1}),
    ("edr", {"r": 0.5}), ("edr", {"r": 0.3, "epsilon": 0.5}),
    ("erp", {"r": 0.5, "g": 0.2}), ("msm", {"r": 0.5, "c": 0.5}),
    ("twe", {"r": 0.5, "penalty": 0.3, "stiffness": 0.01}),
]


def _walk(rng, shape):
    return np.cumsum(rng.standard_normal(shape), axis=-1) * 0.3


def _oracle(X, Y, metric, params):
    return O.pairwise(X, Y, dim=0, metric=metric, metric_params=params)


def _check(metric, got, want, n, m, params=None):
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape
    p = (params or {}).get("p", 0.0)
    if metric == "adtw" and p < 0:
        np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        bound = RTOL * (want[ok] ** 2 + abs(p) * (n + m))
        assert np.all(np.abs(got[ok] ** 2 - want[ok] ** 2) <= bound)
    elif metric in COUNTS:
        diff = np.abs(got - want)
        step = 2.0 / (min(n, m) if metric != "edr" else max(n, m))
        # wlcss sums float32 weights: 1e-6 absorbs their rounding
        assert np.mean(diff > 1e-6) <= 0.01, np.mean(diff > 1e-6)
        assert diff.max() <= step + 1e-12, diff.max()
    else:
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=1e-9)


@pytest.mark.parametrize("metric,params", CASES, ids=[f"{m}-{i}" for i, (m, _) in enumerate(CASES)])
@pytest.mark.parametrize("lx,ly", [(64, 64), (100, 77), (40, 130), (600, 600)])
def test_fp32_pairwise_vs_fp64_oracle(metric, params, lx, ly):
    rng = np.random.default_rng(lx * 7 + ly)
    nx, ny = (37, 9) if lx < 600 else (33, 4)
    X = _walk(rng, (nx, 1, lx))
    Y = _walk(rng, (ny, 1, ly))
    got = pairwise_distance_fp32(X, Y, metric=metric, metric_params=params)
    _check(metric, got, _oracle(X, Y, metric, params), lx, ly, params)


@pytest.mark.parametrize("metric,params", CASES[::2], ids=[m for m, _ in CASES[::2]])
def test_fp32_singleton_upper_triangle(metric, params):
    rng = np.random.default_rng(11)
    X = _walk(rng, (45, 1, 90))
    got = pairwise_distance_fp32(X, metric=metric, metric_params=params)
    want = O.pairwise(X, None, dim=0, metric=metric, metric_params=params)
    assert np.all(np.diag(got) == 0.0)
    np.testing.assert_array_equal(got, got.T)
    _check(metric, got, want, 90, 90, params)


def test_fp32_matches_fp64_api_shapes_and_dims():
    rng = np.random.default_rng(3)
    X = _walk(rng, (12, 3, 50))
    Y = _walk(rng, (7, 3, 50))
    for dim in ("mean", "full", 2):
        a = pairwise_distance(X, Y, dim=dim, metric="msm")
        b = pairwise_distance_fp32(X, Y, dim=dim, metric="msm")
        assert np.shape(a) == np.shape(b)
        np.testing.assert_allclose(b, a, rtol=RTOL)
    # 1-D inputs are squeezed like the FP64 API
    a = pairwise_distance(X[0, 0], Y[:, 0], metric="dtw")
    b = pairwise_distance_fp32(X[0, 0], Y[:, 0], metric="dtw")
    assert np.shape(a) == np.shape(b)
    np.testing.assert_allclose(b, a, rtol=RTOL)


def test_fp32_torch_device_inputs_and_short_series():
    rng = np.random.default_rng(4)
    X = _walk(rng, (20, 1, 2))
    Y = _walk(rng, (5, 1, 2))
    # derivative metrics on series shorter than 3
    got = pairwise_distance_fp32(X, Y, metric="ddtw")
    np.testing.assert_array_equal(got, _oracle(X, Y, "ddtw", {}))
    X = _walk(rng, (20, 1, 33))
    Y = _walk(rng, (5, 1, 1))
    for metric in ("dtw", "erp", "twe", "msm"):
        got = pairwise_distance_fp32(torch.as_tensor(X, device="cuda"),
                                     torch.as_tensor(Y, device="cuda"), metric=metric)
        assert isinstance(got, torch.Tensor) and got.is_cuda
        np.testing.assert_allclose(got.cpu().numpy(), _oracle(X, Y, metric, {}),
                                   rtol=RTOL, atol=1e-9)


def test_fp32_rejects_non_elastic():
    with pytest.raises(ValueError):
        pairwise_distance_fp32(np.zeros((2, 5)), np.zeros((2, 5)), metric="euclidean")
