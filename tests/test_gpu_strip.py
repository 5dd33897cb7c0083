"""Register-strip kernels against the ring kernels: bit-identical FP64.

The pairwise / paired FP64 path runs on the strip kernel; WB_GPU_ELASTIC=ring
selects the thread-per-pair ring kernel, which replays the reference's
two-row buffers directly.  Both must give the same bits for every metric,
band and shape (including unequal lengths, bands wider than the series,
the singleton upper triangle and paired rows), and both must match the
oracle (the parity tests cover the default path).
"""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from wildboar_gb300.distance import paired_distance, pairwise_distance  # noqa: E402

CASES = [
    ("dtw", {"r": 0.1}), ("dtw", {"r": 1.0}), ("dtw", {"r": 0.0}),
    ("wdtw", {"r": 0.4, "g": 0.1}), ("ddtw", {"r": 0.3}), ("wddtw", {"r": 1.0, "g": 0.05}),
    ("adtw", {"r": 0.5, "p": 0.7}), ("adtw", {"r": 1.0, "p": -0.2}),
    ("lcss", {"r": 0.5, "epsilon": 0.6}), ("lcss", {"r": 0.05, "epsilon": 0.3}),
    ("wlcss", {"r": 1.0, "epsilon": 1.0, "g": 0.1}),
    ("edr", {"r": 0.5}), ("edr", {"r": 1.0, "epsilon": 0.4}), ("edr", {"r": 0.02}),
    ("erp", {"r": 0.5, "g": 0.2}), ("erp", {"r": 0.05, "g": 0.0}),
    ("msm", {"r": 0.5, "c": 0.5}), ("msm", {"r": 0.02, "c": 1.0}), ("msm", {"r": 1.0}),
    ("twe", {"r": 0.5, "penalty": 0.3, "stiffness": 0.01}), ("twe", {"r": 0.03}),
]
SHAPES = [(64, 64), (100, 77), (40, 130), (257, 250), (1, 17), (17, 1), (3, 3), (2, 9)]


def _walk(rng, shape):
    return np.cumsum(rng.standard_normal(shape), axis=-1) * 0.4


def _both(fn):
    old = os.environ.get("WB_GPU_ELASTIC")
    try:
        os.environ["WB_GPU_ELASTIC"] = "ring"
        a = fn()
        os.environ["WB_GPU_ELASTIC"] = "strip"
        b = fn()
    finally:
        if old is None:
            os.environ.pop("WB_GPU_ELASTIC", None)
        else:
            os.environ["WB_GPU_ELASTIC"] = old
    return np.asarray(a), np.asarray(b)


@pytest.mark.parametrize("metric,params", CASES, ids=[f"{m}-{i}" for i, (m, _) in enumerate(CASES)])
@pytest.mark.parametrize("lx,ly", SHAPES)
def test_strip_equals_ring_pairwise(metric, params, lx, ly):
    rng = np.random.default_rng(lx * 131 + ly)
    X = _walk(rng, (35, 1, lx))
    Y = _walk(rng, (9, 1, ly))
    a, b = _both(lambda: pairwise_distance(X, Y, metric=metric, metric_params=params))
    np.testing.assert_array_equal(a, b)
    if lx * ly <= 20000:
        want = O.pairwise(X, Y, dim=0, metric=metric, metric_params=params)
        # 1e-12: edr's default epsilon sums x*x where the oracle calls pow
        np.testing.assert_allclose(b, want, rtol=1e-12, atol=0)


@pytest.mark.parametrize("metric,params", CASES, ids=[f"{m}-{i}" for i, (m, _) in enumerate(CASES)])
def test_strip_equals_ring_singleton_and_paired(metric, params):
    rng = np.random.default_rng(7)
    X = _walk(rng, (40, 1, 90))
    Y = _walk(rng, (40, 1, 90))  # paired_distance broadcasts: equal lengths
    a, b = _both(lambda: pairwise_distance(X, metric=metric, metric_params=params))
    np.testing.assert_array_equal(a, b)
    a, b = _both(lambda: paired_distance(X, Y, metric=metric, metric_params=params))
    np.testing.assert_array_equal(a, b)
    np.testing.assert_allclose(
        b, O.paired(X, Y, dim=0, metric=metric, metric_params=params), rtol=1e-12, atol=0)
