"""Batched entry points for the compiled callers (proximity-tree nodes,
shapelet-transform attributes) on the GPU, against the oracle: branches and
argmin windows exact, distances within 1e-12 relative."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from wildboar_gb300.distance._subsequence import _transient_stats  # noqa: E402
from wildboar_gb300.distance.batch import (nearest_pivot,  # noqa: E402
                                           subsequence_distance_views)

RTOL = 1e-12


@pytest.mark.parametrize("on_device", [False, True])
def test_nearest_pivot_vs_oracle(on_device):
    rng = np.random.default_rng(21)
    X = np.cumsum(rng.standard_normal((80, 2, 50)), axis=2)
    metrics = [("dtw", {"r": 0.1}), ("msm", {"c": 0.5}), ("euclidean", None),
               ("twe", {"penalty": 0.3, "stiffness": 0.01}), ("lcss", {"epsilon": 0.8})]
    groups = []
    for g in range(17):
        samples = rng.choice(80, size=int(rng.integers(1, 30)), replace=False)
        pivots = rng.choice(80, size=int(rng.integers(1, 5)), replace=False)
        groups.append((samples, pivots, g % len(metrics)))
    xin = torch.as_tensor(X, device="cuda") if on_device else X
    for dim in (0, 1):
        branch, dist = nearest_pivot(xin, groups, metrics, dim=dim)
        pos = 0
        for samples, pivots, slot in groups:
            name, params = metrics[slot]
            D = O.pairwise(X[samples, dim], X[pivots, dim], metric=name,
                           metric_params=params)
            for r in range(len(samples)):
                best, arg = np.inf, -1
                for c in range(len(pivots)):
                    if D[r, c] < best:
                        best, arg = D[r, c], c
                assert branch[pos] == arg
                np.testing.assert_allclose(dist[pos], best, rtol=RTOL, atol=0)
                pos += 1


@pytest.mark.parametrize("metric,params", [("euclidean", None), ("scaled_euclidean", None),
                                           ("dtw", {"r": 0.2}), ("scaled_dtw", {"r": 0.1}),
                                           ("msm", None)])
@pytest.mark.parametrize("on_device", [False, True])
def test_subsequence_views_vs_oracle(metric, params, on_device):
    rng = np.random.default_rng(22)
    X = np.cumsum(rng.standard_normal((30, 2, 120)), axis=2)
    X[4, 0, 10:40] = 1.5  # a constant view: zero std
    views = np.array([[4, 0, 10, 25]] + [
        [int(rng.integers(30)), int(rng.integers(2)), int(rng.integers(0, 60)),
         int(rng.integers(4, 60))] for _ in range(20)])
    xin = torch.as_tensor(X, device="cuda") if on_device else X
    dist, idx = subsequence_distance_views(xin, views, dim=1, metric=metric,
                                           metric_params=params)
    if on_device:
        dist, idx = dist.cpu().numpy(), idx.cpu().numpy()
    shp = [X[v[0], v[1], v[2]:v[2] + v[3]] for v in views]
    st = [_transient_stats(s) for s in shp]
    od, oi = O.subsequence(shp, X, dim=1, metric=metric, metric_params=params,
                           stats=(np.array([a for a, _ in st]), np.array([b for _, b in st])))
    np.testing.assert_array_equal(idx, oi)
    np.testing.assert_allclose(dist, od, rtol=RTOL, atol=0)
