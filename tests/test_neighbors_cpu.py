"""Host-side checks of dtw_average, KMeans and the neighbour estimators
(argument validation that runs before any device work; no GPU needed)."""

import numpy as np
import pytest

from wildboar_gb300.distance import KMeans, KNeighborsClassifier, NearestNeighbors
from wildboar_gb300.distance.dtw import check_random_state, dtw_average, jeong_weight

X = np.cumsum(np.random.default_rng(0).standard_normal((10, 20)), axis=1)


@pytest.mark.parametrize("kw", [{"n_clusters": 0}, {"metric": "msm"}, {"r": 1.5},
                                {"r": -0.1}, {"g": 0.0}, {"init": "k-means++"},
                                {"n_init": 0}, {"max_iter": 0}, {"tol": 1}])
def test_kmeans_rejects_bad_params(kw):
    with pytest.raises(ValueError):
        KMeans(**kw).fit(X)


def test_kmeans_rejects_3d():
    with pytest.raises(ValueError):
        KMeans(2).fit(X.reshape(10, 1, 20))


@pytest.mark.parametrize("kw,exc", [({"r": 1.5}, ValueError), ({"method": "foo"}, ValueError),
                                    ({"g": 0.0}, ValueError), ({"init": 3}, ValueError),
                                    ({"sample_weight": np.ones(3)}, ValueError)])
def test_dtw_average_rejects_bad_args(kw, exc):
    with pytest.raises(exc):
        dtw_average(X, **kw)


def test_dtw_average_needs_two_samples():
    with pytest.raises(ValueError):
        dtw_average(X[:1])


def test_neighbors_reject_bad_params():
    with pytest.raises(ValueError):
        KNeighborsClassifier(n_neighbors=0).fit(X, np.arange(10) % 2)
    with pytest.raises(ValueError):
        KNeighborsClassifier(metric="nope").fit(X, np.arange(10) % 2)
    with pytest.raises(ValueError):
        KNeighborsClassifier().predict(X)
    with pytest.raises(ValueError):
        NearestNeighbors().kneighbors(X)
    with pytest.raises(ValueError):
        KNeighborsClassifier().fit(X, np.linspace(0, 1, 10))


def test_check_random_state():
    assert isinstance(check_random_state(3), np.random.RandomState)
    rs = np.random.RandomState(1)
    assert check_random_state(rs) is rs
    assert check_random_state(None) is np.random.mtrand._rand
    with pytest.raises(ValueError):
        check_random_state("seed")


def test_jeong_weight_formula():
    w = jeong_weight(10, 0.3)
    want = 1.0 / (1.0 + np.exp(-0.3 * (np.arange(10, dtype=float) - 5.0)))
    np.testing.assert_array_equal(w, want)


def test_dtw_average_ssg_needs_the_device():
    import torch

    if torch.cuda.is_available():  # pragma: no cover
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        dtw_average(X, method="ssg", random_state=0)
