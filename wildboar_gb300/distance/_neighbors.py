"""Neighbour-based estimators on the GPU distance path.

``KMeans`` (distance/_neighbors.py:309-570 of the reference) alternates
``argmin_distance`` (assignment), ``paired_distance`` (cost) and the
centroid update; all three run on the device here, the data uploaded once
per fit.  The dtw / wdtw update is the MM barycenter of every cluster in
lockstep (``dtw._mm_average_groups``); the euclidean update is
``wb_group_mean``.  The cluster loop's bookkeeping (empty clusters take the
sample farthest from its centre, singletons copy their sample, the random
state is drawn in the reference's order) is the reference's, on the host, so
labels, centres, ``inertia_`` and ``n_iter_`` are the reference's.

``KNeighborsClassifier`` and ``NearestNeighbors`` (:17-306) are the
reference's voting and neighbour bookkeeping over ``argmin_distance`` /
``pairwise_distance``.
"""

import ctypes
import math
import numbers
import warnings

import numpy as np

from .. import _lib
from ._distance import InvalidParameterError, argmin_distance, paired_distance, pairwise_distance
from ._metrics import _METRICS
from ._validation import check_array
from .dtw import _mm_average_groups, _torch, check_random_state


def _check_fitted(est, attr):
    if not hasattr(est, attr):
        raise ValueError(
            f"This {type(est).__name__} instance is not fitted yet. Call 'fit' with "
            "appropriate arguments before using this estimator."
        )


def _param_error(name, est, value, expect):
    return InvalidParameterError(
        f"The {name!r} parameter of {type(est).__name__} must be {expect}. Got {value!r} instead."
    )


def _check_int(est, name, value, low):
    if not isinstance(value, numbers.Integral) or isinstance(value, bool) or value < low:
        raise _param_error(name, est, value, f"an int in the range [{low}, inf)")


def _check_n_features(est, x, reset):
    if reset:
        est.n_features_in_ = x.shape[-1]
        est.n_dims_in_ = x.shape[1] if x.ndim == 3 else 1
    elif x.shape[-1] != est.n_features_in_:
        raise ValueError(
            f"X has {x.shape[-1]} timesteps, but {type(est).__name__} is expecting "
            f"{est.n_features_in_} timesteps as input."
        )


def _check_classification_targets(y):
    y = np.asarray(y)
    if y.dtype.kind == "f" and np.any(y != y.astype(int)):
        raise ValueError("Unknown label type: continuous")


# --------------------------------------------------------------------------
# nearest neighbours


class _NeighborsBase:
    def __init__(self, n_neighbors=5, *, metric="euclidean", metric_params=None,
                 n_jobs=None):
        self.n_neighbors = n_neighbors
        self.metric = metric
        self.metric_params = metric_params
        self.n_jobs = n_jobs

    def _validate_params(self):
        _check_int(self, "n_neighbors", self.n_neighbors, 1)
        if self.metric not in _METRICS:
            raise _param_error("metric", self, self.metric,
                               "a str among " + repr(sorted(_METRICS.keys())))
        if self.metric_params is not None and not isinstance(self.metric_params, dict):
            raise _param_error("metric_params", self, self.metric_params, "a dict or None")


class NearestNeighbors(_NeighborsBase):
    """Unsupervised neighbour search (distance/_neighbors.py:17-162)."""

    def fit(self, x, y=None):
        self._validate_params()
        x = check_array(x, allow_3d=True)
        _check_n_features(self, x, True)
        self._fit_X = x.copy()
        return self

    def kneighbors(self, x=None, n_neighbors=None, return_distance=True):
        _check_fitted(self, "_fit_X")
        if n_neighbors is None:
            n_neighbors = self.n_neighbors
        if x is not None:
            query_is_train = False
            x = check_array(x, allow_3d=True)
            _check_n_features(self, x, False)
        else:
            query_is_train = True
            x = self._fit_X
        if x.ndim == 3 and x.shape[1] == 1:
            x = x.reshape(x.shape[0], -1)
        if x.ndim == 3:
            dists = pairwise_distance(x, self._fit_X, dim="mean", metric=self.metric,
                                      metric_params=self.metric_params)
            if query_is_train:
                np.fill_diagonal(dists, np.inf)
            sample_range = np.arange(x.shape[0])[:, None]
            neigh_ind = np.argpartition(dists, n_neighbors - 1, axis=1)[:, :n_neighbors]
            neigh_dist = dists[sample_range, neigh_ind]
            sort_inds = np.argsort(neigh_dist, axis=1)
            neigh_ind = neigh_ind[sample_range, sort_inds]
            if return_distance:
                return neigh_dist[sample_range, sort_inds], neigh_ind
            return neigh_ind
        k = n_neighbors + 1 if query_is_train else n_neighbors
        indices, distances = argmin_distance(
            x, self._fit_X, metric=self.metric, metric_params=self.metric_params, k=k,
            return_distance=True, sorted=True)
        if query_is_train:
            mask = indices != np.arange(x.shape[0])[:, None]
            indices = indices[mask].reshape(x.shape[0], -1)
            distances = distances[mask].reshape(x.shape[0], -1)
        if return_distance:
            return distances, indices
        return indices


class KNeighborsClassifier(_NeighborsBase):
    """k-nearest-neighbour classifier (distance/_neighbors.py:165-306)."""

    def fit(self, x, y):
        self._validate_params()
        x = check_array(x, allow_3d=True)
        y = np.asarray(y)
        if y.ndim != 1 or y.shape[0] != x.shape[0]:
            raise ValueError(
                "Found input variables with inconsistent numbers of samples: "
                f"[{x.shape[0]}, {y.shape[0] if y.ndim else 0}]")
        _check_classification_targets(y)
        _check_n_features(self, x, True)
        self._fit_X = x.copy()
        self.classes_, self._y = np.unique(y, return_inverse=True)
        return self

    def predict_proba(self, x):
        _check_fitted(self, "_fit_X")
        x = check_array(x, allow_3d=True)
        _check_n_features(self, x, False)
        if x.ndim == 3 and x.shape[1] == 1:
            x = x.reshape(x.shape[0], -1)
        if x.ndim == 3:
            dists = pairwise_distance(x, self._fit_X, dim="mean", metric=self.metric,
                                      metric_params=self.metric_params)
            closest = np.argpartition(dists, self.n_neighbors, axis=1)[:, :self.n_neighbors]
        else:
            closest = argmin_distance(x, self._fit_X, metric=self.metric,
                                      metric_params=self.metric_params, k=self.n_neighbors)
        preds = self._y[closest]
        probs = np.empty((x.shape[0], len(self.classes_)), dtype=float)
        for i in range(len(self.classes_)):
            probs[:, i] = np.sum(preds == i, axis=1) / self.n_neighbors
        return probs

    def predict(self, x):
        proba = np.argmax(self.predict_proba(x), axis=1)
        return np.take(self.classes_, proba)

    def score(self, x, y):
        return float(np.mean(self.predict(x) == np.asarray(y)))


# --------------------------------------------------------------------------
# KMeans


class _Cluster:
    """_KMeansCluster (distance/_neighbors.py:309-361) over device-resident data."""

    def __init__(self, xd, centroids, metric, metric_params, random_state):
        self.xd = xd
        self.metric = metric
        self.metric_params = metric_params
        self.centroids_ = centroids
        self.random_state = random_state
        self.assigned_ = None

    def _centroids_dev(self):
        torch = _torch()
        return torch.as_tensor(self.centroids_, device=self.xd.device)

    def cost(self, x):
        if self.assigned_ is None:
            raise ValueError("`assign` must be called before `cost`")
        torch = _torch()
        c = self._centroids_dev()[torch.as_tensor(self.assigned_, device=self.xd.device)]
        d = paired_distance(self.xd, c, dim="mean", metric=self.metric,
                            metric_params=self.metric_params)
        return d.cpu().numpy().sum() / x.shape[0]

    def assign(self, x):
        idx, dist = argmin_distance(self.xd, self._centroids_dev(), k=1, metric=self.metric,
                                    metric_params=self.metric_params, return_distance=True)
        self.assigned_ = np.ravel(idx.cpu().numpy()).astype(np.intp)
        self.distance_ = dist.cpu().numpy()

    def update(self, x):
        groups, targets = [], []
        for c in range(self.centroids_.shape[0]):
            members = np.flatnonzero(self.assigned_ == c)
            if members.shape[0] == 0:
                far_from_center = self.distance_.min(axis=1).argmax()
                self.assigned_[far_from_center] = c
                self.centroids_[c] = x[far_from_center]
            elif members.shape[0] == 1:
                self.centroids_[c] = x[members[0]]
            else:
                self._draw()
                groups.append(members)
                targets.append(c)
        if groups:
            self.centroids_[targets] = self._update_centroids(groups, targets)

    def _draw(self):
        pass


class _EuclideanCluster(_Cluster):
    def __init__(self, xd, centroids, random_state):
        super().__init__(xd, centroids, "euclidean", None, random_state)

    def _update_centroids(self, groups, targets):
        torch = _torch()
        dev = self.xd.device
        counts = np.array([len(g) for g in groups], dtype=np.int64)
        start = np.zeros(len(groups) + 1, dtype=np.int64)
        np.cumsum(counts, out=start[1:])
        member = torch.as_tensor(np.concatenate(groups).astype(np.int64), device=dev)
        gs = torch.as_tensor(start, device=dev)
        out = torch.empty((len(groups), self.xd.shape[1]), dtype=torch.float64, device=dev)
        st = _lib.lib().wb_group_mean(
            self.xd.data_ptr(), self.xd.stride(0), self.xd.shape[1], member.data_ptr(),
            gs.data_ptr(), None, len(groups), out.data_ptr(), _lib.current_stream_handle())
        _lib.check(st)
        return out.cpu().numpy()


class _DtwCluster(_Cluster):
    def __init__(self, xd, centroids, r, g, random_state):
        params = {"r": r} if g is None else {"r": r, "g": g}
        super().__init__(xd, centroids, "dtw" if g is None else "wdtw", params, random_state)
        self.r = r
        self.g = g

    def _draw(self):
        # the reference seeds each dtw_average call with a draw from the
        # estimator's random state (unused with an array init, but drawn)
        self.random_state.randint(np.iinfo(np.int32).max)

    def _update_centroids(self, groups, targets):
        means, _ = _mm_average_groups(self.xd, groups, self.centroids_[targets], r=self.r,
                                      g=self.g)
        return means


class KMeans:
    """KMeans with the euclidean, dtw or weighted dtw metric (distance/_neighbors.py:
    403-588): same parameters, attributes and results as the reference."""

    def __init__(self, n_clusters=8, *, metric="euclidean", r=1.0, g=None, init="random",
                 n_init="auto", max_iter=300, tol=1e-3, verbose=0, random_state=None):
        self.metric = metric
        self.r = r
        self.g = g
        self.n_clusters = n_clusters
        self.init = init
        self.n_init = n_init
        self.max_iter = max_iter
        self.tol = tol
        self.verbose = verbose
        self.random_state = random_state

    def get_params(self, deep=True):
        return {k: getattr(self, k) for k in ("n_clusters", "metric", "r", "g", "init",
                                              "n_init", "max_iter", "tol", "verbose",
                                              "random_state")}

    def _validate_params(self):
        _check_int(self, "n_clusters", self.n_clusters, 1)
        if self.metric not in ("euclidean", "dtw"):
            raise _param_error("metric", self, self.metric, "a str among {'euclidean', 'dtw'}")
        if (not isinstance(self.r, numbers.Real) or isinstance(self.r, bool)
                or not 0 <= self.r <= 1):
            raise _param_error("r", self, self.r, "a float in the range [0, 1]")
        if self.g is not None and (not isinstance(self.g, numbers.Real) or self.g <= 0):
            raise _param_error("g", self, self.g, "None or a float in the range (0, inf)")
        if self.init != "random":
            raise _param_error("init", self, self.init, "a str among {'random'}")
        if self.n_init != "auto":
            _check_int(self, "n_init", self.n_init, 1)
        _check_int(self, "max_iter", self.max_iter, 1)
        if not isinstance(self.tol, float):
            raise _param_error("tol", self, self.tol, "an instance of 'float'")
        if not isinstance(self.verbose, numbers.Integral):
            raise _param_error("verbose", self, self.verbose, "an instance of 'int'")

    def fit(self, x, y=None):
        self._validate_params()
        x = check_array(x, allow_3d=False, ensure_2d=True)
        _check_n_features(self, x, True)
        n_init = 1 if self.n_init == "auto" else self.n_init
        random_state = check_random_state(self.random_state)
        torch = _torch()
        xd = torch.as_tensor(x, device="cuda")
        best_cost = np.inf
        best_cluster = None
        best_reassign = True
        best_iter = None
        for _ in range(n_init):
            it, cost, cluster, reassign = self._fit_one_init(x, xd, random_state)
            if cost < best_cost:
                best_cost = cost
                best_cluster = cluster
                best_reassign = reassign
                best_iter = it
        self.n_iter_ = best_iter
        self.inertia_ = best_cost
        self.cluster_centers_ = best_cluster.centroids_
        if best_reassign:
            best_cluster.assign(x)
        self.labels_ = best_cluster.assigned_
        return self

    def _fit_one_init(self, x, xd, random_state):
        centroids = x[random_state.choice(x.shape[0], size=self.n_clusters, replace=False)]
        if self.metric == "euclidean":
            cluster = _EuclideanCluster(xd, centroids, random_state)
        else:
            cluster = _DtwCluster(xd, centroids, self.r, self.g, random_state)
        prev_cost = np.inf
        cost = -np.inf
        reassign = True
        it = 0
        for it in range(self.max_iter):
            cluster.assign(x)
            prev_cost, cost = cost, cluster.cost(x)
            if self.verbose > 0:
                print(f"Iteration {it}, {cost} (prev_cost = {prev_cost})")
            if math.isclose(cost, prev_cost, rel_tol=self.tol):
                reassign = False
                break
            cluster.update(x)
        return it, cost, cluster, reassign

    def fit_predict(self, x, y=None):
        return self.fit(x).labels_

    def transform(self, x):
        _check_fitted(self, "cluster_centers_")
        x = check_array(x, allow_3d=False, ensure_2d=True)
        _check_n_features(self, x, False)
        metric_params = {}
        metric = self.metric
        if self.metric == "dtw":
            metric_params["r"] = self.r
            if self.g is not None:
                metric_params["g"] = self.g
                metric = "wdtw"
        return pairwise_distance(x, self.cluster_centers_, dim="mean", metric=metric,
                                 metric_params=metric_params)

    def predict(self, x):
        return self.transform(x).argmin(axis=1)


__all__ = ["KMeans", "KNeighborsClassifier", "NearestNeighbors"]
