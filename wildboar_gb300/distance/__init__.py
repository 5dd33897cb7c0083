"""GPU drop-in for wildboar.distance (the distance hot path)."""

from ._distance import (
    InvalidParameterError,
    argmin_distance,
    check_metric,
    check_subsequence_metric,
    paired_distance,
    paired_subsequence_distance,
    pairwise_distance,
    pairwise_subsequence_distance,
)
from ._metrics import _METRICS, _SUBSEQUENCE_METRICS
from ._neighbors import KMeans, KNeighborsClassifier, NearestNeighbors
from ._subsequence import (
    argmin_subsequence_distance,
    distance_profile,
    paired_subsequence_match,
    subsequence_match,
)

__all__ = [
    "pairwise_distance",
    "paired_distance",
    "argmin_distance",
    "pairwise_subsequence_distance",
    "paired_subsequence_distance",
    "distance_profile",
    "argmin_subsequence_distance",
    "subsequence_match",
    "paired_subsequence_match",
    "check_metric",
    "check_subsequence_metric",
    "InvalidParameterError",
    "KMeans",
    "KNeighborsClassifier",
    "NearestNeighbors",
    "_METRICS",
    "_SUBSEQUENCE_METRICS",
]
