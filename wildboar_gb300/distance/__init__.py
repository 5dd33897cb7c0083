"""GPU drop-in for wildboar.distance (the distance hot path)."""

from ._distance import (
    InvalidParameterError,
    argmin_distance,
    check_metric,
    check_subsequence_metric,
    paired_distance,
    pairwise_distance,
    pairwise_subsequence_distance,
)
from ._metrics import _METRICS, _SUBSEQUENCE_METRICS

__all__ = [
    "pairwise_distance",
    "paired_distance",
    "argmin_distance",
    "pairwise_subsequence_distance",
    "check_metric",
    "check_subsequence_metric",
    "InvalidParameterError",
    "_METRICS",
    "_SUBSEQUENCE_METRICS",
]
