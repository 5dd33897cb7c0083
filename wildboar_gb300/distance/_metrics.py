"""Metric registry: names, constructor arguments and their validation.

Restates the constructors of the reference's metric classes
(wildboar src/wildboar/distance/_elastic.pyx:3126-4082 and
distance/_metric.pyx:26-409) so that ``metric_params`` are accepted, rejected
and pickled exactly as there.  Each metric carries the numeric id of the C ABI
(include/wbgpu.h) and packs its arguments into ``wb_params``.
"""

import math
import numbers
import operator
import warnings

from .. import _lib


def check_scalar(x, name, target_type, *, min_val=None, max_val=None,
                 include_boundaries="both"):
    """sklearn.utils.validation.check_scalar, as the reference metrics call it."""
    if not isinstance(x, target_type):
        if isinstance(target_type, tuple):
            types_str = ", ".join(t.__qualname__ for t in target_type)
            target_type_str = f"{{{types_str}}}"
        else:
            target_type_str = target_type.__qualname__
        raise TypeError(
            f"{name} must be an instance of {target_type_str}, not {type(x).__qualname__}."
        )
    lower = operator.lt if include_boundaries in ("left", "both") else operator.le
    if min_val is not None and lower(x, min_val):
        raise ValueError(
            f"{name} == {x}, must be {'>=' if include_boundaries in ('left', 'both') else '>'} "
            f"{min_val}."
        )
    upper = operator.gt if include_boundaries in ("right", "both") else operator.ge
    if max_val is not None and upper(x, max_val):
        raise ValueError(
            f"{name} == {x}, must be {'<=' if include_boundaries in ('right', 'both') else '<'} "
            f"{max_val}."
        )
    return x


def _double(x, name):
    # Cython ``double`` arguments: accept real numbers, convert to float
    if isinstance(x, bool) or not isinstance(x, numbers.Real):
        raise TypeError(f"must be real number, not {type(x).__qualname__}")
    return float(x)


class Metric:
    """Base of the pairwise metrics (the reference's ``Metric`` cdef class)."""

    metric_id = -1
    is_elastic = False
    _args = ()

    def __reduce__(self):
        return self.__class__, tuple(getattr(self, a) for a in self._args)

    def __eq__(self, other):
        return type(self) is type(other) and all(
            _same(getattr(self, a), getattr(other, a)) for a in self._args
        )

    def __hash__(self):
        return hash((type(self).__name__,) + tuple(getattr(self, a) for a in self._args))

    def __repr__(self):
        args = ", ".join(f"{a}={getattr(self, a)!r}" for a in self._args)
        return f"{type(self).__name__}({args})"

    def params(self):
        p = _lib.Params()
        p.r = getattr(self, "r", 1.0)
        p.g = getattr(self, "g", 0.0)
        p.p = getattr(self, "p", 1.0)
        p.epsilon = getattr(self, "epsilon", math.nan)
        p.c = getattr(self, "c", 1.0)
        p.penalty = getattr(self, "penalty", 1.0)
        p.stiffness = getattr(self, "stiffness", 0.001)
        return p


def _same(a, b):
    if isinstance(a, float) and isinstance(b, float) and math.isnan(a) and math.isnan(b):
        return True
    return a == b


class EuclideanMetric(Metric):
    """EuclideanMetric, distance/_metric.pyx:381-409."""

    metric_id = 0

    def __init__(self):
        pass


class DtwMetric(Metric):
    """DtwMetric, distance/_elastic.pyx:3126-3217."""

    metric_id = 1
    is_elastic = True
    _args = ("r",)

    def __init__(self, r=1.0):
        r = _double(r, "r")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        self.r = r


class DerivativeDtwMetric(DtwMetric):
    """DerivativeDtwMetric, distance/_elastic.pyx:3228-3320."""

    metric_id = 3

    def __init__(self, r=1.0):
        super().__init__(r=r)


class WeightedDtwMetric(DtwMetric):
    """WeightedDtwMetric, distance/_elastic.pyx:3322-3341."""

    metric_id = 2
    _args = ("r", "g")

    def __init__(self, r=1.0, g=0.05):
        super().__init__(r=r)
        g = _double(g, "g")
        check_scalar(g, "g", float, min_val=0.0)
        self.g = g


class WeightedDerivativeDtwMetric(DerivativeDtwMetric):
    """WeightedDerivativeDtwMetric, distance/_elastic.pyx:3404-3430 (g unchecked)."""

    metric_id = 4
    _args = ("r", "g")

    def __init__(self, r=1.0, g=0.05):
        super().__init__(r=r)
        self.g = _double(g, "g")


class AmercingDtwMetric(DtwMetric):
    """AmercingDtwMetric, distance/_elastic.pyx:3344-3401."""

    metric_id = 5
    _args = ("r", "p")

    def __init__(self, r=1.0, p=1.0):
        super().__init__(r=r)
        p = _double(p, "p")
        check_scalar(p, "p", float)
        self.p = p


class LcssMetric(Metric):
    """LcssMetric, distance/_elastic.pyx:3433-3539."""

    metric_id = 6
    is_elastic = True
    _args = ("r", "epsilon")

    def __init__(self, r=1.0, epsilon=1.0, threshold=math.nan):
        r = _double(r, "r")
        epsilon = _double(epsilon, "epsilon")
        threshold = _double(threshold, "threshold")
        if not math.isnan(threshold):
            warnings.warn(
                "The parameter threshold has been renamed to epsilon in 1.2 "
                "and will be removed in 1.4.",
                FutureWarning,
            )
            epsilon = threshold
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        check_scalar(epsilon, "epsilon", float, min_val=0, include_boundaries="neither")
        self.r = r
        self.epsilon = epsilon


class WeightedLcssMetric(LcssMetric):
    """WeightedLcssMetric, distance/_elastic.pyx:3542-3561."""

    metric_id = 7
    _args = ("r", "epsilon", "g")

    def __init__(self, r=1.0, epsilon=1.0, g=0.05, threshold=math.nan):
        super().__init__(r=r, epsilon=epsilon, threshold=threshold)
        g = _double(g, "g")
        check_scalar(g, "g", float, min_val=0.0)
        self.g = g


class ErpMetric(Metric):
    """ErpMetric, distance/_elastic.pyx:3564-3668."""

    metric_id = 9
    is_elastic = True
    _args = ("r", "g")

    def __init__(self, r=1.0, g=0.0):
        r = _double(r, "r")
        g = _double(g, "g")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        check_scalar(g, "g", float, min_val=0)
        self.r = r
        self.g = g


class EdrMetric(Metric):
    """EdrMetric, distance/_elastic.pyx:3671-3884 (epsilon=NaN: per-pair default)."""

    metric_id = 8
    is_elastic = True
    _args = ("r", "epsilon")

    def __init__(self, r=1.0, epsilon=math.nan, threshold=math.nan):
        r = _double(r, "r")
        epsilon = _double(epsilon, "epsilon")
        threshold = _double(threshold, "threshold")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        if not math.isnan(threshold):
            warnings.warn(
                "The parameter threshold has been renamed to epsilon in 1.2 "
                "and will be removed in 1.4.",
                FutureWarning,
            )
            epsilon = threshold
        if not math.isnan(epsilon):
            check_scalar(epsilon, "epsilon", float, min_val=0, include_boundaries="neither")
        self.r = r
        self.epsilon = epsilon


class MsmMetric(Metric):
    """MsmMetric, distance/_elastic.pyx:3887-3982."""

    metric_id = 10
    is_elastic = True
    _args = ("r", "c")

    def __init__(self, r=1.0, c=1.0):
        r = _double(r, "r")
        c = _double(c, "c")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        check_scalar(c, "c", float, min_val=0)
        self.r = r
        self.c = c


class TweMetric(Metric):
    """TweMetric, distance/_elastic.pyx:3985-4082."""

    metric_id = 11
    is_elastic = True
    _args = ("r", "penalty", "stiffness")

    def __init__(self, r=1.0, penalty=1.0, stiffness=0.001):
        r = _double(r, "r")
        penalty = _double(penalty, "penalty")
        stiffness = _double(stiffness, "stiffness")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        check_scalar(penalty, "penalty", float, min_val=0.0)
        check_scalar(stiffness, "stiffness", float, min_val=0.0,
                     include_boundaries="neither")
        self.r = r
        self.penalty = penalty
        self.stiffness = stiffness


class SubsequenceMetric:
    metric_id = -1
    _args = ()

    def __init__(self):
        pass

    def __reduce__(self):
        return self.__class__, ()

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self).__name__)


class EuclideanSubsequenceMetric(SubsequenceMetric):
    """EuclideanSubsequenceMetric, distance/_metric.pyx:26-58."""

    metric_id = 0
    scaled = False


class ScaledEuclideanSubsequenceMetric(SubsequenceMetric):
    """ScaledEuclideanSubsequenceMetric, distance/_metric.pyx:96-169."""

    metric_id = 32
    scaled = True


class _ElasticSubsequence(SubsequenceMetric):
    """Base of the elastic subsequence metrics (distance/_elastic.pyx:2206-3124)."""

    scaled = False

    def __reduce__(self):
        return self.__class__, tuple(getattr(self, a) for a in self._args)

    def __eq__(self, other):
        return type(self) is type(other) and all(
            _same(getattr(self, a), getattr(other, a)) for a in self._args)

    def __hash__(self):
        return hash((type(self).__name__,) + tuple(getattr(self, a) for a in self._args))

    params = Metric.params


class DtwSubsequenceMetric(_ElasticSubsequence):
    """DtwSubsequenceMetric, distance/_elastic.pyx:2206-2290."""

    metric_id = 1
    _args = ("r",)

    def __init__(self, r=1.0):
        r = _double(r, "r")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        self.r = r


class ScaledDtwSubsequenceMetric(DtwSubsequenceMetric):
    """ScaledDtwSubsequenceMetric, distance/_elastic.pyx:1928-2204: z-normalised
    dtw with the UCR-suite scan (LB_Kim, LB_Keogh both ways, cumulative-bound
    abandoning) and its warp width (r == 1: length - 1, else floor(length r))."""

    metric_id = 33
    scaled = True


class AmercingDtwSubsequenceMetric(DtwSubsequenceMetric):
    """AmercingDtwSubsequenceMetric, distance/_elastic.pyx:2293-2351 (p unchecked)."""

    metric_id = 5
    _args = ("r", "p")

    def __init__(self, r=1.0, p=1.0):
        super().__init__(r=r)
        self.p = _double(p, "p")


class WeightedDtwSubsequenceMetric(DtwSubsequenceMetric):
    """WeightedDtwSubsequenceMetric, distance/_elastic.pyx:2354-2440."""

    metric_id = 2
    _args = ("r", "g")

    def __init__(self, r=1.0, g=0.05):
        super().__init__(r=r)
        check_scalar(g, "g", float, min_val=0.0)
        self.g = float(g)


class DerivativeDtwSubsequenceMetric(DtwSubsequenceMetric):
    """DerivativeDtwSubsequenceMetric, distance/_elastic.pyx:2443-2519."""

    metric_id = 3


class WeightedDerivativeDtwSubsequenceMetric(DerivativeDtwSubsequenceMetric):
    """WeightedDerivativeDtwSubsequenceMetric, distance/_elastic.pyx:2522-2613."""

    metric_id = 4
    _args = ("r", "g")

    def __init__(self, r=1.0, g=0.05):
        super().__init__(r=r)
        check_scalar(g, "g", float, min_val=0.0)
        self.g = float(g)


class LcssSubsequenceMetric(_ElasticSubsequence):
    """LcssSubsequenceMetric, distance/_elastic.pyx:2616-2705."""

    metric_id = 6
    _args = ("r", "epsilon")

    def __init__(self, r=1.0, epsilon=1.0):
        r = _double(r, "r")
        epsilon = _double(epsilon, "epsilon")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        check_scalar(epsilon, "epsilon", float, min_val=0, include_boundaries="neither")
        self.r = r
        self.epsilon = epsilon


class EdrSubsequenceMetric(_ElasticSubsequence):
    """EdrSubsequenceMetric, distance/_elastic.pyx:2708-2812 (epsilon=NaN: std/4)."""

    metric_id = 8
    _args = ("r", "epsilon")
    needs_std = True

    def __init__(self, r=1.0, epsilon=math.nan):
        r = _double(r, "r")
        epsilon = _double(epsilon, "epsilon")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        if not math.isnan(epsilon):
            check_scalar(epsilon, "epsilon", float, min_val=0, include_boundaries="neither")
        self.r = r
        self.epsilon = epsilon


class TweSubsequenceMetric(_ElasticSubsequence):
    """TweSubsequenceMetric, distance/_elastic.pyx:2815-2911."""

    metric_id = 11
    _args = ("r", "penalty", "stiffness")

    def __init__(self, r=1.0, penalty=1.0, stiffness=0.001):
        r = _double(r, "r")
        penalty = _double(penalty, "penalty")
        stiffness = _double(stiffness, "stiffness")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        check_scalar(penalty, "penalty", float, min_val=0.0)
        check_scalar(stiffness, "stiffness", float, min_val=0.0,
                     include_boundaries="neither")
        self.r = r
        self.penalty = penalty
        self.stiffness = stiffness


class MsmSubsequenceMetric(_ElasticSubsequence):
    """MsmSubsequenceMetric, distance/_elastic.pyx:2914-3010."""

    metric_id = 10
    _args = ("r", "c")

    def __init__(self, r=1.0, c=1.0):
        r = _double(r, "r")
        c = _double(c, "c")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        check_scalar(c, "c", float, min_val=0)
        self.r = r
        self.c = c


class ErpSubsequenceMetric(_ElasticSubsequence):
    """ErpSubsequenceMetric, distance/_elastic.pyx:3013-3124."""

    metric_id = 9
    _args = ("r", "g")

    def __init__(self, r=1.0, g=0.0):
        r = _double(r, "r")
        g = _double(g, "g")
        check_scalar(r, "r", float, min_val=0.0, max_val=1.0)
        check_scalar(g, "g", float, min_val=0)
        self.r = r
        self.g = g


# distance/_distance.py:186-205 (the metrics this implementation provides)
_METRICS = {
    "euclidean": EuclideanMetric,
    "adtw": AmercingDtwMetric,
    "dtw": DtwMetric,
    "ddtw": DerivativeDtwMetric,
    "wdtw": WeightedDtwMetric,
    "wddtw": WeightedDerivativeDtwMetric,
    "lcss": LcssMetric,
    "wlcss": WeightedLcssMetric,
    "erp": ErpMetric,
    "edr": EdrMetric,
    "msm": MsmMetric,
    "twe": TweMetric,
}

# distance/_distance.py:149-183 (subset provided here)
_SUBSEQUENCE_METRICS = {
    "euclidean": EuclideanSubsequenceMetric,
    "scaled_euclidean": ScaledEuclideanSubsequenceMetric,
    "dtw": DtwSubsequenceMetric,
    "scaled_dtw": ScaledDtwSubsequenceMetric,
    "wdtw": WeightedDtwSubsequenceMetric,
    "ddtw": DerivativeDtwSubsequenceMetric,
    "wddtw": WeightedDerivativeDtwSubsequenceMetric,
    "adtw": AmercingDtwSubsequenceMetric,
    "lcss": LcssSubsequenceMetric,
    "edr": EdrSubsequenceMetric,
    "twe": TweSubsequenceMetric,
    "msm": MsmSubsequenceMetric,
    "erp": ErpSubsequenceMetric,
}
