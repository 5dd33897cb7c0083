"""Lower bounds for dtw nearest-neighbour search (wildboar.distance.lb).

``DtwKeoghLowerBound`` (distance/lb.py:314-432) and ``DtwKimLowerBound``
(:198-311) of the reference, computed on the GPU (``wb_lb_keogh``,
``wb_lb_kim``, ``wb_dtw_envelope`` in csrc/lower_bound.cu) with the
reference's values: the envelopes use its streaming min / max with its ring
deques, the LB_Keogh sums run in its order.  Their output feeds
``argmin_distance(..., lower_bound=...)``.
"""

import ctypes
import math
import numbers

import numpy as np

from .. import _lib
from ._distance import InvalidParameterError
from ._validation import check_array

_lib.declare("wb_dtw_envelope", [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                 ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_int32, ctypes.c_void_p])
_lib.declare("wb_lb_keogh", [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                             ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                             ctypes.c_int32, ctypes.c_void_p])
_lib.declare("wb_lb_kim", [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                           ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p])

_KINDS = {"both": 0, "left": 1, "right": 2}


def _compute_warp_size(x_size, r, *, y_size=0):
    """distance/dtw.py:38-40."""
    return max(math.floor(max(x_size, y_size) * r), 1)


def _ts2(X):
    """Rows of dim 0 of a (n, n_timestep) or (n, d, n_timestep) array."""
    X = check_array(X, allow_3d=True, ensure_2d=True)
    if X.ndim == 3:
        X = X[:, 0, :]
    return np.ascontiguousarray(X, dtype=np.float64)


def _check_fitted(est):
    if not hasattr(est, "X_"):
        raise ValueError(
            f"This {type(est).__name__} instance is not fitted yet. Call 'fit' with "
            "appropriate arguments before using this estimator.")


def _check_features(est, X):
    if X.shape[-1] != est.X_.shape[-1]:
        raise ValueError(
            f"X has {X.shape[-1]} timesteps, but {type(est).__name__} is expecting "
            f"{est.X_.shape[-1]} timesteps as input.")


def dtw_envelope(X, warp):
    """_dtw_envelop of every row: (lower, upper), each (n, n_timestep)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    lower = np.empty_like(X)
    upper = np.empty_like(X)
    st = _lib.lib().wb_dtw_envelope(_lib.ptr(X), X.shape[0], X.shape[1], int(warp),
                                    _lib.ptr(lower), _lib.ptr(upper), 0, None)
    _lib.check(st)
    return lower, upper


class DtwKimLowerBound:
    """Constant-time dtw lower bound (distance/lb.py:198-311)."""

    def fit(self, X, y=None):
        X = check_array(X, allow_3d=False, ensure_2d=True)
        self.X_ = np.ascontiguousarray(X, dtype=np.float64)
        return self

    def transform(self, X):
        _check_fitted(self)
        Y = check_array(X, allow_3d=False, ensure_2d=True)
        _check_features(self, Y)
        Xf = _ts2(self.X_)
        Yf = _ts2(Y)
        out = np.empty((Yf.shape[0], Xf.shape[0]))
        st = _lib.lib().wb_lb_kim(_lib.ptr(Yf), Yf.shape[0], _lib.ptr(Xf), Xf.shape[0],
                                  Xf.shape[1], _lib.ptr(out), 0, None)
        _lib.check(st)
        return out

    def fit_transform(self, X, y=None):
        return self.fit(X).transform(X)


class DtwKeoghLowerBound:
    """LB_Keogh dtw lower bound (distance/lb.py:314-432).

    Parameters
    ----------
    r : float
        The warp window for DTW.
    kind : {"both", "left", "right"}
        "both": the larger of the query-side and data-side bounds.
    """

    def __init__(self, r=1.0, *, kind="both"):
        self.r = r
        self.kind = kind

    def _validate_params(self):
        if (not isinstance(self.r, numbers.Real) or isinstance(self.r, bool)
                or not 0 <= self.r <= 1):
            raise InvalidParameterError(
                f"The 'r' parameter of DtwKeoghLowerBound must be a float in the range "
                f"[0, 1]. Got {self.r!r} instead.")
        if self.kind not in _KINDS:
            raise InvalidParameterError(
                "The 'kind' parameter of DtwKeoghLowerBound must be a str among "
                f"{{'both', 'left', 'right'}}. Got {self.kind!r} instead.")

    def _warp(self, n_timesteps):
        warp = _compute_warp_size(n_timesteps, self.r)
        if warp == n_timesteps:
            warp -= 1
        return warp

    def fit(self, X, y=None):
        self._validate_params()
        X = check_array(X, allow_3d=True, ensure_2d=True)
        self.X_ = X.reshape(X.shape[0], 1, -1) if X.ndim == 2 else X
        x0 = _ts2(self.X_)
        self.lower_, self.upper_ = dtw_envelope(x0, self._warp(x0.shape[1]))
        return self

    def transform(self, X):
        _check_fitted(self)
        Y = check_array(X, allow_3d=True, ensure_2d=True)
        _check_features(self, Y)
        Yf = _ts2(Y)
        Xf = _ts2(self.X_)
        out = np.empty((Yf.shape[0], Xf.shape[0]))
        st = _lib.lib().wb_lb_keogh(_lib.ptr(Yf), Yf.shape[0], _lib.ptr(Xf), Xf.shape[0],
                                    Xf.shape[1], self._warp(Yf.shape[1]), _KINDS[self.kind],
                                    _lib.ptr(out), 0, None)
        _lib.check(st)
        return out

    def fit_transform(self, X, y=None):
        return self.fit(X).transform(X)


__all__ = ["DtwKeoghLowerBound", "DtwKimLowerBound", "dtw_envelope"]
