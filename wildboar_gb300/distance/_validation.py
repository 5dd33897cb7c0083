"""Input validation of the distance API.

Restates what the reference's ``check_array`` / ``_check_ts_array``
(wildboar src/wildboar/utils/validation.py:404-620) enforce on the distance
hot path, with the same error messages, without depending on scikit-learn:
float64 conversion, at most three dimensions, at least one sample and one
timestep, rejection of end-of-series markers, NaN and infinity.
"""

import numpy as np

_EOS_LOW_BITS = 9  # utils/variable_len.py:17 (EoS = float32 NaN 0x7F800009)


def is_end_of_series(x):
    """utils/variable_len.py:29-46: NaN whose float32 image has low bits 1001."""
    x = np.asarray(x)
    nan = np.isnan(x)
    if not nan.any():
        return nan
    bits = np.array(x, dtype="f").view(dtype="I")
    return np.logical_and(nan, np.bitwise_and(bits, np.uint32(0xF)) == _EOS_LOW_BITS)


def check_array(array, *, allow_3d=True, ensure_2d=False, ensure_ts_array=False,
                dtype=float, allow_nan=False, input_name=""):
    try:
        array = np.asarray(array, dtype=dtype)
    except (TypeError, ValueError) as e:
        raise ValueError(str(e)) from None
    if array.ndim == 0:
        raise ValueError(
            f"Singleton array {array!r} cannot be considered a valid collection."
        )
    if ensure_2d and array.ndim == 1:
        raise ValueError(
            "Expected 2D array, got 1D array instead:\narray={}.\n"
            "Reshape your data either using array.reshape(-1, 1) if "
            "your data has a single feature or array.reshape(1, -1) "
            "if it contains a single sample.".format(array)
        )
    if not allow_3d and array.ndim >= 3:
        raise ValueError("Found array with dim %d. None expected <= 2." % array.ndim)
    if array.ndim >= 4:
        raise ValueError("Found array with dim %d. None expected <= 3." % array.ndim)
    n_samples = array.shape[0]
    if n_samples < 1:
        raise ValueError(
            "Found array with %d sample(s) (shape=%s) while a minimum of %d is required."
            % (n_samples, array.shape, 1)
        )
    if array.ndim in (2, 3):
        if array.ndim == 3 and array.shape[1] < 1:
            raise ValueError(
                "Found array with %d dimension(s) (shape=%s) while a minimum of %d is "
                "required." % (array.shape[1], array.shape, 1)
            )
        if array.shape[-1] < 1:
            raise ValueError(
                "Found array with %d feature(s) (shape=%s) while a minimum of %d is "
                "required." % (array.shape[-1], array.shape, 1)
            )
    padded = input_name + " " if input_name else ""
    if np.issubdtype(array.dtype, np.floating):
        nan = np.isnan(array)
        if nan.any():
            if is_end_of_series(array).any():
                raise ValueError(f"Input {padded}expected time series of equal length.")
            if not allow_nan:
                raise ValueError(f"Input {padded}contains NaN.")
        if np.isinf(array).any():
            raise ValueError(f"Input {padded}contains infinity.")
    if not ensure_ts_array:
        array = np.ascontiguousarray(array)
    return check_ts_array(array) if ensure_ts_array else array


def check_ts_array(array):
    """_check_ts_array: (n_samples, n_dims, n_timestep), C-contiguous float64."""
    if array.ndim == 1:
        array = array.reshape(1, 1, array.shape[0])
    elif array.ndim == 2:
        array = array.reshape(array.shape[0], 1, array.shape[1])
    return np.ascontiguousarray(array, dtype=np.float64)
