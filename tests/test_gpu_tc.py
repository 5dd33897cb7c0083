"""Tensor-core euclidean (tcgen05, 3xTF32) against the FP64 euclidean matrix."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from wildboar_gb300.distance import precision as P  # noqa: E402

# 3xTF32 products of the series centred on their means, accumulated in FP32
# in tensor memory (one accumulator over the whole length): the squared
# distance carries an error of ~1e-5 of |x|^2 + |y|^2 at length 1000
# (cancellation makes that larger relative to d^2 for close pairs).  Bars:
# |d2_tc - d2| <= 2e-5 (|x|^2 + |y|^2) and 1e-4 relative on d for pairs whose
# d^2 is at least 5% of |x|^2 + |y|^2.
NORM_TOL = 2e-5
TC_RTOL = 1e-4


def _check(got, X, Y):
    nx = (X * X).sum(1)[:, None]
    ny = (Y * Y).sum(1)[None, :]
    d2 = np.maximum(nx + ny - 2 * X @ Y.T, 0)
    want = np.sqrt(d2)
    assert np.max(np.abs(got ** 2 - d2) / (nx + ny)) <= NORM_TOL
    far = d2 >= 0.05 * (nx + ny)
    np.testing.assert_allclose(got[far], want[far], rtol=TC_RTOL)


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (300, 257, 1000), (64, 700, 96),
                                   (513, 129, 4)])
def test_euclidean_tc_vs_fp64(m, n, k):
    rng = np.random.default_rng(m * 7 + n + k)
    X = np.cumsum(rng.standard_normal((m, k)), axis=1)
    Y = np.cumsum(rng.standard_normal((n, k)), axis=1)
    got = P.pairwise_euclidean_tc(torch.as_tensor(X, device="cuda"),
                                  torch.as_tensor(Y, device="cuda")).cpu().numpy()
    _check(got, X, Y)


def test_euclidean_tc_matches_oracle_sample():
    rng = np.random.default_rng(1)
    X = np.cumsum(rng.standard_normal((40, 256)), axis=1)
    Y = np.cumsum(rng.standard_normal((30, 256)), axis=1)
    got = P.pairwise_euclidean_tc(torch.as_tensor(X, device="cuda"),
                                  torch.as_tensor(Y, device="cuda")).cpu().numpy()
    want = O.pairwise(X, Y, metric="euclidean")
    np.testing.assert_allclose(got, want, rtol=TC_RTOL)


def test_dtw_fp32_precision_form():
    rng = np.random.default_rng(2)
    X = np.cumsum(rng.standard_normal((25, 128)), axis=1)
    Y = np.cumsum(rng.standard_normal((19, 128)), axis=1)
    got = P.pairwise_dtw_fp32(torch.as_tensor(X, device="cuda"),
                              torch.as_tensor(Y, device="cuda"), r=0.1).cpu().numpy()
    want = O.pairwise(X.astype(np.float32).astype(np.float64),
                      Y.astype(np.float32).astype(np.float64), metric="dtw",
                      metric_params={"r": 0.1})
    np.testing.assert_allclose(got, want, rtol=1e-5)


def test_euclidean_tc_offset_series():
    # series far from zero: centring keeps the error relative to the centred
    # magnitudes, so distances stay accurate although |x|^2 + |y|^2 >> d^2
    rng = np.random.default_rng(4)
    X = np.cumsum(rng.standard_normal((200, 300)), axis=1) + 1000.0
    Y = np.cumsum(rng.standard_normal((260, 300)), axis=1) + 990.0
    got = P.pairwise_euclidean_tc(torch.as_tensor(X, device="cuda"),
                                  torch.as_tensor(Y, device="cuda")).cpu().numpy()
    want = np.sqrt(((X[:, None, :] - Y[None, :, :]) ** 2).sum(-1))
    Xc = X - X.mean(1, keepdims=True)
    Yc = Y - Y.mean(1, keepdims=True)
    scale = (Xc * Xc).sum(1)[:, None] + (Yc * Yc).sum(1)[None, :]
    assert np.max(np.abs(got ** 2 - want ** 2) / scale) <= NORM_TOL
    far = want ** 2 >= 0.05 * scale
    np.testing.assert_allclose(got[far], want[far], rtol=TC_RTOL)
