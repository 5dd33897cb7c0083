"""Parity at the benchmark workloads' own shapes.

Each test runs the CUDA path on inputs drawn exactly as the benchmark draws
them (seeded Gaussian random walks) and compares with the CPU oracle:

* C1 -- pairwise_distance dtw r=0.1, 100 x 100 distinct random walks, L=128:
  bit-exact.
* C2 -- 8 query rows x 2000 series of length 512 for every metric setting of
  the L=512 sweep (dtw r in {0.1, 1}, wdtw g=0.05, ddtw, adtw, lcss / edr with
  epsilon = 0.1 std(X), erp g=0, msm c=1, twe stiffness=0.001 penalty=1):
  the FP64 drop-in bit-exact; the FP32-compensated form within the per-metric
  bar of tests/test_gpu_precision.py.
* C3 -- 300 shapelets of the shapelet-scan distribution (lengths U{16..128},
  z-normalised random-walk fragments) x 8 series of length 1024, euclidean and
  scaled_euclidean: distances and argmin indices bit-exact.
* C4 -- 256 pairs x 3 dims of the ragged batch (lengths U{32..2048}
  NaN-padded to 2048, r=0.1) through the CUDA-graph runner: within 1e-5
  relative of the FP64 oracle.
* C5 -- differentiable dtw at L=256, r=0.2: distances within 1e-5, gradients
  within 1e-4 of the reference's dtw_alignment + dtw_mapping path.

The reference recurrences are distance/_elastic.pyx:869-940 (dtw) and its
siblings; the oracle restates them in the reference's operation order.
"""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from tests.test_gpu_precision import _check as _check_fp32  # noqa: E402
from wildboar_gb300.distance import pairwise_distance  # noqa: E402
from wildboar_gb300.distance.precision import pairwise_distance_fp32  # noqa: E402

THREADS = os.cpu_count() or 1


def _walks(seed, shape):
    return np.cumsum(np.random.default_rng(seed).standard_normal(shape), axis=-1)


def test_c1_pairwise_dtw_bit_exact():
    X = _walks(101, (100, 128))
    Y = _walks(102, (100, 128))
    got = pairwise_distance(X, Y, metric="dtw", metric_params={"r": 0.1})
    want = O.pairwise(X, Y, metric="dtw", metric_params={"r": 0.1}, n_threads=THREADS)
    assert got.shape == (100, 100)
    np.testing.assert_array_equal(got, want)
    # and through device tensors (the result stays on the GPU)
    gt = pairwise_distance(torch.as_tensor(X, device="cuda"), torch.as_tensor(Y, device="cuda"),
                           metric="dtw", metric_params={"r": 0.1})
    np.testing.assert_array_equal(gt.cpu().numpy(), want)


def _c2_data():
    X = _walks(12, (8, 512))
    Y = _walks(13, (2000, 512))
    return X, Y


def _c2_sweep():
    X, _ = _c2_data()
    eps = 0.1 * float(X.std())
    return [("dtw", {"r": 0.1}), ("dtw", {"r": 1.0}), ("wdtw", {"g": 0.05}), ("ddtw", {}),
            ("adtw", {}), ("lcss", {"epsilon": eps}), ("edr", {"epsilon": eps}),
            ("erp", {"g": 0.0}), ("msm", {"c": 1.0}),
            ("twe", {"stiffness": 0.001, "penalty": 1.0})]


C2 = _c2_sweep()


@pytest.mark.parametrize("metric,params", C2, ids=[f"{m}-{i}" for i, (m, _) in enumerate(C2)])
def test_c2_slice_fp64_bit_exact_and_fp32_bar(metric, params):
    X, Y = _c2_data()
    want = O.pairwise(X, Y, metric=metric, metric_params=params, n_threads=THREADS)
    got = pairwise_distance(X, Y, metric=metric, metric_params=params)
    np.testing.assert_array_equal(got, want)
    got32 = pairwise_distance_fp32(X, Y, metric=metric, metric_params=params)
    n = 510 if metric == "ddtw" else 512
    _check_fp32(metric, got32, want, n, n, params)


def _c3_data(n_series, n_shapelets, seed=6):
    rng = np.random.default_rng(seed)
    X = np.cumsum(rng.standard_normal((n_series, 1024)), axis=1)
    shp = []
    for L in rng.integers(16, 129, size=n_shapelets):
        f = np.cumsum(rng.standard_normal(L))
        sd = f.std()
        shp.append((f - f.mean()) / (sd if sd > 0 else 1.0))
    return X, shp


@pytest.mark.parametrize("metric", ["euclidean", "scaled_euclidean"])
def test_c3_slice_subsequence_bit_exact(metric):
    from wildboar_gb300.distance import pairwise_subsequence_distance

    X, shp = _c3_data(8, 300)
    d, i = pairwise_subsequence_distance(shp, X, metric=metric, return_index=True)
    od, oi = O.subsequence(shp, X, metric=metric, n_threads=THREADS)
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(d, od)


def test_c4_slice_ragged_batch_vs_fp64_oracle():
    from wildboar_gb300.distance.batched import BatchedDTW

    rng = np.random.default_rng(44)
    n, d, L, r = 256, 3, 2048, 0.1
    x = np.cumsum(rng.standard_normal((n, d, L)), axis=-1).astype(np.float32)
    y = np.cumsum(rng.standard_normal((n, d, L)), axis=-1).astype(np.float32)
    lx = rng.integers(32, L + 1, size=(n, d))
    ly = rng.integers(32, L + 1, size=(n, d))
    ar = np.arange(L)
    x[ar[None, None, :] >= lx[..., None]] = np.nan
    y[ar[None, None, :] >= ly[..., None]] = np.nan
    runner = BatchedDTW(torch.as_tensor(x, device="cuda"), torch.as_tensor(y, device="cuda"),
                        r=r, tune=False, graph=True)
    runner.run()
    got = runner.run().cpu().numpy()
    want = np.zeros(n)
    for i in range(n):
        acc = 0.0
        for k in range(d):
            acc += O.distance_1d(x[i, k, : lx[i, k]].astype(np.float64),
                                 y[i, k, : ly[i, k]].astype(np.float64), metric="dtw",
                                 metric_params={"r": r})
        want[i] = acc / d
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=0)


def _near_tie(al, path, rel=1e-9):
    """True if some step of the optimal path had a competing predecessor whose
    cumulative cost is within `rel` of the chosen one (dtw is not
    differentiable at a tie, and the compensated float32 costs resolve
    differences down to about 1e-12 of the path cost)."""
    for a, b in path:
        if a == 0 or b == 0:
            continue
        c = np.sort([al[a - 1, b - 1], al[a - 1, b], al[a, b - 1]])
        if np.isfinite(c[1]) and c[1] - c[0] <= rel * c[0]:
            return True
    return False


def test_c5_slice_gradient_vs_alignment_path():
    from wildboar_gb300.distance import autograd as AG

    rng = np.random.default_rng(55)
    L, r = 256, 0.2
    t = np.linspace(0, 1, L)
    nx, nc = 8, 4
    X = np.stack([np.sin(2 * np.pi * (1 + k / 4) * t) * 3 + 0.1 * rng.standard_normal(L)
                  for k in range(nx)]).astype(np.float32)
    C = np.cumsum(rng.standard_normal((nc, L)), axis=1).astype(np.float32) * 0.3
    gw = rng.standard_normal((nx, nc))
    paths = {}
    for i in range(nx):
        for j in range(nc):
            x64, c64 = X[i].astype(np.float64), C[j].astype(np.float64)
            al = O.dtw_alignment(x64, c64, r=r)
            path = O.dtw_mapping(al)
            if _near_tie(al, path):
                # dtw is differentiable where the optimal path is unique: a
                # pair whose path passes a near-tie is left out of the check
                gw[i, j] = 0.0
            paths[i, j] = (np.sqrt(al[-1, -1]), path)
    assert np.count_nonzero(gw) >= nx * nc // 2
    xt = torch.as_tensor(X, device="cuda").requires_grad_(True)
    ct = torch.as_tensor(C, device="cuda").requires_grad_(True)
    D = AG.dtw_matrix(xt, ct, r)
    (D * torch.as_tensor(gw, device="cuda")).sum().backward()
    gx_want = np.zeros((nx, L))
    gc_want = np.zeros((nc, L))
    for (i, j), (d, path) in paths.items():
        x64, c64 = X[i].astype(np.float64), C[j].astype(np.float64)
        assert abs(D[i, j].item() - d) <= 1e-5 * d
        for a, b in path:
            g = gw[i, j] * (x64[a] - c64[b]) / d
            gx_want[i, a] += g
            gc_want[j, b] -= g
    np.testing.assert_allclose(xt.grad.cpu().numpy(), gx_want, rtol=0, atol=1e-4)
    np.testing.assert_allclose(ct.grad.cpu().numpy(), gc_want, rtol=0, atol=1e-4)
