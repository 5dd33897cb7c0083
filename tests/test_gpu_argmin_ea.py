"""GPU parity of argmin_distance's early-abandoned candidate chunks.

For dtw, wdtw, ddtw, wddtw and adtw (penalty >= 0) with a narrow band the
library walks the candidates in chunks of doubling size and stops a pair as
soon as its running largest row minimum exceeds the k-th distance of the
replayed prefix.  ``WB_GPU_ARGMIN=<c>`` sets the first chunk (small chunks
exercise many bound updates on small inputs), ``WB_GPU_ARGMIN=all`` turns the
chunks off, ``WB_GPU_ARGMIN_FORM=strip`` runs the register-strip form (wide
bands) for any band.  Every form must give the oracle's indices (heap order included)
and distances, and the two GPU forms must agree bit for bit.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from wildboar_gb300.distance import argmin_distance  # noqa: E402

RTOL = 1e-12

EA_METRICS = [("dtw", {"r": 0.1}), ("dtw", {"r": 0.3}), ("wdtw", {"g": 0.1, "r": 0.2}),
              ("ddtw", {"r": 0.2}), ("wddtw", {"g": 0.05, "r": 0.25}),
              ("adtw", {"p": 0.5, "r": 0.2}), ("adtw", {"p": 0.0, "r": 0.1})]


def _walk(rng, shape):
    return np.cumsum(rng.standard_normal(shape), axis=-1)


def _both(monkeypatch, first_chunk, X, Y, **kw):
    monkeypatch.setenv("WB_GPU_ARGMIN", str(first_chunk))
    ea = argmin_distance(X, Y, return_distance=True, **kw)
    monkeypatch.setenv("WB_GPU_ARGMIN", "all")
    full = argmin_distance(X, Y, return_distance=True, **kw)
    monkeypatch.delenv("WB_GPU_ARGMIN")
    return ea, full


@pytest.mark.parametrize("metric,params", EA_METRICS,
                         ids=[f"{m}-{i}" for i, (m, _) in enumerate(EA_METRICS)])
@pytest.mark.parametrize("k,first", [(1, 1), (3, 5), (10, 16)])
def test_argmin_ea_vs_oracle(monkeypatch, metric, params, k, first):
    rng = np.random.default_rng(100 + k)
    X = _walk(rng, (19, 60))
    Y = _walk(rng, (260, 60))
    Y[200] = X[4] + 0.01 * rng.standard_normal(60)  # a close candidate late in the scan
    Y[230] = Y[200]                                 # and a tie after it
    (idx, dist), (fidx, fdist) = _both(monkeypatch, first, X, Y, k=k, metric=metric,
                                       metric_params=params)
    oidx, odist = O.argmin(X, Y, k=k, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))


@pytest.mark.parametrize("metric,params", EA_METRICS,
                         ids=[f"{m}-{i}" for i, (m, _) in enumerate(EA_METRICS)])
@pytest.mark.parametrize("k,first", [(1, 3), (6, 9)])
def test_argmin_ea_strip_form_vs_oracle(monkeypatch, metric, params, k, first):
    monkeypatch.setenv("WB_GPU_ARGMIN_FORM", "strip")
    test_argmin_ea_vs_oracle(monkeypatch, metric, params, k, first)


@pytest.mark.parametrize("metric,params", [("dtw", {"r": 1.0}), ("dtw", {"r": 0.5}),
                                           ("wdtw", {"g": 0.05}), ("wddtw", {"g": 0.1}),
                                           ("adtw", {"p": 0.25, "r": 1.0}),
                                           ("ddtw", {"r": 0.7})])
def test_argmin_ea_wide_band_vs_oracle(monkeypatch, metric, params):
    # series long enough that the ring leaves fewer than two blocks per SM:
    # the strip form by default
    rng = np.random.default_rng(31)
    X = _walk(rng, (9, 170))
    Y = _walk(rng, (120, 170))
    Y[100] = X[2] + 0.01 * rng.standard_normal(170)
    (idx, dist), (fidx, fdist) = _both(monkeypatch, 4, X, Y, k=3, metric=metric,
                                       metric_params=params)
    oidx, odist = O.argmin(X, Y, k=3, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))


@pytest.mark.parametrize("form", ["default", "strip"])
@pytest.mark.parametrize("metric,params", [("dtw", {"r": 0.15}), ("wdtw", {"g": 0.2}),
                                           ("adtw", {"p": 1.0, "r": 0.1})])
def test_argmin_ea_unequal_lengths_vs_oracle(monkeypatch, form, metric, params):
    if form == "strip":
        monkeypatch.setenv("WB_GPU_ARGMIN_FORM", "strip")
    rng = np.random.default_rng(9)
    X = _walk(rng, (11, 48))
    Y = _walk(rng, (150, 71))
    (idx, dist), (fidx, fdist) = _both(monkeypatch, 3, X, Y, k=4, metric=metric,
                                       metric_params=params)
    oidx, odist = O.argmin(X, Y, k=4, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))


@pytest.mark.parametrize("form", ["default", "strip"])
def test_argmin_ea_lower_bound_vs_oracle(monkeypatch, form):
    if form == "strip":
        monkeypatch.setenv("WB_GPU_ARGMIN_FORM", "strip")
    rng = np.random.default_rng(12)
    X = _walk(rng, (13, 64))
    Y = _walk(rng, (220, 64))
    full = O.pairwise(X, Y, metric="dtw", metric_params={"r": 0.2})
    lb = full * rng.uniform(0.2, 1.05, size=full.shape)
    (idx, dist), (fidx, fdist) = _both(monkeypatch, 4, X, Y, k=5, metric="dtw",
                                       metric_params={"r": 0.2}, lower_bound=lb)
    oidx, odist = O.argmin(X, Y, k=5, metric="dtw", metric_params={"r": 0.2},
                           lower_bound=lb)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))


def test_argmin_ea_k_above_first_chunks(monkeypatch):
    # k larger than the first chunks: the bound stays infinite until the
    # heap is full
    rng = np.random.default_rng(5)
    X = _walk(rng, (7, 40))
    Y = _walk(rng, (90, 40))
    (idx, dist), _ = _both(monkeypatch, 2, X, Y, k=40, metric="dtw", metric_params={"r": 0.2})
    oidx, odist = O.argmin(X, Y, k=40, metric="dtw", metric_params={"r": 0.2})
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)


def test_argmin_ea_default_schedule_bitwise(monkeypatch):
    # the default schedule at a size where it chunks (2 000 queries), against
    # the all-pairs form, plus a row sample against the oracle
    rng = np.random.default_rng(21)
    X = _walk(rng, (2000, 128))
    Y = _walk(rng, (1200, 128))
    monkeypatch.delenv("WB_GPU_ARGMIN", raising=False)
    idx, dist = argmin_distance(X, Y, k=5, metric="dtw", metric_params={"r": 0.1},
                                return_distance=True)
    monkeypatch.setenv("WB_GPU_ARGMIN", "all")
    fidx, fdist = argmin_distance(X, Y, k=5, metric="dtw", metric_params={"r": 0.1},
                                  return_distance=True)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))
    rows = [0, 777, 1999]
    oidx, odist = O.argmin(X[rows], Y, k=5, metric="dtw", metric_params={"r": 0.1})
    np.testing.assert_array_equal(idx[rows], oidx)
    np.testing.assert_allclose(dist[rows], odist, rtol=RTOL, atol=0)


@pytest.mark.parametrize("metric,params", [("dtw", {"r": 1.0}), ("lcss", {"epsilon": 0.5}),
                                           ("msm", {"c": 0.5}), ("wdtw", {"g": 0.05})])
def test_argmin_long_series_wide_band_vs_oracle(monkeypatch, metric, params):
    # L = 512 with a full band: the all-pairs form runs the ring kernel with a
    # global ring (its workspace is sized for the keyed kernel), the chunked
    # form the strip kernel
    rng = np.random.default_rng(41)
    X = _walk(rng, (5, 512))
    Y = _walk(rng, (40, 512))
    Y[33] = X[1] + 0.01 * rng.standard_normal(512)
    (idx, dist), (fidx, fdist) = _both(monkeypatch, 2, X, Y, k=3, metric=metric,
                                       metric_params=params)
    oidx, odist = O.argmin(X, Y, k=3, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))


STRIP_EA_METRICS = [("edr", {"epsilon": 0.5}), ("edr", {}), ("edr", {"epsilon": 0.3, "r": 0.2}),
                    ("erp", {"g": 0.2}), ("erp", {"g": 0.0, "r": 0.3}), ("msm", {"c": 0.5}),
                    ("msm", {"c": 1.0, "r": 0.2}), ("twe", {"penalty": 0.5, "stiffness": 0.01}),
                    ("twe", {"penalty": 1.0, "stiffness": 0.001, "r": 0.25})]


@pytest.mark.parametrize("metric,params", STRIP_EA_METRICS,
                         ids=[f"{m}-{i}" for i, (m, _) in enumerate(STRIP_EA_METRICS)])
@pytest.mark.parametrize("k,first", [(1, 2), (4, 7)])
def test_argmin_strip_ea_vs_oracle(monkeypatch, metric, params, k, first):
    # edr / erp / msm / twe: the generic strip form with chunks and bounds
    test_argmin_ea_vs_oracle(monkeypatch, metric, params, k, first)


@pytest.mark.parametrize("metric,params", [("edr", {}), ("erp", {"g": 0.1}),
                                           ("msm", {"c": 0.7}),
                                           ("twe", {"penalty": 0.3, "stiffness": 0.05})])
def test_argmin_strip_ea_unequal_lengths_vs_oracle(monkeypatch, metric, params):
    rng = np.random.default_rng(19)
    X = _walk(rng, (8, 52))
    Y = _walk(rng, (110, 37))
    (idx, dist), (fidx, fdist) = _both(monkeypatch, 3, X, Y, k=4, metric=metric,
                                       metric_params=params)
    oidx, odist = O.argmin(X, Y, k=4, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))


@pytest.mark.parametrize("metric,params", [("lcss", {"epsilon": 0.5}),
                                           ("wlcss", {"epsilon": 0.4, "g": 0.1}),
                                           ("adtw", {"p": -0.2, "r": 1.0})])
def test_argmin_keyed_strip_sweep_vs_oracle(monkeypatch, metric, params):
    # lcss / wlcss / negative-penalty adtw with a band too wide for a shared
    # ring: one chunk through the strip sweep with keys, no bound
    rng = np.random.default_rng(23)
    X = _walk(rng, (6, 240))
    Y = _walk(rng, (45, 240))
    Y[30] = X[2] + 0.01 * rng.standard_normal(240)
    (idx, dist), (fidx, fdist) = _both(monkeypatch, 5, X, Y, k=3, metric=metric,
                                       metric_params=params)
    oidx, odist = O.argmin(X, Y, k=3, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))


@pytest.mark.parametrize("metric,params", [("dtw", {"r": 0.2}), ("msm", {"c": 0.5}),
                                           ("dtw", {"r": 1.0})])
def test_argmin_ea_multivariate_dim_vs_oracle(monkeypatch, metric, params):
    # (n, d, L) inputs (the reference's argmin accepts dim 0 only): the
    # chunked kernels read dimension 0 through the series stride d * L
    rng = np.random.default_rng(61)
    X = _walk(rng, (7, 3, 130))
    Y = _walk(rng, (90, 3, 130))
    (idx, dist), (fidx, fdist) = _both(monkeypatch, 3, X, Y, k=4, metric=metric,
                                       metric_params=params, dim=0)
    oidx, odist = O.argmin(X[:, 0, :], Y[:, 0, :], k=4, metric=metric, metric_params=params)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    np.testing.assert_array_equal(idx, fidx)
    assert np.array_equal(dist.view(np.uint64), fdist.view(np.uint64))


def test_argmin_ea_device_inputs(monkeypatch):
    # torch device tensors (outputs stay on the device) through the chunks
    rng = np.random.default_rng(62)
    X = _walk(rng, (300, 96))
    Y = _walk(rng, (700, 96))
    Xd = torch.as_tensor(X, device="cuda")
    Yd = torch.as_tensor(Y, device="cuda")
    monkeypatch.setenv("WB_GPU_ARGMIN", "16")
    idx, dist = argmin_distance(Xd, Yd, k=5, metric="dtw", metric_params={"r": 0.1},
                                return_distance=True)
    hidx, hdist = argmin_distance(X, Y, k=5, metric="dtw", metric_params={"r": 0.1},
                                  return_distance=True)
    np.testing.assert_array_equal(idx.cpu().numpy(), hidx)
    assert np.array_equal(dist.cpu().numpy().view(np.uint64), hdist.view(np.uint64))
    rows = [0, 150, 299]
    oidx, odist = O.argmin(X[rows], Y, k=5, metric="dtw", metric_params={"r": 0.1})
    np.testing.assert_array_equal(hidx[rows], oidx)
    np.testing.assert_allclose(hdist[rows], odist, rtol=RTOL, atol=0)


@pytest.mark.parametrize("metric,params,first", [("dtw", {"r": 0.2}, "5"), ("msm", {"c": 0.5}, "5"),
                                                 ("lcss", {"epsilon": 0.5}, "all"),
                                                 ("euclidean", {}, "all")])
def test_argmin_query_batches(monkeypatch, metric, params, first):
    # queries in several batches (a pair budget of 7 query rows of 150
    # candidates), with a lower bound: the same result as one batch
    rng = np.random.default_rng(63)
    X = _walk(rng, (31, 64))
    Y = _walk(rng, (150, 64))
    lb = None
    if metric == "dtw":
        full = O.pairwise(X, Y, metric=metric, metric_params=params)
        lb = full * rng.uniform(0.3, 1.02, size=full.shape)
    monkeypatch.setenv("WB_GPU_ARGMIN", first)
    monkeypatch.setenv("WB_GPU_ARGMIN_BATCH", str(7 * 150))
    idx, dist = argmin_distance(X, Y, k=4, metric=metric, metric_params=params,
                                lower_bound=lb, return_distance=True)
    monkeypatch.delenv("WB_GPU_ARGMIN_BATCH")
    sidx, sdist = argmin_distance(X, Y, k=4, metric=metric, metric_params=params,
                                  lower_bound=lb, return_distance=True)
    np.testing.assert_array_equal(idx, sidx)
    assert np.array_equal(dist.view(np.uint64), sdist.view(np.uint64))
    oidx, odist = O.argmin(X, Y, k=4, metric=metric, metric_params=params, lower_bound=lb)
    np.testing.assert_array_equal(idx, oidx)
    np.testing.assert_allclose(dist, odist, rtol=RTOL, atol=0)
    if metric == "dtw":
        Xd = torch.as_tensor(X, device="cuda")
        Yd = torch.as_tensor(Y, device="cuda")
        lbd = torch.as_tensor(lb, device="cuda")
        monkeypatch.setenv("WB_GPU_ARGMIN_BATCH", str(7 * 150))
        didx, ddist = argmin_distance(Xd, Yd, k=4, metric=metric, metric_params=params,
                                      lower_bound=lbd, return_distance=True)
        np.testing.assert_array_equal(didx.cpu().numpy(), idx)
        assert np.array_equal(ddist.cpu().numpy().view(np.uint64), dist.view(np.uint64))


def _golden_argmin_cases():
    from tests import _golden
    return [c for c in _golden.cases("argmin") if c["name"].startswith("argmin_long_")]


@pytest.mark.parametrize("case", _golden_argmin_cases(), ids=lambda c: c["name"])
@pytest.mark.parametrize("first", ["3", "40", "all"])
def test_argmin_long_golden_chunked(monkeypatch, case, first):
    # the reference's own outputs over 400 candidates (golden fixtures),
    # through forced small chunks, larger chunks and the all-pairs form
    a = case["args"]
    inp = case["inputs"]
    monkeypatch.setenv("WB_GPU_ARGMIN", first)
    idx, dist = argmin_distance(inp["x"], inp["y"], k=a["k"], metric=a["metric"],
                                metric_params=a.get("metric_params"), return_distance=True)
    np.testing.assert_array_equal(idx, case["outputs"]["idx"])
    np.testing.assert_allclose(dist, case["outputs"]["dist"], rtol=RTOL, atol=0)
