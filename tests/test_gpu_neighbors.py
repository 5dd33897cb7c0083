"""dtw_average (method="mm"), KMeans, KNeighborsClassifier and NearestNeighbors
on the GPU path.

Parity: the reference's own outputs (golden fixtures made by running it,
tests/golden/make_golden.py) through the public API, and the CPU oracle
(oracle.dtw_average_mm / oracle.kmeans) on larger seeded cases: both
alignment kernels (the row-strip wavefront with 4, 8 and 16 rows per lane and
means longer than one pass of 512 rows; the anti-diagonal form with 1 to 16
register slots per lane), weights, sample weights, unequal lengths, groups
converging at different epochs.  Means, costs and distances within 1e-12 relative (the
kernels perform the reference's operations in its order; 1e-12 absorbs libm
differences between machines), labels, indices and iteration counts exact.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from tests import _golden  # noqa: E402
from wildboar_gb300.distance import KMeans, KNeighborsClassifier, NearestNeighbors  # noqa: E402
from wildboar_gb300.distance.dtw import _mm_average_groups, dtw_average  # noqa: E402

RTOL = 1e-12


def _cases(kind):
    cs = _golden.cases(kind)
    return pytest.mark.parametrize("case", cs, ids=[c["name"] for c in cs])


@_cases("dtw_average")
def test_dtw_average_golden(case):
    a = dict(case["args"])
    inp = case["inputs"]
    kw = {k: a[k] for k in ("r", "g", "tol", "max_epoch", "random_state", "method",
                            "learning_rate", "decay", "max_stable") if k in a}
    init = inp["init"] if "init" in inp else a["init"]
    mean, cost = dtw_average(inp["x"], init=init, sample_weight=inp.get("sample_weight"),
                             return_cost=True, **kw)
    np.testing.assert_allclose(mean, case["outputs"]["mean"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(cost, case["outputs"]["cost"], rtol=RTOL, atol=0)


@_cases("kmeans")
def test_kmeans_golden(case):
    inp = case["inputs"]
    km = KMeans(**case["args"]).fit(inp["x"])
    out = case["outputs"]
    np.testing.assert_array_equal(km.labels_, out["labels"])
    assert km.n_iter_ == int(out["n_iter"])
    np.testing.assert_allclose(km.cluster_centers_, out["centers"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(km.inertia_, out["inertia"], rtol=RTOL, atol=0)
    if "transform" in out:
        np.testing.assert_allclose(km.transform(inp["xt"]), out["transform"], rtol=RTOL,
                                   atol=0)
        np.testing.assert_array_equal(km.predict(inp["xt"]), out["transform"].argmin(axis=1))


@_cases("knn")
def test_knn_golden(case):
    a = case["args"]
    inp = case["inputs"]
    clf = KNeighborsClassifier(n_neighbors=a["n_neighbors"], metric=a["metric"],
                               metric_params=a["metric_params"]).fit(inp["x"], inp["y"])
    np.testing.assert_array_equal(clf.predict_proba(inp["xt"]), case["outputs"]["proba"])
    np.testing.assert_array_equal(clf.predict(inp["xt"]), case["outputs"]["pred"])


@_cases("kneighbors")
def test_kneighbors_golden(case):
    a = case["args"]
    inp = case["inputs"]
    out = case["outputs"]
    nn = NearestNeighbors(n_neighbors=a["n_neighbors"], metric=a["metric"],
                          metric_params=a["metric_params"]).fit(inp["x"])
    d, i = nn.kneighbors()
    np.testing.assert_array_equal(i, out["ind_train"])
    np.testing.assert_allclose(d, out["dist_train"], rtol=RTOL, atol=0)
    d, i = nn.kneighbors(inp["xt"])
    np.testing.assert_array_equal(i, out["ind"])
    np.testing.assert_allclose(d, out["dist"], rtol=RTOL, atol=0)


def _walk(rng, shape):
    return np.cumsum(rng.standard_normal(shape), axis=-1)


# mean length -> strip of 4 (<= 128), 8 (<= 256), 16 rows per lane, two passes (> 512)
@pytest.mark.parametrize("n,T,r,g", [(100, 100, 1.0, None), (250, 250, 0.2, None),
                                     (400, 400, 0.1, None), (600, 600, 0.05, None),
                                     (300, 300, 0.15, 0.05), (90, 120, 0.3, None),
                                     (530, 500, 0.1, None)])
def test_dtw_average_vs_oracle(n, T, r, g):
    rng = np.random.default_rng(n + T)
    X = _walk(rng, (9, T))
    init = _walk(rng, n)
    mean, cost = dtw_average(X, r=r, g=g, init=init, return_cost=True)
    om, oc = O.dtw_average_mm(X, r=r, g=g, init=init)
    np.testing.assert_allclose(mean, om, rtol=RTOL, atol=0)
    np.testing.assert_allclose(cost, oc, rtol=RTOL, atol=0)


def test_mm_epoch_vs_oracle_sample_weight():
    rng = np.random.default_rng(3)
    X = _walk(rng, (15, 180))
    sw = rng.uniform(0.1, 3.0, 15)
    init = X[4].copy()
    mean = dtw_average(X, r=0.25, init=init, sample_weight=sw, max_epoch=1, tol=0.0)
    np.testing.assert_allclose(mean, O.mm_epoch(X, init, r=0.25, sample_weight=sw),
                               rtol=RTOL, atol=0)


def test_groups_in_lockstep_match_one_by_one():
    # groups of different sizes converge at different epochs; the lockstep
    # batch must give each group the result of its own dtw_average
    rng = np.random.default_rng(11)
    X = _walk(rng, (40, 64))
    groups = [np.arange(0, 3), np.arange(3, 20), np.arange(20, 22), np.arange(22, 40)]
    init = X[[0, 5, 21, 30]].copy()
    Xd = torch.as_tensor(X, device="cuda")
    for g in (None, 0.1):
        means, costs = _mm_average_groups(Xd, groups, init, r=0.3, g=g)
        for k, grp in enumerate(groups):
            om, oc = O.dtw_average_mm(X[grp], r=0.3, g=g, init=init[k])
            np.testing.assert_allclose(means[k], om, rtol=RTOL, atol=0)
            np.testing.assert_allclose(costs[k], oc, rtol=RTOL, atol=0)


@pytest.mark.parametrize("metric,r,g,k", [("dtw", 0.2, None, 4), ("euclidean", 1.0, None, 5),
                                          ("dtw", 1.0, 0.3, 3)])
def test_kmeans_vs_oracle(metric, r, g, k):
    rng = np.random.default_rng(k)
    X = _walk(rng, (60, 48))
    X[:20] += 5.0
    X[20:40] -= 5.0
    km = KMeans(k, metric=metric, r=r, g=g, random_state=k, n_init=2).fit(X)
    labels, centers, inertia, n_iter = O.kmeans(X, k, metric=metric, r=r, g=g, n_init=2,
                                                random_state=k)
    np.testing.assert_array_equal(km.labels_, labels)
    assert km.n_iter_ == n_iter
    np.testing.assert_allclose(km.cluster_centers_, centers, rtol=RTOL, atol=0)
    np.testing.assert_allclose(km.inertia_, inertia, rtol=RTOL, atol=0)


def test_mm_step_launches_native_kernels():
    from wildboar_gb300 import _lib

    rng = np.random.default_rng(2)
    X = _walk(rng, (6, 40))
    before = _lib.launch_count()
    dtw_average(X, r=0.5, init=X[0], max_epoch=2, tol=0.0)
    assert _lib.launch_count() - before >= 2


# both alignment kernels (row-strip wavefront, anti-diagonal) on the same cases
@pytest.mark.parametrize("form", ["strip", "antidiag"])
@pytest.mark.parametrize("n,T,r,g", [(40, 40, 1.0, None), (200, 200, 0.2, None),
                                     (300, 300, 1.0, None), (500, 480, 0.1, 0.05),
                                     (64, 100, 0.4, None), (120, 70, 0.25, 0.2),
                                     (33, 33, 0.0, None)])
def test_alignment_forms_vs_oracle(monkeypatch, form, n, T, r, g):
    monkeypatch.setenv("WB_MM_ALIGN", form)
    rng = np.random.default_rng(7 * n + T)
    X = _walk(rng, (6, T))
    init = _walk(rng, n)
    mean, cost = dtw_average(X, r=r, g=g, init=init, return_cost=True, max_epoch=4, tol=0.0)
    om, oc = O.dtw_average_mm(X, r=r, g=g, init=init, max_epoch=4, tol=0.0)
    np.testing.assert_allclose(mean, om, rtol=RTOL, atol=0)
    np.testing.assert_allclose(cost, oc, rtol=RTOL, atol=0)


@pytest.mark.parametrize("form", ["strip", "antidiag"])
def test_dtw_average_ssg_vs_oracle(monkeypatch, form):
    monkeypatch.setenv("WB_MM_ALIGN", form)
    rng = np.random.default_rng(31)
    X = _walk(rng, (12, 90))
    mean, cost = dtw_average(X, method="ssg", r=0.2, max_epoch=5, random_state=9,
                             return_cost=True)
    rs = np.random.RandomState(9)
    init = X[rs.randint(12)]
    om, oc = O.dtw_average_ssg(X, r=0.2, init=init, max_epoch=5, random_state=rs)
    np.testing.assert_allclose(mean, om, rtol=RTOL, atol=0)
    np.testing.assert_allclose(cost, oc, rtol=RTOL, atol=0)


@_cases("dtw_helpers")
def test_dtw_helpers_golden(case):
    from wildboar_gb300.distance import dtw as D

    a, inp, out = case["args"], case["inputs"], case["outputs"]
    r, ha, hb, hc = a["r"], inp["a"], inp["b"], inp["c"]
    np.testing.assert_allclose(D.dtw_distance(ha, hb, r=r), out["dtw"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(D.ddtw_distance(ha, hc, r=r), out["ddtw"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(D.wdtw_distance(hc, hb, r=r, g=0.1), out["wdtw"], rtol=RTOL,
                               atol=0)
    np.testing.assert_allclose(D.wddtw_distance(ha, hb, r=r, g=0.2), out["wddtw"], rtol=RTOL,
                               atol=0)
    lo, up = D.dtw_envelop(ha, r=r)
    np.testing.assert_array_equal(lo, out["lower"])
    np.testing.assert_array_equal(up, out["upper"])
    d1, cb1 = D.dtw_lb_keogh(hb, ha, r=r)
    d2, cb2 = D.dtw_lb_keogh(hb, lower=lo, upper=up)
    np.testing.assert_allclose(d1, out["lb"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(cb1, out["cb"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(d2, out["lb2"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(cb2, out["cb2"], rtol=RTOL, atol=0)
    np.testing.assert_array_equal(D.dtw_mapping(ha, hc, r=r), out["mapping"])
    wal = D.wdtw_alignment(ha, hc, r=r, g=0.3)
    np.testing.assert_allclose(np.where(inp["mask"], wal, 0.0), out["walign"], rtol=RTOL,
                               atol=0)


@_cases("alignment")
def test_dtw_alignment_golden(case):
    from wildboar_gb300.distance import dtw as D

    inp = case["inputs"]
    al = D.dtw_alignment(inp["x"], inp["y"], r=case["args"]["r"])
    np.testing.assert_allclose(np.where(inp["mask"], al, 0.0), case["outputs"]["a"],
                               rtol=RTOL, atol=0)
