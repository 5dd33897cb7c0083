"""Pin the CPU oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by running the reference wildboar build through its
public API (tests/golden/make_golden.py).  On x86-64 the oracle must reproduce
them bit for bit; elsewhere a libm exp/pow that rounds differently may move
WDTW weights or EDR epsilons by an ulp, hence the 1e-12 relative fallback.
"""

import math
import platform

import numpy as np
import pytest

from oracle import oracle as O
from tests import _golden

EXACT = platform.machine() in ("x86_64", "AMD64")


def _ts(x):
    x = np.asarray(x, dtype=float)
    if x.ndim == 1:
        return x.reshape(1, 1, -1)
    if x.ndim == 2:
        return x.reshape(x.shape[0], 1, x.shape[1])
    return x


def _format_return(x, y_dims, x_dims):
    # distance/_distance.py:514-540
    if x_dims == 1 and y_dims == 1 and x.size == 1:
        return x.item()
    elif x_dims == 1 or y_dims == 1:
        return np.squeeze(x)
    return x


def _dims(fn, n_dims, dim):
    if n_dims == 1 and dim == "mean":
        dim = 0
    if dim in ("mean", "full"):
        ds = [fn(d) for d in range(n_dims)]
        return np.mean(ds, axis=0) if dim == "mean" else np.stack(ds, axis=0)
    return fn(dim)


def run_oracle(case):
    a = case["args"]
    metric, params = a.get("metric"), a.get("metric_params", {})
    dim = a.get("dim", "mean")
    kind = case["kind"]
    inp = case["inputs"]
    if kind == "pairwise":
        x, y = inp["x"], inp["y"]
        X, Y = _ts(x), _ts(y)
        d = _dims(lambda k: O.pairwise(X, Y, dim=k, metric=metric, metric_params=params),
                  X.shape[1], dim)
        return {"d": _format_return(d, y.ndim, x.ndim)}
    if kind == "singleton":
        X = _ts(inp["x"])
        d = _dims(lambda k: O.pairwise(X, None, dim=k, metric=metric,
                                       metric_params=params), X.shape[1], dim)
        return {"d": d}
    if kind == "paired":
        x, y = inp["x"], inp["y"]
        X, Y = _ts(x), _ts(y)
        d = _dims(lambda k: O.paired(X, Y, dim=k, metric=metric, metric_params=params),
                  X.shape[1], dim)
        return {"d": _format_return(d, y.ndim, x.ndim)}
    if kind == "argmin":
        idx, dist = O.argmin(inp["x"], inp["y"], k=a["k"], metric=metric,
                             metric_params=params, lower_bound=inp.get("lower_bound"))
        return {"idx": idx, "dist": dist}
    if kind == "subsequence":
        shp = _golden.unpack_shapelets(case)
        d, i = O.subsequence(shp, inp["x"], metric=metric, metric_params=params)
        return {"d": d, "idx": i}
    if kind == "paired_subsequence":
        # _paired_subsequence_distance (distance/_cdistance.pyx:1040-1062) is the
        # pairwise scan of shapelet i against series i
        shp = _golden.unpack_shapelets(case)
        d, i = O.subsequence(shp, inp["x"], metric=metric, metric_params=params)
        n = len(shp)
        return {"d": d[np.arange(n), np.arange(n)], "idx": i[np.arange(n), np.arange(n)]}
    if kind == "argmin_subsequence":
        idx, dist = O.argmin_subsequence(inp["y"], inp["x"], k=a["k"], metric=metric,
                                         metric_params=params, scale=a["scale"])
        return {"idx": idx, "dist": dist}
    if kind == "distance_profile":
        X = _ts(inp["x"])
        q = inp["y"]
        d, _ = O.subsequence_matches([q] * X.shape[0], X, math.inf, metric=metric,
                                     metric_params=params, transient=True)
        return {"d": np.squeeze(d[:, : X.shape[2] - q.shape[0] + 1])}
    if kind == "dilated_profile":
        d = O.dilated_profile(np.atleast_2d(inp["y"]), _ts(inp["x"]), dilation=a["dilation"],
                              padding=a["padding"], dim=a.get("dim", 0), metric=metric,
                              metric_params=params, scale=a.get("scale", False))
        return {"d": np.squeeze(d)}
    if kind == "mass_profile":
        return {"d": np.squeeze(O.mass_profile(inp["y"], _ts(inp["x"])))}
    if kind in ("subsequence_match", "paired_subsequence_match"):
        X = _ts(inp["x"])
        if kind == "subsequence_match":
            shp = [inp["y"]] * X.shape[0]
        else:
            shp = _golden.unpack_shapelets(case)
        return oracle_matches(shp, X, metric, params, dict(a["kw"]), kind)
    if kind == "alignment":
        al = O.dtw_alignment(inp["x"], inp["y"], r=a["r"])
        return {"a": np.where(inp["mask"], al, 0.0)}
    if kind == "dtw_average":
        X = inp["x"]
        rs = np.random.RandomState(a["random_state"]) if "random_state" in a else None
        if "init" in inp:
            init = inp["init"]
        else:  # init="random": dtw_average draws the row (distance/dtw.py:542-543)
            init = X[rs.randint(X.shape[0])]
        if a.get("method") == "ssg":
            kw = {k: a[k] for k in ("max_epoch", "learning_rate", "decay", "max_stable")
                  if k in a}
            mean, cost = O.dtw_average_ssg(X, r=a["r"], g=a.get("g"), init=init,
                                           sample_weight=inp.get("sample_weight"),
                                           random_state=rs, **kw)
            return {"mean": mean, "cost": cost}
        mean, cost = O.dtw_average_mm(X, r=a["r"], g=a.get("g"), init=init,
                                      sample_weight=inp.get("sample_weight"),
                                      tol=a.get("tol", 1e-5), max_epoch=a.get("max_epoch", 50))
        return {"mean": mean, "cost": cost}
    if kind == "kmeans":
        labels, centers, inertia, n_iter = O.kmeans(
            inp["x"], a["n_clusters"], metric=a.get("metric", "euclidean"), r=a.get("r", 1.0),
            g=a.get("g"), n_init=a.get("n_init", "auto"), max_iter=a.get("max_iter", 300),
            random_state=a["random_state"])
        out = {"labels": labels, "centers": centers, "inertia": inertia, "n_iter": n_iter}
        if "xt" in inp:
            metric, params = "euclidean", {}
            if a.get("metric") == "dtw":
                metric = "dtw" if a.get("g") is None else "wdtw"
                params = {"r": a.get("r", 1.0)}
                if a.get("g") is not None:
                    params["g"] = a["g"]
            out["transform"] = O.pairwise(inp["xt"], centers, metric=metric,
                                          metric_params=params)
        return out
    if kind == "knn":
        proba = O.knn_predict_proba(inp["x"], inp["y"], inp["xt"], n_neighbors=a["n_neighbors"],
                                    metric=metric, metric_params=a["metric_params"])
        classes = np.unique(inp["y"])
        return {"proba": proba, "pred": classes[np.argmax(proba, axis=1)]}
    if kind == "kneighbors":
        k = a["n_neighbors"]
        X, Xt = inp["x"], inp["xt"]

        def sorted_argmin(q, kk):
            idx, dist = O.argmin(q, X, k=kk, metric=metric, metric_params=a["metric_params"])
            order = np.argsort(dist, axis=1, kind="stable")
            return np.take_along_axis(idx, order, 1), np.take_along_axis(dist, order, 1)

        ind, dist = sorted_argmin(X, k + 1)
        mask = ind != np.arange(X.shape[0])[:, None]
        ind_tr = ind[mask].reshape(X.shape[0], -1)
        dist_tr = dist[mask].reshape(X.shape[0], -1)
        ind_te, dist_te = sorted_argmin(Xt, k)
        return {"dist_train": dist_tr, "ind_train": ind_tr, "dist": dist_te, "ind": ind_te}
    if kind == "lb_keogh":
        X = inp["x"]
        lo, up = O.dtw_envelope(X, O._warp_size(X.shape[1], a["r"]))
        return {"out": O.lb_keogh(inp["q"], X, r=a["r"], kind=a["kind"]), "lower": lo,
                "upper": up}
    if kind == "lb_kim":
        return {"out": O.lb_kim(inp["q"], inp["x"])}
    if kind == "dtw_helpers":
        r, ha, hb, hc = a["r"], inp["a"], inp["b"], inp["c"]
        warp = max(math.floor(ha.shape[0] * r), 1)
        warp = warp - 1 if warp == ha.shape[0] else warp
        lo, up = O.dtw_envelope(ha, warp)
        lo, up = lo[0], up[0]
        # cumulative_bound at mean 0, std 1 (distance/_elastic.pyx:240-270): a
        # sequential sum of the excursion terms
        cb = np.where(hb > up, (hb - up) ** 2, np.where(hb < lo, (hb - lo) ** 2, 0.0))
        acc = 0.0
        for v in cb.tolist():
            acc += v
        lb = math.sqrt(acc)
        path = O.dtw_mapping(O.dtw_alignment(ha, hc, r=r))
        mapping = np.zeros((ha.shape[0], hc.shape[0]), dtype=bool)
        for i, j in path:
            mapping[i, j] = True
        wal = O.dtw_alignment(ha, hc, r=r, weights=O.jeong_weight(35, 0.3))
        return {"dtw": O.distance_1d(ha, hb, metric="dtw", metric_params={"r": r}),
                "ddtw": O.distance_1d(ha, hc, metric="ddtw", metric_params={"r": r}),
                "wdtw": O.distance_1d(hc, hb, metric="wdtw", metric_params={"r": r, "g": 0.1}),
                "wddtw": O.distance_1d(ha, hb, metric="wddtw",
                                       metric_params={"r": r, "g": 0.2}),
                "lower": lo, "upper": up, "lb": lb, "cb": cb, "lb2": lb, "cb2": cb,
                "mapping": mapping, "walign": np.where(inp["mask"], wal, 0.0)}
    raise AssertionError(kind)


ORACLE_KINDS = {"pairwise", "singleton", "paired", "argmin", "subsequence", "alignment",
                "paired_subsequence"}
ORACLE_KINDS |= {"argmin_subsequence", "distance_profile", "subsequence_match",
                 "paired_subsequence_match"}
ORACLE_KINDS |= {"dtw_average", "kmeans", "knn", "kneighbors", "lb_keogh", "lb_kim",
                 "dtw_helpers", "dilated_profile", "mass_profile"}
# the reference's MASS takes its cross-correlation from its vendored pocketfft,
# the oracle from numpy's FFT: the profiles agree to the FFT's rounding
FFT_ATOL = 1e-9
CASES = [c for c in _golden.cases() if c["kind"] in ORACLE_KINDS]


def oracle_matches(shp, X, metric, params, kw, kind):
    """The oracle's per-window distances and keep flags, then the reference's
    host-side filters (distance/_distance.py:400-512, 732-1080)."""
    from wildboar_gb300.distance import _subsequence as SS

    threshold = kw.get("threshold")
    max_matches = kw.get("max_matches")
    exclude = kw.get("exclude")
    if threshold is None:
        threshold = math.inf
        if max_matches is None:
            max_matches = 10
    dist, keep = O.subsequence_matches(shp, X, threshold, metric=metric,
                                       metric_params=params)
    ind, dis = [], []
    for i, s in enumerate(shp):
        nwin = X.shape[2] - len(s) + 1
        sel = np.flatnonzero(keep[i, :nwin] > 0)
        ind.append(sel.astype(np.intp) if sel.size else None)
        dis.append(dist[i, sel] if sel.size else None)
    if kind == "subsequence_match" and exclude is not None:
        if isinstance(exclude, float):
            exclude = math.ceil(len(shp[0]) * exclude)
        if exclude:
            ind, dis = SS._exclude_trivial_matches(ind, dis, exclude)
    if max_matches:
        ind, dis = SS._filter_by_max_matches(ind, dis, max_matches)
    counts = np.array([0 if a is None else len(a) for a in ind], dtype=np.int64)
    fi = [np.asarray(a, dtype=np.int64) for a in ind if a is not None]
    fd = [np.asarray(a, dtype=float) for a in dis if a is not None]
    return {"counts": counts,
            "idx": np.concatenate(fi) if fi else np.zeros(0, np.int64),
            "dist": np.concatenate(fd) if fd else np.zeros(0)}


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference(case):
    got = run_oracle(case)
    for key, want in case["outputs"].items():
        g = np.asarray(got[key])
        want = np.asarray(want)
        assert g.shape == want.shape, (key, g.shape, want.shape)
        if want.dtype.kind in "iu":
            keep = want >= 0  # -1: the reference leaves the index unset
            np.testing.assert_array_equal(g[keep], want[keep])
        elif case["kind"] == "mass_profile":
            np.testing.assert_allclose(g, want, rtol=0, atol=FFT_ATOL)
        elif EXACT:
            np.testing.assert_array_equal(g, want)
        else:
            np.testing.assert_allclose(g, want, rtol=1e-12, atol=0)


def test_golden_covers_every_metric_and_kind():
    kinds = {c["kind"] for c in CASES}
    assert kinds >= {"pairwise", "singleton", "paired", "argmin", "subsequence",
                     "alignment"}
    metrics = {c["args"].get("metric") for c in CASES}
    assert metrics >= {"dtw", "wdtw", "ddtw", "wddtw", "adtw", "lcss", "wlcss", "edr",
                       "erp", "msm", "twe", "euclidean", "scaled_euclidean"}


def test_alignment_endpoint_equals_dtw():
    # sqrt of the last alignment cell is the dtw distance when the warp widths
    # agree (equal lengths): distance/dtw.py:246-290 vs _elastic.pyx:3167-3186
    rng = np.random.default_rng(5)
    x = np.cumsum(rng.standard_normal(64))
    y = np.cumsum(rng.standard_normal(64))
    for r in (0.1, 0.2, 1.0):
        al = O.dtw_alignment(x, y, r=r)
        d = O.distance_1d(x, y, metric="dtw", metric_params={"r": r})
        assert np.sqrt(al[-1, -1]) == d
