"""Generate the golden fixtures in this folder by running the reference itself.

Usage (in a container where the reference wildboar is built and importable)::

    WILDBOAR_REF_PATH=/path/to/built/wildboar/src python tests/golden/make_golden.py

The reference is imported from ``WILDBOAR_REF_PATH`` and called through its
public API (``wildboar.distance.pairwise_distance``, ``paired_distance``,
``argmin_distance``, ``pairwise_subsequence_distance``,
``paired_subsequence_distance``, ``argmin_subsequence_distance``,
``distance_profile``, ``subsequence_match``, ``paired_subsequence_match`` and
``wildboar.distance.dtw.dtw_alignment``).  Inputs are seeded Gaussian random
walks; every case stores its inputs, its call arguments and the reference's
outputs in ``golden.npz`` with a JSON index in ``golden.json``.  The fixtures
are read by tests/test_oracle_golden.py (oracle pinning) and by the GPU parity
tests.  Nothing at test time imports the reference.
"""

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _walk(rng, shape, scale=1.0):
    return np.cumsum(rng.standard_normal(shape) * scale, axis=-1)


ELASTIC = [
    ("dtw", {"r": 0.0}),
    ("dtw", {"r": 0.1}),
    ("dtw", {"r": 0.3}),
    ("dtw", {"r": 1.0}),
    ("wdtw", {"r": 1.0, "g": 0.05}),
    ("wdtw", {"r": 0.2, "g": 0.5}),
    ("ddtw", {"r": 1.0}),
    ("ddtw", {"r": 0.15}),
    ("wddtw", {"r": 1.0, "g": 0.05}),
    ("adtw", {"r": 1.0, "p": 1.0}),
    ("adtw", {"r": 0.3, "p": 0.1}),
    ("adtw", {"r": 1.0, "p": 10.0}),
    ("lcss", {"r": 1.0, "epsilon": 0.5}),
    ("lcss", {"r": 0.2, "epsilon": 1.0}),
    ("wlcss", {"r": 1.0, "epsilon": 0.8, "g": 0.05}),
    ("edr", {"r": 1.0}),
    ("edr", {"r": 0.25, "epsilon": 0.4}),
    ("erp", {"r": 1.0, "g": 0.0}),
    ("erp", {"r": 0.2, "g": 0.5}),
    ("msm", {"r": 1.0, "c": 1.0}),
    ("msm", {"r": 0.1, "c": 0.5}),
    ("msm", {"r": 0.3, "c": 0.1}),
    ("twe", {"r": 1.0, "penalty": 1.0, "stiffness": 0.001}),
    ("twe", {"r": 0.2, "penalty": 0.5, "stiffness": 0.1}),
    ("euclidean", {}),
]


def main():
    ref = os.environ.get("WILDBOAR_REF_PATH")
    if ref:
        sys.path.insert(0, ref)
    import wildboar
    from wildboar.distance import (
        argmin_distance,
        argmin_subsequence_distance,
        distance_profile,
        paired_distance,
        paired_subsequence_distance,
        paired_subsequence_match,
        pairwise_distance,
        pairwise_subsequence_distance,
        subsequence_match,
    )
    from wildboar.distance.dtw import dtw_alignment

    rng = np.random.default_rng(20261203)
    arrays = {}
    cases = []

    def add(name, kind, inputs, args, outputs):
        entry = {"name": name, "kind": kind, "args": args, "inputs": {}, "outputs": {}}
        for k, v in inputs.items():
            key = f"{name}/in/{k}"
            arrays[key] = np.asarray(v)
            entry["inputs"][k] = key
        for k, v in outputs.items():
            key = f"{name}/out/{k}"
            arrays[key] = np.asarray(v)
            entry["outputs"][k] = key
        cases.append(entry)

    # equal-length pairwise, 6 x 5, L = 40
    X = _walk(rng, (6, 40))
    Y = _walk(rng, (5, 40))
    # unequal lengths: Y shorter, and X shorter
    Xs = _walk(rng, (4, 33))
    Yl = _walk(rng, (5, 47))
    for ci, (metric, params) in enumerate(ELASTIC):
        tag = f"{metric}_{ci}"
        d = pairwise_distance(X, Y, metric=metric, metric_params=params)
        add(f"pairwise_eq_{tag}", "pairwise", {"x": X, "y": Y},
            {"metric": metric, "metric_params": params}, {"d": d})
        d = pairwise_distance(X, metric=metric, metric_params=params)
        add(f"singleton_{tag}", "singleton", {"x": X},
            {"metric": metric, "metric_params": params}, {"d": d})
        if metric != "euclidean":
            d = pairwise_distance(Xs, Yl, metric=metric, metric_params=params)
            add(f"pairwise_uneq_{tag}", "pairwise", {"x": Xs, "y": Yl},
                {"metric": metric, "metric_params": params}, {"d": d})
            # WeightedDerivativeDtwMetric.reset sizes its x-derivative buffer by
            # Y.shape[2] (distance/_elastic.pyx:3420), so a longer x overruns
            # the heap in the reference; that case is not recorded.
            if metric != "wddtw":
                d = pairwise_distance(Yl, Xs, metric=metric, metric_params=params)
                add(f"pairwise_uneq2_{tag}", "pairwise", {"x": Yl, "y": Xs},
                    {"metric": metric, "metric_params": params}, {"d": d})
        d = paired_distance(X[:5], Y, metric=metric, metric_params=params)
        add(f"paired_eq_{tag}", "paired", {"x": X[:5], "y": Y},
            {"metric": metric, "metric_params": params}, {"d": d})
        for k in (1, 3):
            Q = _walk(rng, (4, 30))
            C = _walk(rng, (9, 30))
            idx, dist = argmin_distance(Q, C, k=k, metric=metric, metric_params=params,
                                        return_distance=True)
            add(f"argmin_k{k}_{tag}", "argmin", {"x": Q, "y": C},
                {"metric": metric, "metric_params": params, "k": k},
                {"idx": idx, "dist": dist})
            if metric not in ("euclidean", "wddtw"):
                C2 = _walk(rng, (7, 26))
                idx, dist = argmin_distance(Q, C2, k=k, metric=metric,
                                            metric_params=params, return_distance=True)
                add(f"argmin_uneq_k{k}_{tag}", "argmin", {"x": Q, "y": C2},
                    {"metric": metric, "metric_params": params, "k": k},
                    {"idx": idx, "dist": dist})

    # lower bound pruning on dtw
    Q = _walk(rng, (5, 32))
    C = _walk(rng, (12, 32))
    full = pairwise_distance(Q, C, metric="dtw", metric_params={"r": 0.2})
    lb = full * rng.uniform(0.3, 1.0, size=full.shape)
    idx, dist = argmin_distance(Q, C, k=3, metric="dtw", metric_params={"r": 0.2},
                                lower_bound=lb, return_distance=True)
    add("argmin_lb_dtw", "argmin", {"x": Q, "y": C, "lower_bound": lb},
        {"metric": "dtw", "metric_params": {"r": 0.2}, "k": 3},
        {"idx": idx, "dist": dist})

    # multivariate, dim mean / full / int
    XM = _walk(rng, (4, 3, 25))
    YM = _walk(rng, (3, 3, 25))
    for dim in ("mean", "full", 1):
        for metric, params in (("dtw", {"r": 0.3}), ("msm", {"c": 1.0}),
                               ("edr", {}), ("euclidean", {})):
            d = pairwise_distance(XM, YM, dim=dim, metric=metric, metric_params=params)
            add(f"pairwise_dim_{dim}_{metric}", "pairwise", {"x": XM, "y": YM},
                {"metric": metric, "metric_params": params, "dim": dim}, {"d": d})
            d = paired_distance(XM[:3], YM, dim=dim, metric=metric, metric_params=params)
            add(f"paired_dim_{dim}_{metric}", "paired", {"x": XM[:3], "y": YM},
                {"metric": metric, "metric_params": params, "dim": dim}, {"d": d})

    # short series edge cases
    for L in (1, 2, 3):
        A = _walk(rng, (3, L))
        B = _walk(rng, (2, L))
        for metric, params in (("dtw", {}), ("ddtw", {}), ("msm", {}), ("twe", {}),
                               ("lcss", {}), ("edr", {}), ("erp", {})):
            d = pairwise_distance(A, B, metric=metric, metric_params=params)
            add(f"short_L{L}_{metric}", "pairwise", {"x": A, "y": B},
                {"metric": metric, "metric_params": params}, {"d": d})

    # subsequence (euclidean / scaled_euclidean)
    T = _walk(rng, (6, 120))
    shp = [_walk(rng, (int(n),)) for n in rng.integers(5, 40, size=7)]
    shp.append(T[2, 30:55].copy())  # exact match present
    shp.append(np.full(9, 3.0))     # constant shapelet (std 0)
    packed = np.concatenate(shp)
    lens = np.array([s.shape[0] for s in shp])
    for metric in ("euclidean", "scaled_euclidean"):
        d, i = pairwise_subsequence_distance(shp, T, metric=metric, return_index=True)
        add(f"subseq_{metric}", "subsequence",
            {"x": T, "shapelets": packed, "lengths": lens},
            {"metric": metric}, {"d": d, "idx": i})

    # dtw_alignment (differentiation oracle)
    a = _walk(rng, (30,))
    b = _walk(rng, (24,))
    for r in (0.2, 1.0):
        al = dtw_alignment(a, b, r=r)
        warp = max(math.floor(max(30, 24) * r), 1)
        # only band cells and their +-1 INF sentinels are defined
        mask = np.zeros(al.shape, dtype=bool)
        for i in range(30):
            js = max(0, i - max(0, 30 - 24) - warp + 1)
            je = min(24, i + max(0, 24 - 30) + warp)
            mask[i, js:je] = True
        if True:
            mask[0, : min(24, max(0, 24 - 30) + warp)] = True
        add(f"alignment_r{r}", "alignment", {"x": a, "y": b, "mask": mask},
            {"r": r}, {"a": np.where(mask, al, 0.0)})

    # elastic subsequence metrics (distance/_elastic.pyx:2206-3124)
    T2 = _walk(rng, (5, 80))
    shp2 = [_walk(rng, (int(n),)) for n in (2, 3, 9, 17, 33)]
    shp2.append(T2[1, 10:30].copy())
    packed2 = np.concatenate(shp2)
    lens2 = np.array([s.shape[0] for s in shp2])
    for metric, params in (("dtw", {"r": 0.2}), ("dtw", {}), ("wdtw", {"r": 0.5, "g": 0.1}),
                           ("ddtw", {"r": 0.3}), ("wddtw", {}), ("adtw", {"p": 0.3}),
                           ("lcss", {"r": 0.3, "epsilon": 0.7}), ("edr", {}),
                           ("edr", {"r": 0.4, "epsilon": 0.3}), ("erp", {"g": 0.2}),
                           ("msm", {"r": 0.2}), ("twe", {"r": 0.4})):
        d, i = pairwise_subsequence_distance(shp2, T2, metric=metric,
                                             metric_params=params, return_index=True)
        if metric in ("ddtw", "wddtw"):
            # series shorter than 3 return 0 without setting the index
            i = np.where(lens2[None, :] < 3, -1, i)
        tag = "_".join(f"{k}{v}" for k, v in params.items())
        add(f"subseq_{metric}_{tag}", "subsequence",
            {"x": T2, "shapelets": packed2, "lengths": lens2},
            {"metric": metric, "metric_params": params}, {"d": d, "idx": i})

    def tagof(params, scale=False):
        t = "_".join(f"{k}{v}" for k, v in params.items())
        return t + ("_scaled" if scale else "")

    # paired subsequence distance (distance/_distance.py:639-729)
    T3 = _walk(rng, (6, 70))
    shp3 = [_walk(rng, (int(n),)) for n in (4, 9, 17, 25, 3, 40)]
    shp3[2] = T3[2, 5:22].copy()
    packed3 = np.concatenate(shp3)
    lens3 = np.array([s.shape[0] for s in shp3])
    for metric, params in (("euclidean", {}), ("scaled_euclidean", {}), ("dtw", {"r": 0.3}),
                           ("msm", {}), ("lcss", {"epsilon": 0.8}), ("edr", {}),
                           ("twe", {"r": 0.5}), ("erp", {"g": 0.1})):
        d, i = paired_subsequence_distance(shp3, T3, metric=metric, metric_params=params,
                                           return_index=True)
        add(f"paired_subseq_{metric}_{tagof(params)}", "paired_subsequence",
            {"x": T3, "shapelets": packed3, "lengths": lens3},
            {"metric": metric, "metric_params": params}, {"d": d, "idx": i})

    # argmin subsequence distance (distance/_distance.py:1636-1761): heap order
    T4 = _walk(rng, (5, 60))
    S4 = _walk(rng, (5, 12))
    S4[3] = T4[3, 20:32]
    for metric, params, scale in (("euclidean", {}, False), ("euclidean", {}, True),
                                  ("dtw", {"r": 0.3}, False), ("dtw", {}, True),
                                  ("msm", {}, False), ("adtw", {"p": -0.2}, False),
                                  ("lcss", {"epsilon": 0.5}, False), ("erp", {}, False),
                                  ("twe", {}, True)):
        for k in (1, 4):
            idx, dist = argmin_subsequence_distance(S4, T4, k=k, metric=metric,
                                                    metric_params=params, scale=scale,
                                                    return_distance=True)
            add(f"argmin_subseq_{metric}_{tagof(params, scale)}_k{k}", "argmin_subsequence",
                {"x": T4, "y": S4},
                {"metric": metric, "metric_params": params, "scale": scale, "k": k},
                {"idx": idx, "dist": dist})

    # distance profile (dilation 1, no padding: distance/_distance.py:1477-1620)
    T5 = _walk(rng, (4, 50))
    q5 = _walk(rng, (10,))
    q5b = T5[2, 7:17].copy()
    for metric, params in (("euclidean", {}), ("scaled_euclidean", {}), ("dtw", {"r": 0.3}),
                           ("msm", {}), ("lcss", {"epsilon": 0.6}), ("twe", {}),
                           ("adtw", {"p": -0.3})):
        for qi, q in enumerate((q5, q5b)):
            dp = distance_profile(q, T5, metric=metric, metric_params=params)
            add(f"profile_{metric}_{tagof(params)}_q{qi}", "distance_profile",
                {"x": T5, "y": q}, {"metric": metric, "metric_params": params},
                {"d": dp})

    # subsequence matches (distance/_distance.py:732-1080), stored flat
    def flat(res):
        idx, dist = res
        counts = np.array([0 if a is None else len(a) for a in idx], dtype=np.int64)
        fi = [np.asarray(a, dtype=np.int64) for a in idx if a is not None]
        fd = [np.asarray(a, dtype=float) for a in dist if a is not None]
        return {"counts": counts,
                "idx": np.concatenate(fi) if fi else np.zeros(0, np.int64),
                "dist": np.concatenate(fd) if fd else np.zeros(0)}

    for metric, params, kw in (
            ("euclidean", {}, {"threshold": 4.0}),
            ("euclidean", {}, {}),
            ("euclidean", {}, {"threshold": 6.0, "max_matches": 3}),
            ("euclidean", {}, {"threshold": 6.0, "exclude": 2}),
            ("euclidean", {}, {"exclude": 0.5}),
            ("scaled_euclidean", {}, {"threshold": 2.0}),
            ("dtw", {"r": 0.3}, {"threshold": 3.0}),
            ("msm", {}, {"max_matches": 5}),
            ("adtw", {"p": -0.3}, {"threshold": 3.0})):
        res = subsequence_match(q5b, T5, metric=metric, metric_params=params,
                                return_distance=True, **kw)
        tag = tagof(params) + "_" + "_".join(f"{k}{v}" for k, v in kw.items())
        add(f"match_{metric}_{tag}", "subsequence_match", {"x": T5, "y": q5b},
            {"metric": metric, "metric_params": params, "kw": kw}, flat(res))
    shp6 = [T5[i, 3 + i:13 + i].copy() for i in range(4)]
    for metric, params, kw in (("euclidean", {}, {"threshold": 5.0}),
                               ("euclidean", {}, {"max_matches": 2}),
                               ("dtw", {}, {"threshold": 4.0})):
        res = paired_subsequence_match(shp6, T5, metric=metric, metric_params=params,
                                       return_distance=True, **kw)
        tag = tagof(params) + "_" + "_".join(f"{k}{v}" for k, v in kw.items())
        add(f"paired_match_{metric}_{tag}", "paired_subsequence_match",
            {"x": T5, "shapelets": np.concatenate(shp6),
             "lengths": np.array([10, 10, 10, 10])},
            {"metric": metric, "metric_params": params, "kw": kw}, flat(res))

    # dtw_average (method="mm"), KMeans and the neighbour estimators
    # (distance/dtw.py:429-690, distance/_neighbors.py:17-588)
    from wildboar.distance import KMeans, KNeighborsClassifier, NearestNeighbors
    from wildboar.distance.dtw import dtw_average

    XA = _walk(rng, (12, 30))
    XM = _walk(rng, (5, 200))
    XL = _walk(rng, (4, 540))
    sw = rng.uniform(0.5, 2.0, 12)
    for name, X_, kw in (
            ("dtw_r1", XA, {"r": 1.0, "init": XA[3]}),
            ("dtw_r02", XA, {"r": 0.2, "init": XA[0]}),
            ("wdtw", XA, {"r": 0.5, "g": 0.1, "init": XA[5]}),
            ("sample_weight", XA, {"r": 0.4, "init": XA[1], "sample_weight": sw}),
            ("short_init", XA, {"r": 0.5, "init": XA[2, :24]}),
            ("long_init", XA, {"r": 0.5, "init": np.concatenate([XA[4], XA[4, :6]])}),
            ("epochs3", XA, {"r": 0.3, "init": XA[7], "tol": 0.0, "max_epoch": 3}),
            ("random_init", XA, {"r": 0.6, "init": "random", "random_state": 7}),
            ("len200", XM, {"r": 0.3, "init": XM[1]}),
            ("len540", XL, {"r": 0.1, "init": XL[2]}),
            ("wdtw_len540", XL, {"r": 0.05, "g": 0.05, "init": XL[0]})):
        mean, cost = dtw_average(X_, return_cost=True, **kw)
        inputs = {"x": X_}
        args = {k: v for k, v in kw.items() if k not in ("init", "sample_weight")}
        if isinstance(kw["init"], str):
            args["init"] = kw["init"]
        else:
            inputs["init"] = kw["init"]
        if "sample_weight" in kw:
            inputs["sample_weight"] = kw["sample_weight"]
        add(f"dtw_average_{name}", "dtw_average", inputs, args, {"mean": mean, "cost": cost})

    XK = _walk(rng, (30, 25))
    XK[:10] += 6.0
    XK[10:20] -= 6.0
    U = _walk(rng, (6, 20))
    XD = np.concatenate([U, U, U + 0.01 * rng.standard_normal((6, 20))])
    XT = _walk(rng, (7, 25))
    for name, X_, kw in (
            ("euclidean", XK, {"n_clusters": 3, "random_state": 1}),
            ("dtw", XK, {"n_clusters": 3, "metric": "dtw", "r": 0.5, "random_state": 2}),
            ("wdtw", XK, {"n_clusters": 2, "metric": "dtw", "r": 1.0, "g": 0.2,
                          "random_state": 3}),
            ("n_init2", XK, {"n_clusters": 3, "metric": "dtw", "r": 0.3, "n_init": 2,
                             "max_iter": 5, "random_state": 4}),
            ("empty_euclidean", XD, {"n_clusters": 6, "random_state": 6, "max_iter": 20}),
            ("empty_dtw", XD, {"n_clusters": 6, "metric": "dtw", "r": 0.3,
                               "random_state": 6, "max_iter": 20}),
            ("empty_dtw13", XD, {"n_clusters": 6, "metric": "dtw", "r": 0.3,
                                 "random_state": 13, "max_iter": 20})):
        km = KMeans(**kw).fit(X_)
        outputs = {"labels": km.labels_, "centers": km.cluster_centers_,
                   "inertia": km.inertia_, "n_iter": km.n_iter_}
        inputs = {"x": X_}
        if X_.shape[1] == XT.shape[1]:
            inputs["xt"] = XT
            outputs["transform"] = km.transform(XT)
        add(f"kmeans_{name}", "kmeans", inputs, kw, outputs)

    ytr = rng.integers(0, 3, size=30)
    for name, metric, params, k in (("dtw", "dtw", {"r": 0.3}, 3),
                                    ("euclidean", "euclidean", None, 5),
                                    ("msm", "msm", {"c": 0.5}, 4)):
        clf = KNeighborsClassifier(n_neighbors=k, metric=metric, metric_params=params)
        clf.fit(XK, ytr)
        add(f"knn_{name}", "knn", {"x": XK, "y": ytr, "xt": XT},
            {"metric": metric, "metric_params": params, "n_neighbors": k},
            {"proba": clf.predict_proba(XT), "pred": clf.predict(XT)})
    for name, metric, params in (("erp", "erp", {"g": 0.1}), ("dtw", "dtw", {"r": 0.2})):
        nn = NearestNeighbors(n_neighbors=4, metric=metric, metric_params=params).fit(XK)
        dist_tr, ind_tr = nn.kneighbors()
        dist_te, ind_te = nn.kneighbors(XT)
        add(f"kneighbors_{name}", "kneighbors", {"x": XK, "xt": XT},
            {"metric": metric, "metric_params": params, "n_neighbors": 4},
            {"dist_train": dist_tr, "ind_train": ind_tr, "dist": dist_te, "ind": ind_te})

    # scaled_dtw: the UCR-suite scan (distance/_elastic.pyx:159-620, 1928-2204)
    XS = _walk(rng, (5, 120))
    XS[3, 40:60] = XS[3, 40]  # a constant stretch (ties in the envelope deques)
    shp_s = [XS[1, 10:30].copy(), rng.standard_normal(15), XS[0, 50:90] + 0.1,
             XS[2, 5:8].copy(), np.full(12, 2.5), XS[4, 0:120].copy()[::4].copy(),
             XS[3, 35:70].copy()]
    lens_s = np.array([len(s) for s in shp_s])
    for r in (0.0, 0.1, 0.3, 1.0):
        params = {"r": r}
        d, i = pairwise_subsequence_distance(shp_s, XS, metric="scaled_dtw",
                                             metric_params=params, return_index=True)
        add(f"subseq_scaled_dtw_r{r}", "subsequence",
            {"x": XS, "shapelets": np.concatenate(shp_s), "lengths": lens_s},
            {"metric": "scaled_dtw", "metric_params": params}, {"d": d, "idx": i})
    shp_p = [XS[k, 7 + 3 * k:27 + 3 * k].copy() + 0.05 * rng.standard_normal(20)
             for k in range(5)]
    for r in (0.2, 1.0):
        d, i = paired_subsequence_distance(shp_p, XS, metric="scaled_dtw",
                                           metric_params={"r": r}, return_index=True)
        add(f"paired_scaled_dtw_r{r}", "paired_subsequence",
            {"x": XS, "shapelets": np.concatenate(shp_p),
             "lengths": np.array([20] * 5)},
            {"metric": "scaled_dtw", "metric_params": {"r": r}}, {"d": d, "idx": i})
    qs = XS[2, 30:52].copy() + 0.05 * rng.standard_normal(22)
    for r in (0.1, 0.5):
        dp = distance_profile(qs, XS, metric="scaled_dtw", metric_params={"r": r})
        add(f"profile_scaled_dtw_r{r}", "distance_profile", {"x": XS, "y": qs},
            {"metric": "scaled_dtw", "metric_params": {"r": r}}, {"d": dp})
    for params, kw in (({"r": 0.1}, {"threshold": 2.0}), ({"r": 0.3}, {}),
                       ({"r": 0.2}, {"threshold": 3.0, "max_matches": 4}),
                       ({"r": 1.0}, {"threshold": 2.5, "exclude": 3})):
        res = subsequence_match(qs, XS, metric="scaled_dtw", metric_params=params,
                                return_distance=True, **kw)
        tag = f"r{params['r']}_" + "_".join(f"{k}{v}" for k, v in kw.items())
        add(f"match_scaled_dtw_{tag}", "subsequence_match", {"x": XS, "y": qs},
            {"metric": "scaled_dtw", "metric_params": params, "kw": kw}, flat(res))
    res = paired_subsequence_match(shp_p, XS, metric="scaled_dtw", metric_params={"r": 0.2},
                                   return_distance=True, threshold=2.0)
    add("paired_match_scaled_dtw_r0.2_threshold2.0", "paired_subsequence_match",
        {"x": XS, "shapelets": np.concatenate(shp_p), "lengths": np.array([20] * 5)},
        {"metric": "scaled_dtw", "metric_params": {"r": 0.2}, "kw": {"threshold": 2.0}},
        flat(res))

    # lower-bound producers (distance/lb.py:198-432)
    from wildboar.distance.lb import DtwKeoghLowerBound, DtwKimLowerBound

    XB = _walk(rng, (9, 60))
    XB[2, 10:30] = XB[2, 10]  # constant stretch: ties in the envelope deques
    XB[5, :] = np.repeat(_walk(rng, 12), 5)
    QB = _walk(rng, (5, 60))
    QB[1, 30:50] = 0.25
    for r, kind in ((0.1, "both"), (0.0, "both"), (1.0, "both"), (0.3, "left"),
                    (0.05, "right")):
        lbk = DtwKeoghLowerBound(r=r, kind=kind).fit(XB)
        add(f"lb_keogh_r{r}_{kind}", "lb_keogh", {"x": XB, "q": QB}, {"r": r, "kind": kind},
            {"out": lbk.transform(QB), "lower": lbk.lower_, "upper": lbk.upper_})
    for L in (60, 2, 1):
        add(f"lb_kim_L{L}", "lb_kim", {"x": XB[:, :L], "q": QB[:, :L]}, {},
            {"out": DtwKimLowerBound().fit(XB[:, :L]).transform(QB[:, :L])})

    # edge cases of the rows above: ties everywhere, minimal bands, single windows
    XE = _walk(rng, (4, 16))
    XT2 = np.stack([XE[0], XE[0], XE[0] + 0.0, XE[1]])
    for name, X_, kw in (("ties_r0", XT2, {"r": 0.0, "init": XE[0]}),
                         ("ties_r1", XT2, {"r": 1.0, "init": XE[2]}),
                         ("two_rows", XE[:2], {"r": 0.5, "init": XE[3]}),
                         ("const_init", XE, {"r": 0.3, "init": np.zeros(16)})):
        mean, cost = dtw_average(X_, return_cost=True, **kw)
        add(f"dtw_average_edge_{name}", "dtw_average", {"x": X_, "init": kw["init"]},
            {"r": kw["r"]}, {"mean": mean, "cost": cost})
    km = KMeans(n_clusters=4, metric="dtw", r=0.2, random_state=5).fit(XE)
    add("kmeans_edge_k_eq_n", "kmeans", {"x": XE},
        {"n_clusters": 4, "metric": "dtw", "r": 0.2, "random_state": 5},
        {"labels": km.labels_, "centers": km.cluster_centers_, "inertia": km.inertia_,
         "n_iter": km.n_iter_})
    shp_e = [XS[0].copy(), XS[1, 7:10].copy(), XS[2, 0:119].copy()]
    for r in (1.0, 0.2):
        d, i = pairwise_subsequence_distance(shp_e, XS, metric="scaled_dtw",
                                             metric_params={"r": r}, return_index=True)
        add(f"subseq_scaled_dtw_edge_r{r}", "subsequence",
            {"x": XS, "shapelets": np.concatenate(shp_e),
             "lengths": np.array([len(s) for s in shp_e])},
            {"metric": "scaled_dtw", "metric_params": {"r": r}}, {"d": d, "idx": i})
    for L in (1, 2, 3):
        lbk = DtwKeoghLowerBound(r=0.5).fit(XB[:, :L])
        add(f"lb_keogh_L{L}", "lb_keogh", {"x": XB[:, :L], "q": QB[:, :L]},
            {"r": 0.5, "kind": "both"},
            {"out": lbk.transform(QB[:, :L]), "lower": lbk.lower_, "upper": lbk.upper_})

    # dtw_average(method="ssg") (distance/dtw.py:597-658)
    XG = _walk(rng, (10, 24))
    swg = rng.uniform(0.5, 1.5, 10)
    for name, kw in (("dtw", {"r": 0.5, "random_state": 3, "max_epoch": 8}),
                     ("wdtw", {"r": 1.0, "g": 0.1, "random_state": 4, "max_epoch": 6}),
                     ("sample_weight", {"r": 0.3, "random_state": 5, "max_epoch": 6,
                                        "sample_weight": swg}),
                     ("stable", {"r": 0.2, "random_state": 6, "max_epoch": 40,
                                 "max_stable": 1, "learning_rate": 0.05, "decay": 0.8})):
        mean, cost = dtw_average(XG, method="ssg", return_cost=True, **kw)
        inputs = {"x": XG}
        if "sample_weight" in kw:
            inputs["sample_weight"] = kw["sample_weight"]
        args = {k: v for k, v in kw.items() if k != "sample_weight"}
        args["method"] = "ssg"
        args["init"] = "random"
        add(f"dtw_average_ssg_{name}", "dtw_average", inputs, args,
            {"mean": mean, "cost": cost})

    # single-pair helpers of distance/dtw.py:43-426
    from wildboar.distance.dtw import (ddtw_distance, dtw_distance, dtw_envelop,
                                       dtw_lb_keogh, dtw_mapping, wddtw_distance,
                                       wdtw_alignment, wdtw_distance)

    ha = _walk(rng, 35)
    hb = _walk(rng, 35)
    hc = _walk(rng, 28)
    def band_mask(n, m, r):
        warp = max(math.floor(max(n, m) * r), 1)
        mask = np.zeros((n, m), dtype=bool)
        for i in range(n):
            mask[i, max(0, i - max(0, n - m) - warp + 1):min(m, i + max(0, m - n) + warp)] = True
        return mask

    for r in (0.1, 1.0):
        lo, up = dtw_envelop(ha, r=r)
        d1, cb1 = dtw_lb_keogh(hb, ha, r=r)
        d2, cb2 = dtw_lb_keogh(hb, lower=lo, upper=up)
        wmask = band_mask(35, 28, r)
        wal = wdtw_alignment(ha, hc, r=r, g=0.3)
        add(f"dtw_helpers_r{r}", "dtw_helpers", {"a": ha, "b": hb, "c": hc, "mask": wmask},
            {"r": r},
            {"dtw": dtw_distance(ha, hb, r=r), "ddtw": ddtw_distance(ha, hc, r=r),
             "wdtw": wdtw_distance(hc, hb, r=r, g=0.1),
             "wddtw": wddtw_distance(ha, hb, r=r, g=0.2), "lower": lo, "upper": up,
             "lb": d1, "cb": cb1, "lb2": d2, "cb2": cb2,
             "mapping": dtw_mapping(ha, hc, r=r),
             "walign": np.where(wmask, wal, 0.0)})

    # argmin over long candidate lists: the reference's abandoning and heap over
    # hundreds of candidates, with near matches late in the scan
    LONG = [("dtw", {"r": 0.1}, 64), ("dtw", {"r": 1.0}, 170), ("wdtw", {"g": 0.05}, 64),
            ("adtw", {"p": 0.5, "r": 0.2}, 64), ("edr", {}, 64), ("erp", {"g": 0.1}, 64),
            ("msm", {"c": 0.5}, 64), ("twe", {"penalty": 0.5, "stiffness": 0.01}, 64),
            ("lcss", {"epsilon": 0.5}, 64), ("ddtw", {"r": 0.3}, 64)]
    for ci, (metric, params, L) in enumerate(LONG):
        Q = _walk(rng, (12, L))
        C = _walk(rng, (400, L))
        for t, q in enumerate((2, 5, 9)):
            C[300 + 30 * t] = Q[q] + 0.02 * rng.standard_normal(L)
        for k in (1, 5):
            idx, dist = argmin_distance(Q, C, k=k, metric=metric, metric_params=params,
                                        return_distance=True)
            add(f"argmin_long_k{k}_{metric}_{ci}", "argmin", {"x": Q, "y": C},
                {"metric": metric, "metric_params": params, "k": k},
                {"idx": idx, "dist": dist})

    # distance profile with dilation / padding (distance/_distance.py:1560-1619,
    # _cdistance.pyx:804-933): pairwise metrics on the gathered windows,
    # "mass" / "scaled_*" on z-normalised windows, partial windows rescaled
    TD = _walk(rng, (3, 70))
    QD = _walk(rng, (3, 9))
    for metric, params in (("euclidean", {}), ("mass", {}), ("scaled_euclidean", {}),
                           ("dtw", {"r": 0.3}), ("scaled_dtw", {"r": 0.5}),
                           ("wdtw", {"g": 0.1}), ("ddtw", {}), ("wddtw", {"g": 0.2}),
                           ("lcss", {"epsilon": 0.7}),
                           ("edr", {}), ("erp", {"g": 0.2}), ("msm", {}), ("twe", {}),
                           ("adtw", {"p": 0.5})):
        for dil, pad in ((1, 3), (2, 0), (2, "same"), (3, 6)):
            dp = distance_profile(QD, TD, metric=metric, metric_params=params,
                                  dilation=dil, padding=pad)
            add(f"dprofile_{metric}_{tagof(params)}_d{dil}_p{pad}", "dilated_profile",
                {"x": TD, "y": QD},
                {"metric": metric, "metric_params": params, "dilation": dil,
                 "padding": pad}, {"d": dp})
    # scale=True with a plain metric on 3-d input (dim 0: for dim > 0 the
    # reference reads the one-dim subsequence array at S[i, dim], past its end),
    # and one subsequence broadcast against one series
    TD3 = _walk(rng, (2, 3, 40))
    QD3 = _walk(rng, (2, 7))
    dp = distance_profile(QD3, TD3, metric="dtw", metric_params={"r": 0.2}, dilation=2,
                          padding=4, dim=0, scale=True)
    add("dprofile_dtw_scale_3d", "dilated_profile", {"x": TD3, "y": QD3},
        {"metric": "dtw", "metric_params": {"r": 0.2}, "dilation": 2, "padding": 4,
         "dim": 0, "scale": True}, {"d": dp})
    dp = distance_profile(QD[0], TD[1], metric="euclidean", dilation=4, padding="same")
    add("dprofile_euclidean_1d_same", "dilated_profile", {"x": TD[1], "y": QD[0]},
        {"metric": "euclidean", "metric_params": {}, "dilation": 4, "padding": "same"},
        {"d": dp})
    # the default "mass" profile (dilation 1, no padding): z-normalised
    # euclidean by an FFT cross-correlation; a constant stretch of series 1 and
    # a constant subsequence reach the zero-variance branches
    TM = _walk(rng, (4, 120))
    TM[1, 30:75] = 3.0
    for L in (5, 16, 40):
        QM = _walk(rng, (4, L))
        QM[2] = 1.0
        dp = distance_profile(QM, TM)
        add(f"mass_L{L}", "mass_profile", {"x": TM, "y": QM}, {}, {"d": dp})

    # scaled_euclidean matching stops a window's sum at the first term where it
    # is >= t^2 and keeps the window if that partial sum is <= t^2
    # (distance/_metric.pyx:625-651, 798-860): with t = 0 every window matches
    # with distance 0; one series holds an exact copy of the subsequence
    TZ = _walk(rng, (3, 40))
    qz = TZ[1, 5:14].copy()
    for t in (0.0, 0.5):
        res = subsequence_match(qz, TZ, threshold=t, metric="scaled_euclidean",
                                return_distance=True)
        add(f"match_scaled_euclidean_t{t}", "subsequence_match", {"x": TZ, "y": qz},
            {"metric": "scaled_euclidean", "metric_params": {},
             "kw": {"threshold": t}}, flat(res))
    shpz = [TZ[i, 2 + i:10 + i].copy() for i in range(3)]
    res = paired_subsequence_match(shpz, TZ, threshold=0.0, metric="scaled_euclidean",
                                   return_distance=True)

    add("paired_match_scaled_euclidean_t0", "paired_subsequence_match",
        {"x": TZ, "shapelets": np.concatenate(shpz), "lengths": np.array([8, 8, 8])},
        {"metric": "scaled_euclidean", "metric_params": {}, "kw": {"threshold": 0.0}},
        flat(res))

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"reference_version": getattr(wildboar, "__version__", "?"),
                   "numpy": np.__version__, "cases": cases}, f, indent=1)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
