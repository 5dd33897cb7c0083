"""Benchmark of the distance hot path (one JSON line on rank 0).

Default workload: the plain FP64 drop-in ``pairwise_distance`` with
metric="dtw", r=0.1 on 2000 x 2000 univariate float64 Gaussian random walks of
length 512 (1.966e11 band cells per step).  A step is one call over the whole
matrix.  ``value`` is device-timed GCUPS with inputs resident in HBM; ``e2e``
is the same metric through the public API with pinned host numpy inputs, the
host-to-device copies and the device-to-host copy of the result inside the
timed region.

``--impl reference`` times the reference algorithm on the host cores instead
(the C restatement under oracle/, all threads), on a bounded row sample of the
same workload.

Multi-GPU (torchrun): every rank computes its own 2000-row block of X against
the shared Y (weak scaling, no collective on the data path).
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from wildboar_gb300.distance._band import band_cells  # noqa: E402

WORKLOAD = {
    "name": "pairwise_distance dtw r=0.1, 2000x2000 random walks, L=512, float64",
    "nx": 2000,
    "ny": 2000,
    "L": 512,
    "metric": "dtw",
    "params": {"r": 0.1},
}
FP64_OPS_PER_CELL = 3  # v = x - y, v * v, min + v*v (mins run on the integer pipe)
FP64_OPS_PER_SM_CLK = 2  # GB300 FP64 pipe (ncu sm__inst_executed_pipe_fp64 / pipe activity)
# DRAM bytes (read + write) of one launch of the headline kernel at 2000 x 2000,
# L = 512, from one earlier ncu capture of `python bench.py --no-cpu --no-forms
# --steps 2 --warmup 3` (dram__bytes_read.sum 17.12 MB + dram__bytes_write.sum
# 10.75 KB); it is not measured in the timed run.  The 32 MB output is still in
# L2 when the kernel ends.
HEADLINE_DRAM_BYTES = 17.12e6 + 10.75e3


def _rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def make_data(rank, nx, ny, L, seed=0):
    rng = np.random.default_rng(seed + 1000 * rank)
    X = np.cumsum(rng.standard_normal((nx, L)), axis=1)
    rngy = np.random.default_rng(seed + 7)
    Y = np.cumsum(rngy.standard_normal((ny, L)), axis=1)
    return X, Y


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread is not None:
                self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference(X, Y, wl, budget_s=15.0, n_threads=None, return_rows=False):
    """The reference algorithm (oracle restatement) on the host cores, bounded."""
    from oracle import oracle as O

    n_threads = n_threads or os.cpu_count() or 1
    cells_pair = band_cells(wl["L"], wl["L"], wl["params"]["r"])
    # calibrate on a small slice, then size the sample to the time budget
    rows = max(1, min(X.shape[0], n_threads))
    t0 = time.perf_counter()
    O.pairwise(X[:rows], Y, metric=wl["metric"], metric_params=wl["params"],
               n_threads=n_threads)
    dt = time.perf_counter() - t0
    per_row = dt / rows
    rows = int(max(rows, min(X.shape[0], budget_s / max(per_row, 1e-9))))
    rows = max(n_threads, (rows // n_threads) * n_threads)
    rows = min(rows, X.shape[0])
    t0 = time.perf_counter()
    ref = O.pairwise(X[:rows], Y, metric=wl["metric"], metric_params=wl["params"],
                     n_threads=n_threads)
    dt = time.perf_counter() - t0
    cells = rows * Y.shape[0] * cells_pair
    res = {"value": cells / dt / 1e9, "unit": "GCUPS", "cores": n_threads, "kind": "port",
           "sample": f"{rows} x {Y.shape[0]} pairs of the workload "
                     f"({cells:.3e} cells, {dt:.2f} s), oracle/wb_oracle.c with "
                     f"{n_threads} threads"}
    return (res, ref) if return_rows else res


def run_reference(args):
    rank, world = _rank()
    if rank != 0:
        return
    wl = WORKLOAD
    X, Y = make_data(0, wl["nx"], wl["ny"], wl["L"])
    step_budget = max(2.0, 30.0 / max(1, args.steps))
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        r = cpu_reference(X, Y, wl, budget_s=1.0 if i < args.warmup else step_budget)
        if i >= args.warmup:
            vals.append(r["value"])
        base = r
    v = statistics.median(vals)
    cells_pair = band_cells(wl["L"], wl["L"], wl["params"]["r"])
    total_cells = wl["nx"] * wl["ny"] * cells_pair
    line = {
        "impl": "reference",
        "metric": "DTW cell-updates/s (GCUPS), plain FP64 drop-in",
        "value": v,
        "unit": "GCUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_cells / (v * 1e9) * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Gaussian random walks)",
        "config": {"workload": wl["name"], "n_pairs": wl["nx"] * wl["ny"],
                   "cells_per_step": total_cells,
                   "sample": "each step times a bounded row sample; ms_per_step is "
                             "extrapolated to the full matrix"},
        "cpu_baseline": dict(base, value=v),
        "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _timed(fn, steps, flush=None):
    """Mean device time (ms) of `steps` calls, CUDA events on the current stream."""
    import torch

    ms = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return sum(ms) / len(ms)


def bench_batched(args, dev, flush):
    """Ragged batch: 65,536 pairs x 3 dims, lengths U{32..2048} NaN-padded to
    2048, float32, r=0.1, one persistent launch replayed from a CUDA graph."""
    import torch

    from oracle import oracle as O
    from wildboar_gb300.distance.batched import BatchedDTW

    g = torch.Generator(device=dev)
    g.manual_seed(4)
    N, d, L, r = args.c4_pairs, 3, 2048, 0.1
    x = torch.randn((N, d, L), device=dev, generator=g).cumsum(-1)
    y = torch.randn((N, d, L), device=dev, generator=g).cumsum(-1)
    lx = torch.randint(32, L + 1, (N, d), device=dev, generator=g)
    ly = torch.randint(32, L + 1, (N, d), device=dev, generator=g)
    ar = torch.arange(L, device=dev)
    x.masked_fill_(ar >= lx.unsqueeze(-1), float("nan"))
    y.masked_fill_(ar >= ly.unsqueeze(-1), float("nan"))
    t0 = time.perf_counter()
    tile = tuple(int(v) for v in args.c4_tile.split(",")) if args.c4_tile else None
    runner = BatchedDTW(x, y, r=r, tune=tile is None, graph=True, tile=tile)
    plan_s = time.perf_counter() - t0
    cells = runner.cells
    for _ in range(args.warmup):
        runner.run()
    torch.cuda.synchronize()
    ms = _timed(runner.run, args.steps, flush)
    out = runner.run().cpu().numpy()
    # error against the FP64 oracle on a sample of pairs (same float32 inputs)
    rng = np.random.default_rng(0)
    idx = rng.choice(N, size=min(N, args.err_sample), replace=False)
    xs, ys = x[idx].cpu().numpy(), y[idx].cpu().numpy()
    lxs, lys = lx[idx].cpu().numpy(), ly[idx].cpu().numpy()
    err = 0.0
    cpu_cells = 0
    t0 = time.perf_counter()
    for t, i in enumerate(idx):
        acc = 0.0
        for k in range(d):
            acc += O.distance_1d(xs[t, k, : lxs[t, k]].astype(np.float64),
                                 ys[t, k, : lys[t, k]].astype(np.float64), metric="dtw",
                                 metric_params={"r": r})
            cpu_cells += band_cells(int(lxs[t, k]), int(lys[t, k]), r)
        err = max(err, abs(out[i] - acc / d) / (acc / d))
    cpu_s = time.perf_counter() - t0
    return {
        "gcups": cells / (ms * 1e-3) / 1e9,
        "ms_per_step": ms,
        "cells_per_step": cells,
        "config": f"{N} pairs x {d} dims, lengths U{{32..2048}} NaN-padded to 2048, "
                  f"float32, r={r}, CUDA graph replay (lengths + kernel + dim mean)",
        "tile": {"strip": runner.plan["strip"], "block": runner.plan["block"]},
        "plan_and_autotune_s": plan_s,
        "max_rel_err_vs_fp64": err,
        "err_sample_pairs": int(len(idx)),
        "cpu_oracle": {"gcups": cpu_cells / cpu_s / 1e9, "cores": 1, "kind": "port",
                       "sample": f"the {len(idx)} error-sample pairs x {d} dims, FP64, "
                                 "one call per pair and dim"},
    }


def bench_fwd_bwd(args, dev, flush):
    """Differentiable dtw: 4,096 float32 series of length 256 (32 sine / random
    walk prototypes + N(0, 0.1)) against 32 learnable centroids, r=0.2;
    a step is forward + backward of the soft-assignment barycenter loss and an
    Adam update."""
    import torch

    from oracle import oracle as O
    from wildboar_gb300.distance import autograd as AG
    from wildboar_gb300.distance._band import band_cells

    rng = np.random.default_rng(5)
    L, K, N, r = 256, 32, args.c5_series, 0.2
    t = np.linspace(0, 1, L)
    protos = []
    for k in range(K):
        if k % 2 == 0:
            protos.append(np.sin(2 * np.pi * (1 + k / 4) * t + rng.uniform(0, 6.28)) * 3)
        else:
            protos.append(np.cumsum(rng.standard_normal(L)) * 0.3)
    protos = np.asarray(protos, dtype=np.float32)
    labels = rng.integers(0, K, size=N)
    X = protos[labels] + 0.1 * rng.standard_normal((N, L)).astype(np.float32)
    x = torch.as_tensor(X, device=dev)
    c = torch.as_tensor(X[rng.choice(N, K, replace=False)], device=dev).clone()
    c.requires_grad_(True)
    opt = torch.optim.Adam([c], lr=0.05)
    cells_fwd = N * K * band_cells(L, L, r)

    def step():
        opt.zero_grad(set_to_none=True)
        D = AG.dtw_matrix(x, c, r)
        loss = AG.soft_assignment_loss(D, 1.0)
        loss.backward()
        opt.step()
        return loss

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ms = _timed(step, args.steps, flush)
    ms_fwd = _timed(lambda: AG.dtw_matrix(x, c.detach(), r), args.steps, flush)
    # the configured 100 Adam barycenter steps
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = []
    for _ in range(args.c5_adam_steps):
        losses.append(step())
    torch.cuda.synchronize()
    adam_s = time.perf_counter() - t0
    # errors against FP64 of the plain forward and of the forward that keeps
    # the directions (the one inside the step)
    D = AG.dtw_matrix(x[:16], c.detach(), r).detach().cpu().numpy()
    Dk = AG.dtw_matrix(x[:16], c, r).detach().cpu().numpy()
    Cn = c.detach().cpu().numpy().astype(np.float64)
    err = err_k = 0.0
    for i in range(16):
        for k in range(K):
            want = O.distance_1d(X[i].astype(np.float64), Cn[k], metric="dtw",
                                 metric_params={"r": r})
            err = max(err, abs(D[i, k] - want) / want)
            err_k = max(err_k, abs(Dk[i, k] - want) / want)
    return {
        "gcups": 2 * cells_fwd / (ms * 1e-3) / 1e9,
        "ms_per_step": ms,
        "forward_gcups": cells_fwd / (ms_fwd * 1e-3) / 1e9,
        "cells_per_step": 2 * cells_fwd,
        "config": f"{N} x {K} centroids, L={L}, r={r}, float32; step = forward + "
                  "backward (path traceback, all pairs) + Adam",
        "backward": ("directions kept by the forward, walk only" if AG.keeps_directions(x, c, r)
                     else "checkpointed recompute + walk"),
        "adam_steps": args.c5_adam_steps,
        "adam_total_s": adam_s,
        "loss_first_last": [float(losses[0].detach()), float(losses[-1].detach())],
        "max_rel_err_vs_fp64": err,
        "max_rel_err_vs_fp64_step_forward": err_k,
    }


def c3_data(n_series, n_shapelets, T=1024, seed=6):
    """Config 3 inputs: random-walk series and z-normalised random-walk
    fragments of lengths U{16..128}."""
    rng = np.random.default_rng(seed)
    X = np.cumsum(rng.standard_normal((n_series, T)), axis=1)
    lens = rng.integers(16, 129, size=n_shapelets)
    shp = []
    for L in lens:
        f = np.cumsum(rng.standard_normal(L))
        sd = f.std()
        shp.append((f - f.mean()) / (sd if sd > 0 else 1.0))
    return X, shp


def bench_subsequence(args, dev, flush):
    """pairwise_subsequence_distance of 10,000 shapelets against 1,000 series
    of length 1,024 (float64, return_index), euclidean and scaled_euclidean."""
    import torch

    from oracle import oracle as O
    from wildboar_gb300.distance import pairwise_subsequence_distance

    X, shp = c3_data(args.c3_series, args.c3_shapelets)
    T = X.shape[1]
    elems = int(sum((T - len(s) + 1) * len(s) for s in shp)) * X.shape[0]
    Xd = torch.as_tensor(X, device=dev)
    res = {}
    for metric in ("euclidean", "scaled_euclidean"):
        def call():
            return pairwise_subsequence_distance(shp, Xd, metric=metric, return_index=True)
        call()
        torch.cuda.synchronize()
        ms = _timed(call, max(1, min(args.steps, 2)), flush)
        d, i = call()
        d = d.cpu().numpy()
        i = i.cpu().numpy()
        t0 = time.perf_counter()
        od, oi = O.subsequence(shp, X[:2], metric=metric, n_threads=os.cpu_count() or 1)
        cpu_s = time.perf_counter() - t0
        res[metric] = {
            "ms": ms,
            "g_window_elements_per_s": elems / (ms * 1e-3) / 1e9,
            "argmin_exact_on_sample": bool(np.array_equal(i[:2], oi)),
            "max_rel_err_on_sample": float(np.max(np.abs(d[:2] - od) / np.maximum(od, 1e-300))),
            "cpu_oracle": {"g_window_elements_per_s": 2 * elems / X.shape[0] / cpu_s / 1e9,
                           "cores": os.cpu_count() or 1, "kind": "port",
                           "sample": f"all {len(shp)} shapelets x 2 series"},
        }
    return {"config": f"{args.c3_shapelets} shapelets (L~U{{16..128}}, z-normalised "
                      f"random-walk fragments) x {args.c3_series} series, T={T}, float64",
            "algorithmic_window_elements": elems, **res}


def bench_subsequence_elastic(args, dev, flush):
    """pairwise_subsequence_distance with elastic metrics (dtw r=0.1, dtw r=1,
    lcss): 1,000 of the C3 shapelets against 100 series of length 1,024.
    GCUPS over the algorithmic band cells of every window (abandoned cells
    included in the count).  CPU: the oracle (the reference's sequential scan
    with its early abandoning) on all host threads, one series."""
    import torch

    from oracle import oracle as O
    from wildboar_gb300.distance import pairwise_subsequence_distance

    X, shp = c3_data(100, 1000)
    T = X.shape[1]
    Xd = torch.as_tensor(X, device=dev)
    res = {}
    for name, metric, params in (("dtw_r0.1", "dtw", {"r": 0.1}), ("dtw_r1", "dtw", {"r": 1.0}),
                                 ("lcss", "lcss", {"epsilon": 0.5})):
        r = params.get("r", 1.0)
        cells = X.shape[0] * sum((T - len(s) + 1) * band_cells(len(s), len(s), r) for s in shp)

        def call():
            return pairwise_subsequence_distance(shp, Xd, metric=metric, metric_params=params,
                                                 return_index=True)
        call()
        torch.cuda.synchronize()
        ms = _timed(call, 1, flush)
        d, i = call()
        n_threads = os.cpu_count() or 1
        ns = 200  # CPU sample: the first 200 shapelets against the first series
        cells_s = sum((T - len(s) + 1) * band_cells(len(s), len(s), r) for s in shp[:ns])
        t0 = time.perf_counter()
        od, oi = O.subsequence(shp[:ns], X[:1], metric=metric, metric_params=params,
                               n_threads=n_threads)
        cpu_s = time.perf_counter() - t0
        res[name] = {
            "ms": ms,
            "gcups_algorithmic": cells / (ms * 1e-3) / 1e9,
            "argmin_exact_on_sample": bool(np.array_equal(i[:1, :ns].cpu().numpy(), oi)),
            "max_rel_err_on_sample": float(np.max(np.abs(d[:1, :ns].cpu().numpy() - od) /
                                                  np.maximum(np.abs(od), 1e-300))),
            "cpu_oracle": {"gcups_algorithmic": cells_s / cpu_s / 1e9,
                           "cores": n_threads, "kind": "port",
                           "sample": f"{ns} shapelets x 1 series"},
        }
    return {"config": f"{len(shp)} shapelets (L~U{{16..128}}, z-normalised random-walk "
                      f"fragments) x {X.shape[0]} series, T={T}, float64", **res}


def bench_subsequence_search(args, dev, flush):
    """The subsequence search functions on 2,000 random-walk series of length
    1,024: argmin_subsequence_distance (one length-64 query per series, taken
    from it plus N(0, 1) noise, k=5), distance_profile and subsequence_match
    (one length-64 pattern against every series).  End-to-end host timings of
    the public calls (they return host arrays).  CPU: the oracle on all host
    threads on a row sample."""
    from oracle import oracle as O
    from wildboar_gb300.distance import (argmin_subsequence_distance, distance_profile,
                                         subsequence_match)

    rng = np.random.default_rng(3)
    n, T, L = 2000, 1024, 64
    X = np.cumsum(rng.standard_normal((n, T)), axis=1)
    starts = 100 + (np.arange(n) % 500)
    Yq = np.stack([X[i, starts[i]:starts[i] + L] + rng.standard_normal(L) for i in range(n)])
    pat = X[7, 300:300 + L].copy()
    n_threads = os.cpu_count() or 1
    rows = 32

    def host_ms(fn, reps=3):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            ts.append((time.perf_counter() - t0) * 1e3)
        return statistics.median(ts), out

    res = {"config": f"{n} series, T={T}, queries / pattern of length {L}, float64"}
    for metric, params in (("dtw", {"r": 0.1}), ("scaled_euclidean", {})):
        ms, (idx, dist) = host_ms(lambda: argmin_subsequence_distance(
            Yq, X, k=5, metric=metric, metric_params=params, return_distance=True))
        t0 = time.perf_counter()
        oi, od = O.argmin_subsequence(Yq[:rows], X[:rows], k=5, metric=metric,
                                      metric_params=params, n_threads=n_threads)
        cpu_ms = (time.perf_counter() - t0) * 1e3 * n / rows
        res[f"argmin_subsequence_{metric}"] = {
            "ms": ms, "exact_on_sample": bool(np.array_equal(idx[:rows], oi)),
            "cpu_oracle_ms_extrapolated": cpu_ms,
            "cpu_oracle": {"cores": n_threads, "kind": "port",
                           "sample": f"{rows} pairs, scaled to {n}"}}
    for metric, params in (("euclidean", {}), ("dtw", {"r": 0.1})):
        ms, prof = host_ms(lambda: distance_profile(pat, X, metric=metric,
                                                    metric_params=params))
        t0 = time.perf_counter()
        od, _ = O.subsequence_matches([pat] * rows, X[:rows], np.inf, metric=metric,
                                      metric_params=params, transient=True,
                                      n_threads=n_threads)
        cpu_ms = (time.perf_counter() - t0) * 1e3 * n / rows
        prof = np.asarray(prof)
        res[f"distance_profile_{metric}"] = {
            "ms": ms, "windows": int(prof.size),
            "max_rel_err_on_sample": float(np.nanmax(np.abs(prof[:rows] - od[:, :prof.shape[1]]) /
                                                     np.maximum(np.abs(od[:, :prof.shape[1]]),
                                                                1e-300))),
            "cpu_oracle_ms_extrapolated": cpu_ms}
    thr = 12.0
    ms, (midx, mdist) = host_ms(lambda: subsequence_match(
        pat, X, thr, metric="dtw", metric_params={"r": 0.1}, return_distance=True))
    res["subsequence_match_dtw"] = {
        "ms": ms, "threshold": thr,
        "matches": int(sum(0 if m is None else len(m) for m in midx))}
    return res


def c6_data(n_series=4096, L=256, K=32, seed=5):
    """KMeans / barycenter inputs: float64 series from 32 sine / random-walk
    prototypes + N(0, 0.1), the prototype labels."""
    rng = np.random.default_rng(seed)
    t = np.linspace(0, 1, L)
    protos = []
    for k in range(K):
        if k % 2 == 0:
            protos.append(np.sin(2 * np.pi * (1 + k / 4) * t + rng.uniform(0, 6.28)) * 3)
        else:
            protos.append(np.cumsum(rng.standard_normal(L)) * 0.3)
    protos = np.asarray(protos)
    labels = rng.integers(0, K, size=n_series)
    return protos[labels] + 0.1 * rng.standard_normal((n_series, L)), labels


def bench_barycenter(args, dev, flush):
    """dtw_average (method="mm") epochs and KMeans(metric="dtw") on 4,096 float64
    series of length 256 in 32 groups, r=0.2: one step is one MM epoch of all
    32 groups (alignment + traceback + z / V sums, exact); then a full KMeans
    fit through the public estimator.  CPU: the oracle's C epoch (one thread)
    on a bounded sample."""
    import torch

    from oracle import oracle as O
    from wildboar_gb300 import _lib
    from wildboar_gb300.distance import KMeans
    from wildboar_gb300.distance import dtw as D
    from wildboar_gb300.distance._band import band_cells

    N, L, K, r = args.c6_series, 256, 32, 0.2
    X, labels = c6_data(N, L, K)
    groups = [np.flatnonzero(labels == k) for k in range(K)]
    init = X[[g[0] for g in groups]].copy()
    Xd = torch.as_tensor(X, device=dev)
    means = torch.as_tensor(init, device=dev)
    nxt = torch.empty_like(means)
    last = torch.empty(N, dtype=torch.float64, device=dev)
    lay = D._layout(groups, list(range(K)), torch, Xd.device)
    cells = N * band_cells(L, L, r)

    def epoch():
        D._step(Xd, means, lay, r, None, None, nxt, last, torch)

    for _ in range(3):
        epoch()
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    ms = _timed(epoch, max(3, args.steps), flush)
    launches = (_lib.launch_count() - l0) / max(3, args.steps)
    got = nxt.cpu().numpy()
    exact = all(np.array_equal(got[k], O.mm_epoch(X[groups[k]], init[k], r=r))
                for k in (0, K // 2, K - 1))
    # CPU: the oracle's epoch on a sample of one group's members
    sample = groups[0][:args.c6_cpu_sample]
    t0 = time.perf_counter()
    O.mm_epoch(X[sample], init[0], r=r)
    cpu_s = time.perf_counter() - t0
    cpu_gcups = len(sample) * band_cells(L, L, r) / cpu_s / 1e9
    # a full KMeans fit through the estimator (host data, returns host labels)
    km = KMeans(K, metric="dtw", r=r, random_state=0)
    km.fit(X[:256])  # warm-up on a small slice
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    km = KMeans(K, metric="dtw", r=r, random_state=0).fit(X)
    torch.cuda.synchronize()
    fit_s = time.perf_counter() - t0
    return {
        "config": f"{N} float64 series, L={L}, {K} groups (32 sine / random-walk prototypes "
                  f"+ N(0, 0.1)), r={r}",
        "mm_epoch_ms": ms,
        "mm_epoch_gcups": cells / (ms * 1e-3) / 1e9,
        "alignment_cells_per_epoch": cells,
        "launches_per_epoch": launches,
        "epoch_means_exact_vs_oracle": bool(exact),
        "cpu_oracle_epoch": {"gcups": cpu_gcups, "cores": 1, "kind": "port",
                             "sample": f"{len(sample)} series of one group, one epoch"},
        "kmeans_fit_s": fit_s,
        "kmeans_n_iter": int(km.n_iter_),
        "kmeans_inertia": float(km.inertia_),
    }


def bench_ucr(args, dev, flush):
    """scaled_dtw subsequence distance (the UCR-suite scan) of 1,000 shapelets
    (L~U{16..128}) against series of length 1,024, r=0.1; and the LB_Keogh
    lower-bound matrix of 1,000 queries against 10,000 series of length 256,
    r=0.1.  CPU: the oracle (one core) on bounded samples."""
    import torch

    from oracle import oracle as O
    from wildboar_gb300.distance import pairwise_subsequence_distance
    from wildboar_gb300.distance.lb import DtwKeoghLowerBound

    res = {}
    X, shp = c3_data(args.c7_series, 1000)
    Xd = torch.as_tensor(X, device=dev)

    def scan():
        return pairwise_subsequence_distance(shp, Xd, metric="scaled_dtw",
                                             metric_params={"r": 0.1}, return_index=True)

    scan()
    torch.cuda.synchronize()
    ms = _timed(scan, 1, flush)
    d, i = scan()
    od, oi = O.scaled_dtw_subsequence(shp[:50], X[:2], r=0.1)
    t0 = time.perf_counter()
    O.scaled_dtw_subsequence(shp[:100], X[:3], r=0.1)
    cpu_pair_s = (time.perf_counter() - t0) / 300
    pairs = len(shp) * X.shape[0]
    res["scaled_dtw_subsequence"] = {
        "config": f"{len(shp)} shapelets (L~U{{16..128}}) x {X.shape[0]} series, T=1024, r=0.1",
        "ms": ms,
        "pairs_per_s": pairs / (ms * 1e-3),
        "argmin_exact_on_sample": bool(np.array_equal(i[:2, :50].cpu().numpy(), oi)),
        "max_rel_err_on_sample": float(np.max(np.abs(d[:2, :50].cpu().numpy() - od) /
                                              np.maximum(od, 1e-300))),
        "cpu_oracle": {"pairs_per_s": 1.0 / cpu_pair_s, "cores": 1, "kind": "port",
                       "sample": "100 shapelets x 3 series"},
    }
    rng = np.random.default_rng(8)
    DB = np.cumsum(rng.standard_normal((10000, 256)), axis=1)
    Q = np.cumsum(rng.standard_normal((1000, 256)), axis=1)
    lbk = DtwKeoghLowerBound(r=0.1).fit(DB)
    lbk.transform(Q[:8])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = lbk.transform(Q)
    wall = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = O.lb_keogh(Q[:4], DB, r=0.1)
    cpu_s = (time.perf_counter() - t0) / 4 * Q.shape[0]
    res["lb_keogh"] = {
        "config": "1000 queries x 10000 series, L=256, r=0.1, both sides, host arrays",
        "wall_ms": wall * 1e3,
        "bounds_per_s": Q.shape[0] * DB.shape[0] / wall,
        "exact_on_sample": bool(np.array_equal(out[:4], ref)),
        "cpu_oracle": {"bounds_per_s": Q.shape[0] * DB.shape[0] / cpu_s, "cores": 1,
                       "kind": "port", "sample": "4 queries x 10000 series"},
    }
    return res


def bench_argmin(args, dev, flush):
    """argmin_distance (k=5) of 2,000 random-walk queries against 2,000 series of
    length 512, dtw r=0.1 (the headline data).  Default form: candidates in
    chunks of doubling size, each pair stopped once it crosses the k-th
    distance of the replayed prefix (the reference's own early abandoning,
    made safe for out-of-order evaluation), then the heap replay; beside it
    the all-pairs form (every pair's recurrence with its abandon key).  GCUPS
    over the algorithmic band cells of all pairs (abandoned cells included in
    the count).  CPU: the oracle's argmin (with the reference's early
    abandoning) on all host threads, on a row sample."""
    import torch

    from oracle import oracle as O
    from wildboar_gb300.distance import argmin_distance

    wl = WORKLOAD
    X, Y = make_data(0, wl["nx"], wl["ny"], wl["L"], seed=11)
    Xd = torch.as_tensor(X, device=dev)
    Yd = torch.as_tensor(Y, device=dev)
    cells = X.shape[0] * Y.shape[0] * band_cells(wl["L"], wl["L"], wl["params"]["r"])

    def call():
        return argmin_distance(Xd, Yd, k=5, metric="dtw", metric_params=wl["params"],
                               return_distance=True)

    prev = os.environ.pop("WB_GPU_ARGMIN", None)
    try:
        call()
        torch.cuda.synchronize()
        ms = _timed(call, max(1, min(args.steps, 2)), flush)
        idx, dist = call()
        os.environ["WB_GPU_ARGMIN"] = "all"
        call()
        torch.cuda.synchronize()
        ms_all = _timed(call, max(1, min(args.steps, 2)), flush)
        fidx, fdist = call()
    finally:
        if prev is None:
            os.environ.pop("WB_GPU_ARGMIN", None)
        else:
            os.environ["WB_GPU_ARGMIN"] = prev
    # the metric's default band (r=1) on half the queries: the strip form
    Xw = Xd[:1000]
    cells_w = Xw.shape[0] * Y.shape[0] * band_cells(wl["L"], wl["L"], 1.0)

    def call_w():
        return argmin_distance(Xw, Yd, k=5, metric="dtw", metric_params={"r": 1.0},
                               return_distance=True)

    try:
        call_w()
        torch.cuda.synchronize()
        ms_w = _timed(call_w, 1, flush)
        widx, wdist = call_w()
        os.environ["WB_GPU_ARGMIN"] = "all"
        call_w()
        torch.cuda.synchronize()
        ms_w_all = _timed(call_w, 1, flush)
        wfidx, wfdist = call_w()
    finally:
        if prev is None:
            os.environ.pop("WB_GPU_ARGMIN", None)
        else:
            os.environ["WB_GPU_ARGMIN"] = prev
    wide = {
        "config": f"1000 queries x {Y.shape[0]} series, L={wl['L']}, dtw r=1.0, k=5",
        "ms": ms_w,
        "gcups_algorithmic": cells_w / (ms_w * 1e-3) / 1e9,
        "all_pairs_ms": ms_w_all,
        "all_pairs_gcups": cells_w / (ms_w_all * 1e-3) / 1e9,
        "forms_bit_identical": bool(torch.equal(widx, wfidx) and torch.equal(
            wdist.view(torch.int64), wfdist.view(torch.int64))),
    }
    oi, od = O.argmin(X[:4], Y, k=5, metric="dtw", metric_params=wl["params"],
                      n_threads=os.cpu_count() or 1)
    n_threads = os.cpu_count() or 1
    rows = max(n_threads, 32)
    t0 = time.perf_counter()
    O.argmin(X[:rows], Y, k=5, metric="dtw", metric_params=wl["params"], n_threads=n_threads)
    cpu_s = time.perf_counter() - t0
    return {
        "config": f"{X.shape[0]} queries x {Y.shape[0]} series, L={wl['L']}, dtw r=0.1, k=5",
        "ms": ms,
        "gcups_algorithmic": cells / (ms * 1e-3) / 1e9,
        "all_pairs_ms": ms_all,
        "all_pairs_gcups": cells / (ms_all * 1e-3) / 1e9,
        "indices_exact_on_sample": bool(np.array_equal(idx[:4].cpu().numpy(), oi)),
        "forms_bit_identical": bool(torch.equal(idx, fidx) and torch.equal(
            dist.view(torch.int64), fdist.view(torch.int64))),
        "cpu_oracle": {"gcups_algorithmic": rows * Y.shape[0] *
                       band_cells(wl["L"], wl["L"], wl["params"]["r"]) / cpu_s / 1e9,
                       "cores": n_threads, "kind": "port",
                       "sample": f"{rows} queries x {Y.shape[0]} series"},
        "wide_band": wide,
    }


def bench_euclid_tc(args, dev, flush):
    """Full-series euclidean 8192 x 8192 at length 1024: tensor-core 3xTF32
    GEMM form against the FP64 drop-in kernel on the same device data."""
    import torch

    from wildboar_gb300.distance import pairwise_distance
    from wildboar_gb300.distance.precision import pairwise_euclidean_tc

    n, L = args.c3_full, 1024
    rng = np.random.default_rng(9)
    X = np.cumsum(rng.standard_normal((n, L)), axis=1)
    Y = np.cumsum(rng.standard_normal((n, L)), axis=1)
    Xd = torch.as_tensor(X, device=dev)
    Yd = torch.as_tensor(Y, device=dev)
    pairwise_euclidean_tc(Xd, Yd)
    torch.cuda.synchronize()
    ms_tc = _timed(lambda: pairwise_euclidean_tc(Xd, Yd), max(1, args.steps), flush)
    D = pairwise_euclidean_tc(Xd, Yd)
    # FP64 drop-in on the same data (sequential per-pair sums, the reference's
    # order); the untimed call grows the workspace to this size first
    D64 = pairwise_distance(Xd, Yd, metric="euclidean")
    ms_64 = _timed(lambda: pairwise_distance(Xd, Yd, metric="euclidean"), 1, flush)
    err = (D - D64).abs().max().item()
    rel = ((D - D64).abs() / D64.clamp(min=1e-300)).max().item()
    nx = (Xd * Xd).sum(1, keepdim=True)
    ny = (Yd * Yd).sum(1, keepdim=True).t()
    norm_err = ((D * D - D64 * D64).abs() / (nx + ny)).max().item()
    flops = 2.0 * n * n * L
    # CPU: the oracle's euclidean pairwise (the reference's sequential sums) on
    # all host threads, a row sample
    from oracle import oracle as O

    rows = max(os.cpu_count() or 1, 16)
    t0 = time.perf_counter()
    O.pairwise(X[:rows], Y, metric="euclidean", n_threads=os.cpu_count() or 1)
    cpu_s = time.perf_counter() - t0
    return {
        "config": f"{n} x {n} series, L={L}, float64 in, float64 out",
        "cpu_oracle": {"gflops_useful": 2.0 * rows * n * L / cpu_s / 1e9,
                       "cores": os.cpu_count() or 1, "kind": "port",
                       "sample": f"{rows} rows x {n} series"},
        "tc_ms": ms_tc,
        "tc_tflops_useful": flops / (ms_tc * 1e-3) / 1e12,
        "tc_tflops_issued_3xtf32": 3 * flops / (ms_tc * 1e-3) / 1e12,
        "fp64_dropin_ms": ms_64,
        "speedup_vs_fp64_dropin": ms_64 / ms_tc,
        "max_abs_err_vs_fp64": err,
        "max_rel_err_vs_fp64": rel,
        "max_d2_err_over_norms": norm_err,
    }


def _cells_w(n, m, w):
    mx = max(0, m - n) + w
    mn = max(0, n - m)
    return sum(min(m, i + mx) - max(0, i - mn - w + 1) for i in range(n))


def bench_precision(args, dev, flush):
    """Every elastic metric on n x n univariate random walks of length 512:
    the FP64 drop-in against the FP32-compensated form on the same device
    data; error of the FP32 form against the FP64 drop-in over the whole
    matrix and against the CPU oracle on a 16 x 16 corner."""
    import torch

    from oracle import oracle as O
    from wildboar_gb300.distance import pairwise_distance
    from wildboar_gb300.distance._band import compute_r
    from wildboar_gb300.distance.precision import pairwise_distance_fp32

    n, L = args.c2_series, 512
    rng = np.random.default_rng(12)
    X = np.cumsum(rng.standard_normal((n, L)), axis=1)
    Y = np.cumsum(rng.standard_normal((n, L)), axis=1)
    eps = 0.1 * float(np.concatenate([X, Y]).std())
    Xd = torch.as_tensor(X, device=dev)
    Yd = torch.as_tensor(Y, device=dev)
    sweep = [("dtw", {"r": 0.1}), ("dtw", {"r": 1.0}), ("wdtw", {"g": 0.05}), ("ddtw", {}),
             ("adtw", {}), ("lcss", {"epsilon": eps}), ("edr", {"epsilon": eps}),
             ("erp", {"g": 0.0}), ("msm", {"c": 1.0}),
             ("twe", {"stiffness": 0.001, "penalty": 1.0})]
    out = []
    for metric, params in sweep:
        r = params.get("r", 1.0)
        w = compute_r(L, r)
        lc = L - 2 if metric == "ddtw" else L
        cells = n * n * _cells_w(lc, lc, w)
        res = {"metric": metric, "params": params}
        outs = {}
        for tag, fn in (("fp64", pairwise_distance), ("fp32", pairwise_distance_fp32)):
            fn(Xd[:64], Yd[:64], metric=metric, metric_params=params)
            torch.cuda.synchronize()
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            outs[tag] = fn(Xd, Yd, metric=metric, metric_params=params)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            res[tag + "_ms"] = ms
            res[tag + "_gcups"] = cells / (ms * 1e-3) / 1e9
        D64, D32 = outs["fp64"], outs["fp32"]
        diff = (D32 - D64).abs()
        rel = diff / D64.abs().clamp(min=1e-300)
        res["max_abs_err_vs_fp64"] = diff.max().item()
        res["max_rel_err_vs_fp64"] = rel[D64 != 0].max().item() if bool((D64 != 0).any()) else 0.0
        res["frac_entries_differing"] = (diff > 0).double().mean().item()
        ref = O.pairwise(X[:16, None, :], Y[:16, None, :], dim=0, metric=metric,
                         metric_params=params)
        corner = D32[:16, :16].cpu().numpy()
        res["max_rel_err_vs_oracle_16x16"] = float(
            np.max(np.abs(corner - ref) / np.maximum(np.abs(ref), 1e-300)))
        res["speedup"] = res["fp64_ms"] / res["fp32_ms"]
        out.append(res)
    return {"config": f"{n} x {n} univariate random walks, L={L}, float64 in/out; "
                      f"lcss/edr epsilon = 0.1 std = {eps:.6g}",
            "cells": "evaluated band cells (ddtw on the L-2 slopes)", "metrics": out}


def run_gpu(args):
    import torch

    from wildboar_gb300 import _build, _lib
    from wildboar_gb300.distance import pairwise_distance
    from wildboar_gb300.distance.sharded import max_over_ranks

    rank, world = _rank()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    _build.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    wl = WORKLOAD
    dev = torch.device("cuda", local)
    if args.skip_fp64:
        flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
        forms = {}
        if args.only in ("", "batched"):
            forms["batched_fp32"] = bench_batched(args, dev, flush)
        if args.only in ("", "fwdbwd"):
            forms["fwd_bwd_fp32"] = bench_fwd_bwd(args, dev, flush)
        if args.only in ("", "subseq"):
            forms["subsequence"] = bench_subsequence(args, dev, flush)
        if args.only in ("", "euclid"):
            forms["euclidean_full_tc"] = bench_euclid_tc(args, dev, flush)
        if args.only in ("", "precision"):
            forms["precision_sweep"] = bench_precision(args, dev, flush)
        if args.only in ("", "barycenter"):
            forms["barycenter_kmeans"] = bench_barycenter(args, dev, flush)
        if args.only in ("", "ucr"):
            forms["ucr_lower_bounds"] = bench_ucr(args, dev, flush)
        if args.only in ("", "argmin"):
            forms["argmin_knn"] = bench_argmin(args, dev, flush)
        if args.only in ("", "subseq_elastic"):
            forms["subsequence_elastic"] = bench_subsequence_elastic(args, dev, flush)
        if args.only in ("", "subseq_search"):
            forms["subsequence_search"] = bench_subsequence_search(args, dev, flush)
        if rank == 0:
            print(json.dumps({"forms": forms}), flush=True)
        return
    X, Y = make_data(rank, wl["nx"], wl["ny"], wl["L"])
    cells_pair = band_cells(wl["L"], wl["L"], wl["params"]["r"])
    cells = wl["nx"] * wl["ny"] * cells_pair
    Xd = torch.as_tensor(X, device=dev)
    Yd = torch.as_tensor(Y, device=dev)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def step_device():
        return pairwise_distance(Xd, Yd, metric=wl["metric"], metric_params=wl["params"])

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    barrier()

    _lib.profile_enable(True)
    launches0 = _lib.launch_count()
    step_ms, kern_ms = [], []
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        barrier()
        for _ in range(args.steps):
            flush.zero_()  # evict L2 (512 MB > 129 MB) outside the timed events
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            step_device()
            e1.record()
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            kern_ms.append(_lib.profile_last_ms())
        torch.cuda.synchronize()
        barrier()
    launches = _lib.launch_count() - launches0 - 0
    _lib.profile_enable(False)
    t_step = sum(step_ms) / len(step_ms)
    if dist is not None:
        t_step = max_over_ranks(t_step)
    value = world * cells / (t_step * 1e-3) / 1e9

    # end to end through the public API with pinned host buffers
    Xh = torch.empty(X.shape, dtype=torch.float64).pin_memory().numpy()
    Yh = torch.empty(Y.shape, dtype=torch.float64).pin_memory().numpy()
    Xh[...] = X
    Yh[...] = Y
    pairwise_distance(Xh, Yh, metric=wl["metric"], metric_params=wl["params"])
    torch.cuda.synchronize()
    barrier()
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = pairwise_distance(Xh, Yh, metric=wl["metric"], metric_params=wl["params"])
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    t_e2e = sum(e2e_ms) / len(e2e_ms)
    if dist is not None:
        t_e2e = max_over_ranks(t_e2e)
    e2e = {"value": world * cells / (t_e2e * 1e-3) / 1e9, "unit": "GCUPS",
           "h2d_bytes_per_step": int(Xh.nbytes + Yh.nbytes),
           "d2h_bytes_per_step": int(np.asarray(out).nbytes)}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # roofline of the recurrence kernel: FP64 ops per launch / launch time
    probe_peak = _lib.alu_probe(_lib.WB_F64, 4096)
    kms = [k for k in kern_ms if k > 0]
    k_avg = sum(kms) / len(kms) if kms else t_step
    achieved = FP64_OPS_PER_CELL * cells / (k_avg * 1e-3)
    # the FP64 pipe issues 2 operations per clock per SM (ncu: the probe kernel
    # keeps the pipe 84.2 % busy at 0.0526 FP64 warp-instructions per
    # SM-cycle), times the SM count and the median SM clock sampled during the
    # timed region
    clk = clocks.summary()
    sm_mhz = clk.get("sm_mhz") or 2070.0
    pipe_peak = FP64_OPS_PER_SM_CLK * torch.cuda.get_device_properties(dev).multi_processor_count \
        * sm_mhz * 1e6
    roofline = {
        "bound": "fp64",
        "achieved": achieved / 1e12,
        "peak": pipe_peak / 1e12,
        "unit": "TFLOP/s (FP64 pipe: 2 ops/clk/SM x SMs x the median SM clock of the run)",
        "frac": achieved / pipe_peak,
        "probe_peak": probe_peak / 1e12,
        "frac_of_probe": achieved / probe_peak,
        # measured for the default 2000 x 2000 workload only
        "traffic": HEADLINE_DRAM_BYTES if (wl["nx"], wl["ny"]) == (2000, 2000) else None,
        "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
        "traffic_source": "one earlier ncu capture of this workload, not measured in this run",
        "algorithmic_bytes": int(X.nbytes + Y.nbytes + wl["nx"] * wl["ny"] * 8),
        "kernel": "elastic_pairs_kernel<K_DTW>",
        "kernel_ms": k_avg,
        "ops_per_cell": FP64_OPS_PER_CELL,
    }
    cpu = None
    parity = None
    if world == 1 and not args.no_cpu:
        cpu, ref_rows = cpu_reference(X, Y, wl, budget_s=args.cpu_budget, return_rows=True)
        # the headline output against the oracle on the same rows
        got = np.asarray(out)[: ref_rows.shape[0]]
        rel = np.abs(got - ref_rows) / np.maximum(np.abs(ref_rows), 1e-300)
        parity = {"rows": int(ref_rows.shape[0]), "cols": int(ref_rows.shape[1]),
                  "max_rel_err": float(rel.max()),
                  "bit_exact": bool(np.array_equal(got, ref_rows)),
                  "against": "oracle rows of the cpu_baseline sample"}
    forms = {}
    # the forms are single-GPU measurements: they run in the one-rank job only
    if not args.no_forms and world == 1:
        forms["batched_fp32"] = bench_batched(args, dev, flush)
        forms["fwd_bwd_fp32"] = bench_fwd_bwd(args, dev, flush)
        forms["subsequence"] = bench_subsequence(args, dev, flush)
        forms["euclidean_full_tc"] = bench_euclid_tc(args, dev, flush)
        forms["precision_sweep"] = bench_precision(args, dev, flush)
        forms["barycenter_kmeans"] = bench_barycenter(args, dev, flush)
        forms["ucr_lower_bounds"] = bench_ucr(args, dev, flush)
        forms["argmin_knn"] = bench_argmin(args, dev, flush)
        forms["subsequence_elastic"] = bench_subsequence_elastic(args, dev, flush)
        forms["subsequence_search"] = bench_subsequence_search(args, dev, flush)
    targets = None
    if forms:
        bt, fb = forms["batched_fp32"], forms["fwd_bwd_fp32"]
        targets = {
            "fp64_drop_in_gcups": value,
            "batched_fp32_gcups": bt["gcups"],
            "batched_fp32_max_rel_err_vs_fp64": bt["max_rel_err_vs_fp64"],
            "batched_fp32_over_fp64": bt["gcups"] / value,
            "fwd_bwd_fp32_gcups": fb["gcups"],
            "fwd_bwd_fp32_max_rel_err_vs_fp64": fb["max_rel_err_vs_fp64"],
            "fwd_bwd_fp32_over_fp64": fb["gcups"] / value,
            "both_beat_fp64_drop_in": bool(bt["gcups"] > value and fb["gcups"] > value),
        }
        # the bulky per-form records go on their own line before the headline
        if rank == 0:
            print(json.dumps({"forms": forms}), flush=True)
    line = {
        "metric": "DTW cell-updates/s (GCUPS), plain FP64 drop-in",
        "value": value,
        "unit": "GCUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Gaussian random walks)",
        "config": {"workload": WORKLOAD["name"], "n_pairs": wl["nx"] * wl["ny"],
                   "cells_per_step": cells, "parallelism": f"x-row shards x{world}",
                   "l2": "flushed between timed steps (512 MB write)"},
        "e2e": e2e,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "parity_on_sample": parity,
        "targets": targets,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--nx", type=int, default=WORKLOAD["nx"],
                    help="rows of X (smaller values for profiling captures)")
    ap.add_argument("--ny", type=int, default=WORKLOAD["ny"])
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched FP32 and fwd+bwd measurements")
    ap.add_argument("--c4-pairs", type=int, default=65536)
    ap.add_argument("--c5-series", type=int, default=4096)
    ap.add_argument("--c5-adam-steps", type=int, default=100)
    ap.add_argument("--err-sample", type=int, default=64)
    ap.add_argument("--c4-tile", default="",
                    help="strip,block for the batched form instead of the autotuner")
    ap.add_argument("--skip-fp64", action="store_true",
                    help="only the FP32 forms (profiling captures)")
    ap.add_argument("--only", default="", choices=["", "batched", "fwdbwd", "subseq", "euclid",
                                                     "precision", "barycenter", "ucr",
                                                     "argmin", "subseq_elastic",
                                                     "subseq_search"],
                    help="with --skip-fp64: run one form only")
    ap.add_argument("--c6-series", type=int, default=4096)
    ap.add_argument("--c7-series", type=int, default=200,
                    help="series for the scaled_dtw subsequence form")
    ap.add_argument("--c6-cpu-sample", type=int, default=48)
    ap.add_argument("--c3-series", type=int, default=1000)
    ap.add_argument("--c3-shapelets", type=int, default=10000)
    ap.add_argument("--c3-full", type=int, default=8192)
    ap.add_argument("--c2-series", type=int, default=1000,
                    help="n for the per-metric FP64 vs FP32 sweep (n x n, L=512)")
    args = ap.parse_args()
    if (args.nx, args.ny) != (WORKLOAD["nx"], WORKLOAD["ny"]):
        WORKLOAD["nx"], WORKLOAD["ny"] = args.nx, args.ny
        WORKLOAD["name"] = WORKLOAD["name"].replace("2000x2000", f"{args.nx}x{args.ny}")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
