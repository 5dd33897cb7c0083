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


def cpu_reference(X, Y, wl, budget_s=15.0, n_threads=None):
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
    O.pairwise(X[:rows], Y, metric=wl["metric"], metric_params=wl["params"],
               n_threads=n_threads)
    dt = time.perf_counter() - t0
    cells = rows * Y.shape[0] * cells_pair
    return {"value": cells / dt / 1e9, "unit": "GCUPS", "cores": n_threads, "kind": "port",
            "sample": f"{rows} x {Y.shape[0]} pairs of the workload "
                      f"({cells:.3e} cells, {dt:.2f} s), oracle/wb_oracle.c with "
                      f"{n_threads} threads"}


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


def run_gpu(args):
    import torch

    from wildboar_gb300 import _build, _lib
    from wildboar_gb300.distance import pairwise_distance

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
    X, Y = make_data(rank, wl["nx"], wl["ny"], wl["L"])
    cells_pair = band_cells(wl["L"], wl["L"], wl["params"]["r"])
    cells = wl["nx"] * wl["ny"] * cells_pair
    dev = torch.device("cuda", local)
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
        tt = torch.tensor([t_step], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
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
        tt = torch.tensor([t_e2e], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_e2e = float(tt.item())
    e2e = {"value": world * cells / (t_e2e * 1e-3) / 1e9, "unit": "GCUPS",
           "h2d_bytes_per_step": int(Xh.nbytes + Yh.nbytes),
           "d2h_bytes_per_step": int(np.asarray(out).nbytes)}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # roofline of the recurrence kernel: FP64 ops per launch / launch time
    fp64_peak = _lib.alu_probe(_lib.WB_F64, 4096)
    kms = [k for k in kern_ms if k > 0]
    k_avg = sum(kms) / len(kms) if kms else t_step
    achieved = FP64_OPS_PER_CELL * cells / (k_avg * 1e-3)
    roofline = {
        "bound": "fp64",
        "achieved": achieved / 1e12,
        "peak": fp64_peak / 1e12,
        "unit": "TFLOP/s (FP64 add+mul, peak measured by wb_alu_probe in this run)",
        "frac": achieved / fp64_peak,
        "traffic": None,
        "kernel": "elastic_pairs_kernel<K_DTW>",
        "kernel_ms": k_avg,
        "ops_per_cell": FP64_OPS_PER_CELL,
    }
    cpu = None
    if world == 1 and not args.no_cpu:
        cpu = cpu_reference(X, Y, wl, budget_s=args.cpu_budget)
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
