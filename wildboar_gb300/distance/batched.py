"""Batched FP32 dtw: ragged (NaN-padded) pair batches on the GPU.

Three layers, all on CUDA torch tensors:

* ``dtw32(...)`` -- one call of ``wb_dtw32_distance`` (include/wbgpu.h): FP32
  costs, compensated (TwoSum) accumulation, FP64 sqrt, one persistent
  launch.
* ``paired_dtw_batch(x, y, r)`` -- the reference's ``paired_distance`` with
  ``metric="dtw"`` and ``dim="mean"`` (distance/_distance.py:1082-1175) over a
  batch whose series end at their first NaN (``get_variable_length``
  semantics, utils/variable_len.py:66-115; the reference itself rejects NaN
  and only supports one length per array).  The (pair, dim) problems are
  sorted by their band cell count so every warp gets problems of similar size
  (length bucketing), and the kernel configuration (rows per register strip,
  block size) comes from ``Autotuner``.
* ``BatchedDTW`` -- the same computation on fixed device buffers, captured in
  a CUDA graph after a warm-up and replayed.
"""

import ctypes
import json
import os
import threading
import time

import numpy as np

from .. import _lib


class Dtw32(ctypes.Structure):
    _fields_ = [
        ("x", ctypes.c_void_p),
        ("x_stride", ctypes.c_int64),
        ("x_lengths", ctypes.c_void_p),
        ("x_len", ctypes.c_int32),
        ("nx", ctypes.c_int64),
        ("y", ctypes.c_void_p),
        ("y_stride", ctypes.c_int64),
        ("y_lengths", ctypes.c_void_p),
        ("y_len", ctypes.c_int32),
        ("ny", ctypes.c_int64),
        ("item_x", ctypes.c_void_p),
        ("item_y", ctypes.c_void_p),
        ("n_items", ctypes.c_int64),
        ("r", ctypes.c_double),
        ("weights", ctypes.c_void_p),
        ("strip", ctypes.c_int32),
        ("block", ctypes.c_int32),
        ("grid", ctypes.c_int32),
    ]


_P = ctypes.POINTER
_vp = ctypes.c_void_p
_lib.declare("wb_dtw32_distance", [_P(Dtw32), _vp, _vp, _vp])
_lib.declare("wb_dtw32_backward", [_P(Dtw32), _vp, _vp, ctypes.c_int64, _vp, ctypes.c_int64,
                                   _vp])
_lib.declare("wb_series_lengths_f32", [_vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
                                       _vp, _vp])
_lib.declare("wb_dtw32_keep_bytes", [_P(Dtw32)], ctypes.c_int64)
_lib.declare("wb_dtw32_distance_keep", [_P(Dtw32), _vp, _vp, _vp, ctypes.c_int64, _vp])
_lib.declare("wb_dtw32_backward_keep", [_P(Dtw32), _vp, _vp, _vp, ctypes.c_int64, _vp,
                                        ctypes.c_int64, _vp, ctypes.c_int64, _vp])

STRIPS = (4, 8, 16, 24, 32)
BLOCKS = (64, 128, 256)


def _torch():
    import torch

    return torch


def _stream():
    return _torch().cuda.current_stream().cuda_stream


def _ptr(t):
    return None if t is None else t.data_ptr()


def make_job(x, y, *, r, x_lengths=None, y_lengths=None, item_x=None, item_y=None,
             weights=None, strip=16, block=128, grid=0):
    """wb_dtw32 descriptor; x, y are (n, L) float32 CUDA tensors (row stride L)."""
    torch = _torch()
    for name, t in (("x", x), ("y", y)):
        if not (t.is_cuda and t.dtype == torch.float32 and t.dim() == 2 and t.is_contiguous()):
            raise ValueError(f"{name} must be a contiguous (n, L) float32 CUDA tensor")
    j = Dtw32()
    j.x, j.x_stride, j.x_lengths = x.data_ptr(), x.shape[1], _ptr(x_lengths)
    j.x_len, j.nx = x.shape[1], x.shape[0]
    j.y, j.y_stride, j.y_lengths = y.data_ptr(), y.shape[1], _ptr(y_lengths)
    j.y_len, j.ny = y.shape[1], y.shape[0]
    if item_x is not None:
        j.item_x, j.item_y, j.n_items = item_x.data_ptr(), item_y.data_ptr(), item_x.numel()
    else:
        j.item_x = j.item_y = None
        j.n_items = x.shape[0] * y.shape[0]
    j.r = float(r)
    j.weights = _ptr(weights)
    j.strip, j.block, j.grid = int(strip), int(block), int(grid)
    return j


def dtw32(x, y, *, r, out=None, out_cost=None, **kw):
    """Per-item dtw distances (float64 CUDA tensor of n_items)."""
    torch = _torch()
    job = make_job(x, y, r=r, **kw)
    if out is None:
        out = torch.empty(job.n_items, dtype=torch.float64, device=x.device)
    _lib.check(_lib.lib().wb_dtw32_distance(ctypes.byref(job), out.data_ptr(),
                                            _ptr(out_cost), _stream()))
    return out


def series_lengths(x):
    """Index of the first NaN of every row of a (n, L) float32 CUDA tensor."""
    torch = _torch()
    out = torch.empty(x.shape[0], dtype=torch.int32, device=x.device)
    _lib.check(_lib.lib().wb_series_lengths_f32(x.data_ptr(), x.shape[0], x.shape[1],
                                                x.shape[1], out.data_ptr(), _stream()))
    return out


def logistic_weights(n, g, device):
    """WeightedDtwMetric weights (distance/_elastic.pyx:3333-3341), host libm exp."""
    torch = _torch()
    w = [1.0 / (1.0 + np.exp(-g * (i - n / 2.0))) for i in range(n)]
    return torch.tensor(np.asarray(w, dtype=np.float32), device=device)


# --------------------------------------------------------------------------
# autotuner


class Autotuner:
    """Picks (strip, block) for a batch by timing the candidates on a sample.

    Results are cached per (device name, length bucket, band fraction) in
    memory and in a JSON file (``WB_GPU_AUTOTUNE_CACHE``, default
    ``~/.cache/wildboar_gb300/autotune.json``).
    """

    def __init__(self, path=None):
        self.path = path or os.environ.get(
            "WB_GPU_AUTOTUNE_CACHE",
            os.path.join(os.path.expanduser("~"), ".cache", "wildboar_gb300", "autotune.json"))
        self.lock = threading.Lock()
        self.table = None

    def _load(self):
        if self.table is None:
            try:
                with open(self.path) as f:
                    self.table = json.load(f)
            except (OSError, ValueError):
                self.table = {}
        return self.table

    def _save(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            tmp = self.path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(self.table, f, indent=1)
            os.replace(tmp, self.path)
        except OSError:
            pass

    @staticmethod
    def key(device, max_len, r, weighted):
        torch = _torch()
        name = torch.cuda.get_device_name(device)
        bucket = 1 << max(int(max_len) - 1, 1).bit_length()
        return f"v2|{name}|L<={bucket}|r={r:g}|w={int(bool(weighted))}"

    def pick(self, x, y, *, r, x_lengths, y_lengths, item_x, item_y, weights=None,
             sample=16384, reps=2):
        torch = _torch()
        k = self.key(x.device, max(x.shape[1], y.shape[1]), r, weights is not None)
        with self.lock:
            tab = self._load()
            if k in tab:
                return tab[k]["strip"], tab[k]["block"]
        n = item_x.numel()
        if n > sample:
            idx = torch.linspace(0, n - 1, sample, device=x.device).long()
            sx, sy = item_x[idx].contiguous(), item_y[idx].contiguous()
        else:
            sx, sy = item_x, item_y
        best = None
        out = torch.empty(sx.numel(), dtype=torch.float64, device=x.device)
        for strip, block in [(s_, b_) for s_ in STRIPS for b_ in BLOCKS]:
            kw = dict(r=r, x_lengths=x_lengths, y_lengths=y_lengths, item_x=sx,
                      item_y=sy, weights=weights, strip=strip, block=block)
            dtw32(x, y, out=out, **kw)  # warm-up (workspace growth)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                dtw32(x, y, out=out, **kw)
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / reps
            if best is None or dt < best[0]:
                best = (dt, strip, block)
        with self.lock:
            tab = self._load()
            tab[k] = {"strip": best[1], "block": best[2], "sample_s": best[0]}
            self._save()
        return best[1], best[2]


AUTOTUNER = Autotuner()
# configuration without autotuning: (strip, block)
DEFAULT_TILE = (24, 128)


# --------------------------------------------------------------------------
# ragged paired batches


def band_cost(n, m, r):
    """Exact band cell count of every (n, m) problem (torch int64).

    Closed form of sum_i [min(m, i + mx) - max(0, i - mn - w + 1)], the cells
    dtw_distance evaluates (distance/_elastic.pyx:869-940); zero for empty
    series.  Used as the bucketing sort key and as the GCUPS numerator.
    """
    torch = _torch()
    n = n.long()
    m = m.long()
    w = torch.clamp(torch.floor(torch.minimum(n, m).double() * r), min=1).long()
    mx = torch.clamp(m - n, min=0) + w
    mn = torch.clamp(n - m, min=0)
    a = torch.minimum(torch.clamp(m - mx, min=0), n)
    first = a * mx + a * (a - 1) // 2 + (n - a) * m
    t = torch.clamp(n - (mn + w), min=0)
    cells = first - t * (t + 1) // 2
    return torch.where((n > 0) & (m > 0), cells, torch.zeros_like(cells))


def bucket_order(n, m, r, transpose=True):
    """Processing order of the items.

    The 32 lanes of a warp sweep their items together over the union of their
    column ranges, so neighbours in this order should have their bands in the
    same columns.  A lane's rows are the shorter series when the kernel
    transposes (dtw: ``transpose=True``), else x; its work is (number of
    32-row strips) x (band width min(m, |m - n| + 2r)).  Items are sorted by
    strip count, then by band width, both descending (without transposition
    the orientation n > m comes first, as it places the band on the other
    side of the diagonal); the persistent queue ends on the smallest
    problems.
    """
    torch = _torch()
    n = n.long()
    m = m.long()
    w = torch.clamp(torch.floor(torch.minimum(n, m).double() * r), min=1).long()
    cols = torch.minimum(torch.maximum(n, m), (m - n).abs() + 2 * w).clamp(0, 8191)
    rows = torch.minimum(n, m) if transpose else n
    key = ((rows - 2).clamp(min=0) // 32) * 8192 + cols
    if not transpose:
        key = key + (n > m).long() * (1 << 40)
    return torch.argsort(key, descending=True, stable=True)


def plan_pairs(x, y, r, *, tune=True, weights=None, tile=None):
    """Items, lengths, order and kernel configuration of a paired batch.

    x, y: (N, d, L) float32 CUDA tensors (NaN padded).  Returns a dict with the
    flattened (N*d, L) views, per-series lengths, the sorted item arrays and
    the inverse permutation.
    """
    torch = _torch()
    if x.shape[:2] != y.shape[:2]:
        raise ValueError("x and y must have the same number of pairs and dims")
    N, d = x.shape[0], x.shape[1]
    xf = x.reshape(N * d, x.shape[2]).contiguous()
    yf = y.reshape(N * d, y.shape[2]).contiguous()
    xl = series_lengths(xf)
    yl = series_lengths(yf)
    cost = band_cost(xl, yl, r)
    order = bucket_order(xl, yl, r, transpose=weights is None).to(torch.int32)
    item = order.contiguous()
    plan = {"xf": xf, "yf": yf, "xl": xl, "yl": yl, "item_x": item, "item_y": item,
            "order": order.long(), "N": N, "d": d, "r": float(r), "weights": weights,
            "cells": int(cost.sum().item())}
    if tile is not None:
        plan["strip"], plan["block"] = tile
    elif tune:
        plan["strip"], plan["block"] = AUTOTUNER.pick(
            xf, yf, r=r, x_lengths=xl, y_lengths=yl, item_x=item, item_y=item,
            weights=weights)
    else:
        plan["strip"], plan["block"] = DEFAULT_TILE
    return plan


def run_plan(plan, out_items=None):
    torch = _torch()
    n = plan["item_x"].numel()
    if out_items is None:
        out_items = torch.empty(n, dtype=torch.float64, device=plan["xf"].device)
    dtw32(plan["xf"], plan["yf"], r=plan["r"], out=out_items, x_lengths=plan["xl"],
          y_lengths=plan["yl"], item_x=plan["item_x"], item_y=plan["item_y"],
          weights=plan["weights"], strip=plan["strip"], block=plan["block"])
    return out_items


def combine_dims(plan, out_items):
    """Per-pair mean over dims (np.mean semantics: sequential sum, then divide)."""
    torch = _torch()
    per = torch.empty_like(out_items)
    per[plan["order"]] = out_items
    per = per.reshape(plan["N"], plan["d"])
    acc = per[:, 0].clone()
    for k in range(1, plan["d"]):
        acc += per[:, k]
    return acc / plan["d"]


def paired_dtw_batch(x, y, r=1.0, *, tune=True):
    """dtw distance of every (x[i], y[i]) pair of a NaN-padded float32 batch.

    x, y: (N, L) or (N, d, L) float32 CUDA tensors; a series ends at its first
    NaN.  Returns (N,) float64 distances (mean over dims).
    """
    if x.dim() == 2:
        x = x.unsqueeze(1)
        y = y.unsqueeze(1)
    plan = plan_pairs(x, y, r, tune=tune)
    return combine_dims(plan, run_plan(plan))


class BatchedDTW:
    """A fixed ragged paired batch replayed through a captured CUDA graph.

    ``BatchedDTW(x, y, r)`` plans (lengths, bucketing sort, autotuning) and
    captures lengths + kernel + dim reduction into one graph; ``run()`` replays
    it on whatever the buffers ``x`` / ``y`` currently hold (same shapes).
    """

    def __init__(self, x, y, r=1.0, *, tune=True, graph=True, tile=None):
        torch = _torch()
        if x.dim() == 2:
            x = x.unsqueeze(1)
            y = y.unsqueeze(1)
        self.x, self.y = x, y
        self.plan = plan_pairs(x, y, r, tune=tune, tile=tile)
        self.items = torch.empty(self.plan["item_x"].numel(), dtype=torch.float64,
                                 device=x.device)
        self.out = None
        self.graph = None
        self.cells = self.plan["cells"]
        # warm-up grows the workspace so that capture performs no allocation
        self._body()
        torch.cuda.synchronize()
        if graph:
            # a stream of its own: the library's workspace is per stream, and
            # the captured graph keeps pointing at this stream's workspace
            s = self.stream = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self._body()
            torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                self._body()
            self.graph = g

    def _body(self):
        p = self.plan
        xf = self.x.reshape(p["N"] * p["d"], self.x.shape[2])
        yf = self.y.reshape(p["N"] * p["d"], self.y.shape[2])
        _lib.check(_lib.lib().wb_series_lengths_f32(
            xf.data_ptr(), xf.shape[0], xf.shape[1], xf.shape[1], p["xl"].data_ptr(),
            _stream()))
        _lib.check(_lib.lib().wb_series_lengths_f32(
            yf.data_ptr(), yf.shape[0], yf.shape[1], yf.shape[1], p["yl"].data_ptr(),
            _stream()))
        run_plan(p, self.items)
        self.out = combine_dims(p, self.items)
        return self.out

    def run(self):
        if self.graph is not None:
            self.graph.replay()
            return self.out
        return self._body()
