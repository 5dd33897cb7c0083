"""Differentiable dtw / wdtw: torch.autograd.Functions over the FP32 kernels.

``dtw_matrix(x, y, r)`` returns the (n_x, n_y) matrix of dtw distances
(wildboar's ``pairwise_distance(x, y, metric="dtw", metric_params={"r": r})``)
as a differentiable float64 tensor; ``paired_dtw(x, y, r)`` the distances of
the pairs (x[i], y[i]) of a NaN-padded ragged batch (``paired_distance`` with
``dim="mean"``).  Their backward (wb_dtw32_backward) recomputes the forward
with a 2-bit direction per band cell, checkpointing the band boundary every K
strips for long series, and walks the optimal path back (dtw_mapping's tie
order: diag, up, left -- distance/dtw.py:362-426), adding in the kernel

    dD/dx_i =  sum_{j: (i, j) on the path} w_{|i-j|} (x_i - y_j) / D
    dD/dy_j = -sum_{i: (i, j) on the path} w_{|i-j|} (x_i - y_j) / D

to one gradient row per series: the gradient of D = sqrt(sum over the path
of w (x_i - y_j)^2) with the path fixed (dtw is differentiable wherever the
optimal path is unique).  Workspace per resident thread: the direction words
of one segment and one checkpoint row per segment boundary (bounded in total
by ``WB_GPU_BWD_WORKSPACE_MB``, default 8192).

When an input of ``dtw_matrix`` requires a gradient and the direction words of
all its pairs fit that budget (``wb_dtw32_keep_bytes``), the forward runs the
sweep with directions once and keeps them (wb_dtw32_distance_keep); the
backward then only walks the paths (wb_dtw32_backward_keep) instead of
recomputing the sweep.  The distances of that forward choose predecessors by
compensated comparison, like the backward; they agree with the plain forward
to a few float32 ulps of the path cost.

``barycenter_kmeans`` uses ``dtw_matrix`` for DTW-barycenter updates: Adam on
the centroids with a soft assignment of every series to every centroid, so
every pair takes part in the backward.
"""

import ctypes
import os

import torch

from .. import _lib
from . import batched as _b


def _job(x, y, r, weights):
    return _b.make_job(x, y, r=r, weights=weights, strip=16, block=128)


def _workspace_budget():
    return float(os.environ.get("WB_GPU_BWD_WORKSPACE_MB", "8192")) * 1048576.0


def keeps_directions(x, y, r=1.0, *, g=None):
    """Whether a differentiable ``dtw_matrix(x, y, r, g=g)`` keeps the
    forward's directions (they fit ``WB_GPU_BWD_WORKSPACE_MB``)."""
    weights = None
    if g is not None:
        weights = _b.logistic_weights(max(x.shape[1], y.shape[1]), g, x.device)
    job = _job(x.detach().contiguous(), y.detach().contiguous(), float(r), weights)
    nbytes = _lib.lib().wb_dtw32_keep_bytes(ctypes.byref(job))
    return 0 <= nbytes <= _workspace_budget()


class DTWMatrix(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, r, weights, keep_dirs):
        x = x.contiguous()
        y = y.contiguous()
        out = torch.empty(x.shape[0] * y.shape[0], dtype=torch.float64, device=x.device)
        job = _job(x, y, r, weights)
        keep = None
        if keep_dirs:
            nbytes = _lib.lib().wb_dtw32_keep_bytes(ctypes.byref(job))
            if 0 <= nbytes <= _workspace_budget():
                keep = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
        if keep is not None:
            _lib.check(_lib.lib().wb_dtw32_distance_keep(
                ctypes.byref(job), out.data_ptr(), None, keep.data_ptr(), keep.numel(),
                _b._stream()))
        else:
            _lib.check(_lib.lib().wb_dtw32_distance(ctypes.byref(job), out.data_ptr(), None,
                                                    _b._stream()))
        ctx.save_for_backward(x, y, out)
        ctx.keep = keep
        ctx.r = r
        ctx.weights = weights
        # items are t = j * nx + i: reshape to (ny, nx) and transpose
        return out.view(y.shape[0], x.shape[0]).t()

    @staticmethod
    def backward(ctx, grad):
        x, y, out = ctx.saved_tensors
        # items are t = j * nx + i: the upstream gradient in that order
        g = grad.t().contiguous().to(torch.float64).reshape(-1)
        gx = torch.zeros_like(x)
        gy = torch.zeros_like(y)
        job = _job(x, y, ctx.r, ctx.weights)
        if ctx.keep is not None:
            keep, ctx.keep = ctx.keep, None
            _lib.check(_lib.lib().wb_dtw32_backward_keep(
                ctypes.byref(job), out.data_ptr(), g.data_ptr(), gx.data_ptr(), x.shape[1],
                gy.data_ptr(), y.shape[1], keep.data_ptr(), keep.numel(), _b._stream()))
        else:
            _lib.check(_lib.lib().wb_dtw32_backward(
                ctypes.byref(job), g.data_ptr(), gx.data_ptr(), x.shape[1], gy.data_ptr(),
                y.shape[1], _b._stream()))
        return (gx if ctx.needs_input_grad[0] else None,
                gy if ctx.needs_input_grad[1] else None, None, None, None)


class PairedDTW(torch.autograd.Function):
    """dtw of the pairs of a ragged batch; see ``paired_dtw``."""

    @staticmethod
    def forward(ctx, x, y, r, tile):
        plan = _b.plan_pairs(x.detach(), y.detach(), r, tune=False, tile=tile)
        items = _b.run_plan(plan)
        ctx.plan = plan
        ctx.shape = x.shape
        return _b.combine_dims(plan, items)

    @staticmethod
    def backward(ctx, grad):
        plan = ctx.plan
        N, d, L = ctx.shape
        # the pair distance is the mean over dims: each (pair, dim) item gets
        # grad / d; items run in the plan's (sorted) order
        g = (grad.to(torch.float64) / d).repeat_interleave(d)[plan["order"]].contiguous()
        gx = torch.zeros((N * d, L), dtype=torch.float32, device=grad.device)
        gy = torch.zeros_like(gx)
        job = _b.make_job(plan["xf"], plan["yf"], r=plan["r"], x_lengths=plan["xl"],
                          y_lengths=plan["yl"], item_x=plan["item_x"],
                          item_y=plan["item_y"], weights=plan["weights"])
        _lib.check(_lib.lib().wb_dtw32_backward(
            ctypes.byref(job), g.data_ptr(), gx.data_ptr(), L, gy.data_ptr(), L,
            _b._stream()))
        return gx.view(N, d, L), gy.view(N, d, L), None, None


def paired_dtw(x, y, r=1.0, *, tile=None):
    """Differentiable dtw of the pairs (x[i], y[i]) of a NaN-padded batch.

    x, y: (N, L) or (N, d, L) float32 CUDA tensors; a series ends at its first
    NaN.  Returns the (N,) float64 distances (mean over dims), differentiable
    with respect to x and y (gradients are 0 on the padding).
    """
    if x.dtype != torch.float32 or y.dtype != torch.float32:
        raise ValueError("paired_dtw works on float32 CUDA tensors")
    squeeze = x.dim() == 2
    if squeeze:
        x = x.unsqueeze(1)
        y = y.unsqueeze(1)
    return PairedDTW.apply(x.contiguous(), y.contiguous(), float(r), tile)


def dtw_matrix(x, y, r=1.0, *, g=None):
    """Differentiable (n_x, n_y) dtw (g=None) or wdtw (weight steepness g) matrix.

    x: (n_x, L_x), y: (n_y, L_y) float32 CUDA tensors.  The band follows
    ``_compute_r(min(len), r)``; wdtw weights are WeightedDtwMetric's
    (length max(L_x, L_y)).
    """
    if x.dtype != torch.float32 or y.dtype != torch.float32:
        raise ValueError("dtw_matrix works on float32 CUDA tensors")
    weights = None
    if g is not None:
        weights = _b.logistic_weights(max(x.shape[1], y.shape[1]), g, x.device)
    # keep the directions only when a backward can follow
    keep_dirs = torch.is_grad_enabled() and (x.requires_grad or y.requires_grad)
    return DTWMatrix.apply(x, y, float(r), weights, keep_dirs)


def soft_assignment_loss(D, temperature=1.0):
    """Mean over series of sum_k softmin_k(D / T) * D^2 (every pair contributes)."""
    w = torch.softmax(-D / temperature, dim=1)
    return (w * D * D).sum(dim=1).mean()


def barycenter_kmeans(x, centroids, r=1.0, *, steps=100, lr=0.05, temperature=1.0,
                      callback=None):
    """Adam barycenter updates of ``centroids`` against ``x`` (both float32 CUDA).

    Returns the final centroids and the loss history.
    """
    c = centroids.clone().requires_grad_(True)
    opt = torch.optim.Adam([c], lr=lr)
    losses = []
    for step in range(steps):
        opt.zero_grad(set_to_none=True)
        D = dtw_matrix(x, c, r)
        loss = soft_assignment_loss(D, temperature)
        loss.backward()
        opt.step()
        losses.append(loss.detach())
        if callback is not None:
            callback(step, c, loss)
    return c.detach(), torch.stack(losses).cpu().numpy()
