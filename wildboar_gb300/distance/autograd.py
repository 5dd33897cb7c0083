"""Differentiable dtw / wdtw: a torch.autograd.Function over the FP32 kernels.

``dtw_matrix(x, y, r)`` returns the (n_x, n_y) matrix of dtw distances
(wildboar's ``pairwise_distance(x, y, metric="dtw", metric_params={"r": r})``)
as a differentiable float64 tensor.  Its backward recomputes every pair's
forward with a 2-bit direction per band cell and walks the optimal path back
(dtw_mapping's tie order: diag, up, left -- distance/dtw.py:362-426), giving

    dD/dx_i =  sum_{j: (i, j) on the path} w_{|i-j|} (x_i - y_j) / D
    dD/dy_j = -sum_{i: (i, j) on the path} w_{|i-j|} (x_i - y_j) / D

the gradient of D = sqrt(sum over the path of w (x_i - y_j)^2) with the path
fixed (dtw is differentiable wherever the optimal path is unique).

``barycenter_kmeans`` uses it for DTW-barycenter updates: Adam on the centroids
with a soft assignment of every series to every centroid, so every pair takes
part in the backward.
"""

import ctypes

import torch

from .. import _lib
from . import batched as _b


def _job(x, y, r, weights):
    return _b.make_job(x, y, r=r, weights=weights, strip=16, block=128)


class DTWMatrix(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, r, weights):
        x = x.contiguous()
        y = y.contiguous()
        out = torch.empty(x.shape[0] * y.shape[0], dtype=torch.float64, device=x.device)
        job = _job(x, y, r, weights)
        _lib.check(_lib.lib().wb_dtw32_distance(ctypes.byref(job), out.data_ptr(), None,
                                                _b._stream()))
        ctx.save_for_backward(x, y)
        ctx.r = r
        ctx.weights = weights
        # items are t = j * nx + i: reshape to (ny, nx) and transpose
        return out.view(y.shape[0], x.shape[0]).t()

    @staticmethod
    def backward(ctx, grad):
        x, y = ctx.saved_tensors
        nx, ny = x.shape[0], y.shape[0]
        g = grad.t().contiguous().to(torch.float64).reshape(-1)
        gx = torch.empty((ny * nx, x.shape[1]), dtype=torch.float32, device=x.device)
        gy = torch.empty((ny * nx, y.shape[1]), dtype=torch.float32, device=x.device)
        job = _job(x, y, ctx.r, ctx.weights)
        _lib.check(_lib.lib().wb_dtw32_backward(
            ctypes.byref(job), g.data_ptr(), gx.data_ptr(), x.shape[1], gy.data_ptr(),
            y.shape[1], _b._stream()))
        grad_x = gx.view(ny, nx, x.shape[1]).sum(dim=0) if ctx.needs_input_grad[0] else None
        grad_y = gy.view(ny, nx, y.shape[1]).sum(dim=1) if ctx.needs_input_grad[1] else None
        return grad_x, grad_y, None, None


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
    return DTWMatrix.apply(x, y, float(r), weights)


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
