"""Backward of the FP32 dtw: checkpointed segments, ragged pairs, in-kernel
gradient sums.

Bars (the differentiable form's): gradients within 1e-4 of the gradient
implied by the reference's dtw_alignment + dtw_mapping path
(distance/dtw.py:246-426, restated in the oracle) and of central finite
differences of the FP64 distance, on pairs whose optimal path has no near-tie
(a step where another predecessor's cumulative cost is within 1e-9 relative:
dtw is not differentiable there).  Series of 600 and 2048 points take the
checkpointed path (several segments of strips per item).  dtw_matrix keeps
the forward's directions when they fit the workspace budget; a small budget
forces the recompute path, and both give the same distances and gradients.
"""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from wildboar_gb300.distance import autograd as AG  # noqa: E402

TIE_REL = 1e-9
GRAD_ATOL = 1e-4


def _walk(rng, n):
    return np.cumsum(rng.standard_normal(n)).astype(np.float32)


def _near_tie(al, path, rel=TIE_REL):
    for a, b in path:
        if a == 0 or b == 0:
            continue
        c = np.sort([al[a - 1, b - 1], al[a - 1, b], al[a, b - 1]])
        if np.isfinite(c[1]) and c[1] - c[0] <= rel * c[0]:
            return True
    return False


def _path_grad(x, y, r):
    """Distance and gradient of the reference path (FP64), or None at a near-tie.

    dtw_alignment sizes its band from max(n, m) (distance/dtw.py:246-290),
    dtw_distance from min(n, m) (_elastic.pyx:1924-1925): the alignment is
    given the fraction whose band is the distance's.
    """
    n, m = len(x), len(y)
    band = max(int(np.floor(min(n, m) * r)), 1)
    al = O.dtw_alignment(x, y, r=(band + 0.5) / max(n, m))
    path = O.dtw_mapping(al)
    if _near_tie(al, path):
        return None
    d = np.sqrt(al[-1, -1])
    gx = np.zeros_like(x)
    gy = np.zeros_like(y)
    for i, j in path:
        g = (x[i] - y[j]) / d
        gx[i] += g
        gy[j] -= g
    return d, gx, gy


def _ragged_pairs(rng, n, L, lo):
    x = np.full((n, L), np.nan, dtype=np.float32)
    y = np.full((n, L), np.nan, dtype=np.float32)
    lx = rng.integers(lo, L + 1, size=n)
    ly = rng.integers(lo, L + 1, size=n)
    for i in range(n):
        x[i, : lx[i]] = _walk(rng, lx[i])
        y[i, : ly[i]] = _walk(rng, ly[i])
    return x, y, lx, ly


@pytest.mark.parametrize("L,lo", [(300, 20), (2048, 1024)])
def test_paired_ragged_gradient_vs_alignment_path(L, lo):
    rng = np.random.default_rng(L)
    n, r = 12, 0.1
    x, y, lx, ly = _ragged_pairs(rng, n, L, lo)
    xt = torch.as_tensor(x, device="cuda").requires_grad_(True)
    yt = torch.as_tensor(y, device="cuda").requires_grad_(True)
    D = AG.paired_dtw(xt, yt, r)
    gw = rng.standard_normal(n)
    (D * torch.as_tensor(gw, device="cuda")).sum().backward()
    gxs, gys = xt.grad.cpu().numpy(), yt.grad.cpu().numpy()
    checked = 0
    for i in range(n):
        a, b = x[i, : lx[i]].astype(np.float64), y[i, : ly[i]].astype(np.float64)
        want = _path_grad(a, b, r)
        # padding gets no gradient
        assert np.all(gxs[i, lx[i]:] == 0) and np.all(gys[i, ly[i]:] == 0)
        if want is None:
            continue
        d, gx, gy = want
        assert abs(D[i].item() - d) <= 1e-5 * d
        np.testing.assert_allclose(gxs[i, : lx[i]], gw[i] * gx, rtol=0, atol=GRAD_ATOL)
        np.testing.assert_allclose(gys[i, : ly[i]], gw[i] * gy, rtol=0, atol=GRAD_ATOL)
        checked += 1
    assert checked >= n // 2


def test_paired_gradient_vs_finite_differences_long():
    rng = np.random.default_rng(77)
    n, L, r = 3, 2048, 0.1
    x, y, lx, ly = _ragged_pairs(rng, n, L, 1500)
    xt = torch.as_tensor(x, device="cuda").requires_grad_(True)
    yt = torch.as_tensor(y, device="cuda").requires_grad_(True)
    AG.paired_dtw(xt, yt, r).sum().backward()
    gxs = xt.grad.cpu().numpy()
    h = 1e-4
    checked = 0
    for p in range(n):
        a = x[p, : lx[p]].astype(np.float64)
        b = y[p, : ly[p]].astype(np.float64)
        d0 = O.distance_1d(a, b, metric="dtw", metric_params={"r": r})
        for i in rng.choice(lx[p], size=12, replace=False):
            ap = a.copy()
            ap[i] += h
            dp = O.distance_1d(ap, b, metric="dtw", metric_params={"r": r})
            ap[i] -= 2 * h
            dm = O.distance_1d(ap, b, metric="dtw", metric_params={"r": r})
            fd = (dp - dm) / (2 * h)
            # away from ties the path does not move within +-h
            if abs((dp - d0) / h - fd) > 1e-3 * (1 + abs(fd)):
                continue
            assert abs(gxs[p, i] - fd) <= GRAD_ATOL, (p, i, gxs[p, i], fd)
            checked += 1
    assert checked >= 24


def test_matrix_gradient_multisegment_vs_alignment_path(monkeypatch):
    # 600 points: 38 strips of 16 rows, more direction words than one segment
    # holds, so the backward checkpoints and recomputes segments (a budget
    # below the kept directions' 2.9 MB keeps the forward from storing them)
    monkeypatch.setenv("WB_GPU_BWD_WORKSPACE_MB", "2")
    rng = np.random.default_rng(600)
    L, r = 600, 0.2
    X = np.stack([_walk(rng, L) for _ in range(3)])
    Y = np.stack([_walk(rng, L) for _ in range(2)])
    xt = torch.as_tensor(X, device="cuda").requires_grad_(True)
    yt = torch.as_tensor(Y, device="cuda").requires_grad_(True)
    D = AG.dtw_matrix(xt, yt, r)
    gw = rng.standard_normal((3, 2))
    refs = {}
    for i in range(3):
        for j in range(2):
            refs[i, j] = _path_grad(X[i].astype(np.float64), Y[j].astype(np.float64), r)
            if refs[i, j] is None:
                gw[i, j] = 0.0
    assert np.count_nonzero(gw) >= 3
    (D * torch.as_tensor(gw, device="cuda")).sum().backward()
    gx_want = np.zeros((3, L))
    gy_want = np.zeros((2, L))
    for (i, j), ref in refs.items():
        if ref is None:
            continue
        d, gx, gy = ref
        gx_want[i] += gw[i, j] * gx
        gy_want[j] += gw[i, j] * gy
    np.testing.assert_allclose(xt.grad.cpu().numpy(), gx_want, rtol=0, atol=GRAD_ATOL)
    np.testing.assert_allclose(yt.grad.cpu().numpy(), gy_want, rtol=0, atol=GRAD_ATOL)


def test_small_workspace_budget_gives_the_same_gradients(monkeypatch):
    rng = np.random.default_rng(5)
    x, y, _, _ = _ragged_pairs(rng, 40, 400, 50)

    def grads():
        xt = torch.as_tensor(x, device="cuda").requires_grad_(True)
        yt = torch.as_tensor(y, device="cuda").requires_grad_(True)
        AG.paired_dtw(xt, yt, 0.1).sum().backward()
        return xt.grad.cpu().numpy(), yt.grad.cpu().numpy()

    gx0, gy0 = grads()
    # one resident block: every warp's items run one after another
    monkeypatch.setenv("WB_GPU_BWD_WORKSPACE_MB", "0.01")
    gx1, gy1 = grads()
    np.testing.assert_allclose(gx1, gx0, rtol=0, atol=1e-6)
    np.testing.assert_allclose(gy1, gy0, rtol=0, atol=1e-6)
    assert os.environ["WB_GPU_BWD_WORKSPACE_MB"] == "0.01"


@pytest.mark.parametrize("lx,ly,g", [(300, 300, None), (300, 180, None), (140, 260, 0.05)])
def test_kept_directions_match_the_recompute_path(monkeypatch, lx, ly, g):
    # 40 x 9 pairs: the kept directions take 3.6-8.8 MB (12 batches of 32
    # items); a 2 MB budget sends the same call through the recompute path
    rng = np.random.default_rng(lx * 3 + ly)
    X = np.stack([_walk(rng, lx) for _ in range(40)])
    Y = np.stack([_walk(rng, ly) for _ in range(9)])
    gw = torch.as_tensor(rng.standard_normal((40, 9)), device="cuda")

    def run():
        xt = torch.as_tensor(X, device="cuda").requires_grad_(True)
        yt = torch.as_tensor(Y, device="cuda").requires_grad_(True)
        D = AG.dtw_matrix(xt, yt, 0.2, g=g)
        (D * gw).sum().backward()
        return (D.detach().cpu().numpy(), xt.grad.cpu().numpy(), yt.grad.cpu().numpy())

    d_keep, gx_keep, gy_keep = run()
    monkeypatch.setenv("WB_GPU_BWD_WORKSPACE_MB", "2")
    d_rec, gx_rec, gy_rec = run()
    metric = "dtw" if g is None else "wdtw"
    params = {"r": 0.2} if g is None else {"r": 0.2, "g": g}
    want = O.pairwise(X.astype(np.float64), Y.astype(np.float64), metric=metric,
                      metric_params=params)
    np.testing.assert_allclose(d_keep, want, rtol=1e-5)
    np.testing.assert_allclose(d_keep, d_rec, rtol=1e-6)
    # same directions and paths; only the order of the gradient atomics differs
    np.testing.assert_allclose(gx_keep, gx_rec, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(gy_keep, gy_rec, rtol=1e-5, atol=1e-6)
    assert np.count_nonzero(gx_keep) > 0.9 * gx_keep.size


def test_no_kept_directions_without_grad():
    # under no_grad (or with no input requiring a gradient) the plain forward runs
    rng = np.random.default_rng(8)
    X = torch.as_tensor(np.stack([_walk(rng, 64) for _ in range(5)]), device="cuda")
    Y = torch.as_tensor(np.stack([_walk(rng, 64) for _ in range(3)]), device="cuda")
    D0 = AG.dtw_matrix(X, Y, 0.3)
    assert not D0.requires_grad
    with torch.no_grad():
        D1 = AG.dtw_matrix(X.clone().requires_grad_(True), Y, 0.3)
    np.testing.assert_array_equal(D0.cpu().numpy(), D1.cpu().numpy())


def test_kept_walk_with_foreign_tables_gives_nan_not_reads():
    # a kept-direction buffer that no forward of this job filled: every strip
    # table gives column start 0 and word base 2^30, so the first direction-word
    # index of every walk lies outside the lane's words; the walk stops with
    # NaN gradients at its first row and column instead of reading there
    import ctypes

    from wildboar_gb300 import _lib
    from wildboar_gb300.distance import batched as B

    rng = np.random.default_rng(9)
    x = torch.as_tensor(np.stack([_walk(rng, 40) for _ in range(6)]), device="cuda")
    y = torch.as_tensor(np.stack([_walk(rng, 40) for _ in range(3)]), device="cuda")
    job = B.make_job(x, y, r=0.3, strip=16, block=128)
    nbytes = _lib.lib().wb_dtw32_keep_bytes(ctypes.byref(job))
    # one batch (18 items): tables of 3 strips (cs[3], base[3]) at the start
    strips = (40 - 2) // 16 + 1
    assert nbytes == ((2 * strips * 4 + 255) // 256 * 256
                      + 32 * ((strips * 40 + 7) // 8 * 8) * 4)
    host = np.zeros(nbytes, dtype=np.uint8)
    tables = host[:2 * strips * 4].view(np.int32)
    tables[:strips] = 0
    tables[strips:] = 1 << 30
    keep = torch.as_tensor(host, device="cuda")
    dist = torch.ones(job.n_items, dtype=torch.float64, device="cuda")
    gx = torch.zeros_like(x)
    gy = torch.zeros_like(y)
    _lib.check(_lib.lib().wb_dtw32_backward_keep(
        ctypes.byref(job), dist.data_ptr(), None, gx.data_ptr(), 40, gy.data_ptr(), 40,
        keep.data_ptr(), nbytes, torch.cuda.current_stream().cuda_stream))
    gx = gx.cpu().numpy()
    gy = gy.cpu().numpy()
    assert np.isnan(gx[:, -1]).all() and np.isnan(gy[:, -1]).all()
    assert np.all(gx[:, :-1] == 0) and np.all(gy[:, :-1] == 0)


@pytest.mark.parametrize("lx,ly", [(1, 1), (1, 5), (5, 1), (2, 3), (3, 17), (17, 2)])
def test_kept_directions_short_series(monkeypatch, lx, ly):
    # no strip (one row), one partial strip, a single column: the kept path and
    # the recompute path agree, distances match the oracle
    rng = np.random.default_rng(lx * 31 + ly)
    X = np.stack([_walk(rng, lx) for _ in range(5)])
    Y = np.stack([_walk(rng, ly) for _ in range(4)])
    gw = torch.as_tensor(rng.standard_normal((5, 4)), device="cuda")

    def run():
        xt = torch.as_tensor(X, device="cuda").requires_grad_(True)
        yt = torch.as_tensor(Y, device="cuda").requires_grad_(True)
        D = AG.dtw_matrix(xt, yt, 0.5)
        (D * gw).sum().backward()
        return (D.detach().cpu().numpy(), xt.grad.cpu().numpy(), yt.grad.cpu().numpy())

    d_keep, gx_keep, gy_keep = run()
    monkeypatch.setenv("WB_GPU_BWD_WORKSPACE_MB", "0.0001")
    d_rec, gx_rec, gy_rec = run()
    want = O.pairwise(X.astype(np.float64), Y.astype(np.float64), metric="dtw",
                      metric_params={"r": 0.5})
    np.testing.assert_allclose(d_keep, want, rtol=1e-5)
    np.testing.assert_allclose(d_rec, want, rtol=1e-5)
    np.testing.assert_allclose(gx_keep, gx_rec, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(gy_keep, gy_rec, rtol=1e-5, atol=1e-6)
    assert np.all(np.isfinite(gx_keep)) and np.all(np.isfinite(gy_keep))
