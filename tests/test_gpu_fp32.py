"""FP32 forms: batched / ragged dtw and the differentiable dtw.

Bars: distances within 1e-5 relative of the FP64 oracle on the same (float32)
inputs; gradients within 1e-4 of central finite differences of the FP64
distance and of the gradient implied by the reference's dtw_alignment +
dtw_mapping path (distance/dtw.py:246-426, restated in the oracle).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA device", allow_module_level=True)

from oracle import oracle as O  # noqa: E402
from wildboar_gb300.distance import autograd as AG  # noqa: E402
from wildboar_gb300.distance import batched as B  # noqa: E402

DIST_RTOL = 1e-5


def _walk(rng, shape):
    return np.cumsum(rng.standard_normal(shape), axis=-1).astype(np.float32)


@pytest.mark.parametrize("r", [0.0, 0.1, 0.2, 1.0])
@pytest.mark.parametrize("lx,ly", [(64, 64), (100, 77), (40, 130), (257, 257)])
@pytest.mark.parametrize("strip", [4, 16, 32])
def test_dtw32_grid_vs_fp64_oracle(r, lx, ly, strip):
    rng = np.random.default_rng(lx * 1000 + ly)
    X = _walk(rng, (37, lx))
    Y = _walk(rng, (9, ly))
    xt = torch.as_tensor(X, device="cuda")
    yt = torch.as_tensor(Y, device="cuda")
    got = B.dtw32(xt, yt, r=r, strip=strip).view(9, 37).t().cpu().numpy()
    want = O.pairwise(X.astype(np.float64), Y.astype(np.float64), metric="dtw",
                      metric_params={"r": r})
    np.testing.assert_allclose(got, want, rtol=DIST_RTOL, atol=1e-9)


def test_wdtw32_vs_fp64_oracle():
    rng = np.random.default_rng(2)
    X = _walk(rng, (20, 90))
    Y = _walk(rng, (11, 90))
    w = B.logistic_weights(90, 0.1, "cuda")
    got = B.dtw32(torch.as_tensor(X, device="cuda"), torch.as_tensor(Y, device="cuda"),
                  r=0.3, weights=w).view(11, 20).t().cpu().numpy()
    want = O.pairwise(X.astype(np.float64), Y.astype(np.float64), metric="wdtw",
                      metric_params={"r": 0.3, "g": 0.1})
    # float32 weights vs the oracle's float64 weights: 1e-7 relative per cell
    np.testing.assert_allclose(got, want, rtol=DIST_RTOL, atol=1e-9)


def _ragged(rng, n, d, L, lo, hi):
    x = np.full((n, d, L), np.nan, dtype=np.float32)
    lens = rng.integers(lo, hi + 1, size=(n, d))
    for i in range(n):
        for k in range(d):
            x[i, k, : lens[i, k]] = _walk(rng, (lens[i, k],))
    return x, lens


def test_paired_ragged_batch_vs_oracle():
    rng = np.random.default_rng(7)
    n, d, L = 300, 3, 180
    x, lx = _ragged(rng, n, d, L, 8, L)
    y, ly = _ragged(rng, n, d, L, 8, L)
    got = B.paired_dtw_batch(torch.as_tensor(x, device="cuda"),
                             torch.as_tensor(y, device="cuda"), r=0.1, tune=False)
    got = got.cpu().numpy()
    want = np.zeros(n)
    for i in range(n):
        acc = 0.0
        for k in range(d):
            acc += O.distance_1d(x[i, k, : lx[i, k]].astype(np.float64),
                                 y[i, k, : ly[i, k]].astype(np.float64), metric="dtw",
                                 metric_params={"r": 0.1})
        want[i] = acc / d
    np.testing.assert_allclose(got, want, rtol=DIST_RTOL, atol=1e-9)


TILES = [(8, 128), (16, 256), (24, 128), (32, 64)]


@pytest.mark.parametrize("tile", TILES, ids=lambda t: f"s{t[0]}-b{t[1]}")
def test_ragged_batch_tiles_vs_oracle(tile):
    # ragged lengths from 1 to L on both sides, so the lanes of a warp mix
    # both orientations (n < m, n > m) and single-element series
    rng = np.random.default_rng(17)
    n, d, L = 240, 2, 300
    x, lx = _ragged(rng, n, d, L, 1, L)
    y, ly = _ragged(rng, n, d, L, 1, L)
    plan = B.plan_pairs(torch.as_tensor(x, device="cuda"), torch.as_tensor(y, device="cuda"),
                        0.1, tune=False, tile=tile)
    got = B.combine_dims(plan, B.run_plan(plan)).cpu().numpy()
    want = np.zeros(n)
    for i in range(n):
        acc = 0.0
        for k in range(d):
            acc += O.distance_1d(x[i, k, : lx[i, k]].astype(np.float64),
                                 y[i, k, : ly[i, k]].astype(np.float64), metric="dtw",
                                 metric_params={"r": 0.1})
        want[i] = acc / d
    np.testing.assert_allclose(got, want, rtol=DIST_RTOL, atol=1e-9)


@pytest.mark.parametrize("r", [0.0, 0.1, 1.0])
@pytest.mark.parametrize("lx,ly", [(64, 64), (130, 41), (41, 130), (1, 50), (50, 1)])
@pytest.mark.parametrize("strip", [8, 24])
@pytest.mark.parametrize("g", [None, 0.1])
def test_grid_shapes_vs_fp64_oracle(r, lx, ly, strip, g):
    rng = np.random.default_rng(lx * 1000 + ly)
    X = _walk(rng, (21, lx))
    Y = _walk(rng, (7, ly))
    xt = torch.as_tensor(X, device="cuda")
    yt = torch.as_tensor(Y, device="cuda")
    w = None if g is None else B.logistic_weights(max(lx, ly), g, "cuda")
    got = B.dtw32(xt, yt, r=r, weights=w, strip=strip).view(7, 21).t().cpu().numpy()
    metric, params = ("dtw", {"r": r}) if g is None else ("wdtw", {"r": r, "g": g})
    want = O.pairwise(X.astype(np.float64), Y.astype(np.float64), metric=metric,
                      metric_params=params)
    np.testing.assert_allclose(got, want, rtol=DIST_RTOL, atol=1e-9)


def test_ragged_wdtw_batch_vs_oracle():
    # one side of every pair has the full length L, so the oracle's weights
    # (length max(n, m) of the pair) are the kernel's table of length L; the
    # other side is ragged, on x for half the pairs and on y for the rest
    rng = np.random.default_rng(23)
    n, L = 160, 120
    x, lx = _ragged(rng, n, 1, L, 2, L)
    y, ly = _ragged(rng, n, 1, L, 2, L)
    full_x = rng.random(n) < 0.5
    for i in range(n):
        if full_x[i]:
            x[i, 0] = _walk(rng, (L,))
            lx[i, 0] = L
        else:
            y[i, 0] = _walk(rng, (L,))
            ly[i, 0] = L
    w = B.logistic_weights(L, 0.05, "cuda")
    xt = torch.as_tensor(x[:, 0].copy(), device="cuda")
    yt = torch.as_tensor(y[:, 0].copy(), device="cuda")
    xl, yl = B.series_lengths(xt), B.series_lengths(yt)
    item = B.bucket_order(xl, yl, 0.2, transpose=False).to(torch.int32).contiguous()
    got = B.dtw32(xt, yt, r=0.2, x_lengths=xl, y_lengths=yl, item_x=item, item_y=item,
                  weights=w, strip=8).cpu().numpy()
    for t, i in enumerate(item.cpu().numpy()):
        want = O.distance_1d(x[i, 0, : lx[i, 0]].astype(np.float64),
                             y[i, 0, : ly[i, 0]].astype(np.float64), metric="wdtw",
                             metric_params={"r": 0.2, "g": 0.05})
        assert abs(got[t] - want) <= DIST_RTOL * want, (t, got[t], want)


def test_batched_graph_replay_matches_direct():
    rng = np.random.default_rng(8)
    x, _ = _ragged(rng, 200, 2, 150, 20, 150)
    y, _ = _ragged(rng, 200, 2, 150, 20, 150)
    xt = torch.as_tensor(x, device="cuda")
    yt = torch.as_tensor(y, device="cuda")
    direct = B.paired_dtw_batch(xt, yt, r=0.1, tune=False)
    runner = B.BatchedDTW(xt, yt, r=0.1, tune=False, graph=True)
    a = runner.run().clone()
    b = runner.run().clone()
    torch.testing.assert_close(a, direct, rtol=0, atol=0)
    torch.testing.assert_close(b, direct, rtol=0, atol=0)
    # new data in the same buffers is picked up by the replay
    xt.copy_(torch.as_tensor(y, device="cuda"))
    c = runner.run().clone()
    torch.testing.assert_close(c, B.paired_dtw_batch(xt, yt, r=0.1, tune=False), rtol=0,
                               atol=0)
    assert float(c.abs().max()) == 0.0


def test_autotuner_returns_valid_config(tmp_path):
    rng = np.random.default_rng(9)
    x, _ = _ragged(rng, 64, 1, 120, 30, 120)
    xt = torch.as_tensor(x, device="cuda")
    tuner = B.Autotuner(path=str(tmp_path / "tune.json"))
    plan = B.plan_pairs(xt, xt, 0.1, tune=False)
    s, b = tuner.pick(plan["xf"], plan["yf"], r=0.1, x_lengths=plan["xl"],
                      y_lengths=plan["yl"], item_x=plan["item_x"], item_y=plan["item_y"])
    assert s in B.STRIPS and b in B.BLOCKS
    assert (tmp_path / "tune.json").exists()


# ---------------------------------------------------------------- gradients


def _path_grad(x, y, r):
    """Gradient implied by the reference path: dtw_alignment + dtw_mapping."""
    al = O.dtw_alignment(x, y, r=r)
    D = np.sqrt(al[-1, -1])
    gx = np.zeros_like(x)
    gy = np.zeros_like(y)
    for i, j in O.dtw_mapping(al):
        g = (x[i] - y[j]) / D
        gx[i] += g
        gy[j] -= g
    return D, gx, gy


@pytest.mark.parametrize("lx,ly,r", [(64, 64, 0.2), (50, 50, 1.0), (80, 80, 0.1)])
def test_gradient_vs_alignment_path(lx, ly, r):
    rng = np.random.default_rng(lx + ly)
    X = _walk(rng, (6, lx))
    Y = _walk(rng, (4, ly))
    xt = torch.as_tensor(X, device="cuda").requires_grad_(True)
    yt = torch.as_tensor(Y, device="cuda").requires_grad_(True)
    D = AG.dtw_matrix(xt, yt, r)
    gw = torch.as_tensor(rng.standard_normal(D.shape), device="cuda")
    (D * gw).sum().backward()
    gx_want = np.zeros_like(X, dtype=np.float64)
    gy_want = np.zeros_like(Y, dtype=np.float64)
    for i in range(6):
        for j in range(4):
            d, gx, gy = _path_grad(X[i].astype(np.float64), Y[j].astype(np.float64), r)
            gx_want[i] += gw[i, j].item() * gx
            gy_want[j] += gw[i, j].item() * gy
            assert abs(D[i, j].item() - d) <= DIST_RTOL * d
    np.testing.assert_allclose(xt.grad.cpu().numpy(), gx_want, rtol=0, atol=1e-4)
    np.testing.assert_allclose(yt.grad.cpu().numpy(), gy_want, rtol=0, atol=1e-4)


def test_gradient_vs_finite_differences():
    rng = np.random.default_rng(13)
    L = 48
    x = _walk(rng, (L,)).astype(np.float64)
    y = _walk(rng, (L,)).astype(np.float64)
    r = 0.2
    xt = torch.as_tensor(x[None].astype(np.float32), device="cuda").requires_grad_(True)
    yt = torch.as_tensor(y[None].astype(np.float32), device="cuda").requires_grad_(True)
    AG.dtw_matrix(xt, yt, r).sum().backward()
    gx = xt.grad.cpu().numpy()[0]
    gy = yt.grad.cpu().numpy()[0]
    h = 1e-5
    checked = 0
    for i in range(L):
        for arr, g in ((x, gx), (y, gy)):
            a = arr.copy()
            a[i] += h
            dp = O.distance_1d(x if arr is y else a, a if arr is y else y, metric="dtw",
                               metric_params={"r": r})
            a[i] -= 2 * h
            dm = O.distance_1d(x if arr is y else a, a if arr is y else y, metric="dtw",
                               metric_params={"r": r})
            fd = (dp - dm) / (2 * h)
            # away from ties the path does not move within +-h: one-sided
            # differences agree with the central one
            d0 = O.distance_1d(x, y, metric="dtw", metric_params={"r": r})
            if abs((dp - d0) / h - fd) > 1e-3 * (1 + abs(fd)):
                continue
            assert abs(g[i] - fd) <= 1e-4, (i, g[i], fd)
            checked += 1
    assert checked > L  # most coordinates are away from ties


def test_unequal_lengths_and_wdtw_gradient():
    rng = np.random.default_rng(21)
    X = _walk(rng, (3, 70))
    Y = _walk(rng, (2, 55))
    xt = torch.as_tensor(X, device="cuda").requires_grad_(True)
    yt = torch.as_tensor(Y, device="cuda").requires_grad_(True)
    D = AG.dtw_matrix(xt, yt, 0.3, g=0.05)
    D.sum().backward()
    want = O.pairwise(X.astype(np.float64), Y.astype(np.float64), metric="wdtw",
                      metric_params={"r": 0.3, "g": 0.05})
    np.testing.assert_allclose(D.detach().cpu().numpy(), want, rtol=DIST_RTOL)
    # finite differences on a few coordinates of x[0]
    x0 = X[0].astype(np.float64)
    for i in (0, 10, 35, 69):
        h = 1e-5
        a = x0.copy()
        a[i] += h
        fp = sum(O.distance_1d(a, Y[j].astype(np.float64), metric="wdtw",
                               metric_params={"r": 0.3, "g": 0.05}) for j in range(2))
        a[i] -= 2 * h
        fm = sum(O.distance_1d(a, Y[j].astype(np.float64), metric="wdtw",
                               metric_params={"r": 0.3, "g": 0.05}) for j in range(2))
        assert abs(xt.grad[0, i].item() - (fp - fm) / (2 * h)) <= 1e-4


def test_barycenter_step_decreases_loss():
    rng = np.random.default_rng(5)
    protos = _walk(rng, (4, 64))
    x = np.concatenate([p + 0.1 * rng.standard_normal((32, 64)).astype(np.float32)
                        for p in protos])
    xt = torch.as_tensor(x, device="cuda")
    c0 = torch.as_tensor(protos + rng.standard_normal((4, 64)).astype(np.float32),
                         device="cuda")
    _, losses = AG.barycenter_kmeans(xt, c0, r=0.2, steps=30, lr=0.05)
    assert losses[-1] < losses[0]
