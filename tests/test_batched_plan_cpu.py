"""Host logic of the batched FP32 form on the CPU: the closed-form band cell
count (the GCUPS numerator and part of the sort key) against the per-row sum
of dtw_distance's loop bounds (distance/_elastic.pyx:869-940), and the item
order the persistent kernel's warps take."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from wildboar_gb300.distance import batched as B  # noqa: E402


def _cells(n, m, r):
    if n == 0 or m == 0:
        return 0
    w = max(int(np.floor(min(n, m) * r)), 1)
    mx = max(0, m - n) + w
    mn = max(0, n - m)
    return sum(min(m, i + mx) - max(0, i - mn - w + 1) for i in range(n))


def test_band_cost_matches_the_row_sum():
    rng = np.random.default_rng(0)
    cases = [(0, 5), (5, 0), (1, 1), (1, 7), (7, 1), (2, 2), (3, 200), (200, 3)]
    cases += [tuple(int(v) for v in rng.integers(1, 700, 2)) for _ in range(60)]
    for r in (0.0, 0.05, 0.1, 0.37, 1.0):
        n = torch.tensor([c[0] for c in cases])
        m = torch.tensor([c[1] for c in cases])
        got = B.band_cost(n, m, r).tolist()
        want = [_cells(a, b, r) for a, b in cases]
        assert got == want, r


def test_bucket_order_groups_equal_strips_and_widths():
    rng = np.random.default_rng(1)
    n = torch.as_tensor(rng.integers(32, 2049, 5000))
    m = torch.as_tensor(rng.integers(32, 2049, 5000))
    order = B.bucket_order(n, m, 0.1)
    assert sorted(order.tolist()) == list(range(5000))
    nn, mm = n[order], m[order]
    rows = torch.minimum(nn, mm)
    w = torch.clamp(torch.floor(rows.double() * 0.1), min=1).long()
    cols = torch.minimum(torch.maximum(nn, mm), (mm - nn).abs() + 2 * w)
    strips = (rows - 2).clamp(min=0) // 32
    key = strips * 8192 + cols
    # descending (strip count, band width): the queue ends on the smallest problems
    assert torch.all(key[:-1] >= key[1:])
    assert torch.all(strips[:-1] >= strips[1:])
    # without transposition the orientation comes first
    o2 = B.bucket_order(n, m, 0.1, transpose=False)
    flags = (n[o2] > m[o2]).long()
    assert torch.all(flags[:-1] >= flags[1:])
