"""CPU check of the rule the early-abandoned argmin chunks rely on.

The reference's k-nearest loop (_ArgMinBatch.__call__, distance/_cdistance.pyx:
1302-1345) abandons candidate j iff its abandon key (the largest row minimum
of the recurrence, squared distances for dtw) exceeds the square of the heap's
k-th distance at that point.  The GPU form computes candidates in chunks
[a, b) and stops a pair once its running key exceeds the square of the k-th
distance D_a after the replayed prefix [0, a).  This test restates both
procedures in Python on small dtw problems and checks that every pair the
chunked form stops is abandoned by the sequential loop as well, and that the
heaps (order included) agree.
"""

import heapq
import math

import numpy as np

from oracle import oracle as O


def _dtw_rows(x, y, r):
    """Squared dtw with the reference's band, and the running abandon key
    after each row (rows 1 .. n-1)."""
    n, m = len(x), len(y)
    w = max(int(math.floor(min(n, m) * r)), 1)
    mx, mn = max(0, m - n) + w, max(0, n - m)
    prev = np.full(m, np.inf)
    acc = 0.0
    for j in range(min(m, mx)):
        acc += (x[0] - y[j]) ** 2
        prev[j] = acc
    keys = []
    kmax = -np.inf
    for i in range(1, n):
        cur = np.full(m, np.inf)
        js, je = max(0, i - mn - w + 1), min(m, i + mx)
        left = np.inf
        for j in range(js, je):
            up = prev[j]
            diag = prev[j - 1] if j > 0 else np.inf
            v = min(up, left, diag) + (x[i] - y[j]) ** 2
            cur[j] = v
            left = v
        kmax = max(kmax, np.min(cur[js:je]))
        keys.append(kmax)
        prev = cur
    return prev[m - 1], keys


class _Heap:
    """Heap.push of utils/_misc.pyx:18-107 by value (ties: earlier first)."""

    def __init__(self, k):
        self.k, self.items = k, []

    def push(self, j, d):
        if len(self.items) < self.k:
            heapq.heappush(self.items, (-d, -j))
        elif d < -self.items[0][0]:
            heapq.heapreplace(self.items, (-d, -j))

    def kth(self):
        return -self.items[0][0] if len(self.items) == self.k else math.inf

    def sorted(self):
        return sorted((-d, -j) for d, j in self.items)


def _sequential(xq, Y, r, k, cache):
    h = _Heap(k)
    abandoned = set()
    for j in range(len(Y)):
        d2, keys = cache[j]
        thr = h.kth() ** 2
        if keys and keys[-1] > thr:
            abandoned.add(j)
            continue
        d = math.sqrt(d2)
        if d < h.kth():
            h.push(j, d)
    return h.sorted(), abandoned


def _chunked(xq, Y, r, k, cache, first):
    h = _Heap(k)
    stopped = set()
    a, c = 0, first
    while a < len(Y):
        b = min(len(Y), a + c)
        bound = h.kth() ** 2            # the replayed prefix [0, a)
        for j in range(a, b):           # the chunk, in any order
            _, keys = cache[j]
            if any(kk > bound for kk in keys):
                stopped.add(j)
        for j in range(a, b):           # the exact replay of the chunk
            d2, keys = cache[j]
            if keys and keys[-1] > h.kth() ** 2:
                continue
            d = math.sqrt(d2)
            if d < h.kth():
                h.push(j, d)
        a, c = b, c * 2
    return h.sorted(), stopped


def test_chunk_bound_only_stops_pairs_the_reference_abandons():
    rng = np.random.default_rng(3)
    X = np.cumsum(rng.standard_normal((6, 18)), axis=1)
    Y = np.cumsum(rng.standard_normal((90, 18)), axis=1)
    Y[70] = X[2] + 0.01 * rng.standard_normal(18)
    for r in (0.1, 0.3, 1.0):
        for k in (1, 3):
            for q in range(len(X)):
                cache = [_dtw_rows(X[q], Y[j], r) for j in range(len(Y))]
                seq, abandoned = _sequential(X[q], Y, r, k, cache)
                for first in (1, 4, 16):
                    chunked, stopped = _chunked(X[q], Y, r, k, cache, first)
                    assert stopped <= abandoned
                    assert chunked == seq
                # the restated sequential loop agrees with the oracle's argmin
                oi, od = O.argmin(X[q:q + 1], Y, k=k, metric="dtw", metric_params={"r": r})
                np.testing.assert_allclose(sorted(od[0]), [d for d, _ in seq], rtol=1e-12)
                assert sorted(oi[0].tolist()) == sorted(j for _, j in seq)


def test_restatement_matches_the_oracle_distances():
    rng = np.random.default_rng(4)
    X = np.cumsum(rng.standard_normal((3, 15)), axis=1)
    Y = np.cumsum(rng.standard_normal((7, 15)), axis=1)
    for r in (0.1, 0.5, 1.0):
        want = O.pairwise(X, Y, metric="dtw", metric_params={"r": r})
        for q in range(3):
            for j in range(7):
                d2, _ = _dtw_rows(X[q], Y[j], r)
                assert math.isclose(math.sqrt(d2), want[q, j], rel_tol=1e-12)
