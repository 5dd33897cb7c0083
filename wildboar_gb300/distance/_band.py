"""Band geometry of the elastic recurrences.

``compute_r`` is ``_compute_r`` of the reference (distance/_elastic.pyx:
1924-1925); ``band_cells`` counts the cells the reference's two-row recurrence
evaluates for an (n x m) pair: rows i = 0..n-1 cover columns
[max(0, i - max(0, n-m) - r + 1), min(m, i + max(0, m-n) + r)).
"""

import math


def compute_r(length, r):
    return int(max(math.floor(length * r), 1))


def band_cells(n, m, r):
    """Evaluated band cells of one (n, m) pair with band fraction r."""
    w = compute_r(min(n, m), r)
    mx = max(0, m - n) + w
    mn = max(0, n - m)
    total = 0
    for i in range(n):
        total += min(m, i + mx) - max(0, i - mn - w + 1)
    return total
