// argmin.cuh -- the reference's k-nearest bookkeeping on the device: the
// eadistance threshold each metric's recurrence abandons at, and Heap.push.
#pragma once

#include "elastic.cuh"

namespace wb {

// threshold the recurrence of `metric` compares its row minima with when
// eadistance is called with the current k-th distance (distance/_elastic.pyx
// and distance/_metric.pyx, the *Metric.eadistance / _eadistance methods)
__device__ __forceinline__ double abandon_threshold(int metric, double distance, int xl, int yl) {
    switch (metric) {
        case WB_DTW:
        case WB_WDTW:
        case WB_DDTW:
        case WB_WDDTW:
        case WB_ADTW:
            return distance * distance;
        case WB_LCSS:
        case WB_WLCSS: {
            if (isinf(distance)) return __longlong_as_double(0x7ff0000000000000LL);
            double ml = (double)(xl < yl ? xl : yl);
            return ml - distance * ml;
        }
        case WB_EDR:
            return distance * (double)(xl > yl ? xl : yl);
        default:
            return distance;
    }
}

// Heap.push and its sift helpers (utils/_misc.pyx:18-107)
__device__ inline void heap_push(int64_t *hi, double *hv, int64_t &n, int64_t k, int64_t index,
                          double value) {
    if (n == 0) {
        hi[0] = index;
        hv[0] = value;
        n = 1;
        return;
    }
    if (n < k) {
        // append, then move toward the root while larger than the parent
        int64_t pos = n;
        n += 1;
        while (pos > 0) {
            int64_t parent = (pos - 1) >> 1;
            if (value > hv[parent]) {
                hi[pos] = hi[parent];
                hv[pos] = hv[parent];
                pos = parent;
                continue;
            }
            break;
        }
        hi[pos] = index;
        hv[pos] = value;
    } else if (hv[0] > value) {
        // replace the root: move it to a leaf along larger children, then
        // back toward the root (heapq's _siftup)
        int64_t pos = 0, end = k;
        int64_t child = 1;
        while (child < end) {
            int64_t right = child + 1;
            if (right < end && hv[child] < hv[right]) child = right;
            hi[pos] = hi[child];
            hv[pos] = hv[child];
            pos = child;
            child = 2 * pos + 1;
        }
        while (pos > 0) {
            int64_t parent = (pos - 1) >> 1;
            if (value > hv[parent]) {
                hi[pos] = hi[parent];
                hv[pos] = hv[parent];
                pos = parent;
                continue;
            }
            break;
        }
        hi[pos] = index;
        hv[pos] = value;
    }
}

}  // namespace wb
