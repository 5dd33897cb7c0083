// envelope.cuh -- find_min_max (distance/_elastic.pyx:98-151), the streaming
// min / max envelope of the dtw lower bounds, with the reference's ring
// deques (:37-95) so that the envelopes carry its values exactly (including
// its single front pop per step, which can keep an expired index in the
// lower deque when both fronts expire at once).
#pragma once

#include "common.cuh"

namespace wb {

// the reference's ring deque (distance/_elastic.pyx:37-95): elements are
// pushed at `back`, which moves down; the front element sits just above
// `front`
struct DevDeque {
    int *q;
    int cap, size, front, back;
    __device__ void reset() {
        size = 0;
        front = 0;
        back = cap - 1;
    }
    __device__ void push_back(int v) {
        q[back] = v;
        back -= 1;
        if (back < 0) back = cap - 1;
        size += 1;
    }
    __device__ void pop_front() {
        front -= 1;
        if (front < 0) front = cap - 1;
        size -= 1;
    }
    __device__ void pop_back() {
        back = (back + 1) % cap;
        size -= 1;
    }
    __device__ int front_v() const { return q[front - 1 < 0 ? cap - 1 : front - 1]; }
    __device__ int back_v() const { return q[(back + 1) % cap]; }
};

// find_min_max (distance/_elastic.pyx:98-151)
// lower / upper element k at [k * ostride]
__device__ inline void sdtw_envelope(const double *T, int length, int r, double *lower,
                                     double *upper, DevDeque &dl, DevDeque &du,
                                     int64_t ostride = 1) {
    du.reset();
    dl.reset();
    du.push_back(0);
    dl.push_back(0);
    for (int i = 1; i < length; i++) {
        if (i > r) {
            const int k = i - r - 1;
            upper[k * ostride] = T[du.front_v()];
            lower[k * ostride] = T[dl.front_v()];
        }
        const double cur = T[i], prev = T[i - 1];
        if (cur > prev) {
            du.pop_back();
            while (du.size != 0 && cur > T[du.back_v()]) du.pop_back();
        } else {
            dl.pop_back();
            while (dl.size != 0 && cur < T[dl.back_v()]) dl.pop_back();
        }
        du.push_back(i);
        dl.push_back(i);
        if (i == 2 * r + 1 + du.front_v())
            du.pop_front();
        else if (i == 2 * r + 1 + dl.front_v())
            dl.pop_front();
    }
    for (int i = length; i < length + r + 1; i++) {
        const int k = i - r - 1;
        upper[k * ostride] = T[du.front_v()];
        lower[k * ostride] = T[dl.front_v()];
        if (i - du.front_v() >= 2 * r + 1) du.pop_front();
        if (i - dl.front_v() >= 2 * r + 1) dl.pop_front();
    }
}

}  // namespace wb
