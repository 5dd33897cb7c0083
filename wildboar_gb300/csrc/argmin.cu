// argmin.cu -- k-nearest-neighbour selection with the reference's heap.
//
// The distance kernel has produced, for every (query i, candidate j), the
// distance the metric's eadistance returns when it does not abandon, and the
// abandon key K(i, j): the largest per-row minimum of the recurrence.  The
// reference abandons a pair iff some checked row's minimum exceeds the
// threshold, i.e. iff K(i, j) > threshold.  Replaying _ArgMinBatch.__call__
// (distance/_cdistance.pyx:1302-1345) over j in order with those two numbers
// reproduces its pushes, its heap (utils/_misc.pyx:18-107) and therefore its
// output order exactly, including for metrics whose abandoning is not
// monotone (negative adtw penalty, band-edge zeros of lcss/edr/erp/msm/twe).

#include "argmin.cuh"

namespace wb {

__global__ void argmin_replay_kernel(const ArgminJob J) {
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < J.nx;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t *hi = J.heap_idx + i * J.k;
        double *hv = J.heap_val + i * J.k;
        const double *drow = J.dist + i * J.ny;
        const double *krow = J.key ? J.key + i * J.ny : nullptr;
        const double *lb = J.lower_bound ? J.lower_bound + i * J.ny : nullptr;
        double distance = INF;
        int64_t n = 0;
        if (J.resume) {
            n = J.state_n[i];
            distance = J.state_dist[i];
        }
        const int64_t j1 = J.j1 < 0 ? J.ny : J.j1;
        if (!J.never_push) {
            for (int64_t j = J.j0; j < j1; j++) {
                if (lb && lb[j] >= distance) continue;
                if (krow) {
                    double thr = abandon_threshold(J.metric, distance, J.xl, J.yl);
                    if (krow[j] > thr) continue;  // abandoned: eadistance returns inf
                }
                double d = drow[j];
                if (d < distance) {
                    heap_push(hi, hv, n, J.k, j, d);
                    distance = (n == J.k) ? hv[0] : INF;
                }
            }
        }
        if (J.state_n) {
            J.state_n[i] = n;
            J.state_dist[i] = distance;
        }
        if (!J.finish) continue;
        for (int64_t t = 0; t < J.k; t++) {
            J.out_idx[i * J.k + t] = t < n ? hi[t] : 0;
            J.out_dist[i * J.k + t] = t < n ? hv[t] : 0.0;
        }
    }
}

int launch_argmin_replay(const ArgminJob &J, cudaStream_t s) {
    if (J.nx == 0) return WB_OK;
    int block = 128;
    int64_t g = (J.nx + block - 1) / block;
    argmin_replay_kernel<<<(int)g, block, 0, s>>>(J);
    WB_LAUNCH_CHECK("argmin_replay_kernel");
    return WB_OK;
}

}  // namespace wb
