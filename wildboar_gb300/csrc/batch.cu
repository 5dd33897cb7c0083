// batch.cu -- entry points shaped for the reference's compiled callers, so
// that the proximity trees (tree/_cptree.pyx) and the shapelet transforms
// (transform/_cshapelet.pyx) can hand their metric calls to the GPU in
// batches instead of one pair at a time.
//
//  * wb_nearest_pivot: many nodes at once.  A proximity-tree node sends each
//    of its samples to the branch of the nearest pivot (_partition_pivots,
//    tree/_cptree.pyx:869-894, and find_min_branch, :273-290: the first
//    pivot with the strictly smallest distance, on the metric's full
//    distance -- not argmin_distance, whose early abandoning can pick another
//    pivot for lcss).  Each group (node) has its samples, its pivots and a
//    metric slot; groups run back to back on one stream: rows gathered on the
//    device, the (samples x pivots) distances, a first-strict-minimum pass.
//    A sample whose distances are all +inf or NaN keeps the branch of the
//    previous sample of its group (_partition_pivots does not reset its
//    running pivot between samples), -1 for the first.
//  * wb_subsequence_distance_views: shapelets given as views into a series
//    array (sample, dim, start, length) with the statistics the caller's
//    SubsequenceView holds (_ts_view_update_statistics,
//    distance/_cdistance.pyx:167-185), gathered on the device and scanned
//    against every target series (transient_distance / persistent_distance,
//    :265-299: a zero std is used as 1), as the shapelet transform fills its
//    attribute columns.

#include <algorithm>
#include <vector>

#include "common.cuh"

extern "C" int wb_pairwise_distance(const wb_series *x, const wb_series *y, int64_t dim,
                                    int32_t metric, const wb_params *params, double *out,
                                    int32_t out_on_device, void *stream_);
extern "C" int wb_pairwise_subsequence_distance(
    const double *shapelets, const int64_t *offsets, const int64_t *lengths,
    const double *means, const double *stds, int64_t m, const wb_series *x, int64_t dim,
    int32_t metric, const wb_params *params, double *out_dist, int64_t *out_idx,
    int32_t out_on_device, void *stream_);

namespace wb {

namespace {

// rows idx[0 .. n) of dim `dim` of a (., d, T) device array into (n, 1, T)
__global__ void gather_rows_kernel(const double *x, int64_t d, int64_t T, int64_t dim,
                                   const int64_t *idx, int64_t n, double *out) {
    for (int64_t r = blockIdx.x; r < n; r += gridDim.x) {
        const double *src = x + (idx[r] * d + dim) * T;
        for (int64_t t = threadIdx.x; t < T; t += blockDim.x) out[r * T + t] = src[t];
    }
}

// views (sample, dim, start, length) of a (., d, T) device array, packed
__global__ void gather_views_kernel(const double *x, int64_t d, int64_t T, const int64_t *vi,
                                    const int64_t *vd, const int64_t *vs, const int64_t *vl,
                                    const int64_t *off, int64_t m, double *out) {
    for (int64_t v = blockIdx.x; v < m; v += gridDim.x) {
        const double *src = x + (vi[v] * d + vd[v]) * T + vs[v];
        for (int64_t t = threadIdx.x; t < vl[v]; t += blockDim.x) out[off[v] + t] = src[t];
    }
}

// first pivot with the strictly smallest distance of every row of D (ns, np);
// -1 when no distance is below +inf
__global__ void first_min_kernel(const double *D, int64_t ns, int64_t np, int64_t *branch,
                                 double *dist) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= ns) return;
    double best = __longlong_as_double(0x7ff0000000000000LL);
    int64_t arg = -1;
    for (int64_t c = 0; c < np; c++) {
        const double v = D[r * np + c];
        if (v < best) {
            best = v;
            arg = c;
        }
    }
    branch[r] = arg;
    dist[r] = best;
}

struct DevBuf {
    void *p = nullptr;
    cudaStream_t s = nullptr;
    ~DevBuf() {
        if (p) cudaFreeAsync(p, s);
    }
};

int dev_alloc(DevBuf &b, size_t bytes, cudaStream_t s) {
    b.s = s;
    if (bytes == 0) bytes = 8;
    cudaError_t e = cudaMallocAsync(&b.p, bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync");
    return WB_OK;
}

}  // namespace

}  // namespace wb

using namespace wb;

extern "C" int wb_nearest_pivot(const wb_series *x, int64_t dim, int64_t n_groups,
                                const int64_t *sample_ptr, const int64_t *samples,
                                const int64_t *pivot_ptr, const int64_t *pivots,
                                const int32_t *group_slot, const int32_t *slot_metric,
                                const wb_params *slot_params, int32_t n_slots,
                                int64_t *out_branch, double *out_dist, void *stream) {
    WB_TRACE();
    const cudaStream_t s = (cudaStream_t)stream;
    if (!x || !x->data) return fail(WB_EINVAL, "x is NULL");
    if (x->dtype != WB_F64) return fail(WB_EINVAL, "x must be float64");
    if (dim < 0 || dim >= x->n_dims) return fail(WB_EINVAL, "dim out of range");
    if (n_groups < 0 || n_slots < 1) return fail(WB_EINVAL, "invalid group or slot count");
    if (n_groups == 0) return WB_OK;
    if (!sample_ptr || !samples || !pivot_ptr || !pivots || !group_slot || !slot_metric ||
        !slot_params || !out_branch || !out_dist)
        return fail(WB_EINVAL, "NULL array");
    const int64_t T = x->n_timestep, d = x->n_dims;
    // the series on the device once
    const double *xd = static_cast<const double *>(x->data);
    DevBuf xbuf;
    if (!x->on_device) {
        WB_TRY(dev_alloc(xbuf, (size_t)x->n * d * T * 8, s));
        WB_CUDA(cudaMemcpyAsync(xbuf.p, x->data, (size_t)x->n * d * T * 8,
                                cudaMemcpyHostToDevice, s));
        xd = static_cast<const double *>(xbuf.p);
    }
    int64_t max_s = 0, max_p = 0;
    for (int64_t g = 0; g < n_groups; g++) {
        const int64_t ns = sample_ptr[g + 1] - sample_ptr[g];
        const int64_t np = pivot_ptr[g + 1] - pivot_ptr[g];
        if (ns < 0 || np < 0) return fail(WB_EINVAL, "group pointers must not decrease");
        if (group_slot[g] < 0 || group_slot[g] >= n_slots)
            return fail(WB_EINVAL, "group metric slot out of range");
        max_s = std::max(max_s, ns);
        max_p = std::max(max_p, np);
    }
    const int64_t n_idx = sample_ptr[n_groups], n_piv = pivot_ptr[n_groups];
    for (int64_t i = 0; i < n_idx; i++)
        if (samples[i] < 0 || samples[i] >= x->n) return fail(WB_EINVAL, "sample out of range");
    for (int64_t i = 0; i < n_piv; i++)
        if (pivots[i] < 0 || pivots[i] >= x->n) return fail(WB_EINVAL, "pivot out of range");
    DevBuf ibuf, rows_s, rows_p, obuf_i, obuf_d, dmat;
    WB_TRY(dev_alloc(dmat, (size_t)max_s * max_p * 8, s));
    WB_TRY(dev_alloc(ibuf, (size_t)(n_idx + n_piv) * 8, s));
    WB_TRY(dev_alloc(rows_s, (size_t)max_s * T * 8, s));
    WB_TRY(dev_alloc(rows_p, (size_t)max_p * T * 8, s));
    WB_TRY(dev_alloc(obuf_i, (size_t)n_idx * 8, s));
    WB_TRY(dev_alloc(obuf_d, (size_t)n_idx * 8, s));
    int64_t *di = static_cast<int64_t *>(ibuf.p);
    WB_CUDA(cudaMemcpyAsync(di, samples, n_idx * 8, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(di + n_idx, pivots, n_piv * 8, cudaMemcpyHostToDevice, s));
    int64_t *oi = static_cast<int64_t *>(obuf_i.p);
    double *od = static_cast<double *>(obuf_d.p);
    for (int64_t g = 0; g < n_groups; g++) {
        const int64_t s0 = sample_ptr[g], ns = sample_ptr[g + 1] - s0;
        const int64_t p0 = pivot_ptr[g], np = pivot_ptr[g + 1] - p0;
        if (ns == 0) continue;
        if (np == 0) {
            // no pivot: branch -1 at +inf, as the reference's loop leaves them
            std::vector<int64_t> b(ns, -1);
            std::vector<double> v(ns, __builtin_inf());
            WB_CUDA(cudaMemcpyAsync(oi + s0, b.data(), ns * 8, cudaMemcpyHostToDevice, s));
            WB_CUDA(cudaMemcpyAsync(od + s0, v.data(), ns * 8, cudaMemcpyHostToDevice, s));
            WB_CUDA(cudaStreamSynchronize(s));
            continue;
        }
        gather_rows_kernel<<<(unsigned)std::min<int64_t>(ns, 65535), 128, 0, s>>>(
            xd, d, T, dim, di + s0, ns, static_cast<double *>(rows_s.p));
        WB_LAUNCH_CHECK("gather_rows_kernel");
        gather_rows_kernel<<<(unsigned)std::min<int64_t>(np, 65535), 128, 0, s>>>(
            xd, d, T, dim, di + n_idx + p0, np, static_cast<double *>(rows_p.p));
        WB_LAUNCH_CHECK("gather_rows_kernel");
        wb_series qs{rows_s.p, ns, 1, T, WB_F64, 1};
        wb_series ps{rows_p.p, np, 1, T, WB_F64, 1};
        const int32_t slot = group_slot[g];
        double *D = static_cast<double *>(dmat.p);
        WB_TRY(wb_pairwise_distance(&qs, &ps, 0, slot_metric[slot], &slot_params[slot], D, 1,
                                    (void *)s));
        first_min_kernel<<<(unsigned)((ns + 127) / 128), 128, 0, s>>>(D, ns, np, oi + s0,
                                                                       od + s0);
        WB_LAUNCH_CHECK("first_min_kernel");
    }
    WB_CUDA(cudaMemcpyAsync(out_branch, oi, n_idx * 8, cudaMemcpyDeviceToHost, s));
    WB_CUDA(cudaMemcpyAsync(out_dist, od, n_idx * 8, cudaMemcpyDeviceToHost, s));
    WB_CUDA(cudaStreamSynchronize(s));
    // the running pivot of _partition_pivots carries over samples without one
    for (int64_t g = 0; g < n_groups; g++) {
        int64_t carry = -1;
        for (int64_t i = sample_ptr[g]; i < sample_ptr[g + 1]; i++) {
            if (out_branch[i] < 0)
                out_branch[i] = carry;
            else
                carry = out_branch[i];
        }
    }
    return WB_OK;
}

extern "C" int wb_subsequence_distance_views(const wb_series *x, const int64_t *view_sample,
                                             const int64_t *view_dim,
                                             const int64_t *view_start,
                                             const int64_t *view_length,
                                             const double *view_mean, const double *view_std,
                                             int64_t m, const wb_series *target, int64_t dim,
                                             int32_t metric, const wb_params *params,
                                             double *out_dist, int64_t *out_idx,
                                             void *stream) {
    WB_TRACE();
    const cudaStream_t s = (cudaStream_t)stream;
    if (!x || !x->data || !target) return fail(WB_EINVAL, "x or target is NULL");
    if (x->dtype != WB_F64) return fail(WB_EINVAL, "x must be float64");
    if (m < 0) return fail(WB_EINVAL, "negative number of views");
    if (m == 0 || target->n == 0) return WB_OK;
    if (!view_sample || !view_dim || !view_start || !view_length || !view_mean || !view_std)
        return fail(WB_EINVAL, "NULL view array");
    const int64_t T = x->n_timestep, d = x->n_dims;
    std::vector<int64_t> off(m);
    int64_t total = 0;
    for (int64_t v = 0; v < m; v++) {
        if (view_sample[v] < 0 || view_sample[v] >= x->n || view_dim[v] < 0 ||
            view_dim[v] >= d || view_start[v] < 0 || view_length[v] < 1 ||
            view_start[v] + view_length[v] > T)
            return fail(WB_EINVAL, "view " + std::to_string(v) + " is outside x");
        off[v] = total;
        total += view_length[v];
    }
    std::vector<int64_t> len(view_length, view_length + m);
    if (!x->on_device) {
        // host: pack on the host and hand host arrays over
        std::vector<double> packed(total);
        const double *base = static_cast<const double *>(x->data);
        for (int64_t v = 0; v < m; v++)
            std::copy_n(base + (view_sample[v] * d + view_dim[v]) * T + view_start[v],
                        view_length[v], packed.begin() + off[v]);
        if (target->on_device) {
            DevBuf p, o, l, mu, sd;
            WB_TRY(dev_alloc(p, total * 8, s));
            WB_TRY(dev_alloc(o, m * 8, s));
            WB_TRY(dev_alloc(l, m * 8, s));
            WB_TRY(dev_alloc(mu, m * 8, s));
            WB_TRY(dev_alloc(sd, m * 8, s));
            WB_CUDA(cudaMemcpyAsync(p.p, packed.data(), total * 8, cudaMemcpyHostToDevice, s));
            WB_CUDA(cudaMemcpyAsync(o.p, off.data(), m * 8, cudaMemcpyHostToDevice, s));
            WB_CUDA(cudaMemcpyAsync(l.p, len.data(), m * 8, cudaMemcpyHostToDevice, s));
            WB_CUDA(cudaMemcpyAsync(mu.p, view_mean, m * 8, cudaMemcpyHostToDevice, s));
            WB_CUDA(cudaMemcpyAsync(sd.p, view_std, m * 8, cudaMemcpyHostToDevice, s));
            return wb_pairwise_subsequence_distance(
                static_cast<double *>(p.p), static_cast<int64_t *>(o.p),
                static_cast<int64_t *>(l.p), static_cast<double *>(mu.p),
                static_cast<double *>(sd.p), m, target, dim, metric, params, out_dist, out_idx,
                1, (void *)s);
        }
        return wb_pairwise_subsequence_distance(packed.data(), off.data(), len.data(),
                                                view_mean, view_std, m, target, dim, metric,
                                                params, out_dist, out_idx, 0, (void *)s);
    }
    // device: gather on the device; outputs follow the target's side
    DevBuf p, vi, o, mu, sd;
    WB_TRY(dev_alloc(p, total * 8, s));
    WB_TRY(dev_alloc(vi, (size_t)m * 5 * 8, s));
    WB_TRY(dev_alloc(mu, m * 8, s));
    WB_TRY(dev_alloc(sd, m * 8, s));
    int64_t *dv = static_cast<int64_t *>(vi.p);
    WB_CUDA(cudaMemcpyAsync(dv, view_sample, m * 8, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(dv + m, view_dim, m * 8, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(dv + 2 * m, view_start, m * 8, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(dv + 3 * m, view_length, m * 8, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(dv + 4 * m, off.data(), m * 8, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(mu.p, view_mean, m * 8, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(sd.p, view_std, m * 8, cudaMemcpyHostToDevice, s));
    gather_views_kernel<<<(unsigned)std::min<int64_t>(m, 65535), 128, 0, s>>>(
        static_cast<const double *>(x->data), d, T, dv, dv + m, dv + 2 * m, dv + 3 * m,
        dv + 4 * m, m, static_cast<double *>(p.p));
    WB_LAUNCH_CHECK("gather_views_kernel");
    const int on = target->on_device ? 1 : 0;
    if (!on) {
        // host target: the entry copies it in; shapelet arrays must be host then
        std::vector<double> hp(total);
        std::vector<double> hm(view_mean, view_mean + m), hs(view_std, view_std + m);
        WB_CUDA(cudaMemcpyAsync(hp.data(), p.p, total * 8, cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaStreamSynchronize(s));
        return wb_pairwise_subsequence_distance(hp.data(), off.data(), len.data(), hm.data(),
                                                hs.data(), m, target, dim, metric, params,
                                                out_dist, out_idx, 0, (void *)s);
    }
    return wb_pairwise_subsequence_distance(
        static_cast<double *>(p.p), dv + 4 * m, dv + 3 * m, static_cast<double *>(mu.p),
        static_cast<double *>(sd.p), m, target, dim, metric, params, out_dist, out_idx, 1,
        (void *)s);
}
