// subseq.cu -- minimum subsequence distance (euclidean, scaled euclidean).
//
// One block per (series, chunk of shapelets); the series sits in shared
// memory; each warp takes one shapelet at a time and its 32 lanes take 32
// consecutive windows.  Every window sum runs k = 0..L-1 in order, exactly as
// euclidean_distance / inner_scaled_euclidean_distance
// (distance/_metric.pyx:625-682), and stops once it reaches the best sum of
// the earlier rounds (the reference stops at the best of all earlier windows;
// a weaker bound only evaluates more terms).  The winner of a round is the
// smallest sum, ties to the smaller window, so the result is the reference's
// "first strictly smaller" minimum and index.
//
// The scaled metric z-normalises each window with the running sums the
// reference keeps (scaled_euclidean_distance, distance/_metric.pyx:561-622);
// those sums depend only on (series, length), so one thread per (series,
// length) reproduces their exact sequence into a table first.

#include "subseq.cuh"

namespace wb {

extern __shared__ double wb_smem_sub[];

// Window statistics of scaled_euclidean_distance: for window w of length L
// mean = ex / L, std = sqrt(ex2 / L - mean^2) or 1 when that is <= 0, where
// ex, ex2 are updated by adding T[i] and, after each window, subtracting T[w].
__global__ void window_stats_kernel(const SubseqJob J, double *mean_tab, double *std_tab) {
    const int64_t total = J.x.count * (int64_t)J.n_groups;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(t / J.x.count);
        const int64_t s = t - (int64_t)g * J.x.count;
        const int L = J.group_len[g];
        const double *T = J.x.base + s * J.x.stride;
        const int nt = J.x.len;
        double *mt = mean_tab + t * (int64_t)J.win_stride;
        double *st = std_tab + t * (int64_t)J.win_stride;
        double ex = 0, ex2 = 0;
        for (int i = 0; i < nt; i++) {
            double cv = T[i];
            ex = ex + cv;
            ex2 = ex2 + cv * cv;
            if (i >= L - 1) {
                int w = i - L + 1;
                double mean = ex / (double)L;
                double tmp = ex2 / (double)L - mean * mean;
                mt[w] = mean;
                st[w] = tmp > 0 ? sqrt(tmp) : 1.0;
                double old = T[w];
                ex = ex - old;
                ex2 = ex2 - old * old;
            }
        }
    }
}

// (S[k] - s_mean) / s_std for every packed shapelet value
__global__ void shapelet_norm_kernel(const SubseqJob J, double *norm) {
    for (int64_t s = blockIdx.x; s < J.m; s += gridDim.x) {
        const double mu = J.means[s];
        const double sd = J.stds[s] != 0.0 ? J.stds[s] : 1.0;
        const int64_t off = J.offsets[s];
        const int L = (int)J.lengths[s];
        for (int k = threadIdx.x; k < L; k += blockDim.x)
            norm[off + k] = (J.shapelets[off + k] - mu) / sd;
    }
}

constexpr int kSubThreads = 128;
constexpr int kSubWarps = kSubThreads / 32;

template <bool SCALED>
__global__ void __launch_bounds__(kSubThreads)
subseq_scan_kernel(const SubseqJob J, const double *norm, const double *mean_tab,
                   const double *std_tab) {
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int64_t chunks = (J.m + J.chunk - 1) / J.chunk;
    const int nt = J.x.len;
    double *T = wb_smem_sub;
    for (int64_t b = blockIdx.x; b < J.x.count * chunks; b += gridDim.x) {
        const int64_t si = b / chunks;
        const int64_t c0 = (b - si * chunks) * J.chunk;
        const int64_t c1 = c0 + J.chunk < J.m ? c0 + J.chunk : J.m;
        __syncthreads();
        const double *Tg = J.x.base + si * J.x.stride;
        for (int i = threadIdx.x; i < nt; i += kSubThreads) T[i] = Tg[i];
        __syncthreads();
        for (int64_t sh = c0 + wid; sh < c1; sh += kSubWarps) {
            const int64_t idx = J.order ? J.order[sh] : sh;
            const int L = (int)J.lengths[idx];
            const double *S = (SCALED ? norm : J.shapelets) + J.offsets[idx];
            const int nwin = nt - L + 1;
            const double *mt = nullptr, *st = nullptr;
            if (SCALED) {
                const int64_t row = (int64_t)J.group_of[idx] * J.x.count + si;
                mt = mean_tab + row * J.win_stride;
                st = std_tab + row * J.win_stride;
            }
            double best = INF;
            int bidx = 0;
            for (int base = 0; base < nwin; base += 32) {
                const int w = base + lane;
                double dist = INF;
                if (w < nwin) {
                    dist = 0.0;
                    if (SCALED) {
                        const double mean = mt[w];
                        const double sd = st[w];
                        for (int k = 0; k < L; k++) {
                            if (dist >= best) break;
                            double x = __ldg(S + k);
                            x = x - (T[w + k] - mean) / sd;
                            dist = dist + x * x;
                        }
                    } else {
                        for (int k = 0; k < L; k++) {
                            if (dist >= best) break;
                            double x = T[w + k];
                            x = x - __ldg(S + k);
                            dist = dist + x * x;
                        }
                    }
                    if (!(dist < best)) dist = INF;
                }
                // lexicographic (dist, window) minimum over the warp
                double v = dist;
                int vi = w;
                for (int o = 16; o > 0; o >>= 1) {
                    double ov = __shfl_xor_sync(0xffffffffu, v, o);
                    int oi = __shfl_xor_sync(0xffffffffu, vi, o);
                    if (ov < v || (ov == v && oi < vi)) {
                        v = ov;
                        vi = oi;
                    }
                }
                if (v < best) {
                    best = v;
                    bidx = vi;
                }
            }
            if (lane == 0) {
                J.out_dist[si * J.m + idx] = sqrt(best);
                J.out_idx[si * J.m + idx] = bidx;
            }
        }
    }
}

static int sub_grid(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)device_info().sm_count * 16;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

size_t subseq_workspace_bytes(const SubseqJob &J, bool scaled) {
    if (!scaled) return 0;
    size_t tab = (size_t)J.n_groups * J.x.count * J.win_stride * sizeof(double);
    return 2 * align256(tab) + align256((size_t)J.total_values * sizeof(double));
}

int launch_subseq(const SubseqJob &J, bool scaled, Workspace &ws) {
    cudaStream_t s = ws.stream();
    if (J.m == 0 || J.x.count == 0) return WB_OK;
    const int64_t chunks = (J.m + J.chunk - 1) / J.chunk;
    const int64_t blocks = J.x.count * chunks;
    int64_t cap = (int64_t)device_info().sm_count * 16;
    const int grid = (int)(blocks < cap ? blocks : cap);
    const size_t smem = (size_t)J.x.len * sizeof(double);
    if (scaled) {
        size_t tab = (size_t)J.n_groups * J.x.count * J.win_stride;
        double *mean_tab = ws.take<double>(tab);
        double *std_tab = ws.take<double>(tab);
        double *norm = ws.take<double>((size_t)J.total_values);
        if (!mean_tab || !std_tab || !norm)
            return fail(WB_ENOMEM, "workspace reservation exceeded");
        window_stats_kernel<<<sub_grid(J.x.count * J.n_groups, 128), 128, 0, s>>>(
            J, mean_tab, std_tab);
        WB_LAUNCH_CHECK("window_stats_kernel");
        shapelet_norm_kernel<<<(int)(J.m < 65535 ? J.m : 65535), 128, 0, s>>>(J, norm);
        WB_LAUNCH_CHECK("shapelet_norm_kernel");
        auto k = subseq_scan_kernel<true>;
        WB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        timer_begin("subseq_scan_kernel<scaled>", s);
        k<<<grid, kSubThreads, smem, s>>>(J, norm, mean_tab, std_tab);
        timer_end(s);
        WB_LAUNCH_CHECK("subseq_scan_kernel<scaled>");
    } else {
        auto k = subseq_scan_kernel<false>;
        WB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        timer_begin("subseq_scan_kernel", s);
        k<<<grid, kSubThreads, smem, s>>>(J, nullptr, nullptr, nullptr);
        timer_end(s);
        WB_LAUNCH_CHECK("subseq_scan_kernel");
    }
    return WB_OK;
}

}  // namespace wb
