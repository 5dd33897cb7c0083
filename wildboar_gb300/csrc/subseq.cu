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
    const int64_t total = J.paired ? J.x.count : J.x.count * (int64_t)J.n_groups;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int g = J.paired ? 0 : (int)(t / J.x.count);
        const int64_t s = t - (int64_t)g * J.x.count;
        const int L = J.paired ? (int)J.lengths[s] : J.group_len[g];
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
        const double sd = (J.stds[s] != 0.0 || J.std_as_given) ? J.stds[s] : 1.0;
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

// Scaled metric, tiled: one block per (series, chunk of shapelets of one
// length L).  Windows go in tiles of 32: the block first writes the
// z-normalised tile Z[k][w] = (T[w + k] - mean_w) / std_w (the reference's
// per-element division, correctly rounded, same operands) into shared
// memory, then every shapelet of the chunk scans the tile with it, so each
// division is shared by all shapelets of the chunk instead of being redone
// per shapelet.  Per shapelet, the sum, the early abandoning against the best
// of earlier tiles and the (sum, window) minimum are those of
// subseq_scan_kernel.
__global__ void __launch_bounds__(kSubThreads)
subseq_scaled_tiled_kernel(const SubseqJob J, const double *norm, const double *mean_tab,
                           const double *std_tab) {
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int nt = J.x.len;
    double *T = wb_smem_sub;                      // nt
    double *best = T + nt;                        // chunk
    int *bidx = reinterpret_cast<int *>(best + J.chunk);  // chunk
    double *Z = best + J.chunk + (J.chunk + 1) / 2;      // [max_len][32]
    for (int64_t b = blockIdx.x; b < J.x.count * J.n_chunks; b += gridDim.x) {
        const int64_t si = b / J.n_chunks;
        const int64_t ch = b - si * J.n_chunks;
        const int64_t first = J.chunk_first[ch];
        const int cnt = J.chunk_count[ch];
        const int g = J.chunk_group[ch];
        const int L = J.group_len[g];
        const int nwin = nt - L + 1;
        const int64_t row = (int64_t)g * J.x.count + si;
        const double *mt = mean_tab + row * J.win_stride;
        const double *st = std_tab + row * J.win_stride;
        __syncthreads();
        const double *Tg = J.x.base + si * J.x.stride;
        for (int i = threadIdx.x; i < nt; i += kSubThreads) T[i] = Tg[i];
        for (int q = threadIdx.x; q < cnt; q += kSubThreads) {
            best[q] = INF;
            bidx[q] = 0;
        }
        for (int base = 0; base < nwin; base += 32) {
            __syncthreads();
            for (int e = threadIdx.x; e < L * 32; e += kSubThreads) {
                const int k = e >> 5, w = e & 31;
                double z = 0.0;
                if (base + w < nwin) z = (T[base + w + k] - mt[base + w]) / st[base + w];
                Z[e] = z;
            }
            __syncthreads();
            const int w = base + lane;
            for (int q = wid; q < cnt; q += kSubWarps) {
                const int64_t idx = J.order[first + q];
                const double *S = norm + J.offsets[idx];
                const double bq = best[q];
                double dist = INF;
                if (w < nwin) {
                    dist = 0.0;
                    for (int k = 0; k < L; k++) {
                        if (dist >= bq) break;
                        double x = __ldg(S + k);
                        x = x - Z[k * 32 + lane];
                        dist = dist + x * x;
                    }
                    if (!(dist < bq)) dist = INF;
                }
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
                if (lane == 0 && v < bq) {
                    best[q] = v;
                    bidx[q] = vi;
                }
                __syncwarp();
            }
        }
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += kSubThreads) {
            const int64_t idx = J.order[first + q];
            J.out_dist[si * J.m + idx] = sqrt(best[q]);
            J.out_idx[si * J.m + idx] = bidx[q];
        }
    }
}

// Paired: one warp per (series i, shapelet i), lanes over windows in rounds
// of 32, the series read through L1; sums, early abandoning and the (sum,
// window) minimum as in subseq_scan_kernel.
template <bool SCALED>
__global__ void __launch_bounds__(kSubThreads)
subseq_paired_kernel(const SubseqJob J, const double *norm, const double *mean_tab,
                     const double *std_tab) {
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * kSubThreads + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * kSubThreads) >> 5;
    const int nt = J.x.len;
    for (int64_t si = warp; si < J.x.count; si += nwarps) {
        const int L = (int)J.lengths[si];
        const double *S = (SCALED ? norm : J.shapelets) + J.offsets[si];
        const double *T = J.x.base + si * J.x.stride;
        const double *mt = SCALED ? mean_tab + si * J.win_stride : nullptr;
        const double *st = SCALED ? std_tab + si * J.win_stride : nullptr;
        const int nwin = nt - L + 1;
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
                        x = x - (__ldg(T + w + k) - mean) / sd;
                        dist = dist + x * x;
                    }
                } else {
                    for (int k = 0; k < L; k++) {
                        if (dist >= best) break;
                        double x = __ldg(T + w + k);
                        x = x - __ldg(S + k);
                        dist = dist + x * x;
                    }
                }
                if (!(dist < best)) dist = INF;
            }
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
            J.out_dist[si] = sqrt(best);
            J.out_idx[si] = bidx;
        }
    }
}

static int sub_grid(int64_t n, int block);

// Profile (paired jobs): every window's full sum, no early abandoning -- the
// values euclidean_distance_matches / scaled_euclidean_distance_matches
// (distance/_metric.pyx:762-870) square-root into their distances with an
// infinite threshold.  One thread per (pair, window); raw[pair * ld + w],
// NaN past the pair's last window.
template <bool SCALED>
__global__ void subseq_profile_kernel(const SubseqJob J, const double *norm,
                                      const double *mean_tab, const double *std_tab,
                                      double *raw, int64_t ld) {
    const int nt = J.x.len;
    const int64_t total = J.x.count * ld;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / ld;
        const int w = (int)(t - i * ld);
        const int L = (int)J.lengths[i];
        if (w >= nt - L + 1) {
            raw[t] = __longlong_as_double(0x7ff8000000000000LL);
            continue;
        }
        const double *S = (SCALED ? norm : J.shapelets) + J.offsets[i];
        const double *T = J.x.base + i * J.x.stride;
        double dist = 0.0;
        if (SCALED) {
            const double mean = mean_tab[i * J.win_stride + w];
            const double sd = std_tab[i * J.win_stride + w];
            for (int k = 0; k < L; k++) {
                double x = __ldg(S + k);
                x = x - (__ldg(T + w + k) - mean) / sd;
                dist = dist + x * x;
            }
        } else {
            for (int k = 0; k < L; k++) {
                double x = __ldg(T + w + k);
                x = x - __ldg(S + k);
                dist = dist + x * x;
            }
        }
        raw[t] = dist;
    }
}

int launch_subseq_profile(const SubseqJob &J, bool scaled, Workspace &ws, double *raw,
                          int64_t ld) {
    cudaStream_t s = ws.stream();
    if (J.m == 0 || J.x.count == 0) return WB_OK;
    const int grid = sub_grid(J.x.count * ld, 128);
    if (scaled) {
        const size_t tab = (size_t)J.x.count * J.win_stride;
        double *mean_tab = ws.take<double>(tab);
        double *std_tab = ws.take<double>(tab);
        double *norm = ws.take<double>((size_t)J.total_values);
        if (!mean_tab || !std_tab || !norm)
            return fail(WB_ENOMEM, "workspace reservation exceeded");
        window_stats_kernel<<<sub_grid(J.x.count, 128), 128, 0, s>>>(J, mean_tab, std_tab);
        WB_LAUNCH_CHECK("window_stats_kernel");
        shapelet_norm_kernel<<<(int)(J.m < 65535 ? J.m : 65535), 128, 0, s>>>(J, norm);
        WB_LAUNCH_CHECK("shapelet_norm_kernel");
        subseq_profile_kernel<true><<<grid, 128, 0, s>>>(J, norm, mean_tab, std_tab, raw, ld);
        WB_LAUNCH_CHECK("subseq_profile_kernel<scaled>");
    } else {
        subseq_profile_kernel<false><<<grid, 128, 0, s>>>(J, nullptr, nullptr, nullptr, raw, ld);
        WB_LAUNCH_CHECK("subseq_profile_kernel");
    }
    return WB_OK;
}

static size_t scaled_tiled_smem(const SubseqJob &J) {
    return (size_t)J.x.len * 8 + (size_t)J.chunk * 8 + (size_t)((J.chunk + 1) / 2) * 8 +
           (size_t)J.max_len * 32 * 8;
}

static int sub_grid(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)device_info().sm_count * 16;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

size_t subseq_workspace_bytes(const SubseqJob &J, bool scaled) {
    if (!scaled) return 0;
    const size_t rows = J.paired ? (size_t)J.x.count : (size_t)J.n_groups * J.x.count;
    size_t tab = rows * J.win_stride * sizeof(double);
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
        const size_t rows = J.paired ? (size_t)J.x.count : (size_t)J.n_groups * J.x.count;
        size_t tab = rows * J.win_stride;
        double *mean_tab = ws.take<double>(tab);
        double *std_tab = ws.take<double>(tab);
        double *norm = ws.take<double>((size_t)J.total_values);
        if (!mean_tab || !std_tab || !norm)
            return fail(WB_ENOMEM, "workspace reservation exceeded");
        window_stats_kernel<<<sub_grid((int64_t)rows, 128), 128, 0, s>>>(J, mean_tab, std_tab);
        WB_LAUNCH_CHECK("window_stats_kernel");
        shapelet_norm_kernel<<<(int)(J.m < 65535 ? J.m : 65535), 128, 0, s>>>(J, norm);
        WB_LAUNCH_CHECK("shapelet_norm_kernel");
        if (J.paired) {
            timer_begin("subseq_paired_kernel<scaled>", s);
            subseq_paired_kernel<true><<<sub_grid(J.x.count * 32, kSubThreads), kSubThreads, 0,
                                         s>>>(J, norm, mean_tab, std_tab);
            timer_end(s);
            WB_LAUNCH_CHECK("subseq_paired_kernel<scaled>");
            return WB_OK;
        }
        const size_t tsm = scaled_tiled_smem(J);
        if (J.n_chunks > 0 && tsm <= (size_t)device_info().max_smem_optin) {
            auto kt = subseq_scaled_tiled_kernel;
            WB_CUDA(cudaFuncSetAttribute(kt, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tsm));
            const int64_t tb = J.x.count * J.n_chunks;
            const int tgrid = (int)(tb < cap ? tb : cap);
            timer_begin("subseq_scaled_tiled_kernel", s);
            kt<<<tgrid, kSubThreads, tsm, s>>>(J, norm, mean_tab, std_tab);
            timer_end(s);
            WB_LAUNCH_CHECK("subseq_scaled_tiled_kernel");
            return WB_OK;
        }
        auto k = subseq_scan_kernel<true>;
        WB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        timer_begin("subseq_scan_kernel<scaled>", s);
        k<<<grid, kSubThreads, smem, s>>>(J, norm, mean_tab, std_tab);
        timer_end(s);
        WB_LAUNCH_CHECK("subseq_scan_kernel<scaled>");
    } else if (J.paired) {
        timer_begin("subseq_paired_kernel", s);
        subseq_paired_kernel<false><<<sub_grid(J.x.count * 32, kSubThreads), kSubThreads, 0,
                                      s>>>(J, nullptr, nullptr, nullptr);
        timer_end(s);
        WB_LAUNCH_CHECK("subseq_paired_kernel");
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
