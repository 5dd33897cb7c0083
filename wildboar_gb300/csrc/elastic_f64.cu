// elastic_f64.cu -- FP64 elastic distances, one thread per pair.
//
// Layout.  A warp holds 32 pairs that share one column series (the metric's
// Y, read with warp-uniform broadcast loads) and have 32 different row series
// (the metric's X, one load per recurrence row).  Each thread keeps the live
// band of the previous recurrence row in a ring of P doubles: in shared
// memory, interleaved across the block ([k][thread], conflict-free), or for
// wide bands in a global scratch ring interleaved across the grid
// ([k][global thread], coalesced).  The cost matrix is never materialised.
//
// Arithmetic.  Every cell performs the reference's IEEE double operations in
// the reference's order (the file is compiled with -fmad=false); only the
// comparisons of non-negative costs run on the integer pipe (nn_min/nn_max),
// which gives the same values.  GB300's FP64 pipe, not memory, bounds these
// kernels.
//
// Band semantics restated from distance/_elastic.pyx (two-row recurrences):
// row i covers columns [js, je) with js = max(0, i - max(0, n-m) - r + 1),
// je = min(m, i + max(0, m-n) + r).  Out-of-band neighbours read the value
// the reference writes next to the band: +inf for the dtw family, 0 for
// lcss / edr / erp / twe and for msm's upper edge.  msm's left neighbour of
// the first band cell is never written by the reference and holds the cell
// two rows up (stale buffer content); the ring reproduces that value.

#include "elastic_rec.cuh"

namespace wb {

// --------------------------------------------------------------------------

template <int KIND, class R>
__device__ __forceinline__ double run_pair(const ElasticJob &J, R ring, int P,
                                           int64_t rs, int64_t cs, double &key) {
    const double *X = J.rows.base + rs * J.rows.stride;
    const double *Y = J.cols.base + cs * J.cols.stride;
    const int n = J.rows.len, m = J.cols.len, r = J.band;
    if constexpr (KIND == K_DTW) return rec_dtw<false>(ring, P, X, n, Y, m, r, nullptr, key);
    if constexpr (KIND == K_WDTW) return rec_dtw<true>(ring, P, X, n, Y, m, r, J.weights, key);
    if constexpr (KIND == K_ADTW) return rec_adtw<true>(ring, P, X, n, Y, m, r, J.p, key);
    if constexpr (KIND == K_ADTW_ANY) return rec_adtw<false>(ring, P, X, n, Y, m, r, J.p, key);
    if constexpr (KIND == K_LCSS) return rec_lcss<false>(ring, P, X, n, Y, m, r, J.eps, nullptr, key);
    if constexpr (KIND == K_WLCSS) return rec_lcss<true>(ring, P, X, n, Y, m, r, J.eps, J.weights, key);
    if constexpr (KIND == K_EDR) {
        double eps = J.eps;
        if (J.std_rows) eps = cy_max(J.std_rows[rs], J.std_cols[cs]) / 4.0;
        return rec_edr(ring, P, X, n, Y, m, r, eps, key);
    }
    if constexpr (KIND == K_ERP)
        return rec_erp(ring, P, X, n, Y, m, r, J.g, J.gsum_rows[rs], J.gsum_cols[cs],
                       J.gtab_cols + cs * (int64_t)m, key);
    if constexpr (KIND == K_MSM) return rec_msm(ring, P, X, n, Y, m, r, J.c, key);
    if constexpr (KIND == K_EUCLID) {
        // euclidean_distance with one window (equal lengths),
        // distance/_metric.pyx:654-682: sum_j (y_j - x_j)^2 in order
        double dist = 0.0;
        for (int j = 0; j < m; j++) {
            double v = ldg(Y + j);
            v = v - X[j];
            dist = dist + v * v;
        }
        key = -WB_INF;
        return dist;
    }
    if constexpr (KIND == K_TWE)
        return rec_twe(ring, P, X, n, Y, m, r, J.penalty, J.stiffness,
                       J.dtab_cols + cs * (int64_t)m, J.stab, key);
    return 0.0;
}

__device__ __forceinline__ double finish(const ElasticJob &J, double v) {
    switch (J.result) {
        case R_SQRT: return sqrt(v);
        case R_LCSS: return 1.0 - v / (double)imin(J.len_norm_rows, J.len_norm_cols);
        case R_EDR: return v / (double)imax(J.len_norm_rows, J.len_norm_cols);
        default: return v;
    }
}

constexpr int kThreads = 128;

template <int KIND, bool GRING>
__global__ void __launch_bounds__(kThreads)
elastic_pairs_kernel(const ElasticJob J, double *gring, int P) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * kThreads) >> 5;
    const int64_t gtid = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const int64_t gthreads = (int64_t)gridDim.x * kThreads;

    auto body = [&](auto ring) {
        if (J.mode == PM_PAIRED) {
            for (int64_t s = gtid; s < J.rows.count; s += gthreads) {
                double key, d;
                d = J.all_zero ? 0.0 : finish(J, run_pair<KIND>(J, ring, P, s, s, key));
                J.out[s] = d;
            }
            return;
        }
        const int64_t chunks = (J.rows.count + 31) >> 5;
        const int64_t ntiles = chunks * J.cols.count;
        for (int64_t t = warp; t < ntiles; t += nwarps) {
            const int64_t cs = t / chunks;
            const int64_t rs = (t - cs * chunks) * 32 + lane;
            if (J.mode == PM_UPPER) {
                if (rs >= cs) continue;
            } else if (rs >= J.rows.count) {
                continue;
            }
            double key = 0.0, d;
            if (J.all_zero) d = 0.0;
            else d = finish(J, run_pair<KIND>(J, ring, P, rs, cs, key));
            J.out[rs * J.out_ld + cs] = d;
            if (J.mode == PM_UPPER) J.out[cs * J.out_ld + rs] = d;
            if (J.key) J.key[rs * J.out_ld + cs] = key;
        }
    };
    if constexpr (GRING) {
        body(RingG{gring + gtid, gthreads});
    } else {
        body(RingS{(int)threadIdx.x, kThreads});
    }
}

template <int KIND>
static int launch_kind(const ElasticJob &J, Workspace &ws, int P, bool gring_mode,
                       double *gring, int grid) {
    cudaStream_t s = ws.stream();
    if (gring_mode) {
        timer_begin("elastic_pairs_kernel", s);
        elastic_pairs_kernel<KIND, true><<<grid, kThreads, 0, s>>>(J, gring, P);
    } else {
        size_t smem = (size_t)P * kThreads * sizeof(double);
        auto kfn = elastic_pairs_kernel<KIND, false>;
        WB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        timer_begin("elastic_pairs_kernel", s);
        kfn<<<grid, kThreads, smem, s>>>(J, nullptr, P);
    }
    timer_end(s);
    WB_LAUNCH_CHECK("elastic_pairs_kernel");
    return WB_OK;
}

// decide ring placement and grid size
struct ElasticPlan {
    int P;
    bool gring;
    int grid;
    size_t gring_bytes;
};

static ElasticPlan plan_elastic(const ElasticJob &J) {
    const DeviceInfo &dev = device_info();
    ElasticPlan pl;
    pl.P = imax(2, ring_len(J.rows.len, J.cols.len, J.band));
    const size_t per_block = (size_t)pl.P * kThreads * sizeof(double);
    int64_t work_threads;
    if (J.mode == PM_PAIRED) work_threads = J.rows.count;
    else work_threads = ((J.rows.count + 31) / 32) * 32 * J.cols.count;
    int64_t want_blocks = (work_threads + kThreads - 1) / kThreads;
    int blocks_per_sm = 0;
    if (per_block <= (size_t)dev.smem_per_sm - 2048 && per_block <= (size_t)dev.max_smem_optin) {
        blocks_per_sm = (int)(((size_t)dev.smem_per_sm - 1024) / (per_block + 1024));
        if (blocks_per_sm > 4) blocks_per_sm = 4;
    }
    // a ring that leaves fewer than 4 warps per SM goes to global memory
    if (blocks_per_sm >= 1) {
        pl.gring = false;
        int64_t cap = (int64_t)blocks_per_sm * dev.sm_count;
        pl.grid = (int)(want_blocks < cap ? want_blocks : cap);
        pl.gring_bytes = 0;
    } else {
        pl.gring = true;
        int64_t cap = (int64_t)4 * dev.sm_count;
        pl.grid = (int)(want_blocks < cap ? want_blocks : cap);
        pl.gring_bytes = (size_t)pl.P * pl.grid * kThreads * sizeof(double);
    }
    if (pl.grid < 1) pl.grid = 1;
    return pl;
}

// FP64: the ring kernel keeps a band that fits in shared memory at no extra
// cost per cell, while the strip kernel also evaluates (and discards) the
// cells of each strip's ragged band edges; measured on GB300 (dtw, L = 512)
// the ring kernel wins for shared-memory rings (r = 0.1: 171 vs 152 GCUPS)
// and the strip kernel for global rings (r = 1: 167 vs 128 GCUPS; lcss 168 vs
// 134, erp 127 vs 115, msm 64 vs 58), except twe (53 vs 57).
static bool use_strip_f64(const ElasticJob &J) {
    if (!strip_supported(J)) return false;
    if (strip_forced()) return true;
    return J.kind != K_TWE && plan_elastic(J).gring;
}

size_t elastic_workspace_bytes(const ElasticJob &J) {
    if (use_strip_f64(J)) return strip_workspace_bytes(J, false);
    ElasticPlan pl = plan_elastic(J);
    return align256(pl.gring_bytes);
}

// --------------------------------------------------------------------------
// Euclidean pairwise distance, tiled: a block computes a 64 x 64 tile of
// (row series i, column series j) pairs, 4 x 4 per thread, staging 32 values
// of each of the 64 + 64 series in shared memory per step.  Every pair's sum
// still runs k = 0 .. L-1 in order with the reference's operations (v = y_k -
// x_k, dist = dist + v * v; euclidean_distance with one window,
// distance/_metric.pyx:654-682), so results are bit-identical; the tiling
// only replaces the per-lane strided row reads of the thread-per-pair kernel
// (whose speed depended on the L1 carve-out) by shared-memory reuse.
constexpr int kEuT = 64, kEuK = 32;

__global__ void __launch_bounds__(256) euclid_tiled_kernel(const ElasticJob J) {
    __shared__ double xs[kEuK][kEuT + 1];
    __shared__ double ys[kEuK][kEuT + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int L = J.rows.len;
    const int64_t tiles_c = (J.cols.count + kEuT - 1) / kEuT;
    const int64_t tiles_r = (J.rows.count + kEuT - 1) / kEuT;
    for (int64_t t = blockIdx.x; t < tiles_r * tiles_c; t += gridDim.x) {
        const int64_t tr = t / tiles_c, tc = t - (t / tiles_c) * tiles_c;
        if (J.mode == PM_UPPER && tr > tc) continue;  // the mirror tile fills it
        const int64_t r0 = tr * kEuT, c0 = tc * kEuT;
        double acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
        for (int k0 = 0; k0 < L; k0 += kEuK) {
            __syncthreads();
            for (int e = threadIdx.x; e < kEuK * kEuT; e += 256) {
                const int s = e / kEuK, k = e - (e / kEuK) * kEuK;
                const int64_t ri = r0 + s, ci = c0 + s;
                double xv = 0.0, yv = 0.0;
                if (k0 + k < L) {
                    if (ri < J.rows.count) xv = J.rows.base[ri * J.rows.stride + k0 + k];
                    if (ci < J.cols.count) yv = J.cols.base[ci * J.cols.stride + k0 + k];
                }
                xs[k][s] = xv;
                ys[k][s] = yv;
            }
            __syncthreads();
            const int kn = L - k0 < kEuK ? L - k0 : kEuK;
            for (int k = 0; k < kn; k++) {
                double xv[4], yv[4];
#pragma unroll
                for (int a = 0; a < 4; a++) xv[a] = xs[k][ty + 16 * a];
#pragma unroll
                for (int b = 0; b < 4; b++) yv[b] = ys[k][tx + 16 * b];
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        double v = yv[b];
                        v = v - xv[a];
                        acc[a][b] = acc[a][b] + v * v;
                    }
            }
        }
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int64_t i = r0 + ty + 16 * a;
            if (i >= J.rows.count) continue;
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int64_t j = c0 + tx + 16 * b;
                if (j >= J.cols.count) continue;
                if (J.mode == PM_UPPER) {
                    if (i >= j) continue;
                    const double d = J.all_zero ? 0.0 : sqrt(acc[a][b]);
                    J.out[i * J.out_ld + j] = d;
                    J.out[j * J.out_ld + i] = d;
                } else {
                    J.out[i * J.out_ld + j] = J.all_zero ? 0.0 : sqrt(acc[a][b]);
                }
            }
        }
    }
}

static int launch_euclid_tiled(const ElasticJob &J, cudaStream_t s) {
    const int64_t tiles = ((J.rows.count + kEuT - 1) / kEuT) * ((J.cols.count + kEuT - 1) / kEuT);
    const int64_t cap = (int64_t)device_info().sm_count * 8;
    const int grid = (int)(tiles < cap ? tiles : cap);
    timer_begin("euclid_tiled_kernel", s);
    euclid_tiled_kernel<<<grid, 256, 0, s>>>(J);
    timer_end(s);
    WB_LAUNCH_CHECK("euclid_tiled_kernel");
    return WB_OK;
}

int launch_elastic(const ElasticJob &J, Workspace &ws, size_t *) {
    if (J.rows.count == 0 || J.cols.count == 0) return WB_OK;
    if (use_strip_f64(J)) return launch_strip(J, ws, false);
    ElasticPlan pl = plan_elastic(J);
    double *gring = pl.gring ? ws.take<double>(pl.gring_bytes / sizeof(double)) : nullptr;
    if (pl.gring && !gring) return fail(WB_ENOMEM, "workspace reservation exceeded");
    switch (J.kind) {
        case K_DTW: return launch_kind<K_DTW>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_WDTW: return launch_kind<K_WDTW>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_ADTW: return launch_kind<K_ADTW>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_ADTW_ANY: return launch_kind<K_ADTW_ANY>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_LCSS: return launch_kind<K_LCSS>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_WLCSS: return launch_kind<K_WLCSS>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_EDR: return launch_kind<K_EDR>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_ERP: return launch_kind<K_ERP>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_MSM: return launch_kind<K_MSM>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_TWE: return launch_kind<K_TWE>(J, ws, pl.P, pl.gring, gring, pl.grid);
        case K_EUCLID:
            if (J.mode != PM_PAIRED && J.key == nullptr && J.rows.len == J.cols.len)
                return launch_euclid_tiled(J, ws.stream());
            return launch_kind<K_EUCLID>(J, ws, 2, false, nullptr, pl.grid);
    }
    return fail(WB_EINVAL, "unknown elastic kernel");
}

// --------------------------------------------------------------------------
// elastic subsequence distance: one warp per (series, shapelet), one lane per
// window, the reference's sequential early-abandoning replayed per round.

__device__ __forceinline__ double subseq_threshold(int metric, double min_dist, int L, int T) {
    switch (metric) {
        case WB_LCSS: return isinf(min_dist) ? min_dist : (double)L - min_dist * (double)L;
        case WB_EDR: return min_dist * (double)(L > T ? L : T);
        default: return min_dist;
    }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads)
elastic_subseq_kernel(const SubseqElasticJob J, double *gring, int P) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * kThreads) >> 5;
    const int64_t gtid = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const int64_t gthreads = (int64_t)gridDim.x * kThreads;
    RingG ring{gring + gtid, gthreads};
    const double INF = WB_INF;
    const int64_t ntask = J.paired ? J.x.count : J.x.count * J.m;
    for (int64_t task = warp; task < ntask; task += nwarps) {
        const int64_t si = J.paired ? task : task / J.m;
        const int64_t sh = J.paired ? task : task - si * J.m;
        const int64_t oidx = J.paired ? task : si * J.m + sh;
        const int Lorig = (int)J.len[sh];
        const int L = J.slopes ? Lorig - 2 : Lorig;  // length of the compared rows
        if (J.slopes && Lorig < 3) {
            if (J.prof_raw) {
                // ddtw_subsequence_matches reports no window for such shapelets
                for (int64_t w = lane; w < J.prof_ld; w += 32) {
                    J.prof_raw[oidx * J.prof_ld + w] = __longlong_as_double(0x7ff8000000000000LL);
                    J.prof_key[oidx * J.prof_ld + w] = INF;
                }
                continue;
            }
            // ddtw_subsequence_distance returns 0 for shapelets shorter than 3
            if (lane == 0) {
                J.out_dist[oidx] = 0.0;
                J.out_idx[oidx] = 0;
            }
            continue;
        }
        const double *S = J.shp + J.off[sh];
        const double *T = J.x.base + si * J.x.stride;
        const int nwin = J.x.len - L + 1;  // = series length - shapelet length + 1
        if (J.prof_raw) {
            // windows past this pair's last one
            for (int64_t w = nwin + lane; w < J.prof_ld; w += 32) {
                J.prof_raw[oidx * J.prof_ld + w] = __longlong_as_double(0x7ff8000000000000LL);
                J.prof_key[oidx * J.prof_ld + w] = __longlong_as_double(0x7ff8000000000000LL);
            }
        }
        const int band = J.band_of_len[sh];
        double eps = J.eps;
        if (KIND == K_EDR && J.shp_std) {
            const double sd =
                (J.shp_std[sh] != 0.0 || J.std_as_given) ? J.shp_std[sh] : 1.0;
            eps = sd / 4.0;
        }
        double gx_sum = 0.0;
        if (KIND == K_ERP)
            for (int k = 0; k < L; k++) gx_sum = gx_sum + fabs(S[k] - J.g);
        double min_dist = INF;
        int best = 0;
        for (int base = 0; base < nwin; base += 32) {
            const int w = base + lane;
            double d = INF, key = INF;
            // The round's windows stop at the threshold of the best window of
            // the earlier rounds: the thresholds inside the round are no larger
            // (lcss's threshold falls as the distance grows: no bound), and an
            // abandoned window's partial key already exceeds the threshold its
            // replay compares it with.  Adjacent windows overlap, so a round
            // far from every good match abandons in all its lanes together.
            const double bound =
                (J.prof_raw || KIND == K_LCSS) ? INF
                                               : subseq_threshold(J.metric, min_dist, L,
                                                                  J.t_len_thr);
            if (w < nwin) {
                const double *Y = T + w;
                double raw;
                if constexpr (KIND == K_DTW)
                    raw = rec_dtw<false, RingG, true>(ring, P, S, L, Y, L, band, nullptr, key,
                                                      bound);
                else if constexpr (KIND == K_WDTW)
                    raw = rec_dtw<true, RingG, true>(ring, P, S, L, Y, L, band, J.weights, key,
                                                     bound);
                else if constexpr (KIND == K_ADTW)
                    raw = rec_adtw<true, RingG, true>(ring, P, S, L, Y, L, band, J.p, key,
                                                      bound);
                else if constexpr (KIND == K_ADTW_ANY)
                    raw = rec_adtw<false, RingG, true>(ring, P, S, L, Y, L, band, J.p, key,
                                                       bound);
                else if constexpr (KIND == K_LCSS)
                    raw = rec_lcss<false>(ring, P, S, L, Y, L, band, eps, nullptr, key);
                else if constexpr (KIND == K_EDR)
                    raw = rec_edr<RingG, true>(ring, P, S, L, Y, L, band, eps, key, bound);
                else if constexpr (KIND == K_ERP) {
                    double gy_sum = 0.0;
                    for (int k = 0; k < L; k++) gy_sum = gy_sum + ldg(J.gtab + si * J.t_len + w + k);
                    raw = rec_erp<RingG, true>(ring, P, S, L, Y, L, band, J.g, gx_sum, gy_sum,
                                               J.gtab + si * J.t_len + w, key, bound);
                } else if constexpr (KIND == K_MSM)
                    raw = rec_msm<RingG, true>(ring, P, S, L, Y, L, band, J.c, key, bound);
                else
                    raw = rec_twe<RingG, false, true>(ring, P, S, L, Y, L, band, J.penalty,
                                                      J.stiffness, nullptr, J.stab, key, bound);
                if (KIND == K_LCSS) d = 1.0 - raw / (double)L;
                else if (KIND == K_EDR) d = raw / (double)L;
                else d = raw;
                if (J.prof_raw) {
                    J.prof_raw[oidx * J.prof_ld + w] = raw;
                    J.prof_key[oidx * J.prof_ld + w] = key;
                }
            }
            if (J.prof_raw) continue;
            // replay windows base..base+31 in order, as the reference scans them
            for (int t = 0; t < 32; t++) {
                const double dt = __shfl_sync(0xffffffffu, d, t);
                const double kt = __shfl_sync(0xffffffffu, key, t);
                if (base + t >= nwin) break;
                const double thr = subseq_threshold(J.metric, min_dist, L, J.t_len_thr);
                if (!(kt > thr) && dt < min_dist) {
                    min_dist = dt;
                    best = base + t;
                }
            }
        }
        if (lane == 0 && !J.prof_raw) {
            const bool sq = KIND == K_DTW || KIND == K_WDTW || KIND == K_ADTW ||
                            KIND == K_ADTW_ANY;
            J.out_dist[oidx] = sq ? sqrt(min_dist) : min_dist;
            J.out_idx[oidx] = best;
        }
    }
}

size_t elastic_subseq_ring_bytes(const SubseqElasticJob &J, int max_len, int max_band,
                                 int *P_out, int *grid_out) {
    const DeviceInfo &dev = device_info();
    int P = imax(2, ring_len(max_len, max_len, max_band));
    int64_t warps = J.paired ? J.x.count : J.x.count * J.m;
    int64_t grid = (warps * 32 + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)4 * dev.sm_count;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    *P_out = P;
    *grid_out = (int)grid;
    return align256((size_t)P * grid * kThreads * sizeof(double));
}

int launch_elastic_subseq(const SubseqElasticJob &J, int kind, double *gring, int P, int grid,
                          cudaStream_t s) {
    if (J.x.count == 0 || J.m == 0) return WB_OK;
    timer_begin("elastic_subseq_kernel", s);
    switch (kind) {
#define WB_SUB_CASE(K)                                                           \
    case K:                                                                      \
        elastic_subseq_kernel<K><<<grid, kThreads, 0, s>>>(J, gring, P);         \
        break;
        WB_SUB_CASE(K_DTW)
        WB_SUB_CASE(K_WDTW)
        WB_SUB_CASE(K_ADTW)
        WB_SUB_CASE(K_ADTW_ANY)
        WB_SUB_CASE(K_LCSS)
        WB_SUB_CASE(K_EDR)
        WB_SUB_CASE(K_ERP)
        WB_SUB_CASE(K_MSM)
        WB_SUB_CASE(K_TWE)
#undef WB_SUB_CASE
        default:
            return fail(WB_EINVAL, "unsupported elastic subsequence kernel");
    }
    timer_end(s);
    WB_LAUNCH_CHECK("elastic_subseq_kernel");
    return WB_OK;
}

// slopes of packed shapelets, in place of each shapelet's first len-2 slots
__global__ void shapelet_slopes_kernel(const double *shp, const int64_t *off,
                                       const int64_t *len, int64_t m, double *out) {
    for (int64_t s = blockIdx.x; s < m; s += gridDim.x) {
        const double *q = shp + off[s];
        double *d = out + off[s];
        const int L = (int)len[s];
        for (int i = 1 + threadIdx.x; i < L - 1; i += blockDim.x) {
            double a = q[i] - q[i - 1];
            double b = (q[i + 1] - q[i - 1]) * 0.5;
            d[i - 1] = (a + b) * 0.5;
        }
    }
}

int launch_shapelet_slopes(const double *shp, const int64_t *off, const int64_t *len,
                           int64_t m, double *out, cudaStream_t s) {
    if (m == 0) return WB_OK;
    int grid = (int)(m < 65535 ? m : 65535);
    shapelet_slopes_kernel<<<grid, 64, 0, s>>>(shp, off, len, m, out);
    WB_LAUNCH_CHECK("shapelet_slopes_kernel");
    return WB_OK;
}

// The shared-memory ring form of launch_elastic, which needs no workspace:
// WB_EUNSUPPORTED when the job's band ring does not fit in shared memory (the
// tiled euclidean kernel needs none either).
int launch_elastic_shared_ring(const ElasticJob &J, cudaStream_t s) {
    if (J.rows.count == 0 || J.cols.count == 0) return WB_OK;
    if (J.kind == K_EUCLID && J.mode != PM_PAIRED && J.key == nullptr &&
        J.rows.len == J.cols.len)
        return launch_euclid_tiled(J, s);
    const ElasticPlan pl = plan_elastic(J);
    if (pl.gring) return fail(WB_EUNSUPPORTED, "band ring does not fit in shared memory");
    const size_t smem = (size_t)pl.P * kThreads * sizeof(double);
    switch (J.kind) {
#define WB_SHR_CASE(K)                                                                   \
    case K: {                                                                            \
        auto kfn = elastic_pairs_kernel<K, false>;                                       \
        WB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                     (int)smem));                                        \
        kfn<<<pl.grid, kThreads, smem, s>>>(J, nullptr, pl.P);                            \
        break;                                                                           \
    }
        WB_SHR_CASE(K_DTW)
        WB_SHR_CASE(K_WDTW)
        WB_SHR_CASE(K_ADTW)
        WB_SHR_CASE(K_ADTW_ANY)
        WB_SHR_CASE(K_LCSS)
        WB_SHR_CASE(K_WLCSS)
        WB_SHR_CASE(K_EDR)
        WB_SHR_CASE(K_ERP)
        WB_SHR_CASE(K_MSM)
        WB_SHR_CASE(K_TWE)
        WB_SHR_CASE(K_EUCLID)
#undef WB_SHR_CASE
        default: return fail(WB_EINVAL, "unknown elastic kernel");
    }
    WB_LAUNCH_CHECK("elastic_pairs_kernel");
    return WB_OK;
}

int launch_elastic_external_ring(const ElasticJob &J, double *ring, size_t ring_bytes,
                                 cudaStream_t s) {
    if (J.rows.count == 0 || J.cols.count == 0) return WB_OK;
    const DeviceInfo &dev = device_info();
    const int P = imax(2, ring_len(J.rows.len, J.cols.len, J.band));
    const size_t per_block = (size_t)P * kThreads * sizeof(double);
    const int64_t fit = (int64_t)(ring_bytes / per_block);
    if (fit < 1)
        return fail(WB_EINVAL, "band ring of " + std::to_string(per_block) +
                                   " bytes per block exceeds the static scratch of " +
                                   std::to_string(ring_bytes) + " bytes");
    int64_t work_threads;
    if (J.mode == PM_PAIRED) work_threads = J.rows.count;
    else work_threads = ((J.rows.count + 31) / 32) * 32 * J.cols.count;
    int64_t grid = (work_threads + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)4 * dev.sm_count;
    if (grid > cap) grid = cap;
    if (grid > fit) grid = fit;
    if (grid < 1) grid = 1;
    switch (J.kind) {
#define WB_EXT_CASE(K)                                                              \
    case K:                                                                         \
        elastic_pairs_kernel<K, true><<<(int)grid, kThreads, 0, s>>>(J, ring, P);    \
        break;
        WB_EXT_CASE(K_DTW)
        WB_EXT_CASE(K_WDTW)
        WB_EXT_CASE(K_ADTW)
        WB_EXT_CASE(K_ADTW_ANY)
        WB_EXT_CASE(K_LCSS)
        WB_EXT_CASE(K_WLCSS)
        WB_EXT_CASE(K_EDR)
        WB_EXT_CASE(K_ERP)
        WB_EXT_CASE(K_MSM)
        WB_EXT_CASE(K_TWE)
        WB_EXT_CASE(K_EUCLID)
#undef WB_EXT_CASE
        default:
            return fail(WB_EINVAL, "unknown elastic kernel");
    }
    WB_LAUNCH_CHECK("elastic_pairs_kernel (external ring)");
    return WB_OK;
}

// --------------------------------------------------------------------------
// per-series preparation

// average_slope, distance/_elastic.pyx:3220-3225; out has stride len-2
__global__ void slopes_kernel(const SeriesSet in, double *out) {
    const int L = in.len;
    const int64_t total = in.count * (int64_t)(L - 2);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t s = t / (L - 2);
        int i = (int)(t - s * (L - 2)) + 1;
        const double *q = in.base + s * in.stride;
        double a = q[i] - q[i - 1];
        double b = (q[i + 1] - q[i - 1]) * 0.5;  // x / 2 == x * 0.5 exactly
        out[t] = (a + b) * 0.5;
    }
}

// fast_mean_std, utils/_stats.pyx:22-42 (one thread per series, sequential)
__global__ void mean_std_kernel(const SeriesSet in, double *std_out) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < in.count;
         s += (int64_t)gridDim.x * blockDim.x) {
        const double *x = in.base + s * in.stride;
        double ex = 0, ex2 = 0;
        for (int i = 0; i < in.len; i++) {
            double v = x[i];
            ex = ex + v;
            ex2 = ex2 + v * v;
        }
        double mean = ex / (double)in.len;
        ex2 = ex2 / (double)in.len - mean * mean;
        std_out[s] = ex2 > 1e-13 ? sqrt(ex2) : 0.0;
    }
}

// erp gap tables: tab[s][j] = |y_j - g|, sums[s] = sequential sum
__global__ void erp_tables_kernel(const SeriesSet in, double g, double *tab, double *sums) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < in.count;
         s += (int64_t)gridDim.x * blockDim.x) {
        const double *x = in.base + s * in.stride;
        double acc = 0;
        for (int i = 0; i < in.len; i++) {
            double v = fabs(x[i] - g);
            if (tab) tab[s * in.len + i] = v;
            acc = acc + v;
        }
        sums[s] = acc;
    }
}

// twe column table: tab[s][j] = |y_{j-1} - y_j| with y_{-1} = 0
__global__ void twe_tables_kernel(const SeriesSet in, double *tab) {
    const int L = in.len;
    const int64_t total = in.count * (int64_t)L;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t s = t / L;
        int j = (int)(t - s * L);
        const double *y = in.base + s * in.stride;
        double yp = j == 0 ? 0.0 : y[j - 1];
        tab[t] = fabs(yp - y[j]);
    }
}

__global__ void fill_stab_kernel(double s2, int n, double *stab) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        stab[k] = s2 * (double)k;
}

__global__ void fill_kernel(double *p, double v, int64_t n) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        p[k] = v;
}

static int grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)device_info().sm_count * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

int launch_slopes(const SeriesSet &in, double *out, cudaStream_t s) {
    if (in.len < 3 || in.count == 0) return WB_OK;
    slopes_kernel<<<grid_for(in.count * (in.len - 2), 256), 256, 0, s>>>(in, out);
    WB_LAUNCH_CHECK("slopes_kernel");
    return WB_OK;
}

int launch_mean_std(const SeriesSet &in, double *std_out, cudaStream_t s) {
    if (in.count == 0) return WB_OK;
    mean_std_kernel<<<grid_for(in.count, 128), 128, 0, s>>>(in, std_out);
    WB_LAUNCH_CHECK("mean_std_kernel");
    return WB_OK;
}

int launch_erp_tables(const SeriesSet &in, double g, double *tab, double *sums,
                      cudaStream_t s) {
    if (in.count == 0) return WB_OK;
    erp_tables_kernel<<<grid_for(in.count, 128), 128, 0, s>>>(in, g, tab, sums);
    WB_LAUNCH_CHECK("erp_tables_kernel");
    return WB_OK;
}

int launch_twe_tables(const SeriesSet &in, double *tab, cudaStream_t s) {
    if (in.count == 0) return WB_OK;
    twe_tables_kernel<<<grid_for(in.count * in.len, 256), 256, 0, s>>>(in, tab);
    WB_LAUNCH_CHECK("twe_tables_kernel");
    return WB_OK;
}

int launch_fill_stab(double s2, int n, double *stab, cudaStream_t s) {
    fill_stab_kernel<<<grid_for(n, 256), 256, 0, s>>>(s2, n, stab);
    WB_LAUNCH_CHECK("fill_stab_kernel");
    return WB_OK;
}

int launch_fill(double *p, double v, int64_t n, cudaStream_t s) {
    if (n == 0) return WB_OK;
    fill_kernel<<<grid_for(n, 256), 256, 0, s>>>(p, v, n);
    WB_LAUNCH_CHECK("fill_kernel");
    return WB_OK;
}

}  // namespace wb
