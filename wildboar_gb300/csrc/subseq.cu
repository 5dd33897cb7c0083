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
//
// FP32 pre-filter.  Once a scan has a best sum b, a window is first summed in
// FP32 on float copies t', s' of its values; it is evaluated in FP64 only if
// that cannot prove its FP64 sum d64 > b.  With u = 2^-24, e = u (max|t| +
// max|s|) bounding |(t - s) - (t' - s')| per element, and d32 the FP32 sum
// (one rounding per subtraction and per fused multiply-add):
//   sqrt(d64) >= (sqrt(d32 / F) - e sqrt(L)) (1 - g),
//   F = 1 + (L + 4) u 1.01,  g = (L + 4) 2^-53 1.01
// (sums of non-negative terms; the triangle inequality in the 2-norm for the
// input rounding).  So d32 > F (sqrt(b)(1 + g) + e sqrt(L))^2, rounded up to
// float, implies d64 > b: such a window can be neither the minimum nor the
// first window attaining it, exactly as if the FP64 sum had been abandoned.
// Partial FP32 sums only grow, so the filter abandons early too.  Results are
// unchanged; only the number of FP64 evaluations drops.

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

// Comparisons of the (non-negative or +inf) sums run on their bit patterns:
// for x, y >= +0 the IEEE order is the signed 64-bit order, so the integer
// pipe takes them and the FP64 pipe only does the sums.
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// Float threshold of the FP32 pre-filter, computed in FP32 with every
// operation rounded up (so it is at least the bound of the file header):
// bf >= best (the FP64 sum rounded up), e >= 2^-24 (max|t| + max|s|); the
// factor 1 + 2^-22 covers the FP64 rounding term g and F uses 6.1e-8 > 1.01
// 2^-24.  FP32 keeps the per-tile recomputation off the FP64 pipe.
__device__ __forceinline__ float filter_threshold(float bf, float e, int L) {
    if (isinf(bf)) return __int_as_float(0x7f800000);
    const float F = __fadd_ru(1.0f, __fmul_ru((float)(L + 4), 6.1e-8f));
    const float sb = __fsqrt_ru(bf);
    const float root = __fadd_ru(__fmul_ru(sb, 1.0000003f), __fmul_ru(e, __fsqrt_ru((float)L)));
    return __fmul_ru(F, __fmul_ru(root, root));
}

// e = 2^-24 (max|t| + max|s|) rounded up, plus an absolute term for subnormals
__device__ __forceinline__ float filter_e(float mt, float ms) {
    return __fadd_ru(__fmul_ru(5.9604644775390625e-08f, __fadd_ru(mt, ms)), 1e-37f);
}

// float copies of packed shapelet values and the max |value| of each
__global__ void shapelet_f32_kernel(const double *src, const int64_t *off, const int64_t *len,
                                    int64_t m, float *dst, float *absmax) {
    __shared__ double red[32];
    for (int64_t s = blockIdx.x; s < m; s += gridDim.x) {
        const int L = (int)len[s];
        double mx = 0.0;
        for (int k = threadIdx.x; k < L; k += blockDim.x) {
            const double v = src[off[s] + k];
            dst[off[s] + k] = (float)v;
            mx = fmax(mx, fabs(v));
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) a = fmax(a, red[w]);
            absmax[s] = __double2float_ru(a);
        }
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
    float *Tf = reinterpret_cast<float *>(T + nt);          // nt floats (unscaled filter)
    unsigned int *tmax = reinterpret_cast<unsigned int *>(Tf + nt + (nt & 1));
    const bool filt = !SCALED && J.shp_f32 != nullptr;
    __shared__ int wqueue[kSubWarps][64];
    for (int64_t b = blockIdx.x; b < J.x.count * chunks; b += gridDim.x) {
        const int64_t si = b / chunks;
        const int64_t c0 = (b - si * chunks) * J.chunk;
        const int64_t c1 = c0 + J.chunk < J.m ? c0 + J.chunk : J.m;
        __syncthreads();
        if (filt && threadIdx.x == 0) *tmax = 0u;
        __syncthreads();
        const double *Tg = J.x.base + si * J.x.stride;
        for (int i = threadIdx.x; i < nt; i += kSubThreads) {
            const double v = Tg[i];
            T[i] = v;
            if (filt) {
                Tf[i] = (float)v;
                // max |t| as a float rounded up (non-negative: integer order)
                atomicMax(tmax, __float_as_uint(__double2float_ru(fabs(v))));
            }
        }
        __syncthreads();
        const float MT = filt ? __uint_as_float(*tmax) : 0.0f;
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
            const float *Sf = filt ? J.shp_f32 + J.offsets[idx] : nullptr;
            const float e = filt ? filter_e(MT, J.shp_absmax[idx]) : 0.0f;
            float thr32 = __int_as_float(0x7f800000);
            // Windows that pass the filter wait in a FIFO (ascending window
            // order) and are summed in FP64 32 at a time, so the FP64 pipe
            // works on full warps.  The order of evaluation stays ascending,
            // so "first strictly smaller" keeps its meaning.
            int *wq = wqueue[wid];
            int qh = 0, qn = 0;
            auto eval_batch = [&](int cnt) {
                double dist = INF;
                int w = 0x7fffffff;
                if (lane < cnt) {
                    w = wq[(qh + lane) & 63];
                    dist = 0.0;
                    if (SCALED) {
                        const double mean = mt[w];
                        const double sd = st[w];
                        for (int k = 0; k < L; k++) {
                            if (dbits(dist) >= dbits(best)) break;
                            double x = __ldg(S + k);
                            x = x - (T[w + k] - mean) / sd;
                            dist = dist + x * x;
                        }
                    } else {
                        for (int k = 0; k < L; k++) {
                            if (dbits(dist) >= dbits(best)) break;
                            double x = T[w + k];
                            x = x - __ldg(S + k);
                            dist = dist + x * x;
                        }
                    }
                    if (!(dbits(dist) < dbits(best))) dist = INF;
                }
                // lexicographic (dist, window) minimum over the warp
                double v = dist;
                int vi = w;
                for (int o = 16; o > 0; o >>= 1) {
                    double ov = __shfl_xor_sync(0xffffffffu, v, o);
                    int oi = __shfl_xor_sync(0xffffffffu, vi, o);
                    if (dbits(ov) < dbits(v) || (dbits(ov) == dbits(v) && oi < vi)) {
                        v = ov;
                        vi = oi;
                    }
                }
                if (dbits(v) < dbits(best)) {
                    best = v;
                    bidx = vi;
                    if (filt) thr32 = filter_threshold(__double2float_ru(best), e, L);
                }
                qh = (qh + cnt) & 63;
                qn -= cnt;
                __syncwarp();
            };
            for (int base = 0; base < nwin; base += 32) {
                const int w = base + lane;
                bool cand = w < nwin;
                if (filt && cand && dbits(best) < dbits(INF)) {
                    float d32 = 0.0f;
                    for (int k = 0; k < L; k++) {
                        const float y = __fsub_rn(Tf[w + k], __ldg(Sf + k));
                        d32 = __fmaf_rn(y, y, d32);
                        if (d32 > thr32) {
                            cand = false;
                            break;
                        }
                    }
                }
                const unsigned mask = __ballot_sync(0xffffffffu, cand);
                if (cand) wq[(qh + qn + __popc(mask & ((1u << lane) - 1u))) & 63] = w;
                qn += __popc(mask);
                __syncwarp();
                if (qn >= 32) eval_batch(32);
            }
            if (qn > 0) eval_batch(qn);
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
    float *bestf = reinterpret_cast<float *>(bidx + J.chunk);  // chunk: best rounded up
    double *Z = best + 2 * J.chunk;               // [max_len][32]
    float *Zf = reinterpret_cast<float *>(Z + (size_t)J.max_len * 32);  // [max_len][32]
    unsigned int *zmax = reinterpret_cast<unsigned int *>(Zf + (size_t)J.max_len * 32);
    const bool filt = J.shp_f32 != nullptr;
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
            bestf[q] = __int_as_float(0x7f800000);
            bidx[q] = 0;
        }
        for (int base = 0; base < nwin; base += 32) {
            __syncthreads();
            if (threadIdx.x == 0) *zmax = 0u;
            __syncthreads();
            for (int e = threadIdx.x; e < L * 32; e += kSubThreads) {
                const int k = e >> 5, w = e & 31;
                double z = 0.0;
                if (base + w < nwin) z = (T[base + w + k] - mt[base + w]) / st[base + w];
                Z[e] = z;
                if (filt) {
                    Zf[e] = (float)z;
                    atomicMax(zmax, __float_as_uint(__double2float_ru(fabs(z))));
                }
            }
            __syncthreads();
            const float MZ = filt ? __uint_as_float(*zmax) : 0.0f;
            const int w = base + lane;
            for (int q = wid; q < cnt; q += kSubWarps) {
                const int64_t idx = J.order[first + q];
                const double *S = norm + J.offsets[idx];
                const double bq = best[q];
                double dist = INF;
                bool cand = w < nwin;
                if (filt && cand && dbits(bq) < dbits(INF)) {
                    // FP32 pre-filter (see the file header); e bounds the
                    // rounding of z and of the normalised shapelet to float
                    const float thr32 =
                        filter_threshold(bestf[q], filter_e(MZ, J.shp_absmax[idx]), L);
                    const float *Sf = J.shp_f32 + J.offsets[idx];
                    float d32 = 0.0f;
                    for (int k = 0; k < L; k++) {
                        const float y = __fsub_rn(__ldg(Sf + k), Zf[k * 32 + lane]);
                        d32 = __fmaf_rn(y, y, d32);
                        if (d32 > thr32) {
                            cand = false;
                            break;
                        }
                    }
                }
                if (cand) {
                    dist = 0.0;
                    for (int k = 0; k < L; k++) {
                        if (dbits(dist) >= dbits(bq)) break;
                        double x = __ldg(S + k);
                        x = x - Z[k * 32 + lane];
                        dist = dist + x * x;
                    }
                    if (!(dbits(dist) < dbits(bq))) dist = INF;
                }
                double v = dist;
                int vi = w;
                for (int o = 16; o > 0; o >>= 1) {
                    double ov = __shfl_xor_sync(0xffffffffu, v, o);
                    int oi = __shfl_xor_sync(0xffffffffu, vi, o);
                    if (dbits(ov) < dbits(v) || (dbits(ov) == dbits(v) && oi < vi)) {
                        v = ov;
                        vi = oi;
                    }
                }
                if (lane == 0 && dbits(v) < dbits(bq)) {
                    best[q] = v;
                    bestf[q] = __double2float_ru(v);
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
                        if (dbits(dist) >= dbits(best)) break;
                        double x = __ldg(S + k);
                        x = x - (__ldg(T + w + k) - mean) / sd;
                        dist = dist + x * x;
                    }
                } else {
                    for (int k = 0; k < L; k++) {
                        if (dbits(dist) >= dbits(best)) break;
                        double x = __ldg(T + w + k);
                        x = x - __ldg(S + k);
                        dist = dist + x * x;
                    }
                }
                if (!(dbits(dist) < dbits(best))) dist = INF;
            }
            double v = dist;
            int vi = w;
            for (int o = 16; o > 0; o >>= 1) {
                double ov = __shfl_xor_sync(0xffffffffu, v, o);
                int oi = __shfl_xor_sync(0xffffffffu, vi, o);
                if (dbits(ov) < dbits(v) || (dbits(ov) == dbits(v) && oi < vi)) {
                    v = ov;
                    vi = oi;
                }
            }
            if (dbits(v) < dbits(best)) {
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
            const double stop = J.stop_sq ? J.stop_sq[i] : __longlong_as_double(0x7ff0000000000000LL);
            for (int k = 0; k < L; k++) {
                if (dist >= stop) break;
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
    return (size_t)J.x.len * 8 + (size_t)J.chunk * 16 + (size_t)J.max_len * 32 * 8 +
           (size_t)J.max_len * 32 * 4 + 16;
}

static int sub_grid(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    int64_t cap = (int64_t)device_info().sm_count * 16;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

size_t subseq_workspace_bytes(const SubseqJob &J, bool scaled) {
    // FP32 copies of the (normalised) shapelets and their max |value|
    const size_t filt = align256((size_t)J.total_values * sizeof(float)) +
                        align256((size_t)J.m * sizeof(double));
    if (!scaled) return filt;
    const size_t rows = J.paired ? (size_t)J.x.count : (size_t)J.n_groups * J.x.count;
    size_t tab = rows * J.win_stride * sizeof(double);
    return 2 * align256(tab) + align256((size_t)J.total_values * sizeof(double)) + filt;
}

static int make_f32_copies(const SubseqJob &J, const double *src, Workspace &ws,
                           SubseqJob &out) {
    float *f = ws.take<float>((size_t)J.total_values);
    float *mx = ws.take<float>((size_t)J.m);
    if (!f || !mx) return fail(WB_ENOMEM, "workspace reservation exceeded");
    shapelet_f32_kernel<<<(int)(J.m < 65535 ? J.m : 65535), 128, 0, ws.stream()>>>(
        src, J.offsets, J.lengths, J.m, f, mx);
    WB_LAUNCH_CHECK("shapelet_f32_kernel");
    out.shp_f32 = f;
    out.shp_absmax = mx;
    return WB_OK;
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
            SubseqJob Jf = J;
            WB_TRY(make_f32_copies(J, norm, ws, Jf));
            auto kt = subseq_scaled_tiled_kernel;
            WB_CUDA(cudaFuncSetAttribute(kt, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tsm));
            const int64_t tb = J.x.count * J.n_chunks;
            const int tgrid = (int)(tb < cap ? tb : cap);
            timer_begin("subseq_scaled_tiled_kernel", s);
            kt<<<tgrid, kSubThreads, tsm, s>>>(Jf, norm, mean_tab, std_tab);
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
        SubseqJob Jf = J;
        WB_TRY(make_f32_copies(J, J.shapelets, ws, Jf));
        // T (doubles), its float copy and the max |t| word
        const size_t fsmem = (size_t)J.x.len * 12 + 16;
        auto k = subseq_scan_kernel<false>;
        WB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
        timer_begin("subseq_scan_kernel", s);
        k<<<grid, kSubThreads, fsmem, s>>>(Jf, nullptr, nullptr, nullptr);
        timer_end(s);
        WB_LAUNCH_CHECK("subseq_scan_kernel");
    }
    return WB_OK;
}

}  // namespace wb
