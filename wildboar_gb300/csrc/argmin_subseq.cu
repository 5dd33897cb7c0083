// argmin_subseq.cu -- the k closest windows of subsequence i in series i
// (argmin_subsequence_distance), FP64, in the reference's heap order.
//
// _ArgminSubsequenceDistance / _ScaledArgminSubsequenceDistance
// (distance/_cdistance.pyx:1381-1557) scan the windows j of series i in order
// and call the pairwise metric's pointer-form eadistance on (S_i, window j)
// with the current k-th distance, pushing a window into the k-max Heap when
// it returns true.  Here one warp takes one pair and its 32 lanes evaluate 32
// consecutive windows with the metric's full recurrence (the same two-row
// band recurrences as the pairwise kernels), each giving its distance and its
// abandon key (the largest per-row minimum); lane 0 then replays the 32
// eadistance calls in window order against the heap, abandoning a window iff
// its key exceeds the threshold the metric would have used, which reproduces
// the reference's pushes and heap exactly.
//
// Scaled: the subsequence is z-normalised with its own statistics (computed
// on the host, sequential sums of v and v * v, as the compiled fast_mean_std
// does) and every window with the
// IncStats mean / std sequence of its series (utils/_stats.pyx:45-93), which a
// prepass reproduces per series; normalised windows (or their slopes for the
// derivative metrics) are materialised per batch of pairs.

#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "argmin.cuh"
#include "elastic_rec.cuh"

namespace wb {

struct ArgminSubseqJob {
    const double *S = nullptr;   // compared rows of the subsequences, row p at p * s_stride
    const int64_t *s_len = nullptr;  // original subsequence lengths
    int64_t s_stride = 0;
    SeriesSet x;                 // the series (values, or slopes for ddtw / wddtw)
    int t_len = 0;               // original series length
    const double *W = nullptr;   // scaled: windows [pair - p0][w][w_stride]
    const double *G = nullptr;   // scaled erp: |W - g| in the same layout
    int64_t w_ld = 0;            // windows per pair in W
    int w_stride = 0;
    const double *gtab = nullptr;  // unscaled erp: |x - g| per series (n, t_len)
    int64_t p0 = 0, p1 = 0;      // pairs of this launch
    int metric = WB_EUCLIDEAN;
    int slopes = 0;
    double r = 1.0, eps = 0, p = 0, g = 0, c = 0, penalty = 0, stiffness = 0;
    const double *weights = nullptr;
    const double *stab = nullptr;
    int64_t k = 1;
    int64_t *heap_idx = nullptr;  // (n, k)
    double *heap_val = nullptr;
    int64_t *out_idx = nullptr;   // (n, k)
    double *out_dist = nullptr;
    int no_abandon = 0;           // evaluate every window in full (WB_GPU_ARGMIN=all)
};

// fast_mean_std, utils/_stats.pyx:22-42 (x*x: the reference's pow(x, 2.0) is
// folded into a multiplication by its C compiler)
__device__ __forceinline__ double row_std(const double *x, int n) {
    double ex = 0, ex2 = 0;
    for (int i = 0; i < n; i++) {
        const double v = x[i];
        ex = ex + v;
        ex2 = ex2 + v * v;
    }
    const double mean = ex / (double)n;
    const double var = ex2 / (double)n - mean * mean;
    return var > 1e-13 ? sqrt(var) : 0.0;
}

constexpr int kAsThreads = 128;

template <int KIND>
__global__ void __launch_bounds__(kAsThreads)
argmin_subseq_kernel(const ArgminSubseqJob J, double *gring, int P) {
    const double INF = WB_INF;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * kAsThreads + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * kAsThreads) >> 5;
    const int64_t gtid = (int64_t)blockIdx.x * kAsThreads + threadIdx.x;
    RingG ring{gring + gtid, (int64_t)gridDim.x * kAsThreads};
    for (int64_t pi = J.p0 + warp; pi < J.p1; pi += nwarps) {
        const int L = (int)J.s_len[pi];
        int64_t *hi = J.heap_idx + pi * J.k;
        double *hv = J.heap_val + pi * J.k;
        int64_t n = 0;
        if (!(J.slopes && L < 3)) {
            const int Lc = J.slopes ? L - 2 : L;  // length of the compared rows
            const int nwin = J.t_len - L + 1;
            const int band = (int)fmax(floor((double)Lc * J.r), 1.0);
            const double *S = J.S + pi * J.s_stride;
            double gx_sum = 0.0, sx = 0.0;
            if (KIND == K_ERP)
                for (int q = 0; q < Lc; q++) gx_sum = gx_sum + fabs(S[q] - J.g);
            if (KIND == K_EDR && isnan(J.eps)) sx = row_std(S, Lc);
            double distance = INF;
            // windows abandon at the threshold of the heap after the earlier
            // rounds (it only falls within a round); lcss / wlcss thresholds
            // fall as the k-th distance grows and adtw's square of a negative
            // root is no bound: those evaluate every window in full
            constexpr bool EA = KIND == K_DTW || KIND == K_WDTW || KIND == K_ADTW ||
                                KIND == K_EDR || KIND == K_ERP || KIND == K_MSM ||
                                KIND == K_TWE;
            for (int base = 0; base < nwin; base += 32) {
                const int w = base + lane;
                double d = INF, key = INF;
                const double bound =
                    (EA && !J.no_abandon)
                        ? abandon_threshold(J.metric, __shfl_sync(0xffffffffu, distance, 0), L, L)
                        : INF;
                if (w < nwin) {
                    const double *Y = J.W ? J.W + ((pi - J.p0) * J.w_ld + w) * J.w_stride
                                          : J.x.base + pi * J.x.stride + w;
                    double raw = 0.0;
                    if constexpr (KIND == K_EUCLID) {
                        // euclidean_distance, distance/_metric.pyx:654-682
                        for (int q = 0; q < Lc; q++) {
                            double v = Y[q];
                            v = v - S[q];
                            raw = raw + v * v;
                        }
                        key = -INF;
                        d = sqrt(raw);
                    } else {
                        if constexpr (KIND == K_DTW)
                            raw = rec_dtw<false, RingG, EA>(ring, P, S, Lc, Y, Lc, band, nullptr, key,
                                                            bound);
                        else if constexpr (KIND == K_WDTW)
                            raw = rec_dtw<true, RingG, EA>(ring, P, S, Lc, Y, Lc, band, J.weights,
                                                           key, bound);
                        else if constexpr (KIND == K_ADTW)
                            raw = rec_adtw<true, RingG, EA>(ring, P, S, Lc, Y, Lc, band, J.p, key,
                                                            bound);
                        else if constexpr (KIND == K_ADTW_ANY)
                            raw = rec_adtw<false>(ring, P, S, Lc, Y, Lc, band, J.p, key);
                        else if constexpr (KIND == K_LCSS)
                            raw = rec_lcss<false>(ring, P, S, Lc, Y, Lc, band, J.eps, nullptr,
                                                  key);
                        else if constexpr (KIND == K_WLCSS)
                            raw = rec_lcss<true>(ring, P, S, Lc, Y, Lc, band, J.eps, J.weights,
                                                 key);
                        else if constexpr (KIND == K_EDR) {
                            double eps = J.eps;
                            if (isnan(eps)) eps = fmax(sx, row_std(Y, Lc)) / 4.0;
                            raw = rec_edr<RingG, EA>(ring, P, S, Lc, Y, Lc, band, eps, key, bound);
                        } else if constexpr (KIND == K_ERP) {
                            const double *gY = J.W ? J.G + ((pi - J.p0) * J.w_ld + w) * J.w_stride
                                                   : J.gtab + pi * J.t_len + w;
                            double gy_sum = 0.0;
                            for (int q = 0; q < Lc; q++) gy_sum = gy_sum + gY[q];
                            raw = rec_erp<RingG, EA>(ring, P, S, Lc, Y, Lc, band, J.g, gx_sum, gy_sum,
                                                     gY, key, bound);
                        } else if constexpr (KIND == K_MSM)
                            raw = rec_msm<RingG, EA>(ring, P, S, Lc, Y, Lc, band, J.c, key, bound);
                        else
                            raw = rec_twe<RingG, false, EA>(ring, P, S, Lc, Y, Lc, band, J.penalty,
                                                            J.stiffness, nullptr, J.stab, key,
                                                            bound);
                        if (KIND == K_LCSS || KIND == K_WLCSS) d = 1.0 - raw / (double)Lc;
                        else if (KIND == K_EDR) d = raw / (double)Lc;
                        else if (KIND == K_ERP || KIND == K_MSM || KIND == K_TWE) d = raw;
                        else d = sqrt(raw);
                    }
                }
                // the 32 eadistance calls in window order
                for (int t = 0; t < 32; t++) {
                    const double dt = __shfl_sync(0xffffffffu, d, t);
                    const double kt = __shfl_sync(0xffffffffu, key, t);
                    if (base + t >= nwin) break;
                    if (lane == 0) {
                        const double thr = abandon_threshold(J.metric, distance, L, L);
                        if (!(kt > thr) && dt < distance) {
                            heap_push(hi, hv, n, J.k, base + t, dt);
                            distance = (n == J.k) ? hv[0] : INF;
                        }
                    }
                }
            }
        }
        if (lane == 0) {
            for (int64_t t = 0; t < J.k; t++) {
                J.out_idx[pi * J.k + t] = t < n ? hi[t] : 0;
                J.out_dist[pi * J.k + t] = t < n ? hv[t] : 0.0;
            }
        }
    }
}

// IncStats window statistics of the scaled path, one thread per pair:
// add the first L - 1 values, then per window add the last value, take
// mean / std (variance <= 1e-13 -> 0 -> std 1), remove the first value.
__global__ void incstats_windows_kernel(const ArgminSubseqJob J, const double *T,
                                        int64_t t_stride, double *mean_tab, double *std_tab,
                                        int64_t ld) {
    for (int64_t pi = J.p0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pi < J.p1;
         pi += (int64_t)gridDim.x * blockDim.x) {
        const double *x = T + pi * t_stride;
        const int L = (int)J.s_len[pi];
        const int nwin = J.t_len - L + 1;
        double mean = 0.0, ns = 0.0, ssq = 0.0;
        auto add = [&](double v) {
            ns = ns + 1.0;
            const double next_m = mean + (v - mean) / ns;
            ssq = ssq + (v - mean) * (v - next_m);
            mean = next_m;
        };
        for (int q = 0; q < L - 1; q++) add(x[q]);
        double *mt = mean_tab + (pi - J.p0) * ld;
        double *st = std_tab + (pi - J.p0) * ld;
        for (int w = 0; w < nwin; w++) {
            add(x[w + L - 1]);
            double var = ns <= 1.0 ? 0.0 : ssq / ns;
            if (var < 1e-13) var = 0.0;
            mt[w] = mean;
            st[w] = var == 0.0 ? 1.0 : sqrt(var);
            const double v = x[w];
            if (ns == 1.0) {
                ns = 0.0;
                mean = 0.0;
                ssq = 0.0;
            } else {
                const double old_m = (ns * mean - v) / (ns - 1.0);
                ssq = ssq - (v - mean) * (v - old_m);
                mean = old_m;
                ns = ns - 1.0;
            }
        }
    }
}

// normalised windows (t - mean_w) / std_w of the batch, then their slopes
// for the derivative metrics, and |. - g| for erp
__global__ void normalise_windows_kernel(const ArgminSubseqJob J, const double *T,
                                         int64_t t_stride, const double *mean_tab,
                                         const double *std_tab, int64_t ld, double *W,
                                         double *G, int w_stride) {
    const int64_t total = (J.p1 - J.p0) * ld;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pr = t / ld;
        const int w = (int)(t - pr * ld);
        const int64_t pi = J.p0 + pr;
        const int L = (int)J.s_len[pi];
        if (w >= J.t_len - L + 1) continue;
        const double *x = T + pi * t_stride + w;
        const double mu = mean_tab[pr * ld + w], sd = std_tab[pr * ld + w];
        double *out = W + t * w_stride;
        if (J.slopes) {
            if (L < 3) continue;
            // average_slope of the normalised window, distance/_elastic.pyx:3220-3225
            double zm = (x[0] - mu) / sd, z0 = (x[1] - mu) / sd;
            for (int q = 1; q < L - 1; q++) {
                const double zp = (x[q + 1] - mu) / sd;
                const double a = z0 - zm;
                const double b = (zp - zm) * 0.5;
                out[q - 1] = (a + b) * 0.5;
                zm = z0;
                z0 = zp;
            }
        } else {
            for (int q = 0; q < L; q++) {
                const double z = (x[q] - mu) / sd;
                out[q] = z;
                if (G) G[t * w_stride + q] = fabs(z - J.g);
            }
        }
    }
}

// (S - mean) / std with the given statistics (std 0 -> 1), in place layout
__global__ void normalise_rows_kernel(const double *S, const int64_t *len, int64_t stride,
                                      int64_t n, const double *mean, const double *std,
                                      double *out) {
    for (int64_t pi = blockIdx.x; pi < n; pi += gridDim.x) {
        const double sd = std[pi] != 0.0 ? std[pi] : 1.0;
        for (int q = threadIdx.x; q < (int)len[pi]; q += blockDim.x)
            out[pi * stride + q] = (S[pi * stride + q] - mean[pi]) / sd;
    }
}

int launch_normalise_rows(const double *S, const int64_t *len, int64_t stride, int64_t n,
                          const double *mean, const double *std, double *out,
                          cudaStream_t s) {
    if (n == 0) return WB_OK;
    normalise_rows_kernel<<<(int)(n < 65535 ? n : 65535), 64, 0, s>>>(S, len, stride, n,
                                                                       mean, std, out);
    WB_LAUNCH_CHECK("normalise_rows_kernel");
    return WB_OK;
}

int launch_incstats_windows(const ArgminSubseqJob &J, const double *T, int64_t t_stride,
                            double *mean_tab, double *std_tab, int64_t ld, cudaStream_t s) {
    const int64_t n = J.p1 - J.p0;
    if (n <= 0) return WB_OK;
    incstats_windows_kernel<<<(int)((n + 63) / 64), 64, 0, s>>>(J, T, t_stride, mean_tab,
                                                                  std_tab, ld);
    WB_LAUNCH_CHECK("incstats_windows_kernel");
    return WB_OK;
}

int launch_normalise_windows(const ArgminSubseqJob &J, const double *T, int64_t t_stride,
                             const double *mean_tab, const double *std_tab, int64_t ld,
                             double *W, double *G, int w_stride, cudaStream_t s) {
    const int64_t total = (J.p1 - J.p0) * ld;
    if (total <= 0) return WB_OK;
    int64_t g = (total + 255) / 256, cap = (int64_t)device_info().sm_count * 16;
    normalise_windows_kernel<<<(int)(g < cap ? g : cap), 256, 0, s>>>(
        J, T, t_stride, mean_tab, std_tab, ld, W, G, w_stride);
    WB_LAUNCH_CHECK("normalise_windows_kernel");
    return WB_OK;
}

// ring length and grid of the main kernel for subsequences up to max_len
size_t argmin_subseq_ring_bytes(int64_t n_pairs, int max_len, double r, int *P_out,
                                int *grid_out) {
    const int band = (int)std::max(std::floor((double)max_len * r), 1.0);
    const int P = imax(2, ring_len(max_len, max_len, band));
    int64_t grid = (n_pairs * 32 + kAsThreads - 1) / kAsThreads;
    const int64_t cap = (int64_t)8 * device_info().sm_count;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    *P_out = P;
    *grid_out = (int)grid;
    return align256((size_t)P * grid * kAsThreads * sizeof(double));
}

int launch_argmin_subseq(const ArgminSubseqJob &J, int kind, double *gring, int P, int grid,
                         cudaStream_t s) {
    if (J.p1 <= J.p0) return WB_OK;
    timer_begin("argmin_subseq_kernel", s);
    switch (kind) {
#define WB_AS_CASE(K)                                                        \
    case K:                                                                  \
        argmin_subseq_kernel<K><<<grid, kAsThreads, 0, s>>>(J, gring, P);    \
        break;
        WB_AS_CASE(K_EUCLID)
        WB_AS_CASE(K_DTW)
        WB_AS_CASE(K_WDTW)
        WB_AS_CASE(K_ADTW)
        WB_AS_CASE(K_ADTW_ANY)
        WB_AS_CASE(K_LCSS)
        WB_AS_CASE(K_WLCSS)
        WB_AS_CASE(K_EDR)
        WB_AS_CASE(K_ERP)
        WB_AS_CASE(K_MSM)
        WB_AS_CASE(K_TWE)
#undef WB_AS_CASE
        default:
            return fail(WB_EINVAL, "no argmin subsequence kernel for this metric");
    }
    timer_end(s);
    WB_LAUNCH_CHECK("argmin_subseq_kernel");
    return WB_OK;
}

// --------------------------------------------------------------------------
// host side

static std::vector<double> host_logistic(int64_t n, double g) {
    // WeightedDtwMetric.reset: distance/_elastic.pyx:3333-3341
    std::vector<double> w((size_t)std::max<int64_t>(n, 1));
    for (int64_t i = 0; i < n; i++)
        w[i] = 1.0 / (1.0 + std::exp(-g * ((double)i - (double)n / 2.0)));
    return w;
}

int wb_argmin_subsequence_impl(const double *s, const int64_t *s_len, int64_t s_stride,
                               int64_t n, const double *s_mean, const double *s_std,
                               const wb_series *x, int64_t dim, int32_t metric,
                               const wb_params *params, int32_t scaled, int64_t k,
                               int64_t *indices, double *distances, int32_t out_on_device,
                               cudaStream_t st) {
    if (!x || !params) return fail(WB_EINVAL, "x and params are required");
    if (x->dtype != WB_F64 || x->n_dims < 1 || x->n_timestep < 1 || x->n < 0)
        return fail(WB_EINVAL, "x must be float64 (n, n_dims, n_timestep)");
    if (dim < 0 || dim >= x->n_dims)
        return fail(WB_EINVAL, "The parameter dim must be dim (" + std::to_string(dim) +
                                   ") < n_dims (" + std::to_string(x->n_dims) + ")");
    if (n != x->n) return fail(WB_EINVAL, "both arrays must have the same number of samples.");
    if (n == 0) return WB_OK;
    if (!s || !s_len || !indices || !distances) return fail(WB_EINVAL, "NULL argument");
    if (scaled && (!s_mean || !s_std)) return fail(WB_EINVAL, "scaled needs s_mean and s_std");
    const int T = (int)x->n_timestep;
    int64_t max_len = 0, min_len = INT64_MAX;
    for (int64_t i = 0; i < n; i++) {
        if (s_len[i] < 1 || s_len[i] > s_stride) return fail(WB_EINVAL, "bad subsequence length");
        max_len = std::max(max_len, s_len[i]);
        min_len = std::min(min_len, s_len[i]);
    }
    if (max_len > T)
        return fail(WB_EINVAL, "the longest subsequence must be shorter than samples.");
    if (k < 1 || k > T - s_stride + 1)
        return fail(WB_EINVAL, "k must be less x.shape[-1] - y.shape[-1] + 1.");
    if (!(params->r >= 0.0 && params->r <= 1.0)) return fail(WB_EINVAL, "r must be in [0, 1]");
    int kind;
    const bool deriv = metric == WB_DDTW || metric == WB_WDDTW;
    switch (metric) {
        case WB_EUCLIDEAN: kind = K_EUCLID; break;
        case WB_DTW: case WB_DDTW: kind = K_DTW; break;
        case WB_WDTW: case WB_WDDTW: kind = K_WDTW; break;
        case WB_ADTW: kind = params->p >= 0.0 ? K_ADTW : K_ADTW_ANY; break;
        case WB_LCSS: kind = K_LCSS; break;
        case WB_WLCSS: kind = K_WLCSS; break;
        case WB_EDR: kind = K_EDR; break;
        case WB_ERP: kind = K_ERP; break;
        case WB_MSM: kind = K_MSM; break;
        case WB_TWE: kind = K_TWE; break;
        default:
            return fail(WB_EUNSUPPORTED, "unsupported metric id " + std::to_string(metric));
    }
    if ((kind == K_LCSS || kind == K_WLCSS) && !(params->epsilon > 0.0))
        return fail(WB_EINVAL, "epsilon must be > 0");

    ArgminSubseqJob J;
    J.metric = metric;
    J.slopes = deriv ? 1 : 0;
    J.t_len = T;
    J.r = params->r;
    J.eps = params->epsilon;
    J.p = params->p;
    J.g = params->g;
    J.c = params->c;
    J.penalty = params->penalty;
    J.stiffness = params->stiffness;
    J.k = k;
    J.s_stride = s_stride;
    std::vector<double> w;
    // Metric.reset(t, s): weights sized by max(t.shape[2], s.shape[2])
    if (metric == WB_WDTW || metric == WB_WLCSS) w = host_logistic(std::max<int64_t>(T, s_stride), params->g);
    if (metric == WB_WDDTW) w = host_logistic(std::max<int64_t>(T - 2, s_stride - 2), params->g);
    const int ts = deriv ? std::max(T - 2, 1) : T;      // compared series row length
    const int64_t ld = T - min_len + 1;                  // windows per pair (max)
    const int w_stride = (int)(deriv ? std::max<int64_t>(max_len - 2, 1) : max_len);
    int P = 0, grid = 0;
    const size_t ring = argmin_subseq_ring_bytes(n, (int)max_len, params->r, &P, &grid);
    // scaled: windows materialised per batch of pairs (~512 MB)
    const size_t per_pair = (size_t)ld * w_stride * 8 * (kind == K_ERP ? 2 : 1) + 2 * ld * 8;
    int64_t batch = scaled ? std::max<int64_t>(1, (int64_t)((512ull << 20) / per_pair)) : n;
    if (batch > n) batch = n;
    size_t need = ring + align256((size_t)n * T * 8) + align256((size_t)n * s_stride * 8) * 3 +
                  align256((size_t)n * 8) * 4 + 4 * align256((size_t)n * k * 8) +
                  align256(w.size() * 8 + 8) + align256((size_t)T * 8 + 8) +
                  (deriv ? align256((size_t)n * ts * 8) : 0) +
                  (kind == K_ERP ? align256((size_t)n * T * 8) + align256((size_t)n * 8) : 0) +
                  (scaled ? align256(per_pair * batch) + 4096 : 0);
    Workspace ws(st);
    WB_TRY(ws.reserve(need));
    WB_TAKE(gring, double, ws, ring / sizeof(double));
    // series of this dim
    WB_TAKE(X, double, ws, (size_t)n * T);
    {
        const double *base = static_cast<const double *>(x->data) + dim * T;
        WB_CUDA(cudaMemcpy2DAsync(X, T * sizeof(double), base, x->n_dims * T * sizeof(double),
                                  T * sizeof(double), n,
                                  x->on_device ? cudaMemcpyDeviceToDevice
                                               : cudaMemcpyHostToDevice, st));
    }
    WB_TAKE(dS, double, ws, (size_t)n * s_stride);
    WB_TAKE(dlen, int64_t, ws, n);
    WB_CUDA(cudaMemcpyAsync(dS, s, (size_t)n * s_stride * 8, cudaMemcpyHostToDevice, st));
    WB_CUDA(cudaMemcpyAsync(dlen, s_len, n * 8, cudaMemcpyHostToDevice, st));
    const double *Srow = dS;
    if (scaled) {
        WB_TAKE(dm, double, ws, n);
        WB_TAKE(dsd, double, ws, n);
        WB_TAKE(dSn, double, ws, (size_t)n * s_stride);
        WB_CUDA(cudaMemcpyAsync(dm, s_mean, n * 8, cudaMemcpyHostToDevice, st));
        WB_CUDA(cudaMemcpyAsync(dsd, s_std, n * 8, cudaMemcpyHostToDevice, st));
        WB_TRY(launch_normalise_rows(dS, dlen, s_stride, n, dm, dsd, dSn, st));
        Srow = dSn;
    }
    if (deriv) {
        std::vector<int64_t> off(n);
        for (int64_t i = 0; i < n; i++) off[i] = i * s_stride;
        WB_TAKE(doff, int64_t, ws, n);
        WB_TAKE(dSs, double, ws, (size_t)n * s_stride);
        WB_CUDA(cudaMemcpyAsync(doff, off.data(), n * 8, cudaMemcpyHostToDevice, st));
        WB_TRY(launch_shapelet_slopes(Srow, doff, dlen, n, dSs, st));
        WB_CUDA(cudaStreamSynchronize(st));  // `off` feeds an asynchronous copy
        Srow = dSs;
    }
    J.S = Srow;
    J.s_len = dlen;
    J.x = SeriesSet{X, (int64_t)T, n, T};
    if (deriv && !scaled) {
        WB_TAKE(Xs, double, ws, (size_t)n * ts);
        if (T >= 3) WB_TRY(launch_slopes(J.x, Xs, st));
        J.x = SeriesSet{Xs, (int64_t)ts, n, ts};
    }
    if (kind == K_ERP && !scaled) {
        WB_TAKE(gt, double, ws, (size_t)n * T);
        WB_TAKE(gs, double, ws, n);
        WB_TRY(launch_erp_tables(SeriesSet{X, (int64_t)T, n, T}, params->g, gt, gs, st));
        J.gtab = gt;
    }
    if (!w.empty()) {
        WB_TAKE(dw, double, ws, w.size());
        WB_CUDA(cudaMemcpyAsync(dw, w.data(), w.size() * 8, cudaMemcpyHostToDevice, st));
        J.weights = dw;
    }
    if (kind == K_TWE) {
        WB_TAKE(stb, double, ws, T);
        WB_TRY(launch_fill_stab(params->stiffness * 2.0, T, stb, st));
        J.stab = stb;
    }
    WB_TAKE(hidx, int64_t, ws, (size_t)n * k);
    WB_TAKE(hval, double, ws, (size_t)n * k);
    J.heap_idx = hidx;
    J.heap_val = hval;
    J.no_abandon = argmin_ea_disabled() ? 1 : 0;
    int64_t *oi = indices;
    double *od = distances;
    if (!out_on_device) {
        oi = ws.take<int64_t>((size_t)n * k);
        od = ws.take<double>((size_t)n * k);
        if (!oi || !od) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    J.out_idx = oi;
    J.out_dist = od;
    double *mt = nullptr, *sdt = nullptr, *W = nullptr, *G = nullptr;
    if (scaled) {
        mt = ws.take<double>((size_t)batch * ld);
        sdt = ws.take<double>((size_t)batch * ld);
        W = ws.take<double>((size_t)batch * ld * w_stride);
        if (kind == K_ERP) G = ws.take<double>((size_t)batch * ld * w_stride);
        if (!mt || !sdt || !W || (kind == K_ERP && !G))
            return fail(WB_ENOMEM, "workspace reservation exceeded");
        J.w_ld = ld;
        J.w_stride = w_stride;
    }
    for (int64_t p0 = 0; p0 < n; p0 += batch) {
        J.p0 = p0;
        J.p1 = std::min(n, p0 + batch);
        if (scaled) {
            WB_TRY(launch_incstats_windows(J, X, T, mt, sdt, ld, st));
            WB_TRY(launch_normalise_windows(J, X, T, mt, sdt, ld, W, G, w_stride, st));
            J.W = W;
            J.G = G;
        }
        WB_TRY(launch_argmin_subseq(J, kind, gring, P, grid, st));
    }
    if (!out_on_device) {
        WB_CUDA(cudaMemcpyAsync(indices, oi, (size_t)n * k * 8, cudaMemcpyDeviceToHost, st));
        WB_CUDA(cudaMemcpyAsync(distances, od, (size_t)n * k * 8, cudaMemcpyDeviceToHost, st));
    }
    WB_CUDA(cudaStreamSynchronize(st));
    return WB_OK;
}

}  // namespace wb

using namespace wb;

extern "C" int wb_argmin_subsequence_distance(const double *s, const int64_t *s_len,
                                              int64_t s_stride, int64_t n,
                                              const double *s_mean, const double *s_std,
                                              const wb_series *x, int64_t dim, int32_t metric,
                                              const wb_params *params, int32_t scaled,
                                              int64_t k, int64_t *indices, double *distances,
                                              int32_t out_on_device, void *stream) {
    WB_TRACE();
    return wb_argmin_subsequence_impl(s, s_len, s_stride, n, s_mean, s_std, x, dim, metric,
                                      params, scaled, k, indices, distances, out_on_device,
                                      (cudaStream_t)stream);
}
