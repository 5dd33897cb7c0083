// profile.cu -- distance profile kernels outside the SubsequenceMetric scans:
// the "mass" profile (z-normalised euclidean by the MASS formula) and the
// window gather of the dilated / padded profile.
//
// MASS (distance/_mass.pyx:194-240, ScaledMassSubsequenceMetric): per window
// i of x, with the window's IncStats mean / std (cumulative_mean_std,
// utils/_stats.pyx:95-111) and the subsequence's transient mean / std
// (_ts_view_update_statistics, distance/_cdistance.pyx:167-185):
//   exactly one std <= 1e-10 -> sqrt(L); both -> 0;
//   else z = 2 (L - (QT_i - L mu_i mu) / (sigma_i sigma)), d = z < 1e-10 ? 0 : sqrt(z)
// with QT_i = sum_j x[i + j] y[j].  The reference takes QT from a pocketfft
// cross-correlation; here it is the exact sequential dot product, so the
// profiles agree to the rounding of the FFT, not bit for bit.

#include "common.cuh"

namespace wb {

namespace {

constexpr double kMassEps = 1e-10;  // EPSILON of distance/_mass.pyx
constexpr double kStatsEps = 1e-13;  // EPSILON of utils/_stats.pyx, distance/_cdistance.pxd

// IncStats window statistics of one series (one thread per series): mean and
// sqrt(variance) of every window of length L, variance < 1e-13 -> 0.
__global__ void mass_window_stats_kernel(const double *x, int64_t n, int64_t x_stride, int T,
                                         int L, double *mean_tab, double *std_tab) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *xr = x + i * x_stride;
    const int nwin = T - L + 1;
    double mean = 0.0, ns = 0.0, ssq = 0.0;
    for (int t = 0; t < T; t++) {
        const double v = xr[t];
        ns = ns + 1.0;
        const double next_m = mean + (v - mean) / ns;
        ssq = ssq + (v - mean) * (v - next_m);
        mean = next_m;
        if (t >= L - 1) {
            const int w = t - (L - 1);
            double var = ns <= 1.0 ? 0.0 : ssq / ns;
            if (var < kStatsEps) var = 0.0;
            mean_tab[i * nwin + w] = mean;
            std_tab[i * nwin + w] = sqrt(var);
            const double u = xr[w];
            if (ns == 1.0) {
                ns = 0.0;
                mean = 0.0;
                ssq = 0.0;
            } else {
                const double old_m = (ns * mean - u) / (ns - 1.0);
                ssq = ssq - (u - mean) * (u - old_m);
                mean = old_m;
                ns = ns - 1.0;
            }
        }
    }
}

// One thread per (series, window): the dot product and the MASS formula.
__global__ void mass_profile_kernel(const double *x, int64_t n, int64_t x_stride, int T,
                                    const double *y, int64_t y_stride, int L,
                                    const double *mean_tab, const double *std_tab,
                                    double *out) {
    const int nwin = T - L + 1;
    const int64_t total = n * nwin;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q / nwin;
        const int w = (int)(q - i * nwin);
        const double *xr = x + i * x_stride + w;
        const double *yr = y + i * y_stride;
        // transient statistics of the subsequence
        double ex = 0.0, ex2 = 0.0, qt = 0.0;
        for (int j = 0; j < L; j++) {
            const double v = yr[j];
            ex += v;
            ex2 += v * v;
            qt += xr[j] * v;
        }
        const double mu = ex / L;
        double var = ex2 / L - mu * mu;
        const double sd = var > kStatsEps ? sqrt(var) : 0.0;
        const double mx = mean_tab[q], sx = std_tab[q];
        const bool zx = sx <= kMassEps, zy = sd <= kMassEps;
        double d;
        if (zx != zy) {
            d = sqrt((double)L);
        } else if (zx) {
            d = 0.0;
        } else {
            const double z = 2 * (L - (qt - L * mx * mu) / (sx * sd));
            d = z < kMassEps ? 0.0 : sqrt(z);
        }
        out[q] = d;
    }
}

// Dilated / padded windows (distance/_cdistance.pyx:804-933): for output
// position p of series i, the samples x[input_offset + j] and the kernel
// values y[(j + kernel_offset) / dilation] for j = 0, dilation, ... below the
// convolution size; with `scale`, the window is z-normalised by its own
// sequential mean and variance over the full kernel length L (variance <=
// 1e-13 -> std 1).  Every position of [p0, p0 + np) has k samples (the host
// groups positions by k).  One thread per (series, position).
__global__ void dilated_gather_kernel(const double *x, int64_t n, int64_t x_stride, int T,
                                      const double *y, int64_t y_stride, int L, int dilation,
                                      int padding, int p0, int np, int k, int scale,
                                      double *xw, double *kw) {
    const int64_t rows = n * np;
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
         row += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = row / np;
        const int p = p0 + (int)(row - i * np);
        const int po = padding - p;
        int kernel_offset, input_offset;
        if (po > 0) {
            kernel_offset = po % dilation == 0 ? po : po + dilation - po % dilation;
            input_offset = kernel_offset - po;
        } else {
            kernel_offset = 0;
            input_offset = -po;
        }
        const int ks = (L - 1) * dilation + 1;
        const int conv = imin(T, input_offset + ks - imax(0, po)) - input_offset;
        const double *xr = x + i * x_stride;
        const double *yr = y + i * y_stride;
        double *xo = xw + row * k;
        double *ko = kw + row * k;
        double mean = 0.0, ssq = 0.0;
        int t = 0;
        for (int j = 0; j < conv && t < k; j += dilation) {
            const double v = xr[input_offset + j];
            xo[t] = v;
            ko[t] = yr[(j + kernel_offset) / dilation];
            mean += v;
            ssq += v * v;
            t++;
        }
        if (scale) {
            mean = mean / L;
            double sd = ssq / L - mean * mean;
            sd = sd > kStatsEps ? sqrt(sd) : 1.0;
            for (int u = 0; u < k; u++) xo[u] = (xo[u] - mean) / sd;
        }
    }
}

// out[i, p] = d[row] / ((float) k / (float) L), the reference's rescaling of a
// partial window (the factor is formed in float32)
__global__ void dilated_scatter_kernel(const double *d, int64_t n, int p0, int np, int k,
                                       int L, double *out, int64_t out_ld) {
    const int64_t rows = n * np;
    const float f = (float)k / (float)L;
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
         row += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = row / np;
        const int p = p0 + (int)(row - i * np);
        out[i * out_ld + p] = d[row] / (double)f;
    }
}

int grid_for(int64_t work, int block) {
    int64_t g = (work + block - 1) / block;
    const int64_t cap = (int64_t)device_info().sm_count * 32;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

int launch_dilated_gather(const double *x, int64_t n, int64_t x_stride, int T, const double *y,
                          int64_t y_stride, int L, int dilation, int padding, int p0, int np,
                          int k, int scale, double *xw, double *kw, cudaStream_t s) {
    if (n * np == 0) return WB_OK;
    dilated_gather_kernel<<<grid_for(n * np, 128), 128, 0, s>>>(
        x, n, x_stride, T, y, y_stride, L, dilation, padding, p0, np, k, scale, xw, kw);
    WB_LAUNCH_CHECK("dilated_gather_kernel");
    return WB_OK;
}

int launch_dilated_scatter(const double *d, int64_t n, int p0, int np, int k, int L,
                           double *out, int64_t out_ld, cudaStream_t s) {
    if (n * np == 0) return WB_OK;
    dilated_scatter_kernel<<<grid_for(n * np, 256), 256, 0, s>>>(d, n, p0, np, k, L, out,
                                                                   out_ld);
    WB_LAUNCH_CHECK("dilated_scatter_kernel");
    return WB_OK;
}

int launch_mass_profile(const double *x, int64_t n, int64_t x_stride, int T, const double *y,
                        int64_t y_stride, int L, double *mean_tab, double *std_tab,
                        double *out, cudaStream_t s) {
    if (n == 0) return WB_OK;
    mass_window_stats_kernel<<<grid_for(n, 64), 64, 0, s>>>(x, n, x_stride, T, L, mean_tab,
                                                             std_tab);
    WB_LAUNCH_CHECK("mass_window_stats_kernel");
    timer_begin("mass_profile_kernel", s);
    mass_profile_kernel<<<grid_for(n * (T - L + 1), 128), 128, 0, s>>>(
        x, n, x_stride, T, y, y_stride, L, mean_tab, std_tab, out);
    timer_end(s);
    WB_LAUNCH_CHECK("mass_profile_kernel");
    return WB_OK;
}

}  // namespace wb
