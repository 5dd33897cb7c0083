// elastic_f32.cu -- FP32 (compensated) recurrences of the elastic metrics
// other than the dtw family (adtw, lcss, wlcss, edr, erp, msm, twe): the
// precision form of the pairwise distance.
//
// Same structure as the FP64 kernels (elastic_f64.cu): one thread per pair,
// 32 pairs per warp sharing a column series, the live band of the previous
// row in a per-thread ring (shared memory, else a global scratch ring), the
// reference's band edges and out-of-band values.  Every cumulative cost is a
// (hi, lo) float pair: each addition is a TwoSum whose rounding error goes
// into lo, minima compare hi.  lcss / edr counts are small integers and exact
// in FP32.  Inputs are read as float64 and rounded to float32; the final
// normalisation (lcss 1 - c/min(n,m), edr c/max(n,m)) and the distance are
// formed in FP64 from hi + lo.  The msm split/merge cost is FP32 in the
// reference already (_msm_cost, distance/_elastic.pyx:1583-1587).

#include "elastic.cuh"

namespace wb {

extern __shared__ float2 wb_smem32[];

struct HL32 {
    float h, l;
};

__device__ __forceinline__ HL32 hl(float h) { return HL32{h, 0.0f}; }

__device__ __forceinline__ HL32 add32(HL32 a, float b) {
    float s = __fadd_rn(a.h, b);
    float bb = __fsub_rn(s, a.h);
    float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return HL32{s, __fadd_rn(a.l, err)};
}

__device__ __forceinline__ HL32 min32(HL32 a, HL32 b) { return b.h < a.h ? b : a; }
__device__ __forceinline__ HL32 max32(HL32 a, HL32 b) { return b.h > a.h ? b : a; }

// split a double into (hi, lo) floats
__device__ __forceinline__ HL32 from_double(double v) {
    float h = (float)v;
    return HL32{h, (float)(v - (double)h)};
}

struct Ring32S {
    int off, s;
    __device__ __forceinline__ HL32 ld(int k) const {
        float2 v = wb_smem32[off + k * s];
        return HL32{v.x, v.y};
    }
    __device__ __forceinline__ void st(int k, HL32 v) const {
        wb_smem32[off + k * s] = make_float2(v.h, v.l);
    }
};

struct Ring32G {
    float2 *p;
    int64_t s;
    __device__ __forceinline__ HL32 ld(int k) const {
        float2 v = p[(int64_t)k * s];
        return HL32{v.x, v.y};
    }
    __device__ __forceinline__ void st(int k, HL32 v) const {
        p[(int64_t)k * s] = make_float2(v.h, v.l);
    }
};

#define WB_F32INF __int_as_float(0x7f800000)

__device__ __forceinline__ int winc(int q, int P) { return (q + 1 == P) ? 0 : q + 1; }
__device__ __forceinline__ int wdec(int q, int P) { return (q == 0) ? P - 1 : q - 1; }
__device__ __forceinline__ float ldf(const double *p) { return (float)__ldg(p); }

// adtw: adtw_distance, distance/_elastic.pyx:943-1008
template <class R>
__device__ HL32 r32_adtw(R ring, int P, const double *X, int n, const double *Y, int m, int r,
                         float pen) {
    const int mx = imax(0, m - n) + r, mn = imax(0, n - m);
    const HL32 INF = hl(WB_F32INF);
    const float x0 = (float)X[0];
    float v = __fsub_rn(x0, ldf(Y));
    HL32 acc = hl(__fmul_rn(v, v));
    ring.st(0, acc);
    const int lim = imin(m, mx);
    int q = 1 % P;
    for (int j = 1; j < lim; j++) {
        v = __fsub_rn(x0, ldf(Y + j));
        acc = add32(acc, __fmul_rn(v, v));
        ring.st(q, acc);
        q = winc(q, P);
    }
    if (mx < m) ring.st(mx % P, INF);
    for (int i = 1; i < n; i++) {
        const int js = imax(0, i - mn - r + 1), je = imin(m, i + mx);
        const float xi = (float)X[i];
        q = js % P;
        HL32 diag = js > 0 ? ring.ld(wdec(q, P)) : INF;
        HL32 left = INF;
        for (int j = js; j < je; j++) {
            HL32 up = ring.ld(q);
            HL32 a = add32(up, pen);
            float d = __fsub_rn(xi, ldf(Y + j));
            HL32 mv = min32(min32(a, left), diag);
            HL32 nv = add32(mv, __fmul_rn(d, d));
            ring.st(q, nv);
            diag = up;
            left = add32(nv, pen);
            q = winc(q, P);
        }
        if (je < m) ring.st(q, INF);
    }
    return ring.ld((m - 1) % P);
}

// lcss / wlcss: lcss_distance, distance/_elastic.pyx:1118-1183
template <bool W, class R>
__device__ HL32 r32_lcss(R ring, int P, const double *X, int n, const double *Y, int m, int r,
                         float eps, const float *w) {
    const int mx = imax(0, m - n) + r, mn = imax(0, n - m);
    const int lim = imin(m, mx);
    int q = 0;
    for (int j = 0; j < lim; j++) {
        ring.st(q, hl(0.0f));
        q = winc(q, P);
    }
    if (mx < m) ring.st(mx % P, hl(0.0f));
    for (int i = 0; i < n; i++) {
        const int js = imax(0, i - mn - r + 1), je = imin(m, i + mx);
        const float xi = (float)X[i];
        q = js % P;
        HL32 diag = js > 0 ? ring.ld(wdec(q, P)) : hl(0.0f);
        HL32 left = hl(0.0f);
        for (int j = js; j < je; j++) {
            HL32 up = ring.ld(q);
            float v = fabsf(__fsub_rn(xi, ldf(Y + j)));
            HL32 nv = (v <= eps) ? add32(diag, W ? w[abs(i - j)] : 1.0f) : max32(left, up);
            ring.st(q, nv);
            diag = up;
            left = nv;
            q = winc(q, P);
        }
        if (je < m) ring.st(q, hl(0.0f));
    }
    return ring.ld((m - 1) % P);
}

// edr: edr_distance, distance/_elastic.pyx:1437-1497 (exact small counts)
template <class R>
__device__ HL32 r32_edr(R ring, int P, const double *X, int n, const double *Y, int m, int r,
                        float eps) {
    const int mx = imax(0, m - n) + r, mn = imax(0, n - m);
    const int lim = imin(m, mx);
    int q = 0;
    for (int j = 0; j < lim; j++) {
        ring.st(q, hl(0.0f));
        q = winc(q, P);
    }
    if (mx < m) ring.st(mx % P, hl(0.0f));
    for (int i = 0; i < n; i++) {
        const int js = imax(0, i - mn - r + 1), je = imin(m, i + mx);
        const float xi = (float)X[i];
        q = js % P;
        float diag = js > 0 ? ring.ld(wdec(q, P)).h : 0.0f;
        float left = 0.0f;
        for (int j = js; j < je; j++) {
            float up = ring.ld(q).h;
            float v = fabsf(__fsub_rn(xi, ldf(Y + j)));
            float a = diag + (v < eps ? 0.0f : 1.0f);
            float nv = fminf(fminf(a, up + 1.0f), left + 1.0f);
            ring.st(q, hl(nv));
            diag = up;
            left = nv;
            q = winc(q, P);
        }
        if (je < m) ring.st(q, hl(0.0f));
    }
    return ring.ld((m - 1) % P);
}

// erp: erp_distance, distance/_elastic.pyx:1273-1347
template <class R>
__device__ HL32 r32_erp(R ring, int P, const double *X, int n, const double *Y, int m, int r,
                        float g, HL32 gx_sum, HL32 gy_sum, const double *gY) {
    const int mx = imax(0, m - n) + r, mn = imax(0, n - m);
    const int lim = imin(m, mx);
    int q = 0;
    for (int j = 0; j < lim; j++) {
        ring.st(q, gy_sum);
        q = winc(q, P);
    }
    if (mx < m) ring.st(mx % P, gy_sum);
    for (int i = 0; i < n; i++) {
        const int js = imax(0, i - mn - r + 1), je = imin(m, i + mx);
        const float xi = (float)X[i];
        const float gxi = fabsf(__fsub_rn(xi, g));
        q = js % P;
        HL32 diag, left;
        if (js > 0) {
            diag = ring.ld(wdec(q, P));
            left = hl(0.0f);
        } else {
            diag = (i == 0) ? hl(0.0f) : gx_sum;
            left = gx_sum;
        }
        for (int j = js; j < je; j++) {
            HL32 up = ring.ld(q);
            float v = fabsf(__fsub_rn(xi, ldf(Y + j)));
            HL32 a = add32(diag, v);
            HL32 b = add32(up, gxi);
            HL32 c = add32(left, ldf(gY + j));
            HL32 nv = min32(a, min32(b, c));
            ring.st(q, nv);
            diag = up;
            left = nv;
            q = winc(q, P);
        }
        if (je < m) ring.st(q, hl(0.0f));
    }
    return ring.ld((m - 1) % P);
}

__device__ __forceinline__ float msm_cost32(float x, float y, float z, float c) {
    if ((y <= x && x <= z) || (y >= x && x >= z)) return c;
    float a = fabsf(__fsub_rn(x, y));
    float b = fabsf(__fsub_rn(x, z));
    return __fadd_rn(c, b < a ? b : a);
}

// msm: msm_distance, distance/_elastic.pyx:1592-1647
template <class R>
__device__ HL32 r32_msm(R ring, int P, const double *X, int n, const double *Y, int m, int r,
                        float c) {
    const int mx = imax(0, m - n) + r, mn = imax(0, n - m);
    const float x0 = (float)X[0];
    const float y0 = ldf(Y);
    HL32 acc = hl(fabsf(__fsub_rn(x0, y0)));
    ring.st(0, acc);
    const int lim = imin(m, mx);
    int q = 1 % P;
    float yprev = y0;
    for (int j = 1; j < lim; j++) {
        float yj = ldf(Y + j);
        acc = add32(acc, msm_cost32(yj, yprev, x0, c));
        ring.st(q, acc);
        yprev = yj;
        q = winc(q, P);
    }
    if (mx < m) {
        acc = add32(acc, msm_cost32(ldf(Y + mx), ldf(Y + mx - 1), x0, c));
        ring.st(mx % P, acc);
    }
    HL32 cy = hl(fabsf(__fsub_rn(x0, y0)));
    HL32 stale = hl(0.0f);
    float xprev = x0;
    for (int i = 1; i < n; i++) {
        const float xi = (float)X[i];
        const HL32 cy_prev = cy;
        cy = add32(cy, msm_cost32(xi, xprev, y0, c));
        const int js = imax(1, i - mn - r + 1), je = imin(m, i + mx);
        int q2 = js % P;
        HL32 diag, left;
        if (js == 1) {
            diag = cy_prev;
            left = cy;
        } else {
            diag = ring.ld(wdec(q2, P));
            left = stale;
        }
        float yl = ldf(Y + js - 1);
        for (int j = js; j < je; j++) {
            HL32 up = ring.ld(q2);
            if (j == js) stale = up;
            const float yj = ldf(Y + j);
            HL32 a = add32(diag, fabsf(__fsub_rn(xi, yj)));
            HL32 b = add32(up, msm_cost32(xi, xprev, yj, c));
            HL32 d = add32(left, msm_cost32(yj, xi, yl, c));
            HL32 nv = min32(min32(a, b), d);
            ring.st(q2, nv);
            diag = up;
            left = nv;
            yl = yj;
            q2 = winc(q2, P);
        }
        if (je < m) ring.st(q2, hl(0.0f));
        xprev = xi;
    }
    if (m == 1) return n == 1 ? ring.ld(0) : cy;
    return ring.ld((m - 1) % P);
}

// twe: twe_distance, distance/_elastic.pyx:1733-1829
template <class R>
__device__ HL32 r32_twe(R ring, int P, const double *X, int n, const double *Y, int m, int r,
                        float pen, float s2) {
    const int mx = imax(0, m - n) + r, mn = imax(0, n - m);
    const HL32 INF = hl(WB_F32INF);
    const int lim = imin(m, mx);
    int q = 0;
    for (int j = 0; j < lim; j++) {
        ring.st(q, INF);
        q = winc(q, P);
    }
    if (mx < m) ring.st(mx % P, INF);
    float xp = 0.0f;
    for (int i = 0; i < n; i++) {
        const int js = imax(0, i - mn - r + 1), je = imin(m, i + mx);
        const float xi = (float)X[i];
        const float dxi = fabsf(__fsub_rn(xp, xi));
        q = js % P;
        HL32 left, upleft;
        float yp;
        if (js > 0) {
            left = hl(0.0f);
            upleft = ring.ld(wdec(q, P));
            yp = ldf(Y + js - 1);
        } else {
            left = INF;
            upleft = (i == 0) ? hl(0.0f) : INF;
            yp = 0.0f;
        }
        for (int j = js; j < je; j++) {
            HL32 up = ring.ld(q);
            const float yj = ldf(Y + j);
            HL32 del_x = add32(add32(up, dxi), pen);
            HL32 del_y = add32(add32(left, fabsf(__fsub_rn(yp, yj))), pen);
            HL32 match = add32(add32(add32(upleft, fabsf(__fsub_rn(xi, yj))),
                                     fabsf(__fsub_rn(xp, yp))),
                               __fmul_rn(s2, (float)abs(i - j)));
            HL32 nv = min32(min32(del_x, del_y), match);
            ring.st(q, nv);
            upleft = up;
            left = nv;
            yp = yj;
            q = winc(q, P);
        }
        if (je < m) ring.st(q, hl(0.0f));
        xp = xi;
    }
    return ring.ld((m - 1) % P);
}

constexpr int kT32 = 128;

template <int KIND, class R>
__device__ __forceinline__ double run32(const ElasticJob &J, R ring, int P, int64_t rs,
                                        int64_t cs) {
    const double *X = J.rows.base + rs * J.rows.stride;
    const double *Y = J.cols.base + cs * J.cols.stride;
    const int n = J.rows.len, m = J.cols.len, r = J.band;
    HL32 v;
    if constexpr (KIND == K_ADTW || KIND == K_ADTW_ANY)
        v = r32_adtw(ring, P, X, n, Y, m, r, (float)J.p);
    else if constexpr (KIND == K_LCSS)
        v = r32_lcss<false>(ring, P, X, n, Y, m, r, (float)J.eps, nullptr);
    else if constexpr (KIND == K_WLCSS)
        v = r32_lcss<true>(ring, P, X, n, Y, m, r, (float)J.eps, J.weights32);
    else if constexpr (KIND == K_EDR) {
        double eps = J.eps;
        if (J.std_rows) eps = cy_max(J.std_rows[rs], J.std_cols[cs]) / 4.0;
        v = r32_edr(ring, P, X, n, Y, m, r, (float)eps);
    } else if constexpr (KIND == K_ERP)
        v = r32_erp(ring, P, X, n, Y, m, r, (float)J.g, from_double(J.gsum_rows[rs]),
                    from_double(J.gsum_cols[cs]), J.gtab_cols + cs * (int64_t)m);
    else if constexpr (KIND == K_MSM)
        v = r32_msm(ring, P, X, n, Y, m, r, (float)J.c);
    else
        v = r32_twe(ring, P, X, n, Y, m, r, (float)(J.penalty + J.stiffness),
                    (float)(J.stiffness * 2.0));
    const double c = (double)v.h + (double)v.l;
    switch (J.result) {
        case R_SQRT: return sqrt(c);
        case R_LCSS: return 1.0 - c / (double)imin(J.len_norm_rows, J.len_norm_cols);
        case R_EDR: return c / (double)imax(J.len_norm_rows, J.len_norm_cols);
        default: return c;
    }
}

template <int KIND, bool GRING>
__global__ void __launch_bounds__(kT32) elastic32_pairs_kernel(const ElasticJob J,
                                                                float2 *gring, int P) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * kT32 + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * kT32) >> 5;
    const int64_t gtid = (int64_t)blockIdx.x * kT32 + threadIdx.x;
    const int64_t gthreads = (int64_t)gridDim.x * kT32;
    auto body = [&](auto ring) {
        if (J.mode == PM_PAIRED) {
            for (int64_t s = gtid; s < J.rows.count; s += gthreads)
                J.out[s] = run32<KIND>(J, ring, P, s, s);
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
            const double d = run32<KIND>(J, ring, P, rs, cs);
            J.out[rs * J.out_ld + cs] = d;
            if (J.mode == PM_UPPER) J.out[cs * J.out_ld + rs] = d;
        }
    };
    if constexpr (GRING) body(Ring32G{gring + gtid, gthreads});
    else body(Ring32S{(int)threadIdx.x, kT32});
}

template <int KIND>
static int launch32(const ElasticJob &J, int P, bool gring, float2 *ring, int grid,
                    cudaStream_t s) {
    timer_begin("elastic32_pairs_kernel", s);
    if (gring) {
        elastic32_pairs_kernel<KIND, true><<<grid, kT32, 0, s>>>(J, ring, P);
    } else {
        size_t smem = (size_t)P * kT32 * sizeof(float2);
        auto k = elastic32_pairs_kernel<KIND, false>;
        WB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kT32, smem, s>>>(J, nullptr, P);
    }
    timer_end(s);
    WB_LAUNCH_CHECK("elastic32_pairs_kernel");
    return WB_OK;
}

int launch_elastic32(const ElasticJob &J, Workspace &ws) {
    if (J.rows.count == 0 || J.cols.count == 0) return WB_OK;
    // same placement rule as the FP64 kernel (float2 entries are 8 bytes too)
    const DeviceInfo &dev = device_info();
    const int P = imax(2, ring_len(J.rows.len, J.cols.len, J.band));
    const size_t per_block = (size_t)P * kT32 * sizeof(float2);
    int64_t work;
    if (J.mode == PM_PAIRED) work = J.rows.count;
    else work = ((J.rows.count + 31) / 32) * 32 * J.cols.count;
    int64_t want = (work + kT32 - 1) / kT32;
    int bps = 0;
    if (per_block <= (size_t)dev.smem_per_sm - 2048 && per_block <= (size_t)dev.max_smem_optin) {
        bps = (int)(((size_t)dev.smem_per_sm - 1024) / (per_block + 1024));
        if (bps > 8) bps = 8;
    }
    bool gring = bps < 1;
    int64_t cap = (int64_t)(gring ? 4 : bps) * dev.sm_count;
    int grid = (int)(want < cap ? want : cap);
    if (grid < 1) grid = 1;
    float2 *ring = nullptr;
    if (gring) {
        ring = ws.take<float2>((size_t)P * grid * kT32);
        if (!ring) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    cudaStream_t s = ws.stream();
    switch (J.kind) {
        case K_ADTW:
        case K_ADTW_ANY: return launch32<K_ADTW>(J, P, gring, ring, grid, s);
        case K_LCSS: return launch32<K_LCSS>(J, P, gring, ring, grid, s);
        case K_WLCSS: return launch32<K_WLCSS>(J, P, gring, ring, grid, s);
        case K_EDR: return launch32<K_EDR>(J, P, gring, ring, grid, s);
        case K_ERP: return launch32<K_ERP>(J, P, gring, ring, grid, s);
        case K_MSM: return launch32<K_MSM>(J, P, gring, ring, grid, s);
        case K_TWE: return launch32<K_TWE>(J, P, gring, ring, grid, s);
    }
    return fail(WB_EINVAL, "no FP32 kernel for this metric kind");
}

// float64 rows -> float32 (for the dtw strip kernel)
__global__ void to_f32_kernel(const SeriesSet in, float *out) {
    const int64_t total = in.count * (int64_t)in.len;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t s = t / in.len;
        int i = (int)(t - s * in.len);
        out[t] = (float)in.base[s * in.stride + i];
    }
}

int launch_to_f32(const SeriesSet &in, float *out, cudaStream_t s) {
    if (in.count == 0) return WB_OK;
    int64_t total = in.count * (int64_t)in.len;
    int64_t g = (total + 255) / 256;
    int64_t cap = (int64_t)device_info().sm_count * 16;
    to_f32_kernel<<<(int)(g < cap ? g : cap), 256, 0, s>>>(in, out);
    WB_LAUNCH_CHECK("to_f32_kernel");
    return WB_OK;
}

// float64 weights -> float32
__global__ void weights_f32_kernel(const double *w, int n, float *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (float)w[i];
}

int launch_weights_f32(const double *w, int n, float *out, cudaStream_t s) {
    if (n <= 0) return WB_OK;
    weights_f32_kernel<<<(n + 255) / 256, 256, 0, s>>>(w, n, out);
    WB_LAUNCH_CHECK("weights_f32_kernel");
    return WB_OK;
}

}  // namespace wb
