// elastic_rec.cuh -- the FP64 two-row recurrences of the elastic metrics,
// thread-per-pair with the live band in a ring (shared or global memory).
// Shared by the pairwise / argmin kernels (elastic_f64.cu) and the
// subsequence kernels (elastic_f64.cu, argmin_subseq.cu).  With EA the
// recurrence stops after the first row that lifts the abandon key (the largest
// row minimum so far) above `bound`, returning +inf with that partial key.  Every cell performs
// the reference's IEEE double operations in the reference's order; the
// including file is compiled with -fmad=false.
#pragma once

#include "elastic.cuh"

namespace wb {

extern __shared__ double wb_smem[];

struct RingS {
    int off, s;
    __device__ __forceinline__ double ld(int k) const { return wb_smem[off + k * s]; }
    __device__ __forceinline__ void st(int k, double v) const { wb_smem[off + k * s] = v; }
};

struct RingG {
    double *p;
    int64_t s;
    __device__ __forceinline__ double ld(int k) const { return p[(int64_t)k * s]; }
    __device__ __forceinline__ void st(int k, double v) const { p[(int64_t)k * s] = v; }
};

#define WB_INF __longlong_as_double(0x7ff0000000000000LL)

__device__ __forceinline__ int wrap_inc(int q, int P) { return (q + 1 == P) ? 0 : q + 1; }
__device__ __forceinline__ int wrap_dec(int q, int P) { return (q == 0) ? P - 1 : q - 1; }
__device__ __forceinline__ double ldg(const double *p) { return __ldg(p); }

// --------------------------------------------------------------------------
// dtw / wdtw / ddtw / wddtw: dtw_distance, distance/_elastic.pyx:869-940
template <bool W, class R, bool EA = false>
__device__ double rec_dtw(R ring, int P, const double *__restrict__ X, int n,
                          const double *__restrict__ Y, int m, int r,
                          const double *__restrict__ w, double &key, double bound = HUGE_VAL) {
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const double INF = WB_INF;
    double x0 = X[0];
    double v = x0 - ldg(Y);
    double acc = W ? (v * v) * ldg(w) : v * v;
    ring.st(0, acc);
    const int lim = imin(m, mx);
    int q = 1 % P;
    for (int j = 1; j < lim; j++) {
        v = x0 - ldg(Y + j);
        double c = W ? (v * v) * ldg(w + j - 1) : v * v;
        acc = acc + c;
        ring.st(q, acc);
        q = wrap_inc(q, P);
    }
    if (mx < m) ring.st(mx % P, INF);
    double kmax = -INF;
    for (int i = 1; i < n; i++) {
        const int js = imax(0, i - mn - r + 1);
        const int je = imin(m, i + mx);
        const double xi = X[i];
        q = js % P;
        double diag = js > 0 ? ring.ld(wrap_dec(q, P)) : INF;
        double left = INF;
        double rmin = INF;
        for (int j = js; j < je; j++) {
            double up = ring.ld(q);
            double d = xi - ldg(Y + j);
            double c = W ? (d * d) * ldg(w + abs(i - j)) : d * d;
            double nv = nn_min(nn_min(up, left), diag) + c;
            ring.st(q, nv);
            rmin = nn_min(rmin, nv);
            diag = up;
            left = nv;
            q = wrap_inc(q, P);
        }
        if (je < m) ring.st(q, INF);
        kmax = fmax(kmax, rmin);
        if constexpr (EA) {
            if (kmax > bound) {  // abandoned: the caller's bound is crossed
                key = kmax;
                return WB_INF;
            }
        }
    }
    key = kmax;
    return ring.ld((m - 1) % P);
}

// adtw: adtw_distance, distance/_elastic.pyx:943-1008
template <bool NONNEG, class R, bool EA = false>
__device__ double rec_adtw(R ring, int P, const double *__restrict__ X, int n,
                           const double *__restrict__ Y, int m, int r, double pen,
                           double &key, double bound = HUGE_VAL) {
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const double INF = WB_INF;
    double x0 = X[0];
    double v = x0 - ldg(Y);
    double acc = v * v;
    ring.st(0, acc);
    const int lim = imin(m, mx);
    int q = 1 % P;
    for (int j = 1; j < lim; j++) {
        v = x0 - ldg(Y + j);
        acc = acc + v * v;
        ring.st(q, acc);
        q = wrap_inc(q, P);
    }
    if (mx < m) ring.st(mx % P, INF);
    double kmax = -INF;
    for (int i = 1; i < n; i++) {
        const int js = imax(0, i - mn - r + 1);
        const int je = imin(m, i + mx);
        const double xi = X[i];
        q = js % P;
        double diag = js > 0 ? ring.ld(wrap_dec(q, P)) : INF;
        double prev = INF;  // the left cell: prev_cost = inf before the band
        double rmin = INF;
        for (int j = js; j < je; j++) {
            double up = ring.ld(q);
            double d = xi - ldg(Y + j);
            // min(up + p, prev + p) == min(up, prev) + p exactly (rounding is
            // monotone and the same operand is added): one addition per cell
            double mv;
            if (NONNEG) mv = nn_min(nn_min(up, prev) + pen, diag);
            else mv = cy_min(cy_min(up, prev) + pen, diag);
            double nv = mv + d * d;
            ring.st(q, nv);
            rmin = NONNEG ? nn_min(rmin, nv) : (nv < rmin ? nv : rmin);
            diag = up;
            prev = nv;
            q = wrap_inc(q, P);
        }
        if (je < m) ring.st(q, INF);
        kmax = fmax(kmax, rmin);
        if constexpr (EA) {
            if (kmax > bound) {  // abandoned: the caller's bound is crossed
                key = kmax;
                return WB_INF;
            }
        }
    }
    key = kmax;
    return ring.ld((m - 1) % P);
}

// lcss / wlcss: lcss_distance, distance/_elastic.pyx:1118-1183
template <bool W, class R>
__device__ double rec_lcss(R ring, int P, const double *__restrict__ X, int n,
                           const double *__restrict__ Y, int m, int r, double eps,
                           const double *__restrict__ w, double &key) {
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const double INF = WB_INF;
    const int lim = imin(m, mx);
    int q = 0;
    for (int j = 0; j < lim; j++) {
        ring.st(q, 0.0);
        q = wrap_inc(q, P);
    }
    if (mx < m) ring.st(mx % P, 0.0);
    double kmax = -INF;
    const long long eb = eps_bits(eps);  // v <= eps on the integer pipe
    for (int i = 0; i < n; i++) {
        const int js = imax(0, i - mn - r + 1);
        const int je = imin(m, i + mx);
        const double xi = X[i];
        q = js % P;
        double diag = js > 0 ? ring.ld(wrap_dec(q, P)) : 0.0;
        double left = 0.0;
        double rmin = INF;
        for (int j = js; j < je; j++) {
            double up = ring.ld(q);
            const long long vb = abs_bits(xi - ldg(Y + j));  // |x - y| as bits
            double wt = W ? ldg(w + abs(i - j)) : 1.0;
            double nv = (vb <= eb) ? wt + diag : nn_max(left, up);
            ring.st(q, nv);
            rmin = nn_min(rmin, nv);
            diag = up;
            left = nv;
            q = wrap_inc(q, P);
        }
        if (je < m) ring.st(q, 0.0);
        kmax = fmax(kmax, rmin);
    }
    key = kmax;
    return ring.ld((m - 1) % P);
}

// edr: edr_distance, distance/_elastic.pyx:1437-1497
template <class R, bool EA = false>
__device__ double rec_edr(R ring, int P, const double *__restrict__ X, int n,
                          const double *__restrict__ Y, int m, int r, double eps,
                          double &key, double bound = HUGE_VAL) {
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const double INF = WB_INF;
    const int lim = imin(m, mx);
    int q = 0;
    for (int j = 0; j < lim; j++) {
        ring.st(q, 0.0);
        q = wrap_inc(q, P);
    }
    if (mx < m) ring.st(mx % P, 0.0);
    double kmax = -INF;
    const long long eb = eps_bits(eps);  // v < eps on the integer pipe
    for (int i = 0; i < n; i++) {
        const int js = imax(0, i - mn - r + 1);
        const int je = imin(m, i + mx);
        const double xi = X[i];
        q = js % P;
        double diag = js > 0 ? ring.ld(wrap_dec(q, P)) : 0.0;
        double left = 0.0;
        double rmin = INF;
        for (int j = js; j < je; j++) {
            double up = ring.ld(q);
            const long long vb = abs_bits(xi - ldg(Y + j));  // |x - y| as bits
            // The three moves add 0 or 1 to diag, 1 to up and left.  Rounding is
            // monotone, so min(a + 1, b + 1) == min(a, b) + 1 exactly: a match
            // gives min(diag, min(up, left) + 1), a mismatch
            // min(diag, up, left) + 1 -- one addition per cell either way.
            const bool match = vb < eb;
            const double mul = nn_min(up, left);
            const double r = (match ? mul : nn_min(diag, mul)) + 1.0;
            double nv = match ? nn_min(diag, r) : r;
            ring.st(q, nv);
            rmin = nn_min(rmin, nv);
            diag = up;
            left = nv;
            q = wrap_inc(q, P);
        }
        if (je < m) ring.st(q, 0.0);
        kmax = fmax(kmax, rmin);
        if constexpr (EA) {
            if (kmax > bound) {  // abandoned: the caller's bound is crossed
                key = kmax;
                return WB_INF;
            }
        }
    }
    key = kmax;
    return ring.ld((m - 1) % P);
}

// erp: erp_distance, distance/_elastic.pyx:1273-1347
template <class R, bool EA = false>
__device__ double rec_erp(R ring, int P, const double *__restrict__ X, int n,
                          const double *__restrict__ Y, int m, int r, double g,
                          double gx_sum, double gy_sum, const double *__restrict__ gY,
                          double &key, double bound = HUGE_VAL) {
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const double INF = WB_INF;
    const int lim = imin(m, mx);
    int q = 0;
    for (int j = 0; j < lim; j++) {
        ring.st(q, gy_sum);
        q = wrap_inc(q, P);
    }
    if (mx < m) ring.st(mx % P, gy_sum);
    double kmax = -INF;
    for (int i = 0; i < n; i++) {
        const int js = imax(0, i - mn - r + 1);
        const int je = imin(m, i + mx);
        const double xi = X[i];
        const double gxi = fabs(xi - g);
        q = js % P;
        double diag, left;
        if (js > 0) {
            diag = ring.ld(wrap_dec(q, P));
            left = 0.0;
        } else {
            diag = (i == 0) ? 0.0 : gx_sum;
            left = gx_sum;
        }
        double rmin = INF;
        for (int j = js; j < je; j++) {
            double up = ring.ld(q);
            double v = fabs(xi - ldg(Y + j));
            double a = diag + v;
            double b = up + gxi;
            double c = left + ldg(gY + j);
            double nv = nn_min(a, nn_min(b, c));
            ring.st(q, nv);
            rmin = nn_min(rmin, nv);
            diag = up;
            left = nv;
            q = wrap_inc(q, P);
        }
        if (je < m) ring.st(q, 0.0);
        kmax = fmax(kmax, rmin);
        if constexpr (EA) {
            if (kmax > bound) {  // abandoned: the caller's bound is crossed
                key = kmax;
                return WB_INF;
            }
        }
    }
    key = kmax;
    return ring.ld((m - 1) % P);
}

// _msm_cost, distance/_elastic.pyx:1583-1587: arguments narrowed to float,
// comparisons and differences in float, the sum in double.
__device__ __forceinline__ double msm_cost(float x, float y, float z, float c) {
    if ((y <= x && x <= z) || (y >= x && x >= z)) return (double)c;
    float a = fabsf(__fsub_rn(x, y));
    float b = fabsf(__fsub_rn(x, z));
    return (double)c + f2d_nonneg(b < a ? b : a);  // exact widening, integer pipe
}

// msm: msm_distance, distance/_elastic.pyx:1592-1647
template <class R, bool EA = false>
__device__ double rec_msm(R ring, int P, const double *__restrict__ X, int n,
                          const double *__restrict__ Y, int m, int r, double cd,
                          double &key, double bound = HUGE_VAL) {
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const double INF = WB_INF;
    const float c = (float)cd;
    const float x0f = (float)X[0];
    double acc = fabs(X[0] - ldg(Y));
    ring.st(0, acc);
    const int lim = imin(m, mx);
    int q = 1 % P;
    float yprev = (float)ldg(Y);
    for (int j = 1; j < lim; j++) {
        float yj = (float)ldg(Y + j);
        acc = acc + msm_cost(yj, yprev, x0f, c);
        ring.st(q, acc);
        yprev = yj;
        q = wrap_inc(q, P);
    }
    if (mx < m) {
        acc = acc + msm_cost((float)ldg(Y + mx), (float)ldg(Y + mx - 1), x0f, c);
        ring.st(mx % P, acc);
    }
    double cy = fabs(X[0] - ldg(Y));   // cost_y[0]
    const float y0f = (float)ldg(Y);
    double stale = 0.0;
    double kmax = -INF;
    float xprevf = x0f;
    for (int i = 1; i < n; i++) {
        const double xi = X[i];
        const float xif = (float)xi;
        const double cy_prev = cy;
        cy = cy + msm_cost(xif, xprevf, y0f, c);
        const int js = imax(1, i - mn - r + 1);
        const int je = imin(m, i + mx);
        q = js % P;
        double diag, left;
        if (js == 1) {
            diag = cy_prev;
            left = cy;
        } else {
            diag = ring.ld(wrap_dec(q, P));
            left = stale;
        }
        double rmin = cy;
        float ylf = (float)ldg(Y + js - 1);
        for (int j = js; j < je; j++) {
            double up = ring.ld(q);
            if (j == js) stale = up;
            const double yj = ldg(Y + j);
            const float yjf = (float)yj;
            double a = diag + fabs(xi - yj);
            double b = up + msm_cost(xif, xprevf, yjf, c);
            double d = left + msm_cost(yjf, xif, ylf, c);
            double nv = nn_min(nn_min(a, b), d);
            ring.st(q, nv);
            rmin = nn_min(rmin, nv);
            diag = up;
            left = nv;
            ylf = yjf;
            q = wrap_inc(q, P);
        }
        if (je < m) ring.st(q, 0.0);
        kmax = fmax(kmax, rmin);
        if constexpr (EA) {
            if (kmax > bound) {  // abandoned: the caller's bound is crossed
                key = kmax;
                return WB_INF;
            }
        }
        xprevf = xif;
    }
    key = kmax;
    if (m == 1) return n == 1 ? ring.ld(0) : cy;
    return ring.ld((m - 1) % P);
}

// twe: twe_distance, distance/_elastic.pyx:1733-1829.  DYTAB: |y_{j-1} - y_j|
// from a per-series table; otherwise computed (windows of a longer series
// start with y_{-1} = 0, which no whole-series table holds).
template <class R, bool DYTAB = true, bool EA = false>
__device__ double rec_twe(R ring, int P, const double *__restrict__ X, int n,
                          const double *__restrict__ Y, int m, int r, double penalty,
                          double stiffness, const double *__restrict__ dY,
                          const double *__restrict__ stab, double &key,
                          double bound = HUGE_VAL) {
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const double INF = WB_INF;
    const int lim = imin(m, mx);
    int q = 0;
    for (int j = 0; j < lim; j++) {
        ring.st(q, INF);
        q = wrap_inc(q, P);
    }
    if (mx < m) ring.st(mx % P, INF);
    const double pen = penalty + stiffness;
    double kmax = -INF;
    double xp = 0.0;
    for (int i = 0; i < n; i++) {
        const int js = imax(0, i - mn - r + 1);
        const int je = imin(m, i + mx);
        const double xi = X[i];
        const double dxi = fabs(xp - xi);
        q = js % P;
        double left, upleft, yp;
        if (js > 0) {
            left = 0.0;
            upleft = ring.ld(wrap_dec(q, P));
            yp = ldg(Y + js - 1);
        } else {
            left = INF;
            upleft = (i == 0) ? 0.0 : INF;
            yp = 0.0;
        }
        double rmin = INF;
        for (int j = js; j < je; j++) {
            double up = ring.ld(q);
            const double yj = ldg(Y + j);
            const double dyj = DYTAB ? ldg(dY + j) : fabs(yp - yj);
            // min((up + dxi) + pen, (left + dyj) + pen) equals
            // min(up + dxi, left + dyj) + pen exactly (rounding is monotone and
            // the same operand is added last): one addition fewer per cell
            double del = nn_min(up + dxi, left + dyj) + pen;
            double match = ((upleft + fabs(xi - yj)) + fabs(xp - yp)) + ldg(stab + abs(i - j));
            double nv = nn_min(del, match);
            ring.st(q, nv);
            rmin = nn_min(rmin, nv);
            upleft = up;
            left = nv;
            yp = yj;
            q = wrap_inc(q, P);
        }
        if (je < m) ring.st(q, 0.0);
        kmax = fmax(kmax, rmin);
        if constexpr (EA) {
            if (kmax > bound) {  // abandoned: the caller's bound is crossed
                key = kmax;
                return WB_INF;
            }
        }
        xp = xi;
    }
    key = kmax;
    return ring.ld((m - 1) % P);
}

}  // namespace wb
