/*
 * wb_oracle.c -- CPU restatement of wildboar's distance hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may
 * load it; the product path (wildboar_gb300) never links or calls it.
 *
 * Every routine restates the algorithm of the reference file/line cited beside
 * it, in plain C99, double precision, built with -O2 -ffp-contract=off so that
 * every multiply and add rounds on its own (as gcc -O2 on x86-64 does for the
 * Cython-generated C of the reference).
 *
 * Citations are to wildboar (src/wildboar/...).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define INF ((double)INFINITY)

typedef int64_t idx_t;

/* metric ids; the same numbering is used by include/wbgpu.h */
enum {
    WBO_EUCLIDEAN = 0,
    WBO_DTW = 1,
    WBO_WDTW = 2,
    WBO_DDTW = 3,
    WBO_WDDTW = 4,
    WBO_ADTW = 5,
    WBO_LCSS = 6,
    WBO_WLCSS = 7,
    WBO_EDR = 8,
    WBO_ERP = 9,
    WBO_MSM = 10,
    WBO_TWE = 11,
    /* subsequence-only */
    WBO_SCALED_EUCLIDEAN = 32,
};

typedef struct {
    double r, g, p, epsilon, c, penalty, stiffness;
} wbo_params;

static inline idx_t imax(idx_t a, idx_t b) { return a > b ? a : b; }
static inline idx_t imin(idx_t a, idx_t b) { return a < b ? a : b; }
/* Cython lowers builtin min/max on C doubles to "b < a ? b : a" */
static inline double dmin(double a, double b) { return b < a ? b : a; }
static inline double dmax(double a, double b) { return b > a ? b : a; }

/* _compute_r: distance/_elastic.pyx:1924-1925 */
static idx_t compute_r(idx_t length, double r)
{
    double v = floor((double)length * r);
    return (idx_t)(v > 1.0 ? v : 1.0);
}

/* fast_mean_std: utils/_stats.pyx:22-42.  ex2 accumulates pow(x, 2.0), the
 * call Cython emits for `x ** 2`; gcc -O2 folds it into x * x here as in the
 * reference's own build. */
static void fast_mean_std(const double *x, idx_t n, double *mean, double *std)
{
    double ex = 0, ex2 = 0;
    for (idx_t i = 0; i < n; i++) {
        double v = x[i];
        ex += v;
        ex2 = ex2 + pow(v, 2.0);
    }
    *mean = ex / (double)n;
    ex2 = ex2 / (double)n - *mean * *mean;
    *std = ex2 > 1e-13 ? sqrt(ex2) : 0.0;
}

/* average_slope: distance/_elastic.pyx:3220-3225 */
static void average_slope(const double *q, idx_t len, double *d)
{
    idx_t j = 0;
    for (idx_t i = 1; i < len - 1; i++) {
        d[j] = ((q[i] - q[i - 1]) + ((q[i + 1] - q[i - 1]) / 2)) / 2;
        j++;
    }
}

/* ---------------------------------------------------------------------- */
/* Elastic kernels: two-row band recurrences                              */
/* ---------------------------------------------------------------------- */

/* dtw_distance: distance/_elastic.pyx:869-940 (also WDTW/DDTW via w, inputs) */
static double dtw_rows(const double *X, idx_t xl, const double *Y, idx_t yl, idx_t r,
                       double *cost, double *cost_prev, const double *wv, double min_dist)
{
    idx_t mx = imax(0, yl - xl) + r;
    idx_t mn = imax(0, xl - yl);
    double v, w = 1.0;
    v = X[0] - Y[0];
    if (wv) w = wv[0];
    cost_prev[0] = v * v * w;
    for (idx_t i = 1; i < imin(yl, mx); i++) {
        v = X[0] - Y[i];
        if (wv) w = wv[i - 1];
        cost_prev[i] = cost_prev[i - 1] + v * v * w;
    }
    if (mx < yl) cost_prev[mx] = INF;
    for (idx_t i = 1; i < xl; i++) {
        idx_t js = imax(0, i - mn - r + 1);
        idx_t je = imin(yl, i + mx);
        if (js > 0) cost[js - 1] = INF;
        double min_cost = INF;
        for (idx_t j = js; j < je; j++) {
            double x = cost_prev[j], y, z;
            if (j > 0) { y = cost[j - 1]; z = cost_prev[j - 1]; }
            else { y = INF; z = INF; }
            v = X[i] - Y[j];
            if (wv) w = wv[labs((long)(i - j))];
            cost[j] = dmin(dmin(x, y), z) + v * v * w;
            if (cost[j] < min_cost) min_cost = cost[j];
        }
        if (min_cost > min_dist) return INF;
        if (je < yl) cost[je] = INF;
        double *t = cost; cost = cost_prev; cost_prev = t;
    }
    return cost_prev[yl - 1];
}

/* adtw_distance: distance/_elastic.pyx:943-1008 */
static double adtw_rows(const double *X, idx_t xl, const double *Y, idx_t yl, idx_t r,
                        double *cost, double *cost_prev, double penalty, double min_dist)
{
    idx_t mx = imax(0, yl - xl) + r;
    idx_t mn = imax(0, xl - yl);
    double v = X[0] - Y[0];
    cost_prev[0] = v * v;
    for (idx_t i = 1; i < imin(yl, mx); i++) {
        v = X[0] - Y[i];
        cost_prev[i] = cost_prev[i - 1] + v * v;
    }
    if (mx < yl) cost_prev[mx] = INF;
    for (idx_t i = 1; i < xl; i++) {
        idx_t js = imax(0, i - mn - r + 1);
        idx_t je = imin(yl, i + mx);
        if (js > 0) cost[js - 1] = INF;
        double prev_cost = INF, min_cost = INF;
        for (idx_t j = js; j < je; j++) {
            double x = cost_prev[j] + penalty, y, z;
            if (j > 0) { y = prev_cost + penalty; z = cost_prev[j - 1]; }
            else { y = INF; z = INF; }
            v = X[i] - Y[j];
            cost[j] = dmin(dmin(x, y), z) + v * v;
            if (cost[j] < min_cost) min_cost = cost[j];
            prev_cost = cost[j];
        }
        if (min_cost > min_dist) return INF;
        if (je < yl) cost[je] = INF;
        double *t = cost; cost = cost_prev; cost_prev = t;
    }
    return cost_prev[yl - 1];
}

/* lcss_distance: distance/_elastic.pyx:1118-1183 */
static double lcss_rows(const double *X, idx_t xl, const double *Y, idx_t yl, idx_t r,
                        double eps, double *cost, double *cost_prev, const double *wv,
                        double min_dist)
{
    idx_t mx = imax(0, yl - xl) + r;
    idx_t mn = imax(0, xl - yl);
    double w = 1.0;
    for (idx_t i = 0; i < imin(yl, mx); i++) cost_prev[i] = 0;
    if (mx < yl) cost_prev[mx] = 0;
    for (idx_t i = 0; i < xl; i++) {
        idx_t js = imax(0, i - mn - r + 1);
        idx_t je = imin(yl, i + mx);
        if (js > 0) cost[js - 1] = 0;
        double min_cost = INF;
        for (idx_t j = js; j < je; j++) {
            double x = cost_prev[j], y, z;
            if (j > 0) { y = cost_prev[j - 1]; z = cost[j - 1]; }
            else { y = 0; z = 0; }
            double v = fabs(X[i] - Y[j]);
            if (wv) w = wv[labs((long)(i - j))];
            if (v <= eps) cost[j] = w + y;
            else cost[j] = dmax(z, x);
            if (cost[j] < min_cost) min_cost = cost[j];
        }
        if (min_cost > min_dist) return INF;
        if (je < yl) cost[je] = 0;
        double *t = cost; cost = cost_prev; cost_prev = t;
    }
    return 1 - (cost_prev[yl - 1] / (double)imin(xl, yl));
}

/* erp_distance: distance/_elastic.pyx:1273-1347 */
static double erp_rows(const double *X, idx_t xl, const double *Y, idx_t yl, idx_t r,
                       double g, double *gX, double *gY, double *cost, double *cost_prev,
                       double min_dist)
{
    double gx_sum = 0, gy_sum = 0;
    for (idx_t i = 0; i < xl; i++) { double v = fabs(X[i] - g); gX[i] = v; gx_sum += v; }
    for (idx_t i = 0; i < yl; i++) { double v = fabs(Y[i] - g); gY[i] = v; gy_sum += v; }
    idx_t mx = imax(0, yl - xl) + r;
    idx_t mn = imax(0, xl - yl);
    for (idx_t i = 0; i < imin(yl, mx); i++) cost_prev[i] = gy_sum;
    if (mx < yl) cost_prev[mx] = gy_sum;
    for (idx_t i = 0; i < xl; i++) {
        idx_t js = imax(0, i - mn - r + 1);
        idx_t je = imin(yl, i + mx);
        if (js > 0) cost[js - 1] = 0;
        double min_cost = INF;
        for (idx_t j = js; j < je; j++) {
            double x = cost_prev[j], y, z;
            if (j > 0) { y = cost_prev[j - 1]; z = cost[j - 1]; }
            else { y = (i == 0) ? 0 : gx_sum; z = gx_sum; }
            double v = fabs(X[i] - Y[j]);
            cost[j] = dmin(y + v, dmin(x + gX[i], z + gY[j]));
            if (cost[j] < min_cost) min_cost = cost[j];
        }
        if (min_cost > min_dist) return INF;
        if (je < yl) cost[je] = 0;
        double *t = cost; cost = cost_prev; cost_prev = t;
    }
    return cost_prev[yl - 1];
}

/* edr_distance: distance/_elastic.pyx:1437-1497 */
static double edr_rows(const double *X, idx_t xl, const double *Y, idx_t yl, idx_t r,
                       double eps, double *cost, double *cost_prev, double min_dist)
{
    idx_t mx = imax(0, yl - xl) + r;
    idx_t mn = imax(0, xl - yl);
    for (idx_t i = 0; i < imin(yl, mx); i++) cost_prev[i] = 0;
    if (mx < yl) cost_prev[mx] = 0;
    for (idx_t i = 0; i < xl; i++) {
        idx_t js = imax(0, i - mn - r + 1);
        idx_t je = imin(yl, i + mx);
        if (js > 0) cost[js - 1] = 0;
        double min_cost = INF;
        for (idx_t j = js; j < je; j++) {
            double x = cost_prev[j], y, z;
            if (j > 0) { y = cost_prev[j - 1]; z = cost[j - 1]; }
            else { y = 0; z = 0; }
            double v = fabs(X[i] - Y[j]);
            /* Cython 3-arg min: keep the first of equal values */
            double a = y + (v < eps ? 0.0 : 1.0), b = x + 1, c = z + 1;
            double m = a;
            if (b < m) m = b;
            if (c < m) m = c;
            cost[j] = m;
            if (cost[j] < min_cost) min_cost = cost[j];
        }
        if (min_cost > min_dist) return INF;
        if (je < yl) cost[je] = 0;
        double *t = cost; cost = cost_prev; cost_prev = t;
    }
    return cost_prev[yl - 1] / (double)imax(xl, yl);
}

/* _msm_cost: distance/_elastic.pyx:1583-1587 (arguments narrowed to float) */
static inline double msm_cost(float x, float y, float z, float c)
{
    if ((y <= x && x <= z) || (y >= x && x >= z)) return c;
    double a = fabs((double)(float)(x - y));
    double b = fabs((double)(float)(x - z));
    return (double)c + dmin(a, b);
}

/* msm_distance: distance/_elastic.pyx:1592-1647 */
static double msm_rows(const double *X, idx_t xl, const double *Y, idx_t yl, idx_t r,
                       double c, double *cost, double *cost_prev, double *cost_y,
                       double min_dist)
{
    float cf = (float)c;
    idx_t mx = imax(0, yl - xl) + r;
    idx_t mn = imax(0, xl - yl);
    cost_prev[0] = fabs(X[0] - Y[0]);
    for (idx_t i = 1; i < imin(yl, mx); i++)
        cost_prev[i] = cost_prev[i - 1] + msm_cost((float)Y[i], (float)Y[i - 1], (float)X[0], cf);
    if (mx < yl)
        cost_prev[mx] = cost_prev[mx - 1] + msm_cost((float)Y[mx], (float)Y[mx - 1], (float)X[0], cf);
    cost_y[0] = cost_prev[0];
    for (idx_t i = 1; i < xl; i++)
        cost_y[i] = cost_y[i - 1] + msm_cost((float)X[i], (float)X[i - 1], (float)Y[0], cf);
    for (idx_t i = 1; i < xl; i++) {
        idx_t js = imax(1, i - mn - r + 1);
        idx_t je = imin(yl, i + mx);
        cost[0] = cost_y[i];
        double min_cost = cost[0];
        for (idx_t j = js; j < je; j++) {
            double a = cost_prev[j - 1] + fabs(X[i] - Y[j]);
            double b = cost_prev[j] + msm_cost((float)X[i], (float)X[i - 1], (float)Y[j], cf);
            double d = cost[j - 1] + msm_cost((float)Y[j], (float)X[i], (float)Y[j - 1], cf);
            double m = a;
            if (b < m) m = b;
            if (d < m) m = d;
            cost[j] = m;
            if (cost[j] < min_cost) min_cost = cost[j];
        }
        if (min_cost > min_dist) return INF;
        if (je < yl) cost[je] = 0;
        double *t = cost; cost = cost_prev; cost_prev = t;
    }
    return cost_prev[yl - 1];
}

/* twe_distance: distance/_elastic.pyx:1733-1829 */
static double twe_rows(const double *X, idx_t xl, const double *Y, idx_t yl, idx_t r,
                       double penalty, double stiffness, double *cost, double *cost_prev,
                       double min_dist)
{
    idx_t mx = imax(0, yl - xl) + r;
    idx_t mn = imax(0, xl - yl);
    for (idx_t i = 0; i < imin(yl, mx); i++) cost_prev[i] = INF;
    if (mx < yl) cost_prev[mx] = INF;
    penalty = penalty + stiffness;
    for (idx_t i = 0; i < xl; i++) {
        idx_t js = imax(0, i - mn - r + 1);
        idx_t je = imin(yl, i + mx);
        if (js > 0) cost[js - 1] = 0;
        double min_cost = INF;
        for (idx_t j = js; j < je; j++) {
            double up = cost_prev[j], left, up_left, x, y;
            if (j == 0) { left = INF; up_left = (i == 0) ? 0 : INF; }
            else { left = cost[j - 1]; up_left = cost_prev[j - 1]; }
            x = (i == 0) ? 0 : X[i - 1];
            y = X[i];
            double del_x = up + fabs(x - y) + penalty;
            x = (j == 0) ? 0 : Y[j - 1];
            y = Y[j];
            double del_y = left + fabs(x - y) + penalty;
            x = (i == 0) ? 0 : X[i - 1];
            y = (j == 0) ? 0 : Y[j - 1];
            double match = up_left + fabs(X[i] - Y[j]) + fabs(x - y)
                           + stiffness * 2.0 * (double)labs((long)(i - j));
            double m = del_x;
            if (del_y < m) m = del_y;
            if (match < m) m = match;
            cost[j] = m;
            if (cost[j] < min_cost) min_cost = cost[j];
        }
        if (min_cost > min_dist) return INF;
        if (je < yl) cost[je] = 0;
        double *t = cost; cost = cost_prev; cost_prev = t;
    }
    return cost_prev[yl - 1];
}

/* euclidean_distance: distance/_metric.pyx:654-682 */
static double euclid_scan(const double *S, idx_t sl, const double *T, idx_t tl,
                          double min_dist, idx_t *index)
{
    for (idx_t i = 0; i < tl - sl + 1; i++) {
        double dist = 0;
        for (idx_t j = 0; j < sl; j++) {
            if (dist >= min_dist) break;
            double x = T[i + j];
            x -= S[j];
            dist += x * x;
        }
        if (dist < min_dist) {
            min_dist = dist;
            if (index) *index = i;
        }
    }
    return sqrt(min_dist);
}

/* scaled_euclidean_distance + inner_scaled_euclidean_distance:
 * distance/_metric.pyx:561-651 */
static double scaled_euclid_scan(const double *S, idx_t sl, double s_mean, double s_std,
                                 const double *T, idx_t tl, double *buf, idx_t *index)
{
    double mean = 0, std = 0, dist = 0, min_dist = INF, ex = 0, ex2 = 0;
    for (idx_t i = 0; i < tl; i++) {
        double cv = T[i];
        ex += cv;
        ex2 += cv * cv;
        idx_t bp = i % sl;
        buf[bp] = cv;
        buf[bp + sl] = cv;
        if (i >= sl - 1) {
            idx_t j = (i + 1) % sl;
            mean = ex / (double)sl;
            double tmp = ex2 / (double)sl - mean * mean;
            std = tmp > 0 ? sqrt(tmp) : 1.0;
            dist = 0;
            for (idx_t k = 0; k < sl; k++) {
                if (dist >= min_dist) break;
                double x = (S[k] - s_mean) / s_std;
                x -= (buf[k + j] - mean) / std;
                dist += x * x;
            }
            if (dist < min_dist) {
                min_dist = dist;
                if (index) *index = (i + 1) - sl;
            }
            cv = buf[j];
            ex -= cv;
            ex2 -= cv * cv;
        }
    }
    return sqrt(min_dist);
}

/* IncStats (Welford updates with unit weights): utils/_stats.pyx:45-93 */
typedef struct { double mean, n_samples, sum_square, sum; } incstats;

static void inc_init(incstats *s) { s->mean = s->n_samples = s->sum_square = s->sum = 0.0; }

static void inc_add(incstats *s, double w, double v)
{
    double next_m;
    s->n_samples += w;
    next_m = s->mean + (v - s->mean) / s->n_samples;
    s->sum_square += (v - s->mean) * (v - next_m);
    s->mean = next_m;
    s->sum += w * v;
}

static void inc_remove(incstats *s, double w, double v)
{
    if (s->n_samples == 1.0) {
        s->n_samples = 0.0;
        s->mean = 0.0;
        s->sum_square = 0.0;
    } else {
        double old_m = (s->n_samples * s->mean - v) / (s->n_samples - w);
        s->sum_square -= (v - s->mean) * (v - old_m);
        s->mean = old_m;
        s->n_samples -= w;
    }
    s->sum -= w * v;
}

static double inc_variance(const incstats *s)
{
    double n = s->n_samples;
    if (n <= 1) return 0;
    double var = s->sum_square / n;
    if (var < 1e-13) var = 0.0;
    return var;
}

/* ---------------------------------------------------------------------- */
/* Metric objects: reset / distance / eadistance                          */
/* ---------------------------------------------------------------------- */

typedef struct {
    int id;
    wbo_params p;
    double *weights;           /* WDTW / WDDTW / WLCSS */
    double *std_x, *std_y;     /* EDR default epsilon tables */
    idx_t xn, xd, xL, yn, yd, yL;
} wbo_metric;

typedef struct {
    double *cost, *cost_prev, *gX, *gY, *cost_y, *d_x, *d_y;
} wbo_scratch;

static void scratch_init(wbo_scratch *s, idx_t L)
{
    idx_t n = L + 4;
    s->cost = malloc(sizeof(double) * n);
    s->cost_prev = malloc(sizeof(double) * n);
    s->gX = malloc(sizeof(double) * n);
    s->gY = malloc(sizeof(double) * n);
    s->cost_y = malloc(sizeof(double) * n);
    s->d_x = malloc(sizeof(double) * n);
    s->d_y = malloc(sizeof(double) * n);
}

static void scratch_free(wbo_scratch *s)
{
    free(s->cost); free(s->cost_prev); free(s->gX); free(s->gY);
    free(s->cost_y); free(s->d_x); free(s->d_y);
}

static double *logistic_weights(idx_t n, double g)
{
    /* WeightedDtwMetric.reset: distance/_elastic.pyx:3333-3341 */
    double *w = malloc(sizeof(double) * (size_t)imax(n, 1));
    for (idx_t i = 0; i < n; i++)
        w[i] = 1.0 / (1.0 + exp(-g * ((double)i - (double)n / 2.0)));
    return w;
}

/* Metric.reset for each metric class (X, Y are (n, d, L) C-contiguous) */
static void metric_reset(wbo_metric *M, const double *X, idx_t xn, idx_t xd, idx_t xL,
                         const double *Y, idx_t yn, idx_t yd, idx_t yL)
{
    M->xn = xn; M->xd = xd; M->xL = xL; M->yn = yn; M->yd = yd; M->yL = yL;
    M->weights = NULL; M->std_x = NULL; M->std_y = NULL;
    if (M->id == WBO_WDTW || M->id == WBO_WLCSS) {
        M->weights = logistic_weights(imax(xL, yL), M->p.g);
    } else if (M->id == WBO_WDDTW) {
        /* WeightedDerivativeDtwMetric.reset: distance/_elastic.pyx:3415-3430 */
        M->weights = logistic_weights(imax(xL - 2, yL - 2), M->p.g);
    } else if (M->id == WBO_EDR && isnan(M->p.epsilon)) {
        /* EdrMetric.reset: distance/_elastic.pyx:3731-3752 */
        double mean, std;
        M->std_x = malloc(sizeof(double) * (size_t)(xn * xd));
        M->std_y = malloc(sizeof(double) * (size_t)(yn * yd));
        for (idx_t i = 0; i < xn; i++)
            for (idx_t d = 0; d < xd; d++) {
                fast_mean_std(X + (i * xd + d) * xL, xL, &mean, &std);
                M->std_x[d * xn + i] = std;
            }
        for (idx_t i = 0; i < yn; i++)
            for (idx_t d = 0; d < yd; d++) {
                fast_mean_std(Y + (i * yd + d) * yL, yL, &mean, &std);
                M->std_y[d * yn + i] = std;
            }
    }
}

static void metric_free(wbo_metric *M)
{
    free(M->weights); free(M->std_x); free(M->std_y);
    M->weights = M->std_x = M->std_y = NULL;
}

/*
 * One call to the metric's distance (ea == 0) or eadistance (ea == 1).
 * For eadistance, *min_dist is the in/out threshold and the return value is
 * the bint result; for distance, the return value is the distance.
 * x/y point at the row (already offset by index and dim).
 */
static double metric_call(const wbo_metric *M, wbo_scratch *s, const double *x, idx_t xl,
                          idx_t x_index, const double *y, idx_t yl, idx_t y_index,
                          idx_t dim, int ea, double *min_dist)
{
    const wbo_params *p = &M->p;
    double dist, thr = 0;
    switch (M->id) {
    case WBO_EUCLIDEAN:
        /* EuclideanMetric: distance/_metric.pyx:381-409 */
        if (!ea) return euclid_scan(x, xl, y, yl, INF, NULL);
        dist = euclid_scan(x, xl, y, yl, *min_dist * *min_dist, NULL);
        break;
    case WBO_DTW:
    case WBO_WDTW:
        /* DtwMetric: distance/_elastic.pyx:3167-3213 */
        thr = ea ? *min_dist * *min_dist : INF;
        dist = sqrt(dtw_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), s->cost,
                             s->cost_prev, M->weights, thr));
        if (!ea) return dist;
        break;
    case WBO_DDTW:
    case WBO_WDDTW:
        /* DerivativeDtwMetric: distance/_elastic.pyx:3262-3320 */
        if (imin(xl, yl) < 3) return 0;
        average_slope(x, xl, s->d_x);
        average_slope(y, yl, s->d_y);
        if (!ea) {
            return sqrt(dtw_rows(s->d_x, xl - 2, s->d_y, yl - 2,
                                 compute_r(imin(xl, yl), p->r), s->cost, s->cost_prev,
                                 M->weights, INF));
        }
        dist = sqrt(dtw_rows(s->d_x, xl - 2, s->d_y, yl - 2,
                             compute_r(imin(xl - 2, yl - 2), p->r), s->cost, s->cost_prev,
                             M->weights, *min_dist * *min_dist));
        break;
    case WBO_ADTW:
        /* AmercingDtwMetric: distance/_elastic.pyx:3354-3401 */
        thr = ea ? *min_dist * *min_dist : INF;
        dist = sqrt(adtw_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), s->cost,
                              s->cost_prev, p->p, thr));
        if (!ea) return dist;
        break;
    case WBO_LCSS:
    case WBO_WLCSS: {
        /* LcssMetric: distance/_elastic.pyx:3483-3535 */
        if (ea) {
            double ml = (double)imin(xl, yl);
            thr = isinf(*min_dist) == 0 ? ml - *min_dist * ml : INF;
        } else {
            thr = INF;
        }
        dist = lcss_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), p->epsilon, s->cost,
                         s->cost_prev, M->weights, thr);
        if (!ea) return dist;
        break;
    }
    case WBO_EDR: {
        double eps;
        if (x_index < 0) {
            /* EdrMetric._distance / _eadistance (pointer forms, x_index < 0):
             * _elastic.pyx:3785-3880 -- epsilon from the two inputs themselves */
            if (isnan(p->epsilon)) {
                double mean, sx, sy;
                fast_mean_std(x, xl, &mean, &sx);
                fast_mean_std(y, yl, &mean, &sy);
                eps = dmax(sx, sy) / 4.0;
            } else {
                eps = p->epsilon;
            }
            if (!ea)
                return edr_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), eps, s->cost,
                                s->cost_prev, INF);
            dist = edr_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), eps, s->cost,
                            s->cost_prev, *min_dist * (double)imax(xl, yl));
            break;
        }
        /* EdrMetric.distance / eadistance (TSArray forms): _elastic.pyx:3754-3845 */
        if (isnan(p->epsilon))
            eps = dmax(M->std_x[dim * M->xn + x_index], M->std_y[dim * M->yn + y_index]) / 4.0;
        else
            eps = p->epsilon;
        if (!ea)
            return edr_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), eps, s->cost,
                            s->cost_prev, INF);
        /* the reference passes min(X.shape[2], X.shape[2]) here */
        dist = edr_rows(x, xl, y, yl, compute_r(imin(xl, xl), p->r), eps, s->cost,
                        s->cost_prev, *min_dist * (double)imax(xl, yl));
        break;
    }
    case WBO_ERP:
        /* ErpMetric: distance/_elastic.pyx:3612-3664 */
        thr = ea ? *min_dist : INF;
        dist = erp_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), p->g, s->gX, s->gY,
                        s->cost, s->cost_prev, thr);
        if (!ea) return dist;
        break;
    case WBO_MSM:
        /* MsmMetric: distance/_elastic.pyx:3933-3978 */
        thr = ea ? *min_dist : INF;
        dist = msm_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), p->c, s->cost,
                        s->cost_prev, s->cost_y, thr);
        if (!ea) return dist;
        break;
    case WBO_TWE:
        /* TweMetric: distance/_elastic.pyx:4038-4078 */
        thr = ea ? *min_dist : INF;
        dist = twe_rows(x, xl, y, yl, compute_r(imin(xl, yl), p->r), p->penalty,
                        p->stiffness, s->cost, s->cost_prev, thr);
        if (!ea) return dist;
        break;
    default:
        return NAN;
    }
    if (dist < *min_dist) {
        *min_dist = dist;
        return 1;
    }
    return 0;
}

/* Elastic subsequence distance: the *_subsequence_distance functions of
 * distance/_elastic.pyx (dtw :622-655, adtw :701-731, ddtw :769-806, lcss
 * :1186-1217, erp :1350-1382, edr :1500-1534, msm :1650-1681, twe :1832-1866)
 * with the metric classes' parameters (:2206-3124).  Every window T[i:i+L] is
 * compared with S, early abandoning at the running minimum (transformed as the
 * reference does), keeping the first strictly smaller window. */
static double subseq_elastic(int metric, const wbo_params *p, const double *S, idx_t sl,
                             double s_std, const double *T, idx_t tl, wbo_scratch *s,
                             const double *weights, double *sbuf, double *tbuf,
                             idx_t *index)
{
    idx_t r = compute_r(sl, p->r);
    idx_t length = tl - sl + 1;
    double min_dist = INF, dist = 0;
    if ((metric == WBO_DDTW || metric == WBO_WDDTW) && sl < 3) return 0;
    if (metric == WBO_DDTW || metric == WBO_WDDTW) average_slope(S, sl, sbuf);
    for (idx_t i = 0; i < length; i++) {
        switch (metric) {
        case WBO_DTW:
        case WBO_WDTW:
            dist = dtw_rows(S, sl, T + i, sl, r, s->cost, s->cost_prev, weights, min_dist);
            break;
        case WBO_ADTW:
            dist = adtw_rows(S, sl, T + i, sl, r, s->cost, s->cost_prev, p->p, min_dist);
            break;
        case WBO_DDTW:
        case WBO_WDDTW:
            average_slope(T + i, sl, tbuf);
            dist = dtw_rows(sbuf, sl - 2, tbuf, sl - 2, r, s->cost, s->cost_prev, weights,
                            min_dist);
            break;
        case WBO_LCSS: {
            double ml = (double)imin(sl, tl);
            double thr = isinf(min_dist) == 0 ? ml - min_dist * ml : min_dist;
            dist = lcss_rows(S, sl, T + i, sl, r, p->epsilon, s->cost, s->cost_prev, NULL,
                             thr);
            break;
        }
        case WBO_EDR: {
            double eps = isnan(p->epsilon) ? s_std / 4.0 : p->epsilon;
            dist = edr_rows(S, sl, T + i, sl, r, eps, s->cost, s->cost_prev,
                            min_dist * (double)imax(sl, tl));
            break;
        }
        case WBO_ERP:
            dist = erp_rows(S, sl, T + i, sl, r, p->g, s->gX, s->gY, s->cost, s->cost_prev,
                            min_dist);
            break;
        case WBO_MSM:
            dist = msm_rows(S, sl, T + i, sl, r, p->c, s->cost, s->cost_prev, s->cost_y,
                            min_dist);
            break;
        case WBO_TWE:
            dist = twe_rows(S, sl, T + i, sl, r, p->penalty, p->stiffness, s->cost,
                            s->cost_prev, min_dist);
            break;
        default:
            return NAN;
        }
        if (dist < min_dist) {
            if (index) *index = i;
            min_dist = dist;
        }
    }
    switch (metric) {
    case WBO_DTW:
    case WBO_WDTW:
    case WBO_ADTW:
    case WBO_DDTW:
    case WBO_WDDTW:
        return sqrt(min_dist);
    default:
        return min_dist;
    }
}

/* SubsequenceMetric._matches for one (S, T) pair: every window's distance
 * and whether the reference keeps it for `threshold` --
 * euclidean_distance_matches / scaled_euclidean_distance_matches
 * (distance/_metric.pyx:762-870) and the elastic *_subsequence_matches
 * (distance/_elastic.pyx:658-1910), each called with the threshold the
 * metric class passes.  dist[i] is the value the reference computes for
 * window i (its stored distance when kept); keep[i] is 1 when kept. */
static void subseq_matches(int metric, const wbo_params *p, const double *S, idx_t sl,
                           double s_mean, double s_std, const double *T, idx_t tl,
                           wbo_scratch *s, const double *weights, double *sbuf,
                           double *tbuf, double threshold, double *dist_out,
                           double *keep_out)
{
    idx_t length = tl - sl + 1;
    if (metric == WBO_EUCLIDEAN) {
        double thr = threshold * threshold;
        for (idx_t i = 0; i < length; i++) {
            double dist = 0;
            for (idx_t j = 0; j < sl; j++) {
                if (dist > thr) break;
                double x = T[i + j];
                x -= S[j];
                dist += x * x;
            }
            dist_out[i] = sqrt(dist);
            keep_out[i] = dist <= thr;
        }
        return;
    }
    if (metric == WBO_SCALED_EUCLIDEAN) {
        double thr = threshold * threshold, ex = 0, ex2 = 0;
        for (idx_t i = 0; i < tl; i++) {
            double cv = T[i];
            ex += cv;
            ex2 += cv * cv;
            idx_t bp = i % sl;
            sbuf[bp] = cv;
            sbuf[bp + sl] = cv;
            if (i >= sl - 1) {
                idx_t j = (i + 1) % sl;
                double mean = ex / (double)sl;
                double tmp = ex2 / (double)sl - mean * mean;
                double std = tmp > 0 ? sqrt(tmp) : 1.0;
                double dist = 0;
                for (idx_t k = 0; k < sl; k++) {
                    if (dist >= thr) break;
                    double x = (S[k] - s_mean) / s_std;
                    x -= (sbuf[k + j] - mean) / std;
                    dist += x * x;
                }
                dist_out[i + 1 - sl] = sqrt(dist);
                keep_out[i + 1 - sl] = dist <= thr;
                cv = sbuf[j];
                ex -= cv;
                ex2 -= cv * cv;
            }
        }
        return;
    }
    idx_t r = compute_r(sl, p->r);
    int sq = metric == WBO_DTW || metric == WBO_WDTW || metric == WBO_ADTW ||
             metric == WBO_DDTW || metric == WBO_WDDTW;
    if ((metric == WBO_DDTW || metric == WBO_WDDTW) && sl < 3) {
        for (idx_t i = 0; i < length; i++) {
            dist_out[i] = NAN;
            keep_out[i] = 0;
        }
        return;
    }
    if (metric == WBO_DDTW || metric == WBO_WDDTW) average_slope(S, sl, sbuf);
    double thr = sq ? threshold * threshold : threshold;
    for (idx_t i = 0; i < length; i++) {
        double dist;
        switch (metric) {
        case WBO_DTW:
        case WBO_WDTW:
            dist = dtw_rows(S, sl, T + i, sl, r, s->cost, s->cost_prev, weights, thr);
            break;
        case WBO_ADTW:
            dist = adtw_rows(S, sl, T + i, sl, r, s->cost, s->cost_prev, p->p, thr);
            break;
        case WBO_DDTW:
        case WBO_WDDTW:
            average_slope(T + i, sl, tbuf);
            dist = dtw_rows(sbuf, sl - 2, tbuf, sl - 2, r, s->cost, s->cost_prev, weights,
                            thr);
            break;
        case WBO_LCSS: {
            double ml = (double)imin(sl, tl);
            double t2 = isinf(threshold) == 0 ? ml - threshold * ml : threshold;
            dist = lcss_rows(S, sl, T + i, sl, r, p->epsilon, s->cost, s->cost_prev, NULL,
                             t2);
            break;
        }
        case WBO_EDR: {
            double eps = isnan(p->epsilon) ? s_std / 4.0 : p->epsilon;
            dist = edr_rows(S, sl, T + i, sl, r, eps, s->cost, s->cost_prev,
                            threshold * (double)imax(sl, tl));
            break;
        }
        case WBO_ERP:
            dist = erp_rows(S, sl, T + i, sl, r, p->g, s->gX, s->gY, s->cost, s->cost_prev,
                            thr);
            break;
        case WBO_MSM:
            dist = msm_rows(S, sl, T + i, sl, r, p->c, s->cost, s->cost_prev, s->cost_y, thr);
            break;
        case WBO_TWE:
            dist = twe_rows(S, sl, T + i, sl, r, p->penalty, p->stiffness, s->cost,
                            s->cost_prev, thr);
            break;
        default:
            dist = NAN;
        }
        keep_out[i] = dist <= thr;
        if (metric == WBO_LCSS || metric == WBO_EDR) keep_out[i] = dist <= threshold;
        dist_out[i] = sq ? sqrt(dist) : dist;
    }
}

/* ---------------------------------------------------------------------- */
/* Heap keeping the k smallest: utils/_misc.pyx:18-107                     */
/* ---------------------------------------------------------------------- */
typedef struct { idx_t index; double value; } heap_el;

static void heap_sift_toward_root(heap_el *h, idx_t start, idx_t pos)
{
    heap_el e = h[pos];
    while (pos > start) {
        idx_t parent = (pos - 1) >> 1;
        if (e.value > h[parent].value) {
            h[pos] = h[parent];
            pos = parent;
            continue;
        }
        break;
    }
    h[pos] = e;
}

static void heap_sift_to_leaf(heap_el *h, idx_t pos, idx_t end)
{
    idx_t start = pos;
    heap_el e = h[pos];
    idx_t child = 2 * pos + 1;
    while (child < end) {
        idx_t right = child + 1;
        if (right < end && h[child].value < h[right].value) child = right;
        h[pos] = h[child];
        pos = child;
        child = 2 * pos + 1;
    }
    h[pos] = e;
    heap_sift_toward_root(h, start, pos);
}

static void heap_push(heap_el *h, idx_t *n, idx_t k, idx_t index, double value)
{
    heap_el e = {index, value};
    if (*n == 0) {
        h[0] = e;
        *n = 1;
    } else if (*n < k) {
        h[*n] = e;
        *n += 1;
        heap_sift_toward_root(h, 0, *n - 1);
    } else if (h[0].value > value) {
        h[0] = e;
        heap_sift_to_leaf(h, 0, k);
    }
}

/* ---------------------------------------------------------------------- */
/* Drivers (run_in_parallel: contiguous batches over the outer axis,       */
/* utils/_parallel.py:7-43)                                                */
/* ---------------------------------------------------------------------- */

typedef struct {
    int kind;                 /* 0 pairwise, 1 singleton, 2 paired, 3 argmin, 4 subseq */
    const wbo_metric *M;
    const double *X, *Y;
    idx_t xn, xd, xL, yn, yd, yL, dim;
    double *out;
    idx_t *out_idx;
    idx_t k;
    const double *lower_bound;
    /* subsequence */
    const double *shp;
    const idx_t *shp_off, *shp_len;
    const double *shp_mean, *shp_std;
    const double *sub_weights;
    wbo_params sub_params;
    idx_t m;
    double threshold;          /* matches */
    double *out_keep;          /* matches: (n, ld) */
    idx_t ld;
    idx_t s_stride;            /* argmin subsequence: row stride of the subsequences */
    int scaled;
    idx_t begin, end;
} job_t;

static void *run_job(void *arg)
{
    job_t *J = arg;
    const wbo_metric *M = J->M;
    wbo_scratch s;
    idx_t L = imax(J->xL, J->yL);
    scratch_init(&s, L);
    double *sbuf = NULL;
    heap_el *heap = NULL;
    if (J->kind == 3) heap = malloc(sizeof(heap_el) * (size_t)imax(J->k, 1));
    double *tbuf = NULL;
    if (J->kind >= 4) {
        sbuf = malloc(sizeof(double) * (size_t)(2 * J->xL + 2));
        tbuf = malloc(sizeof(double) * (size_t)(2 * J->xL + 2));
    }
    if (J->kind == 5) heap = malloc(sizeof(heap_el) * (size_t)imax(J->k, 1));
    for (idx_t i = J->begin; i < J->end; i++) {
        const double *xr = J->X + (i * J->xd + J->dim) * J->xL;
        if (J->kind == 0) {
            for (idx_t j = 0; j < J->yn; j++) {
                const double *yr = J->Y + (j * J->yd + J->dim) * J->yL;
                J->out[i * J->yn + j] =
                    metric_call(M, &s, xr, J->xL, i, yr, J->yL, j, J->dim, 0, NULL);
            }
        } else if (J->kind == 1) {
            for (idx_t j = i + 1; j < J->xn; j++) {
                const double *yr = J->X + (j * J->xd + J->dim) * J->xL;
                double d = metric_call(M, &s, xr, J->xL, i, yr, J->xL, j, J->dim, 0, NULL);
                J->out[i * J->xn + j] = d;
                J->out[j * J->xn + i] = d;
            }
        } else if (J->kind == 2) {
            const double *yr = J->Y + (i * J->yd + J->dim) * J->yL;
            J->out[i] = metric_call(M, &s, xr, J->xL, i, yr, J->yL, i, J->dim, 0, NULL);
        } else if (J->kind == 3) {
            /* _ArgMinBatch.__call__: distance/_cdistance.pyx:1302-1345 */
            double distance = INF;
            idx_t hn = 0;
            for (idx_t j = 0; j < J->yn; j++) {
                if (J->lower_bound && J->lower_bound[i * J->yn + j] >= distance) continue;
                const double *yr = J->Y + (j * J->yd + J->dim) * J->yL;
                if (metric_call(M, &s, xr, J->xL, i, yr, J->yL, j, J->dim, 1, &distance)) {
                    heap_push(heap, &hn, J->k, j, distance);
                    distance = (hn == J->k) ? heap[0].value : INF;
                }
            }
            /* the output array is zero-initialised; unfilled heap slots keep
             * whatever the heap array held (never read when hn == k) */
            for (idx_t j = 0; j < J->k; j++) {
                if (j < hn) {
                    J->out_idx[i * J->k + j] = heap[j].index;
                    J->out[i * J->k + j] = heap[j].value;
                }
            }
        } else if (J->kind == 4) {
            /* _PairwiseSubsequenceDistance.__call__: distance/_cdistance.pyx:1001-1015 */
            for (idx_t j = 0; j < J->m; j++) {
                const double *S = J->shp + J->shp_off[j];
                idx_t sl = J->shp_len[j];
                idx_t mi = 0;
                double d;
                if (M->id == WBO_SCALED_EUCLIDEAN) {
                    double sstd = J->shp_std[j] != 0 ? J->shp_std[j] : 1.0;
                    d = scaled_euclid_scan(S, sl, J->shp_mean[j], sstd, xr, J->xL, sbuf, &mi);
                } else if (M->id == WBO_EUCLIDEAN) {
                    d = euclid_scan(S, sl, xr, J->xL, INF, &mi);
                } else {
                    double sstd = J->shp_std && J->shp_std[j] != 0 ? J->shp_std[j] : 1.0;
                    d = subseq_elastic(M->id, &J->sub_params, S, sl, sstd, xr, J->xL, &s,
                                       J->sub_weights, sbuf, tbuf, &mi);
                }
                J->out[i * J->m + j] = d;
                J->out_idx[i * J->m + j] = mi;
            }
        } else if (J->kind == 6) {
            /* _subsequence_match / _paired_subsequence_match / _distance_profile:
             * _cdistance.pyx:1065-1141, :345-403; pair i = (shapelet i, series i) */
            const double *S = J->shp + J->shp_off[i];
            idx_t sl = J->shp_len[i];
            double smean = J->shp_mean ? J->shp_mean[i] : 0.0;
            double sstd = J->shp_std && (J->shp_std[i] != 0 || J->scaled) ? J->shp_std[i] : 1.0;
            subseq_matches(M->id, &J->sub_params, S, sl, smean, sstd, xr, J->xL, &s,
                           J->sub_weights, sbuf, tbuf, J->threshold, J->out + i * J->ld,
                           J->out_keep + i * J->ld);
        } else if (J->kind == 5) {
            /* _ArgminSubsequenceDistance / _ScaledArgminSubsequenceDistance:
             * _cdistance.pyx:1381-1557 */
            idx_t sl = J->shp_len[i];
            const double *S = J->shp + i * J->s_stride;
            const double *sv = S;
            idx_t nwin = J->xL - sl + 1;
            incstats st;
            if (J->scaled) {
                double mean, std;
                fast_mean_std(S, sl, &mean, &std);
                if (std == 0.0) std = 1.0;
                inc_init(&st);
                for (idx_t n = 0; n < sl - 1; n++) {
                    sbuf[n] = (S[n] - mean) / std;
                    inc_add(&st, 1.0, xr[n]);
                }
                sbuf[sl - 1] = (S[sl - 1] - mean) / std;
                sv = sbuf;
            }
            double distance = INF;
            idx_t hn = 0;
            for (idx_t j = 0; j < nwin; j++) {
                const double *wv = xr + j;
                if (J->scaled) {
                    inc_add(&st, 1.0, xr[j + sl - 1]);
                    double sd = inc_variance(&st);
                    if (sd == 0.0) sd = 1.0;
                    else sd = sqrt(sd);
                    double mu = st.mean;
                    for (idx_t n = 0; n < sl; n++) tbuf[n] = (xr[j + n] - mu) / sd;
                    inc_remove(&st, 1.0, xr[j]);
                    wv = tbuf;
                }
                if (metric_call(M, &s, sv, sl, -1, wv, sl, -1, 0, 1, &distance))
                    heap_push(heap, &hn, J->k, j, distance);
                distance = (hn == J->k) ? heap[0].value : INF;
            }
            for (idx_t j = 0; j < J->k && j < hn; j++) {
                J->out_idx[i * J->k + j] = heap[j].index;
                J->out[i * J->k + j] = heap[j].value;
            }
        }
    }
    free(heap);
    free(sbuf);
    free(tbuf);
    scratch_free(&s);
    return NULL;
}

static void run_parallel(job_t *proto, idx_t n_work, int n_threads)
{
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_work) n_threads = (int)(n_work > 0 ? n_work : 1);
    pthread_t *th = malloc(sizeof(pthread_t) * (size_t)n_threads);
    job_t *jobs = malloc(sizeof(job_t) * (size_t)n_threads);
    idx_t base = n_work / n_threads, rem = n_work % n_threads, off = 0;
    for (int t = 0; t < n_threads; t++) {
        idx_t sz = base + (t < rem ? 1 : 0);
        jobs[t] = *proto;
        jobs[t].begin = off;
        jobs[t].end = off + sz;
        off += sz;
        if (n_threads == 1) run_job(&jobs[t]);
        else pthread_create(&th[t], NULL, run_job, &jobs[t]);
    }
    if (n_threads > 1)
        for (int t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
}

/* ---------------------------------------------------------------------- */
/* Exported entry points (ctypes)                                          */
/* ---------------------------------------------------------------------- */

/* _pairwise_distance / _singleton_pairwise_distance: _cdistance.pyx:1184-1267.
 * Y == NULL selects the singleton (x is y) path; out must be zero-filled. */
int wbo_pairwise(const double *X, idx_t xn, idx_t xd, idx_t xL, const double *Y, idx_t yn,
                 idx_t yd, idx_t yL, idx_t dim, int metric, const wbo_params *p,
                 double *out, int n_threads)
{
    wbo_metric M = {0};
    M.id = metric;
    M.p = *p;
    job_t J = {0};
    J.M = &M;
    J.X = X; J.xn = xn; J.xd = xd; J.xL = xL; J.dim = dim; J.out = out;
    if (Y == NULL) {
        metric_reset(&M, X, xn, xd, xL, X, xn, xd, xL);
        J.kind = 1;
        J.Y = X; J.yn = xn; J.yd = xd; J.yL = xL;
    } else {
        metric_reset(&M, X, xn, xd, xL, Y, yn, yd, yL);
        J.kind = 0;
        J.Y = Y; J.yn = yn; J.yd = yd; J.yL = yL;
    }
    run_parallel(&J, xn, n_threads);
    metric_free(&M);
    return 0;
}

/* _paired_distance: _cdistance.pyx:1597-1652.  A and B are the API's x and y;
 * the metric sees (B, A): rows of the DP come from the second argument. */
int wbo_paired(const double *A, const double *B, idx_t n, idx_t d, idx_t AL, idx_t BL,
               idx_t dim, int metric, const wbo_params *p, double *out, int n_threads)
{
    wbo_metric M = {0};
    M.id = metric;
    M.p = *p;
    metric_reset(&M, B, n, d, BL, A, n, d, AL);
    job_t J = {0};
    J.kind = 2; J.M = &M;
    J.X = B; J.xn = n; J.xd = d; J.xL = BL;
    J.Y = A; J.yn = n; J.yd = d; J.yL = AL;
    J.dim = dim; J.out = out;
    run_parallel(&J, n, n_threads);
    metric_free(&M);
    return 0;
}

/* _argmin_distance: _cdistance.pyx:1348-1378 (outputs zero-filled by caller) */
int wbo_argmin(const double *X, idx_t xn, idx_t xd, idx_t xL, const double *Y, idx_t yn,
               idx_t yd, idx_t yL, idx_t dim, int metric, const wbo_params *p, idx_t k,
               const double *lower_bound, idx_t *out_idx, double *out_dist, int n_threads)
{
    wbo_metric M = {0};
    M.id = metric;
    M.p = *p;
    metric_reset(&M, X, xn, xd, xL, Y, yn, yd, yL);
    job_t J = {0};
    J.kind = 3; J.M = &M;
    J.X = X; J.xn = xn; J.xd = xd; J.xL = xL;
    J.Y = Y; J.yn = yn; J.yd = yd; J.yL = yL;
    J.dim = dim; J.k = k; J.lower_bound = lower_bound;
    J.out = out_dist; J.out_idx = out_idx;
    run_parallel(&J, xn, n_threads);
    metric_free(&M);
    return 0;
}

/* _pairwise_subsequence_distance (euclidean / scaled_euclidean):
 * _cdistance.pyx:956-1037.  Shapelets are packed; mean/std come from
 * np.mean/np.std on the caller side (ScaledSubsequenceMetric.from_array,
 * _cdistance.pyx:453-467). */
int wbo_subsequence(const double *shp, const idx_t *off, const idx_t *len,
                    const double *smean, const double *sstd, idx_t m, const double *X,
                    idx_t xn, idx_t xd, idx_t xL, idx_t dim, int metric,
                    const wbo_params *p, double *out_dist, idx_t *out_idx, int n_threads)
{
    wbo_metric M = {0};
    M.id = metric;
    job_t J = {0};
    J.kind = 4; J.M = &M;
    J.X = X; J.xn = xn; J.xd = xd; J.xL = xL; J.yL = xL; J.dim = dim;
    J.shp = shp; J.shp_off = off; J.shp_len = len; J.shp_mean = smean; J.shp_std = sstd;
    J.m = m; J.out = out_dist; J.out_idx = out_idx;
    double *w = NULL;
    if (p) J.sub_params = *p;
    /* WeightedDtwSubsequenceMetric.reset (_elastic.pyx:2364-2376): n = X.shape[2];
     * WeightedDerivativeDtwSubsequenceMetric.reset (:2533-2546): n = X.shape[2] - 2 */
    if (metric == WBO_WDTW) w = logistic_weights(xL, p->g);
    if (metric == WBO_WDDTW) w = logistic_weights(xL - 2 > 0 ? xL - 2 : 0, p->g);
    J.sub_weights = w;
    run_parallel(&J, xn, n_threads);
    free(w);
    return 0;
}

/* SubsequenceMetric._matches for pairs (shapelet i, x[i, dim]):
 * out_dist / out_keep are (n, ld), windows past a pair's last untouched.
 * std_as_given: a zero shapelet std is not replaced by 1 (the distance
 * profile passes its transient statistics as they are). */
int wbo_subsequence_matches(const double *shp, const idx_t *off, const idx_t *len,
                            const double *smean, const double *sstd, idx_t n,
                            const double *X, idx_t xd, idx_t xL, idx_t dim, int metric,
                            const wbo_params *p, double threshold, double *out_dist,
                            double *out_keep, idx_t ld, int std_as_given, int n_threads)
{
    wbo_metric M = {0};
    M.id = metric;
    job_t J = {0};
    J.kind = 6; J.M = &M;
    J.X = X; J.xn = n; J.xd = xd; J.xL = xL; J.yL = xL; J.dim = dim;
    J.shp = shp; J.shp_off = off; J.shp_len = len; J.shp_mean = smean; J.shp_std = sstd;
    J.m = n; J.out = out_dist; J.out_keep = out_keep; J.ld = ld; J.threshold = threshold;
    J.scaled = std_as_given;  /* kind 6: a zero std is used as is */
    double *w = NULL;
    if (p) J.sub_params = *p;
    if (metric == WBO_WDTW) w = logistic_weights(xL, p->g);
    if (metric == WBO_WDDTW) w = logistic_weights(xL - 2 > 0 ? xL - 2 : 0, p->g);
    J.sub_weights = w;
    run_parallel(&J, n, n_threads);
    free(w);
    return 0;
}

/* _argmin_subsequence_distance: _cdistance.pyx:1559-1594.  S is (n, s_stride)
 * (the reference's (n, 1, max_len) subsequence array), s_len the lengths;
 * metric reset with (x, S) as the reference does.  Outputs zero-filled by the
 * caller; (n, k) in heap order. */
int wbo_argmin_subsequence(const double *S, const idx_t *s_len, idx_t s_stride, idx_t n,
                           const double *X, idx_t xd, idx_t xL, idx_t dim, int metric,
                           const wbo_params *p, int scaled, idx_t k, idx_t *out_idx,
                           double *out_dist, int n_threads)
{
    wbo_metric M = {0};
    M.id = metric;
    M.p = *p;
    metric_reset(&M, X, n, xd, xL, S, n, 1, s_stride);
    job_t J = {0};
    J.kind = 5; J.M = &M;
    J.X = X; J.xn = n; J.xd = xd; J.xL = xL; J.yL = s_stride; J.dim = dim;
    J.shp = S; J.shp_len = s_len; J.s_stride = s_stride; J.scaled = scaled; J.k = k;
    J.out = out_dist; J.out_idx = out_idx;
    run_parallel(&J, n, n_threads);
    metric_free(&M);
    return 0;
}

/* single pair, full-matrix-free: distance of two 1-D rows (used by tests) */
double wbo_distance_1d(const double *x, idx_t xl, const double *y, idx_t yl, int metric,
                       const wbo_params *p)
{
    wbo_metric M = {0};
    M.id = metric;
    M.p = *p;
    metric_reset(&M, x, 1, 1, xl, y, 1, 1, yl);
    wbo_scratch s;
    scratch_init(&s, imax(xl, yl));
    double d = metric_call(&M, &s, x, xl, 0, y, yl, 0, 0, 0, NULL);
    scratch_free(&s);
    metric_free(&M);
    return d;
}

/* _dilated_distance_profile with dilated_distance_profile /
 * scaled_dilated_distance_profile (distance/_cdistance.pyx:804-933,
 * 1809-1841): S (n, L) kernels (scaled by the caller when `scaled`), X
 * (n, xd, T); out (n, T + 2 padding - (L - 1) dilation).  Positions where the
 * metric's _eadistance returns false (an infinite distance) are NAN here; the
 * reference leaves them unwritten. */
int wbo_dilated_profile(const double *S, idx_t L, const double *X, idx_t n, idx_t xd,
                        idx_t T, idx_t dim, int metric, const wbo_params *p, idx_t dilation,
                        idx_t padding, int scaled, double *out)
{
    idx_t input_size = T + 2 * padding;
    idx_t kernel_size = (L - 1) * dilation + 1;
    if (dilation < 1 || padding < 0 || kernel_size > input_size) return -1;
    idx_t output_size = input_size - kernel_size + 1;
    double *xb = malloc(sizeof(double) * (size_t)L);
    double *kb = malloc(sizeof(double) * (size_t)L);
    wbo_metric M = {0};
    M.id = metric;
    M.p = *p;
    /* Metric.reset(X, X): weights sized from the series length */
    metric_reset(&M, X, n, xd, T, X, n, xd, T);
    wbo_scratch s;
    scratch_init(&s, imax(L, T));
    for (idx_t i = 0; i < n; i++) {
        const double *x = X + (i * xd + dim) * T;
        const double *kernel = S + i * L;
        for (idx_t o = 0; o < output_size; o++) {
            idx_t padding_offset = padding - o;
            idx_t kernel_offset, input_offset;
            if (padding_offset > 0) {
                if (padding_offset % dilation == 0)
                    kernel_offset = padding_offset;
                else
                    kernel_offset = padding_offset + dilation - (padding_offset % dilation);
                input_offset = kernel_offset - padding_offset;
            } else {
                kernel_offset = 0;
                input_offset = -padding_offset;
            }
            idx_t conv = imin(T, input_offset + kernel_size - imax(0, padding_offset)) -
                         input_offset;
            idx_t k = 0;
            double mean = 0, std = 0;
            for (idx_t j = 0; j < conv; j += dilation) {
                double v = x[input_offset + j];
                xb[k] = v;
                kb[k] = kernel[(j + kernel_offset) / dilation];
                mean += v;
                std += v * v;
                k++;
            }
            if (scaled) {
                mean = mean / L;
                std = std / L - mean * mean;
                if (std > 1e-13) std = sqrt(std);
                else std = 1;
                for (idx_t j = 0; j < k; j++) xb[j] = (xb[j] - mean) / std;
            }
            double md = INF;
            if (metric_call(&M, &s, xb, k, -1, kb, k, -1, 0, 1, &md))
                out[i * output_size + o] = md / (double)((float)k / (float)L);
            else
                out[i * output_size + o] = NAN;
        }
    }
    scratch_free(&s);
    metric_free(&M);
    free(xb);
    free(kb);
    return 0;
}

/* cumulative_mean_std (utils/_stats.pyx:95-111): IncStats mean and std of
 * every window of length L of x (n_windows = T - L + 1) */
void wbo_cumulative_mean_std(const double *x, idx_t T, idx_t L, double *mean, double *std)
{
    double m = 0, ns = 0, ssq = 0;
    for (idx_t i = 0; i < T; i++) {
        double v = x[i], next_m;
        ns += 1.0;
        next_m = m + (v - m) / ns;
        ssq += (v - m) * (v - next_m);
        m = next_m;
        if (i >= L - 1) {
            double var = ns <= 1 ? 0 : ssq / ns;
            if (var < 1e-13) var = 0.0;
            mean[i - (L - 1)] = m;
            std[i - (L - 1)] = sqrt(var);
            double u = x[i - (L - 1)];
            if (ns == 1.0) {
                ns = 0.0;
                m = 0.0;
                ssq = 0.0;
            } else {
                double old_m = (ns * m - u) / (ns - 1.0);
                ssq -= (u - m) * (u - old_m);
                m = old_m;
                ns -= 1.0;
            }
        }
    }
}

/* fast_mean_std, exported for tests */
void wbo_fast_mean_std(const double *x, idx_t n, double *mean, double *std)
{
    fast_mean_std(x, n, mean, std);
}

/* _dtw_alignment: distance/_elastic.pyx:1011-1073.  out is (n, m); cells
 * outside the band are left as the caller filled them. */
int wbo_dtw_alignment(const double *X, idx_t n, const double *Y, idx_t m, idx_t r,
                      const double *weights, double *out)
{
    if (!(0 < r && r <= imax(n, m))) return -1;
    double v, w = 1.0;
#define OUT(i, j) out[(i) * m + (j)]
    v = X[0] - Y[0];
    if (weights) w = weights[0];
    OUT(0, 0) = v * v * w;
    for (idx_t i = 1; i < imin(n, r + 1); i++) {
        v = X[i] - Y[0];
        if (weights) w = weights[i];
        OUT(i, 0) = OUT(i - 1, 0) + v * v * w;
    }
    for (idx_t i = 1; i < imin(m, imax(0, m - n) + r); i++) {
        v = X[0] - Y[i];
        if (weights) w = weights[i];
        OUT(0, i) = OUT(0, i - 1) + v * v * w;
    }
    if (imax(0, m - n) + r < m) OUT(0, imax(0, m - n) + r) = INF;
    for (idx_t i = 1; i < n; i++) {
        idx_t js = imax(0, i - imax(0, n - m) - r + 1);
        idx_t je = imin(m, i + imax(0, m - n) + r);
        if (js > 0) OUT(i, js - 1) = INF;
        for (idx_t j = js; j < je; j++) {
            v = X[i] - Y[j];
            double x = OUT(i - 1, j);
            double y = j > 0 ? OUT(i, j - 1) : INF;
            double z = j > 0 ? OUT(i - 1, j - 1) : INF;
            if (weights) w = weights[labs((long)(i - j))];
            OUT(i, j) = dmin(dmin(x, y), z) + v * v * w;
        }
        if (je < m) OUT(i, je) = INF;
    }
#undef OUT
    return 0;
}

/* One epoch of _mm_dtw_average (distance/dtw.py:661-690): for every sample i
 * in order, the alignment of `mean` (nm values) with X[i] (T values,
 * _dtw_alignment with warp r and optional weights), the traceback of
 * dtw_mapping (distance/dtw.py:362-426: from the last cell, np.argmin over
 * [diag, up, left], the first minimum winning; along the first row or column
 * the only finite option), then V[m] += w and z[m] += X[i, x] * w over the
 * path cells in row-major order (indicator.nonzero()); out_mean = z / V.
 * `work` holds nm * T doubles, `path` 2 * (nm + T) indices. */
int wbo_mm_epoch(const double *X, idx_t n_samples, idx_t T, const double *mean, idx_t nm,
                 idx_t r, const double *weights, const double *sample_weight,
                 double *out_mean, double *work, idx_t *path, double *last)
{
    double *z = (double *)calloc((size_t)nm, sizeof(double));
    double *V = (double *)calloc((size_t)nm, sizeof(double));
    if (!z || !V) {
        free(z);
        free(V);
        return -2;
    }
    for (idx_t s = 0; s < n_samples; s++) {
        const double *Xs = X + s * T;
        if (wbo_dtw_alignment(mean, nm, Xs, T, r, weights, work) != 0) {
            free(z);
            free(V);
            return -1;
        }
        if (last) last[s] = work[(nm - 1) * T + (T - 1)];
        idx_t i = nm - 1, j = T - 1, len = 0;
        while (i > 0 || j > 0) {
            path[2 * len] = i;
            path[2 * len + 1] = j;
            len++;
            double diag = (i > 0 && j > 0) ? work[(i - 1) * T + (j - 1)] : INF;
            double up = i > 0 ? work[(i - 1) * T + j] : INF;
            double left = j > 0 ? work[i * T + (j - 1)] : INF;
            int move = 0;
            double best = diag;
            if (up < best) {
                best = up;
                move = 1;
            }
            if (left < best) move = 2;
            if (move == 0) {
                i--;
                j--;
            } else if (move == 1) {
                i--;
            } else {
                j--;
            }
        }
        path[2 * len] = 0;
        path[2 * len + 1] = 0;
        len++;
        const double w = sample_weight ? sample_weight[s] : 1.0;
        for (idx_t k = len - 1; k >= 0; k--) {
            const idx_t pm = path[2 * k], px = path[2 * k + 1];
            V[pm] += w;
            z[pm] += Xs[px] * w;
        }
    }
    for (idx_t k = 0; k < nm; k++) out_mean[k] = z[k] / V[k];
    free(z);
    free(V);
    return 0;
}

/* ------------------------------------------------------------------------
 * scaled_dtw subsequence metric: ScaledDtwSubsequenceMetric
 * (distance/_elastic.pyx:1928-2204) with the UCR-suite scan
 * scaled_dtw_subsequence_distance / scaled_dtw_matches (:353-620).
 */

/* the reference's ring deque (_elastic.pyx:37-95): push at `back`, moving
 * down; the front element sits just above `front` */
typedef struct {
    idx_t *q;
    idx_t cap, size, front, back;
} sdq;

static void sdq_reset(sdq *c) { c->size = 0; c->front = 0; c->back = c->cap - 1; }
static void sdq_push_back(sdq *c, idx_t v)
{
    c->q[c->back] = v;
    c->back -= 1;
    if (c->back < 0) c->back = c->cap - 1;
    c->size += 1;
}
static void sdq_pop_front(sdq *c)
{
    c->front -= 1;
    if (c->front < 0) c->front = c->cap - 1;
    c->size -= 1;
}
static void sdq_pop_back(sdq *c) { c->back = (c->back + 1) % c->cap; c->size -= 1; }
static idx_t sdq_front(const sdq *c)
{
    idx_t t = c->front - 1;
    if (t < 0) t = c->cap - 1;
    return c->q[t];
}
static idx_t sdq_back(const sdq *c) { return c->q[(c->back + 1) % c->cap]; }

/* find_min_max (_elastic.pyx:98-151): streaming envelope of T with warp r,
 * including the reference's single front pop per step */
static void sdtw_envelope(const double *T, idx_t length, idx_t r, double *lower, double *upper,
                          sdq *dl, sdq *du)
{
    sdq_reset(du);
    sdq_reset(dl);
    sdq_push_back(du, 0);
    sdq_push_back(dl, 0);
    for (idx_t i = 1; i < length; i++) {
        if (i > r) {
            idx_t k = i - r - 1;
            upper[k] = T[sdq_front(du)];
            lower[k] = T[sdq_front(dl)];
        }
        double cur = T[i], prev = T[i - 1];
        if (cur > prev) {
            sdq_pop_back(du);
            while (du->size != 0 && cur > T[sdq_back(du)]) sdq_pop_back(du);
        } else {
            sdq_pop_back(dl);
            while (dl->size != 0 && cur < T[sdq_back(dl)]) sdq_pop_back(dl);
        }
        sdq_push_back(du, i);
        sdq_push_back(dl, i);
        if (i == 2 * r + 1 + sdq_front(du))
            sdq_pop_front(du);
        else if (i == 2 * r + 1 + sdq_front(dl))
            sdq_pop_front(dl);
    }
    for (idx_t i = length; i < length + r + 1; i++) {
        idx_t k = i - r - 1;
        upper[k] = T[sdq_front(du)];
        lower[k] = T[sdq_front(dl)];
        if (i - sdq_front(du) >= 2 * r + 1) sdq_pop_front(du);
        if (i - sdq_front(dl) >= 2 * r + 1) sdq_pop_front(dl);
    }
}

static inline double sd2(double x, double y) { double s = x - y; return s * s; }

/* constant_lower_bound (_elastic.pyx:159-237), LB_Kim of the first and last
 * three points (the reference's second end term compares t_y1 with s_y1 twice) */
/* (the reference reads T[1], T[2], T[L - 2], T[L - 3] and the same points
 * of S whatever L is; for L < 3 those reads leave the arrays, here they are
 * clamped to [0, L - 1]) */
static inline idx_t sdtw_ix(idx_t k, idx_t L) { return k < 0 ? 0 : (k >= L ? L - 1 : k); }

static double sdtw_kim(const double *S, double sm, double ss, const double *T, double tm,
                       double ts, idx_t L, double best)
{
    if (ts == 0) return 0;
    const idx_t a1 = sdtw_ix(1, L), a2 = sdtw_ix(2, L), b1 = sdtw_ix(L - 2, L),
                b2 = sdtw_ix(L - 3, L);
    double tx0 = (T[0] - tm) / ts, ty0 = (T[L - 1] - tm) / ts;
    double sx0 = (S[0] - sm) / ss, sy0 = (S[L - 1] - sm) / ss;
    double md = sd2(tx0, sx0) + sd2(ty0, sy0);
    if (md >= best) return md;
    double tx1 = (T[a1] - tm) / ts, sx1 = (S[a1] - sm) / ss;
    md += dmin(dmin(sd2(tx1, sx0), sd2(tx0, sx1)), sd2(tx1, sx1));
    if (md >= best) return md;
    double ty1 = (T[b1] - tm) / ts, sy1 = (S[b1] - sm) / ss;
    md += dmin(dmin(sd2(ty1, sy1), sd2(ty0, sy1)), sd2(ty1, sy1));
    if (md >= best) return md;
    double tx2 = (T[a2] - tm) / ts, sx2 = (S[a2] - sm) / ss;
    md += dmin(dmin(dmin(sd2(tx0, sx2), dmin(sd2(tx1, sx2), sd2(tx2, sx2))), sd2(tx2, sx1)),
               sd2(tx2, sx0));
    if (md >= best) return md;
    double ty2 = (T[b2] - tm) / ts, sy2 = (S[b2] - sm) / ss;
    md += dmin(dmin(dmin(sd2(ty0, sy2), dmin(sd2(ty1, sy2), sd2(ty2, sy2))), sd2(ty2, sy1)),
               sd2(ty2, sy0));
    return md;
}

/* cumulative_bound (_elastic.pyx:240-270): LB_Keogh of T (normalised with
 * mean/std) against an envelope normalised with lu_mean/lu_std */
static double sdtw_keogh(const double *T, idx_t L, double mean, double std, double lu_mean,
                         double lu_std, const double *lower, const double *upper, double *cb,
                         double best)
{
    double md = 0;
    for (idx_t i = 0; i < L; i++) {
        if (md >= best) break;
        double x = (T[i] - mean) / std;
        double us = (upper[i] - lu_mean) / lu_std;
        double ls = (lower[i] - lu_mean) / lu_std;
        double d;
        if (x > us) d = sd2(x, us);
        else if (x < ls) d = sd2(x, ls);
        else d = 0;
        md += d;
        cb[i] = d;
    }
    return md;
}

/* inner_scaled_dtw_subsequence_distance (_elastic.pyx:273-344): Sakoe-Chiba
 * band |i - j| <= r, rows abandoned on row min + cb[i + r + 1] >= min_dist */
static double sdtw_inner(const double *S, idx_t L, double sm, double ss, const double *X,
                         double mean, double std, idx_t r, const double *cb, double *cost,
                         double *cost_prev, double min_dist)
{
    int std_zero = std == 0, s_std_zero = ss == 0;
    if (std_zero && s_std_zero) return 0;
    for (idx_t i = 0; i < 2 * r + 1; i++) {
        cost[i] = INF;
        cost_prev[i] = INF;
    }
    idx_t k = 0;
    for (idx_t i = 0; i < L; i++) {
        k = imax(0, r - i);
        double min_cost = INF;
        for (idx_t j = imax(0, i - r); j < imin(L, i + r + 1); j++) {
            double v;
            if (i == 0 && j == 0) {
                v = !s_std_zero ? (S[0] - sm) / ss : 0;
                if (!std_zero) v -= (X[0] - mean) / std;
                cost[k] = v * v;
            } else {
                double y = (j - 1 < 0 || k - 1 < 0) ? INF : cost[k - 1];
                double x = (i - 1 < 0 || k + 1 > 2 * r) ? INF : cost_prev[k + 1];
                double z = (i - 1 < 0 || j - 1 < 0) ? INF : cost_prev[k];
                v = (S[i] - sm) / ss;
                if (!std_zero) v -= (X[j] - mean) / std;
                cost[k] = dmin(dmin(x, y), z) + v * v;
            }
            if (cost[k] < min_cost) min_cost = cost[k];
            k += 1;
        }
        if (i + r < L - 1 && min_cost + cb[i + r + 1] >= min_dist)
            return min_cost + cb[i + r + 1];
        double *t = cost;
        cost = cost_prev;
        cost_prev = t;
    }
    return cost_prev[k - 1];
}

typedef struct {
    double *xbuf, *tl, *tu, *cost, *cost_prev, *cb, *cb1, *cb2;
} sdtw_work;

/* the UCR scan of one series (scaled_dtw_subsequence_distance and
 * scaled_dtw_matches share it): threshold < 0 gives the minimum (and its
 * first window in *index); otherwise every window with distance <= threshold
 * goes to distances[] / matches[] in order and the count is returned */
static idx_t sdtw_scan(const double *S, idx_t L, double sm, double ss, const double *sl,
                       const double *su, const double *T, idx_t n, idx_t r, sdtw_work *w,
                       double threshold, double *min_out, idx_t *index, double *distances,
                       idx_t *matches)
{
    double ex = 0, ex2 = 0, min_dist = INF;
    int find_min = threshold < 0;
    double thr = find_min ? 0 : threshold * threshold;
    idx_t n_matches = 0;
    for (idx_t i = 0; i < n; i++) {
        double cv = T[i];
        ex += cv;
        ex2 += cv * cv;
        idx_t pos = i % L;
        w->xbuf[pos] = cv;
        w->xbuf[pos + L] = cv;
        if (i >= L - 1) {
            idx_t j = (i + 1) % L;
            idx_t I = i - (L - 1);
            double mean = ex / L;
            double tmp = ex2 / L - mean * mean;
            double std = tmp > 0 ? sqrt(tmp) : 1.0;
            double bound = find_min ? min_dist : thr;
            double lb_kim = sdtw_kim(S, sm, ss, w->xbuf + j, mean, std, L, bound);
            if (lb_kim < bound) {
                double lb_k = sdtw_keogh(w->xbuf + j, L, mean, std, sm, ss, sl, su, w->cb1, bound);
                if (lb_k < bound) {
                    double lb_k2 = sdtw_keogh(S, L, sm, ss, mean, std, w->tl + I, w->tu + I,
                                              w->cb2, bound);
                    if (lb_k2 < bound) {
                        const double *src = lb_k > lb_k2 ? w->cb1 : w->cb2;
                        w->cb[L - 1] = src[L - 1];
                        for (idx_t k = L - 2; k >= 0; k--) w->cb[k] = w->cb[k + 1] + src[k];
                        double dist = sdtw_inner(S, L, sm, ss, w->xbuf + j, mean, std, r, w->cb,
                                                 w->cost, w->cost_prev, bound);
                        if (find_min) {
                            if (dist < min_dist) {
                                if (index) *index = (i + 1) - L;
                                min_dist = dist;
                            }
                        } else if (dist <= thr) {
                            if (matches) matches[n_matches] = (i + 1) - L;
                            distances[n_matches] = sqrt(dist);
                            n_matches++;
                        }
                    }
                }
            }
            cv = w->xbuf[j];
            ex -= cv;
            ex2 -= cv * cv;
        }
    }
    if (min_out) *min_out = sqrt(min_dist);
    return n_matches;
}

static idx_t sdtw_warp(idx_t length, double r)
{
    /* _compute_warp_width (_elastic.pyx:1917-1921) */
    if (r == 1) return length - 1;
    return (idx_t)floor(length * r);
}

/* pairwise (paired = 0: every shapelet against every x[i, dim]) or paired
 * (shapelet i against x[i, dim]) scaled_dtw subsequence scans.  threshold < 0:
 * minimum distance and first argmin window into out_dist / out_idx
 * ((xn, m) or (m,)); threshold >= 0 (paired only): the matched windows'
 * distances at out_dist[i * ld + window] with out_keep = 1.  smean / sstd as
 * ScaledSubsequenceMetric.from_array gives them (std <= EPSILON -> 0); a zero
 * std is taken as 1 unless std_as_given (the transient statistics of the
 * distance profile are used as they are). */
int wbo_scaled_dtw_subsequence(const double *shp, const idx_t *off, const idx_t *len,
                               const double *smean, const double *sstd, idx_t m,
                               const double *X, idx_t xn, idx_t xd, idx_t xL, idx_t dim,
                               double r, int paired, double threshold, int std_as_given,
                               double *out_dist, idx_t *out_idx, double *out_keep, idx_t ld)
{
    idx_t cap = 2 * sdtw_warp(xL, r) + 2;
    sdq du = {0}, dl = {0};
    du.cap = dl.cap = cap;
    du.q = (idx_t *)malloc(sizeof(idx_t) * cap);
    dl.q = (idx_t *)malloc(sizeof(idx_t) * cap);
    idx_t maxL = 0;
    for (idx_t s = 0; s < m; s++) maxL = imax(maxL, len[s]);
    sdtw_work w;
    w.xbuf = (double *)malloc(sizeof(double) * 2 * xL);
    w.tl = (double *)malloc(sizeof(double) * xL);
    w.tu = (double *)malloc(sizeof(double) * xL);
    w.cost = (double *)malloc(sizeof(double) * (2 * xL + 1));
    w.cost_prev = (double *)malloc(sizeof(double) * (2 * xL + 1));
    w.cb = (double *)malloc(sizeof(double) * xL);
    w.cb1 = (double *)malloc(sizeof(double) * xL);
    w.cb2 = (double *)malloc(sizeof(double) * xL);
    double *sl = (double *)malloc(sizeof(double) * (maxL > 0 ? maxL : 1));
    double *su = (double *)malloc(sizeof(double) * (maxL > 0 ? maxL : 1));
    double *dbuf = (double *)malloc(sizeof(double) * xL);
    idx_t *ibuf = (idx_t *)malloc(sizeof(idx_t) * xL);
    idx_t npairs = paired ? m : xn * m;
    for (idx_t p = 0; p < npairs; p++) {
        idx_t si = paired ? p : p / m, sh = paired ? p : p % m;
        const double *S = shp + off[sh];
        idx_t L = len[sh];
        idx_t wr = sdtw_warp(L, r);
        double sm = smean[sh];
        double ss = (sstd[sh] != 0 || std_as_given) ? sstd[sh] : 1.0;
        sdtw_envelope(S, L, wr, sl, su, &dl, &du);
        const double *T = X + (si * xd + dim) * xL;
        sdtw_envelope(T, xL, wr, w.tl, w.tu, &dl, &du);
        if (threshold < 0) {
            double d;
            idx_t idx = 0;
            sdtw_scan(S, L, sm, ss, sl, su, T, xL, wr, &w, -1.0, &d, &idx, NULL, NULL);
            out_dist[p] = d;
            out_idx[p] = idx;
        } else {
            idx_t cnt = sdtw_scan(S, L, sm, ss, sl, su, T, xL, wr, &w, threshold, NULL, NULL,
                                  dbuf, ibuf);
            for (idx_t k = 0; k < cnt; k++) {
                out_dist[p * ld + ibuf[k]] = dbuf[k];
                out_keep[p * ld + ibuf[k]] = 1.0;
            }
        }
    }
    free(du.q); free(dl.q);
    free(w.xbuf); free(w.tl); free(w.tu); free(w.cost); free(w.cost_prev);
    free(w.cb); free(w.cb1); free(w.cb2); free(sl); free(su); free(dbuf); free(ibuf);
    return 0;
}

/* ------------------------------------------------------------------------
 * lower bounds of distance/lb.py */

/* _dtw_envelop (distance/_elastic.pyx:1076-1092): deques of capacity 2r + 2 */
int wbo_dtw_envelope(const double *x, idx_t n, idx_t L, idx_t r, double *lower, double *upper)
{
    if (!(0 <= r && r < L)) return -1;
    sdq du = {0}, dl = {0};
    du.cap = dl.cap = 2 * r + 2;
    du.q = (idx_t *)malloc(sizeof(idx_t) * du.cap);
    dl.q = (idx_t *)malloc(sizeof(idx_t) * dl.cap);
    for (idx_t i = 0; i < n; i++)
        sdtw_envelope(x + i * L, L, r, lower + i * L, upper + i * L, &dl, &du);
    free(du.q);
    free(dl.q);
    return 0;
}

/* DtwKeoghLowerBound.transform (distance/lb.py:390-432): kind 0 both,
 * 1 left (query vs fitted envelope), 2 right (fitted vs query envelope);
 * each side sqrt(cumulative_bound at mean 0, std 1) (_dtw_lb_keogh,
 * _elastic.pyx:1095-1115); out (nq, nx) = max(left, right) */
int wbo_lb_keogh(const double *q, idx_t nq, const double *x, idx_t nx, idx_t L, idx_t r,
                 int kind, double *out)
{
    double *xl = (double *)malloc(sizeof(double) * nx * L);
    double *xu = (double *)malloc(sizeof(double) * nx * L);
    double *ql = (double *)malloc(sizeof(double) * L);
    double *qu = (double *)malloc(sizeof(double) * L);
    double *cb = (double *)malloc(sizeof(double) * L);
    if (wbo_dtw_envelope(x, nx, L, r, xl, xu) != 0) return -1;
    for (idx_t i = 0; i < nq; i++) {
        const double *qi = q + i * L;
        if (kind != 1) wbo_dtw_envelope(qi, 1, L, r, ql, qu);
        for (idx_t j = 0; j < nx; j++) {
            double d1 = -INF, d2 = -INF;
            if (kind != 2)
                d1 = sqrt(sdtw_keogh(qi, L, 0, 1, 0, 1, xl + j * L, xu + j * L, cb, INF));
            if (kind != 1)
                d2 = sqrt(sdtw_keogh(x + j * L, L, 0, 1, 0, 1, ql, qu, cb, INF));
            out[i * nx + j] = d2 > d1 ? d2 : d1;
        }
    }
    free(xl); free(xu); free(ql); free(qu); free(cb);
    return 0;
}
