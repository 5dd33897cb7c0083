// scaled_dtw.cu -- the scaled_dtw subsequence metric (ScaledDtwSubsequenceMetric,
// distance/_elastic.pyx:1928-2204) with the UCR-suite scan of
// scaled_dtw_subsequence_distance / scaled_dtw_matches (:159-620), FP64.
//
// The reference scans the windows of a series in order.  For window I it
// takes the running mean / std of the stream (sums ex, ex2 updated by adding
// the newest and subtracting the oldest value; std 1 when the variance is
// not positive), and skips the window when LB_Kim (first / last three
// points), then LB_Keogh of the window against the shapelet's envelope, then
// LB_Keogh of the shapelet against the window's slice of the series
// envelope reaches the best distance so far; otherwise it runs a
// Sakoe-Chiba-banded dtw on the z-normalised values that gives up as soon
// as a row minimum plus the cumulative bound of the remaining rows reaches
// the best.  Each test is "value >= best" on a sum of non-negative terms, so
// the reference's decision for a window equals comparing the window's full
// values with the best at that point:
//   key(I) = max(LB_Kim, LB_Keogh, LB_Keogh2, max over rows of
//                (row minimum + cumulative bound)),   raw(I) = the dtw,
// window I is evaluated iff key(I) < best, and then replaces the best iff
// raw(I) < best.  Here one warp takes one (shapelet, series) pair, its lanes
// compute (key, raw) of 32 consecutive windows -- each lane stops early once
// a value reaches the best at the start of the 32 (the best only decreases,
// so such a window fails the exact test too) -- and the 32 decisions are
// replayed in window order.  For thresholds (subsequence_match, the distance
// profile) the same (key, raw) pair decides: a window matches threshold t
// iff key < t^2 and raw <= t^2.
//
// Prepasses: the envelopes (find_min_max, :98-151, restated with the same
// ring deques -- including its single front pop per step -- so the
// envelopes carry the reference's values) of every shapelet and, per
// shapelet length, of every series; the running window statistics per
// (series, length); the z-normalised shapelet and shapelet envelope.

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "elastic.cuh"
#include "envelope.cuh"

namespace wb {

namespace {

constexpr int kSdThreads = 128;

// persistent grid: 8 blocks per SM, lane scratch bounded to about 512 MiB
inline int64_t sdtw_grid(int slots, int sm_count) {
    const int64_t per_block = (int64_t)slots * kSdThreads * 8;
    return std::max<int64_t>(
        1, std::min<int64_t>((int64_t)8 * sm_count, (512LL << 20) / per_block));
}

// length groups whose prep arrays (envelope, window statistics, deques)
// stay resident together: about 2 GiB
inline int64_t sdtw_chunk_groups(int64_t n_series, int n, int cap, int64_t n_groups) {
    const int64_t per_group = n_series * ((int64_t)n * 4 * 8 + (int64_t)cap * 2 * 4);
    const int64_t fit = std::max<int64_t>(1, (2LL << 30) / std::max<int64_t>(per_group, 1));
    return std::min(fit, n_groups);
}

// _compute_warp_width (distance/_elastic.pyx:1917-1921)
inline int sdtw_warp(int64_t length, double r) {
    if (r == 1.0) return (int)(length - 1);
    return (int)std::floor((double)length * r);
}

// Per shapelet: z-normalised values and envelope (the reference normalises
// them on the fly with the same two operations).  sstd: 0 is taken as 1
// unless std_as_given.
__global__ void sdtw_shapelet_prep_kernel(const double *shp, const int64_t *off,
                                          const int64_t *len, const double *mean,
                                          const double *sstd, int64_t m, double r,
                                          int std_as_given, int cap, int *dq, double *Sn,
                                          double *SnL, double *SnU, double *sstd_eff) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    const double *S = shp + off[s];
    const int L = (int)len[s];
    const int w = r == 1.0 ? L - 1 : (int)floor((double)L * r);
    const double sm = mean[s];
    const double ss = (sstd[s] != 0.0 || std_as_given) ? sstd[s] : 1.0;
    sstd_eff[s] = ss;
    DevDeque dl{dq + s * 2 * cap, cap, 0, 0, 0}, du{dq + s * 2 * cap + cap, cap, 0, 0, 0};
    double *lo = SnL + off[s], *up = SnU + off[s];
    sdtw_envelope(S, L, w, lo, up, dl, du);
    for (int k = 0; k < L; k++) {
        Sn[off[s] + k] = (S[k] - sm) / ss;
        up[k] = (up[k] - sm) / ss;
        lo[k] = (lo[k] - sm) / ss;
    }
}

// Per prep item (series, shapelet length L, warp w): the series envelope
// and the running window statistics of scaled_dtw_subsequence_distance
// (:380-398, 455-460).  Paired (pair_len set): item i is series i with the
// length of shapelet i; otherwise item i is series i % n_series with length
// group_len[i / n_series].
__global__ void sdtw_series_prep_kernel(SeriesSet X, const int64_t *pair_len,
                                        const int32_t *group_len, int64_t n_items, double r,
                                        int cap, int *dq, double *tl, double *tu, double *wmean,
                                        double *wstd) {
    const int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= n_items) return;
    const int n = X.len;
    const int64_t series = pair_len ? it : it % X.count;
    const double *T = X.base + series * X.stride;
    const int L = pair_len ? (int)pair_len[it] : group_len[it / X.count];
    const int w = r == 1.0 ? L - 1 : (int)floor((double)L * r);
    DevDeque dl{dq + it * 2 * cap, cap, 0, 0, 0}, du{dq + it * 2 * cap + cap, cap, 0, 0, 0};
    sdtw_envelope(T, n, w, tl + it * n, tu + it * n, dl, du);
    double ex = 0.0, ex2 = 0.0;
    double *mo = wmean + it * n, *so = wstd + it * n;
    for (int i = 0; i < n; i++) {
        const double v = T[i];
        ex = ex + v;
        ex2 = ex2 + v * v;
        if (i >= L - 1) {
            const int I = i - (L - 1);
            const double mu = ex / (double)L;
            const double tmp = ex2 / (double)L - mu * mu;
            mo[I] = mu;
            so[I] = tmp > 0.0 ? sqrt(tmp) : 1.0;
            const double o = T[I];
            ex = ex - o;
            ex2 = ex2 - o * o;
        }
    }
}

struct SdtwScanJob {
    SeriesSet x;
    const int64_t *off = nullptr;   // packed shapelet offsets (Sn, SnL, SnU)
    const int64_t *len = nullptr;
    const double *Sn = nullptr, *SnL = nullptr, *SnU = nullptr;
    const double *sstd_eff = nullptr;  // the shapelet std the scan uses (0 kept when given)
    double r = 1.0;
    // tasks: pairwise: shapelets task_shp[0 .. n_shp) x all series, prep item
    // task_group[k] * series count + series; paired: task t = (shapelet t,
    // series t), prep item t
    const int32_t *task_shp = nullptr;
    const int32_t *task_group = nullptr;
    int64_t n_shp = 0;
    int paired = 0;
    int64_t m = 0;  // shapelets in the output row
    const double *tl = nullptr, *tu = nullptr, *wmean = nullptr, *wstd = nullptr;
    double *out_dist = nullptr;
    int64_t *out_idx = nullptr;
    double *prof_raw = nullptr, *prof_key = nullptr;
    int64_t prof_ld = 0;
    int64_t scr_stride = 0;  // threads of the launch (scratch stride)
    int xn_off = 0, t1_off = 0, t2_off = 0, c0_off = 0, c1_off = 0;  // lane scratch slots
};

__device__ __forceinline__ double sq(double a) { return a * a; }
__device__ __forceinline__ double dmin2(double a, double b) { return b < a ? b : a; }

// LB_Kim of constant_lower_bound (:159-237), all six terms (the reference's
// early returns only stop at a partial sum that already fails).  For L < 3
// the reference reads outside the arrays; indices are clamped here.
__device__ double sdtw_kim(const double *Sn, const double *W, double tm, double ts, int L) {
    const int a1 = L > 1 ? 1 : L - 1, a2 = L > 2 ? 2 : L - 1;
    const int b1 = L - 2 >= 0 ? L - 2 : 0, b2 = L - 3 >= 0 ? L - 3 : 0;
    const double tx0 = (W[0] - tm) / ts, ty0 = (W[L - 1] - tm) / ts;
    const double sx0 = Sn[0], sy0 = Sn[L - 1];
    double md = sq(tx0 - sx0) + sq(ty0 - sy0);
    const double tx1 = (W[a1] - tm) / ts, sx1 = Sn[a1];
    md = md + dmin2(dmin2(sq(tx1 - sx0), sq(tx0 - sx1)), sq(tx1 - sx1));
    const double ty1 = (W[b1] - tm) / ts, sy1 = Sn[b1];
    md = md + dmin2(dmin2(sq(ty1 - sy1), sq(ty0 - sy1)), sq(ty1 - sy1));
    const double tx2 = (W[a2] - tm) / ts, sx2 = Sn[a2];
    md = md + dmin2(dmin2(dmin2(sq(tx0 - sx2), dmin2(sq(tx1 - sx2), sq(tx2 - sx2))),
                          sq(tx2 - sx1)),
                    sq(tx2 - sx0));
    const double ty2 = (W[b2] - tm) / ts, sy2 = Sn[b2];
    md = md + dmin2(dmin2(dmin2(sq(ty0 - sy2), dmin2(sq(ty1 - sy2), sq(ty2 - sy2))),
                          sq(ty2 - sy1)),
                    sq(ty2 - sy0));
    return md;
}

// one term of cumulative_bound (:240-270)
__device__ __forceinline__ double keogh_term(double x, double us, double ls) {
    if (x > us) return sq(x - us);
    if (x < ls) return sq(x - ls);
    return 0.0;
}

// Per-lane scratch, strided by the launch's thread count: the normalised
// window, the terms of the two LB_Keogh sums (the larger one's become the
// cumulative bound in place), two cost rows of the banded recurrence.
struct LaneScratch {
    double *xn, *t1, *t2, *c0, *c1;
    int64_t st;
};

struct SdtwPair {
    int L, w;
    const double *Sn, *SnL, *SnU;
    bool ss_zero;
    const double *T, *tl, *tu, *wm, *ws;
};

// Everything after LB_Kim for window I: LB_Keogh (window vs shapelet
// envelope), LB_Keogh (shapelet vs window envelope), the cumulative bound of
// the larger, the banded recurrence.  Each stage runs only while its value
// stays below `bound`; returns key (the largest value met) and raw (the dtw,
// +inf when a stage reached the bound).
__device__ void sdtw_eval(const SdtwPair &P, const LaneScratch &S, int I, double kim,
                          double bound, double &key, double &raw) {
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    const int L = P.L, w = P.w;
    const int64_t st = S.st;
    const double tm = P.wm[I], ts = P.ws[I];
    const double *W = P.T + I;
    key = kim;
    raw = INF;
    if (!(kim < bound)) return;
    double lbk = 0.0;
    for (int k = 0; k < L; k++) {
        const double x = (W[k] - tm) / ts;
        S.xn[(int64_t)k * st] = x;
        const double d = keogh_term(x, P.SnU[k], P.SnL[k]);
        S.t1[(int64_t)k * st] = d;
        lbk = lbk + d;
    }
    key = key > lbk ? key : lbk;
    if (!(lbk < bound)) return;
    double lbk2 = 0.0;
    for (int k = 0; k < L; k++) {
        const double d = keogh_term(P.Sn[k], (P.tu[I + k] - tm) / ts, (P.tl[I + k] - tm) / ts);
        S.t2[(int64_t)k * st] = d;
        lbk2 = lbk2 + d;
    }
    key = key > lbk2 ? key : lbk2;
    if (!(lbk2 < bound)) return;
    // cb[k] = cb[k + 1] + term[k] from the larger bound, in place
    double *cb = lbk > lbk2 ? S.t1 : S.t2;
    double acc = 0.0;
    for (int k = L - 1; k >= 0; k--) {
        const double d = cb[(int64_t)k * st];
        acc = k == L - 1 ? d : acc + d;
        cb[(int64_t)k * st] = acc;
    }
    // inner_scaled_dtw_subsequence_distance (:273-344)
    const int W2 = 2 * w + 1;
    double *c = S.c0, *pv = S.c1;
    for (int k = 0; k < W2; k++) {
        c[(int64_t)k * st] = INF;
        pv[(int64_t)k * st] = INF;
    }
    int kk = 0;
    double kmax = -INF;
    for (int i = 0; i < L; i++) {
        kk = w - i > 0 ? w - i : 0;
        double minc = INF;
        const int j0 = i - w > 0 ? i - w : 0;
        const int j1 = i + w + 1 < L ? i + w + 1 : L;
        double left = INF;
        double pk = (i >= 1) ? pv[(int64_t)kk * st] : INF;
        const double si_v = P.Sn[i];
        for (int j = j0; j < j1; j++) {
            double v;
            if (i == 0 && j == 0) {
                v = P.ss_zero ? 0.0 : P.Sn[0];
                v = v - S.xn[0];
                v = v * v;
            } else {
                const double y = (j - 1 < 0 || kk - 1 < 0) ? INF : left;
                const double pk1 =
                    (kk + 1 <= 2 * w && i >= 1) ? pv[(int64_t)(kk + 1) * st] : INF;
                const double x = (i - 1 < 0 || kk + 1 > 2 * w) ? INF : pk1;
                const double z = (i - 1 < 0 || j - 1 < 0) ? INF : pk;
                const double dv = si_v - S.xn[(int64_t)j * st];
                v = dmin2(dmin2(x, y), z) + dv * dv;
                pk = pk1;
            }
            c[(int64_t)kk * st] = v;
            left = v;
            if (v < minc) minc = v;
            kk += 1;
        }
        if (i + w < L - 1) {
            const double val = minc + cb[(int64_t)(i + w + 1) * st];
            kmax = kmax > val ? kmax : val;
            if (val >= bound) {
                key = key > kmax ? key : kmax;
                return;
            }
        }
        double *t = c;
        c = pv;
        pv = t;
    }
    key = key > kmax ? key : kmax;
    raw = pv[(int64_t)(kk - 1) * st];
}

constexpr int kSdQueue = 64;

template <bool PROFILE>
__global__ void __launch_bounds__(kSdThreads) sdtw_scan_kernel(const SdtwScanJob J,
                                                               double *scr) {
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    const double QNAN = __longlong_as_double(0x7ff8000000000000LL);
    __shared__ int q_win[kSdThreads / 32][kSdQueue];
    __shared__ double q_kim[kSdThreads / 32][kSdQueue];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t warp = gtid >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t st = J.scr_stride;
    LaneScratch S;
    S.st = st;
    S.xn = scr + gtid + (int64_t)J.xn_off * st;
    S.t1 = scr + gtid + (int64_t)J.t1_off * st;
    S.t2 = scr + gtid + (int64_t)J.t2_off * st;
    S.c0 = scr + gtid + (int64_t)J.c0_off * st;
    S.c1 = scr + gtid + (int64_t)J.c1_off * st;
    const int n = J.x.len;
    const int64_t ntask = J.paired ? J.m : J.n_shp * J.x.count;
    for (int64_t task = warp; task < ntask; task += nwarps) {
        int64_t sh, si, item, oidx;
        if (J.paired) {
            sh = si = item = oidx = task;
        } else {
            const int64_t k = task / J.x.count;
            sh = J.task_shp[k];
            si = task - k * J.x.count;
            item = (int64_t)J.task_group[k] * J.x.count + si;
            oidx = si * J.m + sh;
        }
        SdtwPair P;
        P.L = (int)J.len[sh];
        P.w = J.r == 1.0 ? P.L - 1 : (int)floor((double)P.L * J.r);
        P.Sn = J.Sn + J.off[sh];
        P.SnL = J.SnL + J.off[sh];
        P.SnU = J.SnU + J.off[sh];
        P.ss_zero = J.sstd_eff[sh] == 0.0;
        P.T = J.x.base + si * J.x.stride;
        P.tl = J.tl + item * n;
        P.tu = J.tu + item * n;
        P.wm = J.wmean + item * n;
        P.ws = J.wstd + item * n;
        const int nwin = n - P.L + 1;
        if (PROFILE) {
            for (int64_t I = nwin + lane; I < J.prof_ld; I += 32) {
                J.prof_raw[oidx * J.prof_ld + I] = QNAN;
                J.prof_key[oidx * J.prof_ld + I] = QNAN;
            }
            for (int base = 0; base < nwin; base += 32) {
                const int I = base + lane;
                if (I < nwin) {
                    double key, raw;
                    const double kim =
                        sdtw_kim(P.Sn, P.T + I, P.wm[I], P.ws[I], P.L);
                    sdtw_eval(P, S, I, kim, INF, key, raw);
                    J.prof_raw[oidx * J.prof_ld + I] = raw;
                    J.prof_key[oidx * J.prof_ld + I] = key;
                }
            }
            continue;
        }
        // Minimum: LB_Kim for 32 windows at a time at full width; windows
        // that pass it against the current best wait in a FIFO (ascending
        // window order) and go through the remaining stages 32 at a time, so
        // the expensive stages run on full warps; each batch is replayed in
        // window order against the running best.  A window dropped by LB_Kim
        // here is dropped by the reference too (the best only decreases).
        int *qw = q_win[wid];
        double *qk = q_kim[wid];
        int qh = 0, qn = 0;
        double best = INF;
        int bidx = 0;
        auto run_batch = [&](int cnt) {
            double key = INF, raw = INF;
            int I = 0x7fffffff;
            if (lane < cnt) {
                I = qw[(qh + lane) % kSdQueue];
                sdtw_eval(P, S, I, qk[(qh + lane) % kSdQueue], best, key, raw);
            }
            for (int t = 0; t < cnt; t++) {
                const double kt = __shfl_sync(0xffffffffu, key, t);
                const double rt = __shfl_sync(0xffffffffu, raw, t);
                const int it = __shfl_sync(0xffffffffu, I, t);
                if (kt < best && rt < best) {
                    best = rt;
                    bidx = it;
                }
            }
            qh = (qh + cnt) % kSdQueue;
            qn -= cnt;
            __syncwarp();
        };
        for (int base = 0; base < nwin; base += 32) {
            const int I = base + lane;
            bool pass = false;
            double kim = INF;
            if (I < nwin) {
                kim = sdtw_kim(P.Sn, P.T + I, P.wm[I], P.ws[I], P.L);
                pass = kim < best;
            }
            const unsigned mask = __ballot_sync(0xffffffffu, pass);
            if (pass) {
                const int slot = (qh + qn + __popc(mask & ((1u << lane) - 1u))) % kSdQueue;
                qw[slot] = I;
                qk[slot] = kim;
            }
            qn += __popc(mask);
            __syncwarp();
            if (qn >= 32) run_batch(32);
        }
        if (qn > 0) run_batch(qn);
        if (lane == 0) {
            J.out_dist[oidx] = sqrt(best);
            J.out_idx[oidx] = bidx;
        }
        __syncwarp();
    }
}

}  // namespace

// Host driver; shapelet arrays (shp, off, len, means, stds) are device
// pointers here, X is staged.
int subseq_scaled_dtw(const double *shp, const int64_t *off, const int64_t *len,
                      const double *means, const double *stds, int64_t m,
                      const std::vector<int64_t> &hlen, int64_t total, const SeriesSet &X,
                      int64_t n_timestep, double r,
                      bool paired, int std_as_given, double *out_dist, int64_t *out_idx,
                      double *prof_raw, double *prof_key, int64_t prof_ld, Workspace &ws,
                      cudaStream_t s) {
    if (!(r >= 0.0 && r <= 1.0)) return fail(WB_EINVAL, "r must be in [0, 1]");
    const int n = X.len;
    const int cap = 2 * sdtw_warp(n_timestep, r) + 2;
    const bool profile = prof_raw != nullptr;
    int max_len = 1, max_w = 0;
    for (int64_t i = 0; i < m; i++) {
        max_len = std::max<int>(max_len, (int)hlen[i]);
        max_w = std::max(max_w, sdtw_warp(hlen[i], r));
    }
    // shapelet prep
    WB_TAKE(Sn, double, ws, total);
    WB_TAKE(SnL, double, ws, total);
    WB_TAKE(SnU, double, ws, total);
    WB_TAKE(sstd_eff, double, ws, m);
    WB_TAKE(dq_s, int, ws, (size_t)m * 2 * cap);
    sdtw_shapelet_prep_kernel<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(
        shp, off, len, means, stds, m, r, std_as_given, cap, dq_s, Sn, SnL, SnU, sstd_eff);
    WB_LAUNCH_CHECK("sdtw_shapelet_prep_kernel");
    // per-lane scratch: xn, t1, t2 [max_len], two cost rows [2 w + 1]
    const int slots = 3 * max_len + 2 * (2 * max_w + 1);
    const DeviceInfo &dev = device_info();
    SdtwScanJob J;
    J.x = X;
    J.off = off;
    J.len = len;
    J.Sn = Sn;
    J.SnL = SnL;
    J.SnU = SnU;
    J.sstd_eff = sstd_eff;
    J.r = r;
    J.paired = paired ? 1 : 0;
    J.m = m;
    J.xn_off = 0;
    J.t1_off = max_len;
    J.t2_off = 2 * max_len;
    J.c0_off = 3 * max_len;
    J.c1_off = 3 * max_len + 2 * max_w + 1;
    J.prof_raw = prof_raw;
    J.prof_key = prof_key;
    J.prof_ld = prof_ld;
    J.out_dist = out_dist;
    J.out_idx = out_idx;

    // Length groups (descending, so long shapelets start first); the prep
    // arrays of a chunk of groups are resident together so one scan launch
    // covers every shapelet of the chunk against every series.
    std::vector<int64_t> order(m);
    for (int64_t i = 0; i < m; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t b) { return hlen[a] > hlen[b]; });
    std::vector<int32_t> glen;
    std::vector<int64_t> gfirst;
    for (int64_t t = 0; t < m; t++) {
        if (glen.empty() || glen.back() != (int32_t)hlen[order[t]]) {
            glen.push_back((int32_t)hlen[order[t]]);
            gfirst.push_back(t);
        }
    }
    gfirst.push_back(m);
    const int64_t n_groups = (int64_t)glen.size();
    const int64_t chunk_groups = paired ? 1 : sdtw_chunk_groups(X.count, n, cap, n_groups);
    const int64_t items = paired ? m : chunk_groups * X.count;
    WB_TAKE(dq, int, ws, (size_t)items * 2 * cap);
    WB_TAKE(tl, double, ws, (size_t)items * n);
    WB_TAKE(tu, double, ws, (size_t)items * n);
    WB_TAKE(wm, double, ws, (size_t)items * n);
    WB_TAKE(wsd, double, ws, (size_t)items * n);
    const int64_t grid = sdtw_grid(slots, dev.sm_count);
    WB_TAKE(scr, double, ws, (size_t)grid * kSdThreads * slots);
    J.tl = tl;
    J.tu = tu;
    J.wmean = wm;
    J.wstd = wsd;
    J.scr_stride = grid * kSdThreads;

    auto launch_scan = [&](int64_t n_items, const int32_t *group_len, int64_t warps) -> int {
        sdtw_series_prep_kernel<<<(unsigned)((n_items + 63) / 64), 64, 0, s>>>(
            X, paired ? len : nullptr, group_len, n_items, r, cap, dq, tl, tu, wm, wsd);
        WB_LAUNCH_CHECK("sdtw_series_prep_kernel");
        const int64_t g = std::max<int64_t>(
            1, std::min<int64_t>(grid, (warps * 32 + kSdThreads - 1) / kSdThreads));
        timer_begin("sdtw_scan_kernel", s);
        if (profile)
            sdtw_scan_kernel<true><<<(unsigned)g, kSdThreads, 0, s>>>(J, scr);
        else
            sdtw_scan_kernel<false><<<(unsigned)g, kSdThreads, 0, s>>>(J, scr);
        timer_end(s);
        WB_LAUNCH_CHECK("sdtw_scan_kernel");
        return WB_OK;
    };

    if (paired) return launch_scan(m, nullptr, m);
    // per shapelet (in length order): its index and its group within the chunk
    std::vector<int32_t> tshp(m), tgrp(m);
    WB_TAKE(d_tshp, int32_t, ws, m);
    WB_TAKE(d_tgrp, int32_t, ws, m);
    WB_TAKE(d_glen, int32_t, ws, n_groups);
    for (int64_t g0 = 0; g0 < n_groups; g0 += chunk_groups) {
        const int64_t g1 = std::min(n_groups, g0 + chunk_groups);
        for (int64_t g = g0; g < g1; g++)
            for (int64_t t = gfirst[g]; t < gfirst[g + 1]; t++) {
                tshp[t] = (int32_t)order[t];
                tgrp[t] = (int32_t)(g - g0);
            }
    }
    WB_CUDA(cudaMemcpyAsync(d_tshp, tshp.data(), m * 4, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(d_tgrp, tgrp.data(), m * 4, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(d_glen, glen.data(), n_groups * 4, cudaMemcpyHostToDevice, s));
    for (int64_t g0 = 0; g0 < n_groups; g0 += chunk_groups) {
        const int64_t g1 = std::min(n_groups, g0 + chunk_groups);
        J.task_shp = d_tshp + gfirst[g0];
        J.task_group = d_tgrp + gfirst[g0];
        J.n_shp = gfirst[g1] - gfirst[g0];
        WB_TRY(launch_scan((g1 - g0) * X.count, d_glen + g0, J.n_shp * X.count));
    }
    // the host arrays above feed asynchronous copies
    WB_CUDA(cudaStreamSynchronize(s));
    return WB_OK;
}

size_t subseq_scaled_dtw_bytes(int64_t m, int64_t total, int64_t n_series, int n,
                               const std::vector<int64_t> &hlen, double r, int64_t n_timestep,
                               bool paired) {
    int max_len = 1, max_w = 0;
    std::vector<int64_t> ls(hlen.begin(), hlen.end());
    std::sort(ls.begin(), ls.end());
    const int64_t n_groups = (int64_t)(std::unique(ls.begin(), ls.end()) - ls.begin());
    for (int64_t i = 0; i < m; i++) {
        max_len = std::max<int>(max_len, (int)hlen[i]);
        max_w = std::max(max_w, sdtw_warp(hlen[i], r));
    }
    const int cap = 2 * sdtw_warp(n_timestep, r) + 2;
    const int slots = 3 * max_len + 2 * (2 * max_w + 1);
    const int64_t items =
        paired ? m : sdtw_chunk_groups(n_series, n, cap, n_groups) * n_series;
    const int64_t grid = sdtw_grid(slots, device_info().sm_count);
    return 3 * align256(total * 8) + align256(m * 8) + align256((size_t)m * 2 * cap * 4) +
           align256((size_t)items * 2 * cap * 4) + 4 * align256((size_t)items * n * 8) +
           align256((size_t)grid * kSdThreads * slots * 8) + 2 * align256(m * 4) +
           align256(n_groups * 4) + 4096;
}

}  // namespace wb
