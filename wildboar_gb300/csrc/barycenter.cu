// barycenter.cu -- the majorize-minimize DTW barycenter (dtw_average with
// method="mm") and the group means of KMeans, FP64, bit-exact.
//
// One MM epoch of the reference (distance/dtw.py:661-690) aligns the current
// mean with every sample (dtw_alignment, distance/_elastic.pyx:1011-1073),
// walks the optimal path back (dtw_mapping, distance/dtw.py:362-426: from the
// last cell, argmin of [diag, up, left] with the first minimum winning) and
// then, for every mean element m, sums V[m] += w and z[m] += X[i, x] * w over
// the path cells (m, x) of every sample i in sample order and, within a
// sample, in ascending x; the new mean is z / V.
//
// Here:
//  * mm_align_kernel: one warp per (mean, sample) pair runs the banded
//    alignment recurrence as a wavefront: lane l owns S consecutive rows
//    (mean elements) and handles column j = t - l at step t, receiving the
//    row above its strip from lane l - 1 by shuffle (rows beyond 32 S go in
//    passes through a boundary row in global memory).  Each cell keeps, in
//    2 bits, the move the traceback would take from it -- the same three
//    values the recurrence reads (up, left, diag), so no matrix is stored --
//    and the warp then walks the path back and records, per row, the first
//    and last column of the path in that row (a DTW path visits a contiguous
//    run of columns in each row).  The final cell is also returned: for dtw
//    with equal lengths it is the squared dtw distance of the pair.
//  * mm_accumulate_kernel: one thread per (group, mean element) adds the
//    path cells of the group's samples in the reference's order (sample
//    order, ascending x), so z and V carry the reference's rounding, and
//    writes z / V.  Without paths (KMeans with the euclidean metric) it is
//    group.mean(axis=0): a sequential sum over the group's rows divided by
//    the count, numpy's order for an axis-0 mean of a C-contiguous array.

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "common.cuh"

namespace wb {

namespace {

constexpr int kMmThreads = 128;
constexpr int kMmWarps = kMmThreads / 32;

template <int S>
struct DirWord;
template <>
struct DirWord<4> { using T = uint8_t; };
template <>
struct DirWord<8> { using T = uint16_t; };
template <>
struct DirWord<16> { using T = uint32_t; };

struct MmAlignJob {
    const double *x = nullptr;      // samples, row s at x + s * x_stride
    int64_t x_stride = 0;
    int m = 0;                      // sample length (columns)
    const double *means = nullptr;  // group means, row g at means + g * n
    int n = 0;                      // mean length (rows)
    const int64_t *member = nullptr;     // pair q aligns sample member[q]
    const int32_t *pair_group = nullptr; // with mean pair_group[q]
    int64_t q0 = 0, q1 = 0;         // pairs of this launch
    int r = 1;                      // warp size max(floor(max(n, m) r), 1)
    const double *weights = nullptr;  // weights[|i - j|] or nullptr
    void *dir = nullptr;            // per pair: (ceil(n / S), m) or (n + m - 1, 32) words
    int64_t dir_pair_words = 0;
    double *bnd = nullptr;          // per warp slot: boundary row (m doubles)
    int32_t *path_lo = nullptr;     // (n_pairs, n)
    int32_t *path_hi = nullptr;
    double *last = nullptr;         // (n_pairs,) final cell, or nullptr
    double *full = nullptr;         // (n, m) cost matrix of pair q0 (dtw_alignment), or nullptr
};

__device__ __forceinline__ long long dbits(double v) { return __double_as_longlong(v); }

// move codes of the traceback: 0 diag, 1 up, 2 left (np.argmin's first minimum
// over [diag, up, left]); values are non-negative or +inf, so integer order
// of the bit patterns is their order
__device__ __forceinline__ uint32_t move_code(long long diag, long long up, long long left) {
    if (diag <= up && diag <= left) return 0u;
    return up <= left ? 1u : 2u;
}

template <int S, bool W>
__global__ void __launch_bounds__(kMmThreads) mm_align_kernel(const MmAlignJob J) {
    using Word = typename DirWord<S>::T;
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    const int lane = threadIdx.x & 31;
    const int slot = blockIdx.x * kMmWarps + (threadIdx.x >> 5);
    const int n = J.n, m = J.m;
    const int mx = imax(0, m - n) + J.r;   // columns j < i + mx
    const int mn = imax(0, n - m);         // columns j >= i - mn - r + 1
    double *bnd = J.bnd ? J.bnd + (int64_t)slot * m : nullptr;
    for (int64_t q = J.q0 + slot; q < J.q1; q += (int64_t)gridDim.x * kMmWarps) {
        const double *Y = J.x + J.member[q] * J.x_stride;
        const double *X = J.means + (int64_t)J.pair_group[q] * n;
        Word *dir = reinterpret_cast<Word *>(J.dir) + (q - J.q0) * J.dir_pair_words;
        double fin = INF;
        for (int p0 = 0; p0 < n; p0 += 32 * S) {
            const int i0 = p0 + lane * S;
            double a[S], left[S];
#pragma unroll
            for (int k = 0; k < S; k++) {
                a[k] = i0 + k < n ? X[i0 + k] : 0.0;
                left[k] = INF;
            }
            double send = INF;       // this lane's last row at its last column
            double prev_up0 = INF;   // row above the strip at the previous column
            for (int t = 0; t < m + 31; t++) {
                const double recv = __shfl_up_sync(0xffffffffu, send, 1);
                const int j = t - lane;
                if (j >= 0 && j < m) {
                    double up0;
                    if (lane == 0)
                        up0 = p0 == 0 ? INF : bnd[j];
                    else
                        up0 = recv;
                    const double y = Y[j];
                    double up = up0, diag = prev_up0;
                    uint32_t word = 0;
#pragma unroll
                    for (int k = 0; k < S; k++) {
                        const int i = i0 + k;
                        const double lf = left[k];
                        double v = INF;
                        if (i < n && j >= i - mn - J.r + 1 && j < i + mx) {
                            const double d = a[k] - y;
                            double c = d * d;
                            if (W) c = c * J.weights[i > j ? i - j : j - i];
                            if (i == 0 && j == 0) {
                                v = c;
                            } else {
                                const long long bu = dbits(up), bl = dbits(lf), bd = dbits(diag);
                                const long long mu = bl < bu ? bl : bu;
                                v = __longlong_as_double(bd < mu ? bd : mu) + c;
                                word |= move_code(bd, bu, bl) << (2 * k);
                            }
                        }
                        if (i == n - 1 && j == m - 1) fin = v;
                        if (J.full && q == J.q0 && i < n && j >= i - mn - J.r + 1 && j < i + mx)
                            J.full[(int64_t)i * m + j] = v;
                        diag = lf;
                        left[k] = v;
                        up = v;
                    }
                    if (i0 < n) dir[(int64_t)(i0 / S) * m + j] = (Word)word;
                    send = up;
                    prev_up0 = up0;
                    if (lane == 31 && bnd) bnd[j] = up;
                }
            }
            __syncwarp();
        }
        // the lane that owns row n - 1 saw the final cell
        const int owner = ((n - 1) % (32 * S)) / S;
        fin = __shfl_sync(0xffffffffu, fin, owner);
        if (lane == 0 && J.last) J.last[q] = fin;
        // The whole warp walks the path back in lockstep (i, j are
        // warp-uniform): a window of 32 consecutive direction words of one
        // strip (columns base .. base + 31) sits one per lane and the word
        // of column j comes by shuffle, so a global load is paid once per
        // window instead of once per step.  The path only moves up and left:
        // a window is reloaded when the path leaves its strip or its columns.
        int32_t *lo = J.path_lo + q * (int64_t)n;
        int32_t *hi = J.path_hi + q * (int64_t)n;
        int i = n - 1, j = m - 1;
        int strip = -1, base = 0;
        uint32_t wreg = 0;
        if (lane == 0) hi[i] = j;
        while (i > 0 || j > 0) {
            uint32_t code;
            if (i == 0) {
                code = 2u;
            } else if (j == 0) {
                code = 1u;
            } else {
                if (i / S != strip || j < base) {
                    strip = i / S;
                    base = j >= 31 ? j - 31 : 0;
                    const int col = base + lane;
                    wreg = col < m ? (uint32_t)dir[(int64_t)strip * m + col] : 0u;
                }
                const uint32_t w = __shfl_sync(0xffffffffu, wreg, j - base);
                code = (w >> (2 * (i % S))) & 3u;
            }
            if (code == 2u) {
                j -= 1;
            } else {
                if (lane == 0) lo[i] = j;
                i -= 1;
                if (code == 0u) j -= 1;
                if (lane == 0) hi[i] = j;
            }
        }
        if (lane == 0) lo[0] = 0;
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Anti-diagonal form for narrow bands.  In the row-strip wavefront above a
// lane's rows meet their band for only (band width + S) of the m + 31 steps,
// and an FP64 warp instruction costs the FP64 pipe the same whatever its
// active lanes, so a narrow band pays for the whole matrix.  Here the warp
// walks the anti-diagonals d = i + j: the in-band cells of diagonal d are
// rows ilo(d) .. ihi(d), and slot s = i - ilo(d) goes to lane s % 32,
// register s / 32 (K registers).  A cell reads up (i - 1, j) and left
// (i, j - 1) from diagonal d - 1 and diag (i - 1, j - 1) from d - 2; since
// ilo grows by 0 or 1 per diagonal those are the previous diagonals' slots
// shifted by -1, 0 or +1: one warp shuffle each.  Register slots past the
// diagonal's cells are skipped by a warp-uniform test, so FP64 instructions
// run only for in-band cells (up to 31 idle lanes per diagonal).  The move
// codes go to one word per (diagonal, lane) (2 bits per register slot); the
// traceback reads them through a shared-memory window of 16 diagonals.

template <int K>
struct AdWord { using T = uint32_t; };
template <>
struct AdWord<1> { using T = uint8_t; };
template <>
struct AdWord<2> { using T = uint8_t; };
template <>
struct AdWord<4> { using T = uint8_t; };
template <>
struct AdWord<8> { using T = uint16_t; };

__host__ __device__ __forceinline__ int floordiv2(int a) { return a >= 0 ? a / 2 : -((1 - a) / 2); }

// in-band rows of anti-diagonal d (band rows i: columns
// [max(0, i - mn - r + 1), min(m, i + mx)))
__host__ __device__ __forceinline__ void ad_bounds(int d, int n, int m, int r, int mx, int mn,
                                                   int &ilo, int &ihi) {
    int lo = d - m + 1 > 0 ? d - m + 1 : 0;
    const int l2 = floordiv2(d - mx) + 1;
    lo = l2 > lo ? l2 : lo;
    int hi = n - 1 < d ? n - 1 : d;
    const int h2 = floordiv2(d + mn + r - 1);
    hi = h2 < hi ? h2 : hi;
    ilo = lo;
    ihi = hi;
}

// slot (lane + 32 k) + SH of the K-slot array P (SH in {-1, 0, +1}); slots
// outside [0, 32 K) read +inf
template <int K, int SH>
__device__ __forceinline__ void ad_shift(const double (&P)[K], double (&out)[K], int lane) {
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    if constexpr (SH == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) out[k] = P[k];
    } else {
        double t[K];
#pragma unroll
        for (int k = 0; k < K; k++) t[k] = __shfl_sync(0xffffffffu, P[k], (lane + SH) & 31);
#pragma unroll
        for (int k = 0; k < K; k++) {
            if (SH < 0)
                out[k] = lane == 0 ? (k == 0 ? INF : t[k == 0 ? 0 : k - 1]) : t[k];
            else
                out[k] = lane == 31 ? (k == K - 1 ? INF : t[k == K - 1 ? 0 : k + 1]) : t[k];
        }
    }
}

constexpr int kAdWindow = 16;

template <int K, bool W>
__global__ void __launch_bounds__(kMmThreads) mm_align_ad_kernel(const MmAlignJob J) {
    using Word = typename AdWord<K>::T;
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    __shared__ uint32_t win_all[kMmWarps][kAdWindow * 32];
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    const int slot = blockIdx.x * kMmWarps + wid;
    uint32_t *win = win_all[wid];
    const int n = J.n, m = J.m, r = J.r;
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const int D = n + m - 1;
    for (int64_t q = J.q0 + slot; q < J.q1; q += (int64_t)gridDim.x * kMmWarps) {
        const double *Y = J.x + J.member[q] * J.x_stride;
        const double *X = J.means + (int64_t)J.pair_group[q] * n;
        Word *dir = reinterpret_cast<Word *>(J.dir) + (q - J.q0) * J.dir_pair_words;
        double P1[K], P2[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            P1[k] = INF;
            P2[k] = INF;
        }
        int lo1 = 0, lo2 = 0;
        double fin = INF;
        for (int d = 0; d < D; d++) {
            int ilo, ihi;
            ad_bounds(d, n, m, r, mx, mn, ilo, ihi);
            const int cnt = ihi - ilo + 1;
            const int d1 = ilo - lo1, d2 = ilo - lo2;
            double up[K], left[K], diag[K];
            if (d1 == 0) {
                ad_shift<K, -1>(P1, up, lane);
                ad_shift<K, 0>(P1, left, lane);
            } else {
                ad_shift<K, 0>(P1, up, lane);
                ad_shift<K, 1>(P1, left, lane);
            }
            if (d2 == 0)
                ad_shift<K, -1>(P2, diag, lane);
            else if (d2 == 1)
                ad_shift<K, 0>(P2, diag, lane);
            else
                ad_shift<K, 1>(P2, diag, lane);
            uint32_t word = 0;
#pragma unroll
            for (int k = 0; k < K; k++) {
                double v = INF;
                if (32 * k < cnt) {
                    const int s = lane + 32 * k;
                    if (s < cnt) {
                        const int i = ilo + s, j = d - i;
                        const double dd = __ldg(X + i) - __ldg(Y + j);
                        double c = dd * dd;
                        if (W) c = c * __ldg(J.weights + (i > j ? i - j : j - i));
                        if (d == 0) {
                            v = c;
                        } else {
                            const long long bu = dbits(up[k]), bl = dbits(left[k]),
                                            bd = dbits(diag[k]);
                            const long long mu = bl < bu ? bl : bu;
                            v = __longlong_as_double(bd < mu ? bd : mu) + c;
                            word |= move_code(bd, bu, bl) << (2 * k);
                        }
                        if (d == D - 1) fin = v;
                        if (J.full && q == J.q0) J.full[(int64_t)i * m + j] = v;
                    }
                }
                P2[k] = P1[k];
                P1[k] = v;
            }
            dir[(int64_t)d * 32 + lane] = (Word)word;
            lo2 = lo1;
            lo1 = ilo;
        }
        // the last diagonal has one cell, in slot 0
        fin = __shfl_sync(0xffffffffu, fin, 0);
        if (lane == 0 && J.last) J.last[q] = fin;
        __syncwarp();
        int32_t *lo = J.path_lo + q * (int64_t)n;
        int32_t *hi = J.path_hi + q * (int64_t)n;
        int i = n - 1, j = m - 1;
        int wtop = -1;  // the window holds diagonals wtop - 15 .. wtop
        if (lane == 0) hi[i] = j;
        while (i > 0 || j > 0) {
            uint32_t code;
            if (i == 0) {
                code = 2u;
            } else if (j == 0) {
                code = 1u;
            } else {
                const int d = i + j;
                if (d > wtop || d <= wtop - kAdWindow) {
                    __syncwarp();
                    wtop = d;
#pragma unroll
                    for (int t = 0; t < kAdWindow; t++)
                        win[t * 32 + lane] = d - t >= 0 ? (uint32_t)dir[(int64_t)(d - t) * 32 + lane]
                                                        : 0u;
                    __syncwarp();
                }
                int ilo, ihi;
                ad_bounds(d, n, m, r, mx, mn, ilo, ihi);
                const int s = i - ilo;
                code = (win[(wtop - d) * 32 + (s & 31)] >> (2 * (s >> 5))) & 3u;
            }
            if (code == 2u) {
                j -= 1;
            } else {
                if (lane == 0) lo[i] = j;
                i -= 1;
                if (code == 0u) j -= 1;
                if (lane == 0) hi[i] = j;
            }
        }
        if (lane == 0) lo[0] = 0;
        __syncwarp();
    }
}

// Thread (group gi, row): pairs group_start[gi] .. group_start[gi + 1] - 1 of
// the group in sample order; path_lo / path_hi null: the single cell x = row.
// The result goes to row groups[gi] (gi when groups is null) of out.
__global__ void mm_accumulate_kernel(const double *x, int64_t x_stride, const int64_t *member,
                                     const int64_t *group_start, const int32_t *groups,
                                     int64_t n_groups, const int32_t *path_lo,
                                     const int32_t *path_hi, const double *sample_weight,
                                     int n, double *out, int64_t out_stride) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n_groups * (int64_t)n) return;
    const int64_t gi = tid / n;
    const int row = (int)(tid - gi * n);
    const int32_t g = groups ? groups[gi] : (int32_t)gi;
    double z = 0.0, V = 0.0;
    const int64_t qa = group_start[gi], qb = group_start[gi + 1];
    for (int64_t q = qa; q < qb; q++) {
        const int64_t s = member[q];
        const double *Xs = x + s * x_stride;
        int lo = row, hi = row;
        if (path_lo) {
            lo = path_lo[q * n + row];
            hi = path_hi[q * n + row];
        }
        if (sample_weight) {
            const double w = sample_weight[q];
            for (int c = lo; c <= hi; c++) {
                V = V + w;
                z = z + Xs[c] * w;
            }
        } else {
            for (int c = lo; c <= hi; c++) {
                V = V + 1.0;
                z = z + Xs[c];
            }
        }
    }
    out[g * out_stride + row] = z / V;
}

template <int S, bool W>
int launch_align(const MmAlignJob &J, int grid, cudaStream_t st) {
    mm_align_kernel<S, W><<<grid, kMmThreads, 0, st>>>(J);
    WB_LAUNCH_CHECK("mm_align_kernel");
    return WB_OK;
}

template <int K, bool W>
int launch_ad(const MmAlignJob &J, int grid, cudaStream_t st) {
    mm_align_ad_kernel<K, W><<<grid, kMmThreads, 0, st>>>(J);
    WB_LAUNCH_CHECK("mm_align_ad_kernel");
    return WB_OK;
}

int pick_strip(int n) {
    if (n <= 32 * 4) return 4;
    if (n <= 32 * 8) return 8;
    return 16;
}

}  // namespace

}  // namespace wb

using namespace wb;

namespace wb {
namespace {

// which alignment kernel, and its direction-word layout, for (n x m) pairs
struct AlignPlan {
    int n = 0, m = 0, warp = 1;
    bool antidiag = false;
    int S = 16, K = 1;
    int64_t pair_words = 0, word_bytes = 4;
    bool passes = false;
};

AlignPlan plan_alignment(int n, int m, double r) {
    AlignPlan P;
    P.n = n;
    P.m = m;
    const int64_t big = n > m ? n : m;
    const double wv = std::floor((double)big * r);
    P.warp = (int)(wv > 1.0 ? wv : 1.0);
    // FP64 warp-instruction slots of the two forms: the strip wavefront runs
    // 32 S rows x (m + 31) steps per pass, the anti-diagonal form
    // 32 ceil(cnt / 32) slots per diagonal
    P.S = pick_strip(n);
    const int mxb = imax(0, m - n) + P.warp, mnb = imax(0, n - m);
    int maxcnt = 0;
    int64_t slots_ad = 0;
    for (int d = 0; d < n + m - 1; d++) {
        int ilo, ihi;
        ad_bounds(d, n, m, P.warp, mxb, mnb, ilo, ihi);
        const int cnt = ihi - ilo + 1;
        maxcnt = cnt > maxcnt ? cnt : maxcnt;
        slots_ad += 32LL * ((cnt + 31) / 32);
    }
    const int64_t slots_strip =
        (int64_t)((n + 32 * P.S - 1) / (32 * P.S)) * (m + 31) * 32 * P.S;
    while (32 * P.K < maxcnt) P.K *= 2;
    P.antidiag = P.K <= 16 && slots_ad < slots_strip;
    if (const char *f = std::getenv("WB_MM_ALIGN")) {
        if (std::strcmp(f, "strip") == 0) P.antidiag = false;
        if (std::strcmp(f, "antidiag") == 0 && P.K <= 16) P.antidiag = true;
    }
    if (P.antidiag) {
        P.pair_words = (int64_t)(n + m - 1) * 32;
        P.word_bytes = P.K <= 4 ? 1 : (P.K <= 8 ? 2 : 4);
    } else {
        P.pair_words = (int64_t)((n + P.S - 1) / P.S) * m;
        P.word_bytes = P.S / 4;
    }
    P.passes = !P.antidiag && n > 32 * P.S;
    return P;
}

int run_alignment(const AlignPlan &P, const MmAlignJob &J, int grid, cudaStream_t st) {
    const bool w = J.weights != nullptr;
    if (P.antidiag) {
        switch (P.K) {
            case 1: return w ? launch_ad<1, true>(J, grid, st) : launch_ad<1, false>(J, grid, st);
            case 2: return w ? launch_ad<2, true>(J, grid, st) : launch_ad<2, false>(J, grid, st);
            case 4: return w ? launch_ad<4, true>(J, grid, st) : launch_ad<4, false>(J, grid, st);
            case 8: return w ? launch_ad<8, true>(J, grid, st) : launch_ad<8, false>(J, grid, st);
            default:
                return w ? launch_ad<16, true>(J, grid, st) : launch_ad<16, false>(J, grid, st);
        }
    }
    if (P.S == 4) return w ? launch_align<4, true>(J, grid, st) : launch_align<4, false>(J, grid, st);
    if (P.S == 8) return w ? launch_align<8, true>(J, grid, st) : launch_align<8, false>(J, grid, st);
    return w ? launch_align<16, true>(J, grid, st) : launch_align<16, false>(J, grid, st);
}

// One stochastic-subgradient step of _ssg_dtw_average (distance/dtw.py:
// 622-633) from the path of (mean, sample): z[m] = sum over the path cells
// (m, x) in order of (mean[m] - X[x] w), then mean[m] -= lr z[m].  One thread
// per mean element (each reads and writes only its own element).
__global__ void ssg_update_kernel(const double *X, const int32_t *lo, const int32_t *hi, int n,
                                  double w, int weighted, double lr, double *mean) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double mv = mean[i];
    double z = 0.0;
    for (int c = lo[i]; c <= hi[i]; c++) {
        const double xv = weighted ? X[c] * w : X[c];
        z = z + (mv - xv);
    }
    mean[i] = mv - lr * z;
}

__global__ void fill_kernel(double *p, int64_t n, double v) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = v;
}

}  // namespace
}  // namespace wb

extern "C" int wb_dtw_alignment(const double *x, int64_t n, const double *y, int64_t m, double r,
                                const double *weights, double *out, int32_t on_device,
                                void *stream) {
    WB_TRACE();
    const cudaStream_t st = (cudaStream_t)stream;
    if (n < 1 || m < 1 || n > INT32_MAX / 2 || m > INT32_MAX / 2)
        return fail(WB_EINVAL, "dtw_alignment: invalid sizes");
    if (!(r >= 0.0 && r <= 1.0)) return fail(WB_EINVAL, "r must be in [0, 1]");
    if (!x || !y || !out) return fail(WB_EINVAL, "NULL array");
    const AlignPlan P = plan_alignment((int)n, (int)m, r);
    const int64_t big = std::max(n, m);
    const size_t cells = (size_t)n * m;
    Workspace ws(st);
    const size_t need = align256(P.pair_words * P.word_bytes) +
                        align256(P.passes ? (size_t)kMmWarps * m * 8 : 0) +
                        2 * align256((size_t)n * 4) + align256(8) + align256(4) +
                        (on_device ? 0 : align256(n * 8) + align256(m * 8) +
                                             align256(cells * 8) +
                                             (weights ? align256(big * 8) : 0)) +
                        4096;
    WB_TRY(ws.reserve(need));
    WB_TAKE(dirbuf, char, ws, P.pair_words * P.word_bytes);
    double *bnd = nullptr;
    if (P.passes) {
        bnd = ws.take<double>((size_t)kMmWarps * m);
        if (!bnd) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    WB_TAKE(lo, int32_t, ws, n);
    WB_TAKE(hi, int32_t, ws, n);
    WB_TAKE(member, int64_t, ws, 1);
    WB_TAKE(group, int32_t, ws, 1);
    WB_CUDA(cudaMemsetAsync(member, 0, 8, st));
    WB_CUDA(cudaMemsetAsync(group, 0, 4, st));
    const double *dx = x, *dy = y, *dw = weights;
    double *dout = out;
    if (!on_device) {
        WB_TAKE(hx, double, ws, n);
        WB_TAKE(hy, double, ws, m);
        WB_TAKE(ho, double, ws, cells);
        WB_CUDA(cudaMemcpyAsync(hx, x, n * 8, cudaMemcpyHostToDevice, st));
        WB_CUDA(cudaMemcpyAsync(hy, y, m * 8, cudaMemcpyHostToDevice, st));
        if (weights) {
            WB_TAKE(hw, double, ws, big);
            WB_CUDA(cudaMemcpyAsync(hw, weights, big * 8, cudaMemcpyHostToDevice, st));
            dw = hw;
        }
        dx = hx;
        dy = hy;
        dout = ho;
    }
    fill_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(
        dout, (int64_t)cells, HUGE_VAL);
    WB_LAUNCH_CHECK("fill_kernel");
    MmAlignJob J;
    J.x = dy;
    J.x_stride = m;
    J.m = (int)m;
    J.means = dx;
    J.n = (int)n;
    J.member = member;
    J.pair_group = group;
    J.r = P.warp;
    J.weights = dw;
    J.dir = dirbuf;
    J.dir_pair_words = P.pair_words;
    J.bnd = bnd;
    J.path_lo = lo;
    J.path_hi = hi;
    J.full = dout;
    J.q0 = 0;
    J.q1 = 1;
    WB_TRY(run_alignment(P, J, 1, st));
    if (!on_device) WB_CUDA(cudaMemcpyAsync(out, dout, cells * 8, cudaMemcpyDeviceToHost, st));
    WB_CUDA(cudaStreamSynchronize(st));
    return WB_OK;
}

extern "C" int wb_dtw_average_mm_step(const double *x, int64_t x_stride, int64_t n_timestep,
                                      const double *means, int64_t mean_len,
                                      const int64_t *member, const int32_t *pair_group,
                                      const int64_t *group_start, const int32_t *groups,
                                      int64_t n_groups, int64_t n_pairs, double r,
                                      const double *weights, const double *sample_weight,
                                      double *new_means, double *last, void *stream) {
    WB_TRACE();
    const cudaStream_t st = (cudaStream_t)stream;
    if (n_pairs < 0 || n_groups < 0 || n_timestep < 1 || mean_len < 1)
        return fail(WB_EINVAL, "dtw_average: invalid sizes");
    if (!(r >= 0.0 && r <= 1.0)) return fail(WB_EINVAL, "dtw_average: r must be in [0, 1]");
    if (n_timestep > INT32_MAX / 2 || mean_len > INT32_MAX / 2)
        return fail(WB_EINVAL, "dtw_average: series too long");
    if (n_pairs == 0) return WB_OK;
    if (!x || !means || !member || !pair_group || !group_start)
        return fail(WB_EINVAL, "dtw_average: null pointer");
    const int n = (int)mean_len, m = (int)n_timestep;
    const AlignPlan P = plan_alignment(n, m, r);
    const int64_t pair_bytes = P.pair_words * P.word_bytes;
    const DeviceInfo &dev = device_info();
    const int max_grid = dev.sm_count * 8;
    // direction words per launch bounded to about 1 GiB
    int64_t chunk = std::max<int64_t>(1, (1LL << 30) / std::max<int64_t>(pair_bytes, 1));
    chunk = std::min<int64_t>(chunk, n_pairs);
    const int grid = (int)std::min<int64_t>((chunk + kMmWarps - 1) / kMmWarps, max_grid);
    Workspace ws(st);
    const size_t need = align256(chunk * pair_bytes) +
                        align256(P.passes ? (size_t)grid * kMmWarps * m * sizeof(double) : 0) +
                        2 * align256((size_t)n_pairs * n * sizeof(int32_t)) + 4096;
    WB_TRY(ws.reserve(need));
    WB_TAKE(dirbuf, char, ws, chunk * pair_bytes);
    double *bnd = nullptr;
    if (P.passes) {
        bnd = ws.take<double>((size_t)grid * kMmWarps * m);
        if (!bnd) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    WB_TAKE(lo, int32_t, ws, (size_t)n_pairs * n);
    WB_TAKE(hi, int32_t, ws, (size_t)n_pairs * n);
    MmAlignJob J;
    J.x = x;
    J.x_stride = x_stride;
    J.m = m;
    J.means = means;
    J.n = n;
    J.member = member;
    J.pair_group = pair_group;
    J.r = P.warp;
    J.weights = weights;
    J.dir = dirbuf;
    J.dir_pair_words = P.pair_words;
    J.bnd = bnd;
    J.path_lo = lo;
    J.path_hi = hi;
    J.last = last;
    timer_begin(P.antidiag ? "mm_align_ad_kernel" : "mm_align_kernel", st);
    for (int64_t q0 = 0; q0 < n_pairs; q0 += chunk) {
        J.q0 = q0;
        J.q1 = std::min(n_pairs, q0 + chunk);
        WB_TRY(run_alignment(P, J, grid, st));
    }
    timer_end(st);
    if (new_means && n_groups > 0) {
        const int64_t threads = n_groups * (int64_t)n;
        mm_accumulate_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(
            x, x_stride, member, group_start, groups, n_groups, lo, hi, sample_weight, n,
            new_means, n);
        WB_LAUNCH_CHECK("mm_accumulate_kernel");
    }
    return WB_OK;
}

extern "C" int wb_dtw_average_ssg_epoch(const double *x, int64_t x_stride, int64_t n_timestep,
                                        double *mean, int64_t mean_len, const int64_t *order,
                                        const double *lr, int64_t n_steps, double r,
                                        const double *weights, const double *sample_weight,
                                        void *stream) {
    WB_TRACE();
    const cudaStream_t st = (cudaStream_t)stream;
    if (n_steps < 0 || n_timestep < 1 || mean_len < 1)
        return fail(WB_EINVAL, "dtw_average: invalid sizes");
    if (!(r >= 0.0 && r <= 1.0)) return fail(WB_EINVAL, "dtw_average: r must be in [0, 1]");
    if (n_timestep > INT32_MAX / 2 || mean_len > INT32_MAX / 2)
        return fail(WB_EINVAL, "dtw_average: series too long");
    if (n_steps == 0) return WB_OK;
    if (!x || !mean || !order || !lr) return fail(WB_EINVAL, "dtw_average: null pointer");
    const int n = (int)mean_len, m = (int)n_timestep;
    const AlignPlan P = plan_alignment(n, m, r);
    const int64_t pair_bytes = P.pair_words * P.word_bytes;
    Workspace ws(st);
    const size_t need = align256(pair_bytes) +
                        align256(P.passes ? (size_t)kMmWarps * m * sizeof(double) : 0) +
                        2 * align256((size_t)n * sizeof(int32_t)) +
                        align256((size_t)n_steps * 8) + align256(4) + 4096;
    WB_TRY(ws.reserve(need));
    WB_TAKE(dirbuf, char, ws, pair_bytes);
    double *bnd = nullptr;
    if (P.passes) {
        bnd = ws.take<double>((size_t)kMmWarps * m);
        if (!bnd) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    WB_TAKE(lo, int32_t, ws, n);
    WB_TAKE(hi, int32_t, ws, n);
    WB_TAKE(dorder, int64_t, ws, n_steps);
    WB_TAKE(zero, int32_t, ws, 1);
    WB_CUDA(cudaMemcpyAsync(dorder, order, n_steps * 8, cudaMemcpyHostToDevice, st));
    WB_CUDA(cudaMemsetAsync(zero, 0, 4, st));
    MmAlignJob J;
    J.x = x;
    J.x_stride = x_stride;
    J.m = m;
    J.means = mean;
    J.n = n;
    J.pair_group = zero;
    J.r = P.warp;
    J.weights = weights;
    J.dir = dirbuf;
    J.dir_pair_words = P.pair_words;
    J.bnd = bnd;
    J.path_lo = lo;
    J.path_hi = hi;
    J.q0 = 0;
    J.q1 = 1;
    for (int64_t i = 0; i < n_steps; i++) {
        J.member = dorder + i;
        WB_TRY(run_alignment(P, J, 1, st));
        const double w = sample_weight ? sample_weight[order[i]] : 1.0;
        ssg_update_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(
            x + order[i] * x_stride, lo, hi, n, w, sample_weight ? 1 : 0, lr[i], mean);
        WB_LAUNCH_CHECK("ssg_update_kernel");
    }
    WB_CUDA(cudaStreamSynchronize(st));
    return WB_OK;
}

extern "C" int wb_group_mean(const double *x, int64_t x_stride, int64_t n_timestep,
                             const int64_t *member, const int64_t *group_start,
                             const int32_t *groups, int64_t n_groups, double *out,
                             void *stream) {
    WB_TRACE();
    const cudaStream_t st = (cudaStream_t)stream;
    if (n_groups < 0 || n_timestep < 1 || n_timestep > INT32_MAX / 2)
        return fail(WB_EINVAL, "group_mean: invalid sizes");
    if (n_groups == 0) return WB_OK;
    if (!x || !member || !group_start || !out) return fail(WB_EINVAL, "group_mean: null pointer");
    const int n = (int)n_timestep;
    const int64_t threads = n_groups * (int64_t)n;
    mm_accumulate_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(
        x, x_stride, member, group_start, groups, n_groups, nullptr, nullptr, nullptr, n, out, n);
    WB_LAUNCH_CHECK("mm_accumulate_kernel");
    return WB_OK;
}
