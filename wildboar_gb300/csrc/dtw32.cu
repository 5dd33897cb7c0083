// dtw32.cu -- FP32 dtw / wdtw with compensated accumulation, forward and
// backward, for batches of (possibly ragged) pairs.
//
// One thread per (x, y) problem, persistent: warps take 32 consecutive items
// at a time from an atomic counter, so a batch sorted by cost keeps the 32
// lanes of a warp on problems of similar size.  dtw items are transposed so
// that the rows of the recurrence are the shorter series (wdtw keeps x on the
// rows: its row-0 weight index makes it asymmetric).  A thread sweeps its band
// in strips of S rows: the S cells of one column live in registers as (hi, lo)
// float pairs, the previous strip's bottom row is read from, and the strip's
// own bottom row written to, a ring in global memory laid out
// [column][thread].  The loop bounds of every strip are the union of the 32
// lanes' column ranges, so lanes never diverge on ragged shapes; cells outside
// a lane's own band take the masked path with an infinite cost.  The cells of
// a column are written to the other of two register sets, which alternate
// between columns, so no cell value is copied to free its register.
//
// Arithmetic: the cost (x_i - y_j)^2 (times the wdtw weight) is FP32 (two
// columns' differences and squares as packed f32x2 operations, each half
// rounded as the scalar operation); the minimum of the three hi parts is one
// 3-input min, the lo of a candidate holding it comes with it, and the new
// partial sum is a Fast2Sum of (minimum, cost), whose error term is exact
// when the minimum is at least the cost and within one rounding of the sum
// otherwise, so the cumulative cost carries ~48 bits.  The final distance
// sqrt(hi + lo) is formed in FP64.  Band, row-0 weights and out-of-band +inf
// follow dtw_distance (distance/_elastic.pyx:869-940).
//
// Backward (second half of the file): checkpointed recomputation with 2-bit
// traceback directions and an in-kernel walk of the optimal path that adds
// dD/dx_i = sum_{j:(i,j) on path} w_{|i-j|} (x_i - y_j) / D and the negative
// column sums dD/dy_j to per-series gradient rows (D = sqrt of the path cost).
// Kept directions (end of the file): the same sweep run once by the forward
// of a differentiable call, its directions kept per batch of 32 items, and a
// walk-only backward over them.

#include "dtw32.cuh"

namespace wb {

struct HL {
    float h, l;
};

#define WB_FINF __int_as_float(0x7f800000)

__device__ __forceinline__ HL hl_inf() { return HL{WB_FINF, 0.0f}; }

// TwoSum (Knuth): s + err == a.h + b exactly; err joins the lo part.
__device__ __forceinline__ HL add_c(HL a, float b) {
    float s = __fadd_rn(a.h, b);
    float bb = __fsub_rn(s, a.h);
    float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return HL{s, __fadd_rn(a.l, err)};
}

__device__ __forceinline__ int band_of(int n, int m, double r) {
    double v = floor((double)(n < m ? n : m) * r);
    return (int)(v > 1.0 ? v : 1.0);
}

struct Item {
    const float *X, *Y;
    int n, m, r, mx, mn;
};

__device__ __forceinline__ Item load_item(const Dtw32Job &J, int64_t t) {
    int64_t cx, cy;
    if (J.item_x) {
        cx = J.item_x[t];
        cy = J.item_y[t];
    } else {
        cy = t / J.nx;
        cx = t - cy * J.nx;
    }
    Item it;
    it.X = J.x + cx * J.x_stride;
    it.Y = J.y + cy * J.y_stride;
    it.n = J.xlen ? J.xlen[cx] : J.x_len;
    it.m = J.ylen ? J.ylen[cy] : J.y_len;
    it.r = J.band_fixed > 0 ? J.band_fixed : band_of(it.n, it.m, J.r);
    it.mx = imax(0, it.m - it.n) + it.r;
    it.mn = imax(0, it.n - it.m);
    return it;
}

// two floats as one packed f32x2 operand (adjacent registers)
__device__ __forceinline__ uint64_t pack2(float a, float b) {
    uint64_t p;
    asm("mov.b64 %0, {%1, %2};" : "=l"(p) : "f"(a), "f"(b));
    return p;
}

// (x0 - y)^2 and (x1 - y)^2 from the packed pairs x2 = {x0, x1}, y2 = {y, y}:
// one packed f32x2 subtraction and one packed multiplication (each half
// rounded as the scalar operation would be)
__device__ __forceinline__ void sqdiff2p(uint64_t x2, uint64_t y2, float &c0, float &c1) {
    asm("{\n\t.reg .b64 pa;\n\t"
        "sub.rn.f32x2 pa, %2, %3;\n\t"
        "mul.rn.f32x2 pa, pa, pa;\n\t"
        "mov.b64 {%0, %1}, pa;\n\t}"
        : "=f"(c0), "=f"(c1)
        : "l"(x2), "l"(y2));
}

// Bits k (k < 32) with 0 <= e - k < width: the strip rows in band at a
// column, e = c - i0 - lo.
__device__ __forceinline__ unsigned band_bits(int e, int width) {
    const unsigned upper = e < 0 ? 0u : (e >= 31 ? 0xffffffffu : (0xffffffffu >> (31 - e)));
    const int lb = e - width + 1;
    const unsigned lower = lb <= 0 ? 0u : (lb >= 32 ? 0xffffffffu : ((1u << lb) - 1u));
    return upper & ~lower;
}

// One column of a strip in the forward sweep (no traceback directions):
// the minimum of the three hi parts with the lo of a candidate holding it
// (left, then up, then diag on equal hi), Fast2Sum for the new partial sum.
// The column reads the previous column's cells from Pin and writes its own
// to Pout (two register sets alternating between columns, so no cell value
// has to be copied to free its register).  With MASK, rows whose bit of M
// is clear are out of band (infinite cost).
template <int S, bool W, bool MASK>
__device__ __forceinline__ void fwd_column(const HL (&Pin)[S], HL (&Pout)[S], HL bup,
                                           HL bdiag, float yc, const float (&xr)[S],
                                           const uint64_t (&xr2)[S / 2], int d0, unsigned M,
                                           const float *__restrict__ w, int valid) {
    float cpair[2];
    const uint64_t yp = W ? 0ull : pack2(yc, yc);
#pragma unroll
    for (int k = 0; k < S; k++) {
        if (!W && (k & 1) == 0) sqdiff2p(xr2[k / 2], yp, cpair[0], cpair[1]);
        const HL dg = k == 0 ? bdiag : Pin[k - 1];  // cell (i0 + k - 1, c - 1)
        const HL up = k == 0 ? bup : Pout[k - 1];   // cell (i0 + k - 1, c)
        const HL lf = Pin[k];                       // cell (i0 + k, c - 1)
        float cst;
        if (W) {
            const float vv = __fsub_rn(xr[k], yc);
            cst = __fmul_rn(__fmul_rn(vv, vv), w[(!MASK || k < valid) ? abs(d0 - k) : 0]);
        } else {
            cst = cpair[k & 1];
        }
        if (MASK) cst = ((M >> k) & 1u) ? cst : WB_FINF;
        HL best;
        asm("min.f32 %0, %1, %2, %3;" : "=f"(best.h) : "f"(dg.h), "f"(up.h), "f"(lf.h));
        best.l = (up.h == best.h) ? up.l : dg.l;
        best.l = (lf.h == best.h) ? lf.l : best.l;
        // Fast2Sum: exact when best.h >= cst; otherwise (a partial sum
        // smaller than the next cost, near the start of a path) the error
        // term is off by at most half an ulp of the new partial sum, and such
        // steps at least double it, so they add at most one unit roundoff of
        // the path cost in all
        const float sh = __fadd_rn(best.h, cst);
        const float err = __fsub_rn(cst, __fsub_rn(sh, best.h));
        Pout[k] = HL{sh, __fadd_rn(best.l, err)};
    }
}

// The forward sweep of the 32 lanes of a warp with warp-uniform loop bounds:
// every strip runs over the union of the lanes' column ranges, so lanes whose
// items differ in shape never diverge; a lane's cells outside its own band
// (or past its own series) get an infinite cost on the masked path.  Columns
// where every row of every lane's strip is in band take the mask-free path.
// Called by all 32 lanes; `active` lanes return the (hi, lo) cost of their
// cell (n-1, m-1), the others run masked and return +inf.
template <int S, bool W>
__device__ HL sweep_uniform(Item it, bool active, const float *__restrict__ w, float2 *ring,
                            int64_t nth) {
    const unsigned FULL = 0xffffffffu;
    if (!active) it.n = it.m = 0;
    if (!W && it.n > it.m) {
        // dtw: rows are the shorter series (the transposed problem has the
        // same band, the same costs and the same minima), so the lanes of a
        // warp, sorted by the shorter length, have their bands in the same
        // columns
        const float *tp = it.X;
        it.X = it.Y;
        it.Y = tp;
        const int tn = it.n;
        it.n = it.m;
        it.m = tn;
        it.mx = imax(0, it.m - it.n) + it.r;
        it.mn = imax(0, it.n - it.m);
    }
    const float *__restrict__ X = it.X;
    const float *__restrict__ Y = it.Y;
    const int n = it.n, m = it.m, r = it.r, mx = it.mx, mn = it.mn;
    const float qnan = __int_as_float(0x7fc00000);
    // row 0: cumulative, weight index j-1 for j >= 1
    const int lim = active ? imin(m, mx) : 0;
    const int lim_w = __reduce_max_sync(FULL, lim);
    HL acc = hl_inf();
    const float x0 = active ? X[0] : qnan;
    for (int c = 0; c < lim_w; c++) {
        if (c < lim) {
            const float v = __fsub_rn(x0, Y[c]);
            float cc = __fmul_rn(v, v);
            if (W) cc = __fmul_rn(cc, w[c > 0 ? c - 1 : 0]);
            acc = c == 0 ? HL{cc, 0.0f} : add_c(acc, cc);
            ring[(int64_t)c * nth] = make_float2(acc.h, acc.l);
        }
    }
    HL result = acc;
    int pstart = 0, pend = lim;
    const int lo = -(mn + r - 1);
    const int hi = mx - 1;
    const unsigned width = (unsigned)(hi - lo + 1);
    const int n_w = __reduce_max_sync(FULL, n);
    for (int i0 = 1; i0 < n_w; i0 += S) {
        const int rows = imax(0, imin(S, n - i0));
        float xr[S];
#pragma unroll
        for (int k = 0; k < S; k++) xr[k] = (k < rows) ? X[i0 + k] : qnan;
        uint64_t xr2[S / 2];
#pragma unroll
        for (int k = 0; k < S / 2; k++) xr2[k] = W ? 0ull : pack2(xr[2 * k], xr[2 * k + 1]);
        int cstart = imax(0, i0 - mn - r + 1);
        int cend = imin(m, i0 + rows - 1 + mx);
        if (rows == 0) {
            cstart = 0x7fffffff;
            cend = 0;
        }
        // columns where every row of a full strip is in band
        int bstart = 0x7fffffff, bend = 0;
        if (rows == S) {
            bstart = imax(cstart, i0 + S - 1 + lo);
            bend = imin(cend, i0 + hi + 1);
        }
        const int cs_w = __reduce_min_sync(FULL, cstart);
        const int ce_w = __reduce_max_sync(FULL, cend);
        const int bs_w = __reduce_max_sync(FULL, bstart);
        const int be_w = __reduce_min_sync(FULL, bend);
        HL P[S], Q[S];
#pragma unroll
        for (int k = 0; k < S; k++) P[k] = hl_inf();
        HL bdiag = hl_inf();
        if (cs_w - 1 >= pstart && cs_w - 1 < pend) {
            const float2 t2 = ring[(int64_t)(cs_w - 1) * nth];
            bdiag = HL{t2.x, t2.y};
        }
        auto load_up = [&](int c) {
            HL b = hl_inf();
            if (c >= pstart && c < pend) {
                const float2 t2 = ring[(int64_t)c * nth];
                b = HL{t2.x, t2.y};
            }
            return b;
        };
        // a lane reads y only inside its own series
        auto load_y = [&](int c) { return c < m ? Y[c] : 0.0f; };
        HL nb0 = load_up(cs_w), nb1 = load_up(cs_w + 1);
        float ny0 = load_y(cs_w), ny1 = load_y(cs_w + 1);
        const bool last = rows > 0 && (i0 + rows == n);
        const int krow = rows - 1;
        // column c from the cells of column c - 1 (Pin) into Pout
        auto column = [&](int c, const HL(&Pin)[S], HL(&Pout)[S]) {
            const HL bup = nb0;
            const float yc = ny0;
            nb0 = nb1;
            ny0 = ny1;
            nb1 = load_up(c + 2);
            ny1 = load_y(c + 2);
            if (c >= bs_w && c < be_w) {
                fwd_column<S, W, false>(Pin, Pout, bup, bdiag, yc, xr, xr2, c - i0, 0u, w,
                                        rows);
            } else {
                // past the lane's series end every row is out of band
                const unsigned M = c < m ? band_bits(c - i0 - lo, (int)width) : 0u;
                fwd_column<S, W, true>(Pin, Pout, bup, bdiag, yc, xr, xr2, c - i0, M, w,
                                       rows);
            }
            if (last && c == m - 1) {
#pragma unroll
                for (int k = 0; k < S; k++)
                    if (k <= krow) result = Pout[k];
            }
            ring[(int64_t)c * nth] = make_float2(Pout[S - 1].h, Pout[S - 1].l);
            bdiag = bup;
        };
        int c = cs_w;
        for (; c + 1 < ce_w; c += 2) {
            if (c >= bs_w && c + 1 < be_w) {
                // two band-interior columns as one straight-line block, so
                // the cells of column c + 1 can issue beside those of c
                const HL bup0 = nb0, bup1 = nb1;
                const float y0 = ny0, y1 = ny1;
                nb0 = load_up(c + 2);
                nb1 = load_up(c + 3);
                ny0 = load_y(c + 2);
                ny1 = load_y(c + 3);
                fwd_column<S, W, false>(P, Q, bup0, bdiag, y0, xr, xr2, c - i0, 0u, w, rows);
                fwd_column<S, W, false>(Q, P, bup1, bup0, y1, xr, xr2, c + 1 - i0, 0u, w,
                                        rows);
                if (last && (c == m - 1 || c + 1 == m - 1)) {
#pragma unroll
                    for (int k = 0; k < S; k++)
                        if (k <= krow) result = c == m - 1 ? Q[k] : P[k];
                }
                ring[(int64_t)c * nth] = make_float2(Q[S - 1].h, Q[S - 1].l);
                ring[(int64_t)(c + 1) * nth] = make_float2(P[S - 1].h, P[S - 1].l);
                bdiag = bup1;
            } else {
                column(c, P, Q);
                column(c + 1, Q, P);
            }
        }
        if (c < ce_w) column(c, P, Q);
        if (rows > 0) {
            pstart = cstart;
            pend = cend;
        }
    }
    return active ? result : hl_inf();
}

__device__ __forceinline__ int64_t take_items(unsigned long long *q, int lane) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(q, 32ull);
    return (int64_t)__shfl_sync(0xffffffffu, base, 0);
}

template <int S, bool W>
__global__ void __launch_bounds__(256) dtw32_forward_kernel(const Dtw32Job J) {
    const int lane = threadIdx.x & 31;
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    float2 *ring = J.ring + gtid;
    for (;;) {
        const int64_t base = take_items(J.queue, lane);
        if (base >= J.n_items) break;
        const int64_t t = base + lane;
        Item it{};
        bool active = false;
        if (t < J.n_items) {
            it = load_item(J, t);
            active = !(it.n < 1 || it.m < 1 || it.m >= J.ring_cols);
        }
        // all 32 lanes sweep together (warp-uniform bounds)
        const HL h = sweep_uniform<S, W>(it, active, J.weights, ring, nth);
        if (t < J.n_items) {
            double res = __longlong_as_double(0x7ff8000000000000LL);  // NaN: empty series
            if (active) {
                const double cost = (double)h.h + (double)h.l;
                if (J.out_cost) J.out_cost[t] = cost;
                res = sqrt(cost);
            } else if (J.out_cost) {
                J.out_cost[t] = res;
            }
            J.out[t] = res;
        }
    }
}

// ---------------------------------------------------------------------------
// Backward.
//
// A warp takes 32 consecutive items and sweeps them together in strips of 16
// rows (one 32-bit word of 2-bit directions per strip column) over rows
// 1..n-1, with warp-uniform column bounds as in the forward and dtw items
// transposed so that rows are the shorter series.  The predecessor of a cell
// is the one with the smallest compensated value (hi - hi') + (lo - lo'),
// ties in dtw_mapping's order (diag, up, left; distance/dtw.py:362-426), so
// the path is the one the FP64 reference takes except at exact ties.
//
// Memory: the strips of an item are cut into segments of K strips.  Items of
// one segment store all their directions and walk back directly.  Longer
// items first sweep the strips once without directions, saving the bottom
// row of every segment but the last (a checkpoint of the band boundary);
// then, from the last segment to the first, each segment is recomputed from
// the checkpoint above it with its directions and the path is walked through
// its rows.  Per resident thread this holds K strips of direction words, the
// checkpoints and one working row, instead of the directions of the whole
// band.
//
// Gradients are added in the kernel (atomically) to per-series rows:
//   dD/dr_i += g / D * sum_{j:(i,j) on path} w (r_i - c_j)
//   dD/dc_j -= g / D * sum_{i:(i,j) on path} w (r_i - c_j)
// (r the row series, c the column series, w the wdtw weight of the cell;
// cells of row 0 use the row-0 weight index j - 1 of the forward).

constexpr int kGradStrip = 16;      // rows per strip (2-bit words of 32 bits)
constexpr int kMaxSegStrips = 64;   // strips per segment (shared-memory tables)
constexpr int kBwdBlock = 128;      // threads per block of the backward kernel

// (a.h + a.l) < (b.h + b.l) for the compensated pairs of two cumulative costs,
// as (a.h - b.h) < (b.l - a.l): the hi difference of close values is exact
// (Sterbenz) and the comparison of the two rounded differences has the sign
// of the exact compensated difference.  An unreachable cell (+inf, 0) is never
// preferred to a finite one; two of them compare false (NaN difference).
__device__ __forceinline__ bool hl_less(HL a, HL b) {
    return __fsub_rn(a.h, b.h) < __fsub_rn(b.l, a.l);
}

// Direction words are stored in groups of 8 consecutive words of one thread
// (one 32-byte sector): word w of thread g at ((w / 8) * nth + g) * 8 + w % 8,
// so a path walked left or diagonally reads words of one cached sector.
__device__ __forceinline__ int64_t dir_index(int64_t w, int64_t g, int64_t nth) {
    return (((w >> 3) * nth + g) << 3) + (w & 7);
}

// One column of a backward strip: Fast2Sum accumulation, the predecessor by
// compensated comparison, its 2-bit code (0 diag, 1 up, 2 left) per row into
// `word`.  Reads the previous column from Pin and writes Pout (register sets
// alternating between columns, as in fwd_column).  With MASK, rows whose bit
// of M is clear are out of band and hold (+inf, 0).
template <bool W, bool MASK>
__device__ __forceinline__ void bwd_column(const HL (&Pin)[kGradStrip], HL (&Pout)[kGradStrip],
                                           HL bup, HL bdiag, float yc,
                                           const float (&xr)[kGradStrip],
                                           const uint64_t (&xr2)[kGradStrip / 2], int d0,
                                           unsigned M, const float *__restrict__ w, int valid,
                                           uint32_t &word) {
    float cpair[2];
    const uint64_t yp = W ? 0ull : pack2(yc, yc);
#pragma unroll
    for (int k = 0; k < kGradStrip; k++) {
        if (!W && (k & 1) == 0) sqdiff2p(xr2[k / 2], yp, cpair[0], cpair[1]);
        const HL dg = k == 0 ? bdiag : Pin[k - 1];
        const HL up = k == 0 ? bup : Pout[k - 1];
        const HL lf = Pin[k];
        HL best = dg;
        uint32_t dir = 0;
        if (hl_less(up, best)) {
            best = up;
            dir = 1;
        }
        if (hl_less(lf, best)) {
            best = lf;
            dir = 2;
        }
        float cst;
        if (W) {
            const float vv = __fsub_rn(xr[k], yc);
            cst = __fmul_rn(__fmul_rn(vv, vv), w[(!MASK || k < valid) ? abs(d0 - k) : 0]);
        } else {
            cst = cpair[k & 1];
        }
        // Fast2Sum (see fwd_column)
        const float sh = __fadd_rn(best.h, cst);
        HL nv{sh, __fadd_rn(best.l, __fsub_rn(cst, __fsub_rn(sh, best.h)))};
        if (MASK && !((M >> k) & 1u)) nv = hl_inf();
        word |= dir << (2 * k);
        Pout[k] = nv;
    }
}

// Per-lane geometry of a backward item (rows: r series, columns: c series).
struct BwdItem {
    const float *R = nullptr, *C = nullptr;
    float *GR = nullptr, *GC = nullptr;  // gradient rows of the r and c series
    int capR = 0, capC = 0;              // positions every gradient row has (padded lengths)
    int n = 0, m = 0, r = 1, mx = 0, mn = 0, lo = 0;
    int width = 0;
    int nstrips = 0;                     // strips over rows 1..n-1
};

// own column range [cs, ce) of strip s (s = -1: row 0, columns [0, lim))
__device__ __forceinline__ void bwd_range(const BwdItem &B, int s, int &cs, int &ce) {
    if (B.n < 1 || s >= B.nstrips) {
        cs = 0x7fffffff;
        ce = 0;
        return;
    }
    if (s < 0) {
        cs = 0;
        ce = imin(B.m, B.mx);
        return;
    }
    const int i0 = 1 + s * kGradStrip;
    const int rows = imin(kGradStrip, B.n - i0);
    cs = imax(0, i0 - B.mn - B.r + 1);
    ce = imin(B.m, i0 + rows - 1 + B.mx);
}

// Row 0 of every lane into `ring` (warp-uniform loop); lanes with n == 1 get
// their cost of cell (0, m-1) in `result`.
template <bool W>
__device__ void bwd_row0(const BwdItem &B, const float *__restrict__ w, float2 *ring,
                         int64_t nth, HL &result) {
    int cs, lim;
    bwd_range(B, -1, cs, lim);
    const int lim_w = __reduce_max_sync(0xffffffffu, lim);
    HL acc = hl_inf();
    const float x0 = B.n > 0 ? B.R[0] : 0.0f;
    for (int c = 0; c < lim_w; c++) {
        if (c < lim) {
            const float v = __fsub_rn(x0, B.C[c]);
            float cc = __fmul_rn(v, v);
            if (W) cc = __fmul_rn(cc, w[c > 0 ? c - 1 : 0]);
            acc = c == 0 ? HL{cc, 0.0f} : add_c(acc, cc);
            ring[(int64_t)c * nth] = make_float2(acc.h, acc.l);
        }
    }
    if (B.n == 1) result = acc;
}

// Strips [s0, s1) of every lane with warp-uniform column bounds.  The row above
// strip s0 is read from `src`; each strip's bottom row goes to `ring`, the last
// one's to `last_dst` when it is set (ring rows have stride nth).  With DIRS,
// the direction words of the strips go to word base + c - cs_w of thread
// dir_g of dir_n (dir_index) and (cs_w, base) of each strip to the warp's
// tables; returns false (for every lane) if the words would not fit
// in dir_words.  A lane whose last strip is in the range gets its cost of cell
// (n-1, m-1) in `result`.
template <bool W, bool DIRS>
__device__ bool bwd_strips(const BwdItem &B, int s0, int s1, const float2 *src, float2 *ring,
                           float2 *last_dst, uint32_t *dirs, int64_t dir_words, int *tab_cs,
                           int *tab_base, uint32_t *stage, int64_t dir_g, int64_t dir_n,
                           int64_t nth, const float *__restrict__ w, HL &result) {
    constexpr int S = kGradStrip;
    const unsigned FULL = 0xffffffffu;
    const float qnan = __int_as_float(0x7fc00000);
    const int lane = threadIdx.x & 31;
    int pstart, pend;
    bwd_range(B, s0 - 1, pstart, pend);
    int64_t base = 0;
    for (int s = s0; s < s1; s++) {
        const int i0 = 1 + s * S;
        const int rows = imax(0, imin(S, B.n - i0));
        float xr[S];
#pragma unroll
        for (int k = 0; k < S; k++) xr[k] = (k < rows) ? B.R[i0 + k] : qnan;
        int cstart, cend;
        bwd_range(B, s, cstart, cend);
        int bstart = 0x7fffffff, bend = 0;
        if (rows == S) {
            bstart = imax(cstart, i0 + S - 1 + B.lo);
            bend = imin(cend, i0 + (B.mx - 1) + 1);
        }
        const int cs_w = __reduce_min_sync(FULL, cstart);
        const int ce_w = __reduce_max_sync(FULL, cend);
        const int bs_w = __reduce_max_sync(FULL, bstart);
        const int be_w = __reduce_min_sync(FULL, bend);
        if (ce_w <= cs_w) continue;  // no lane has rows here
        if (DIRS) {
            if (base + (ce_w - cs_w) > dir_words) return false;
            if (lane == 0) {
                tab_cs[s - s0] = cs_w;
                tab_base[s - s0] = (int)base;
            }
        }
        const float2 *in = (s == s0) ? src : ring;
        float2 *out = (s == s1 - 1 && last_dst) ? last_dst : ring;
        uint64_t xr2[S / 2];
#pragma unroll
        for (int k = 0; k < S / 2; k++) xr2[k] = W ? 0ull : pack2(xr[2 * k], xr[2 * k + 1]);
        HL P[S], Q[S];
#pragma unroll
        for (int k = 0; k < S; k++) P[k] = hl_inf();
        auto load_up = [&](int c) {
            HL b = hl_inf();
            if (c >= pstart && c < pend) {
                const float2 t2 = in[(int64_t)c * nth];
                b = HL{t2.x, t2.y};
            }
            return b;
        };
        auto load_y = [&](int c) { return c < B.m ? B.C[c] : 0.0f; };
        HL bdiag = load_up(cs_w - 1);
        HL nb0 = load_up(cs_w), nb1 = load_up(cs_w + 1);
        float ny0 = load_y(cs_w), ny1 = load_y(cs_w + 1);
        const bool last = rows > 0 && (i0 + rows == B.n);
        const int krow = rows - 1;
        // the column's direction word into the stage; a full group of 8 (or
        // the strip's last column) goes out as two 16-byte stores
        auto put_word = [&](int c, uint32_t word) {
            if (DIRS) {
                const int64_t wi = base + (c - cs_w);
                stage[(wi & 7) * 33] = word;
                if ((wi & 7) == 7 || c == ce_w - 1) {
                    uint4 *dst = reinterpret_cast<uint4 *>(
                        dirs + dir_index(wi & ~(int64_t)7, dir_g, dir_n));
                    dst[0] = make_uint4(stage[0], stage[33], stage[66], stage[99]);
                    dst[1] = make_uint4(stage[132], stage[165], stage[198], stage[231]);
                }
            }
        };
        // column c from the cells of column c - 1 (Pin) into Pout
        auto column = [&](int c, const HL(&Pin)[S], HL(&Pout)[S]) {
            const HL bup = nb0;
            const float yc = ny0;
            nb0 = nb1;
            ny0 = ny1;
            nb1 = load_up(c + 2);
            ny1 = load_y(c + 2);
            uint32_t word = 0;
            if (c >= bs_w && c < be_w) {
                bwd_column<W, false>(Pin, Pout, bup, bdiag, yc, xr, xr2, c - i0, 0u, w, rows,
                                     word);
            } else {
                const unsigned M = c < B.m ? band_bits(c - i0 - B.lo, B.width) : 0u;
                bwd_column<W, true>(Pin, Pout, bup, bdiag, yc, xr, xr2, c - i0, M, w, rows,
                                    word);
            }
            put_word(c, word);
            if (last && c == B.m - 1) {
#pragma unroll
                for (int k = 0; k < S; k++)
                    if (k == krow) result = Pout[k];
            }
            out[(int64_t)c * nth] = make_float2(Pout[S - 1].h, Pout[S - 1].l);
            bdiag = bup;
        };
        int c = cs_w;
        for (; c + 1 < ce_w; c += 2) {
            if (c >= bs_w && c + 1 < be_w) {
                // two band-interior columns as one straight-line block
                const HL bup0 = nb0, bup1 = nb1;
                const float y0 = ny0, y1 = ny1;
                nb0 = load_up(c + 2);
                nb1 = load_up(c + 3);
                ny0 = load_y(c + 2);
                ny1 = load_y(c + 3);
                uint32_t w0 = 0, w1 = 0;
                bwd_column<W, false>(P, Q, bup0, bdiag, y0, xr, xr2, c - i0, 0u, w, rows, w0);
                bwd_column<W, false>(Q, P, bup1, bup0, y1, xr, xr2, c + 1 - i0, 0u, w, rows,
                                     w1);
                put_word(c, w0);
                put_word(c + 1, w1);
                if (last && (c == B.m - 1 || c + 1 == B.m - 1)) {
#pragma unroll
                    for (int k = 0; k < S; k++)
                        if (k == krow) result = c == B.m - 1 ? Q[k] : P[k];
                }
                out[(int64_t)c * nth] = make_float2(Q[S - 1].h, Q[S - 1].l);
                out[(int64_t)(c + 1) * nth] = make_float2(P[S - 1].h, P[S - 1].l);
                bdiag = bup1;
            } else {
                column(c, P, Q);
                column(c + 1, Q, P);
            }
        }
        if (c < ce_w) column(c, P, Q);
        base += ce_w - cs_w;
        if (rows > 0) {
            pstart = cstart;
            pend = cend;
        }
    }
    return true;
}

// Gradients of four consecutive positions of one gradient row (positions
// 4 g .. 4 g + 3), added with one 16-byte vector atomic when the walk leaves
// the group: a path leaves every row and every column exactly once, in
// decreasing order, so each position is assigned once.  Rows that are not
// 16-byte aligned, or groups that reach past the positions every row has
// (cap: the padded series length), take scalar atomics (positions below the
// item's length only).
struct GradQuad {
    float *base;
    int cap, len;
    bool vec;
    int g = -1;
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
    __device__ __forceinline__ GradQuad(float *b, int c, int l)
        : base(b), cap(c), len(l), vec((reinterpret_cast<uintptr_t>(b) & 15) == 0) {}
    __device__ __forceinline__ void flush() {
        if (g < 0) return;
        const int p0 = 4 * g;
        if (vec && p0 + 3 < cap) {
            atomicAdd(reinterpret_cast<float4 *>(base + p0), make_float4(s0, s1, s2, s3));
        } else {
            if (p0 < len) atomicAdd(base + p0, s0);
            if (p0 + 1 < len) atomicAdd(base + p0 + 1, s1);
            if (p0 + 2 < len) atomicAdd(base + p0 + 2, s2);
            if (p0 + 3 < len) atomicAdd(base + p0 + 3, s3);
        }
        g = -1;
    }
    __device__ __forceinline__ void put(int idx, float v) {
        if ((idx >> 2) != g) {
            flush();
            g = idx >> 2;
            s0 = s1 = s2 = s3 = 0.0f;
        }
        const int u = idx & 3;
        s0 = u == 0 ? v : s0;
        s1 = u == 1 ? v : s1;
        s2 = u == 2 ? v : s2;
        s3 = u == 3 ? v : s3;
    }
};

// Walk of one lane through the rows of segment g (strips [g K, (g+1) K), and
// row 0 when g == 0), from (i, j) upward, adding the gradient of every row and
// column the path leaves.  Returns with i below the segment (or done).  The
// walk keeps in registers the 8-word group (one 32-byte sector) of direction
// words it reads from, the strip's table entries and the current r_i and c_j,
// so a step that stays in the group (a move up, or left within 8 columns)
// issues no dependent load.  dir_cap: the words each lane owns; an index
// outside them ends the walk with NaN gradients.
template <bool W>
__device__ __forceinline__ void bwd_walk(const BwdItem &B, int g, int K, const uint32_t *dirs,
                                         int64_t dir_cap, const int *tab_cs,
                                         const int *tab_base, int64_t gtid, int64_t nth,
                                         const float *__restrict__ w, float sc, int &i, int &j,
                                         float &gr, float &gc, bool &done) {
    const int first_row = g == 0 ? 0 : 1 + g * K * kGradStrip;
    if (done || i < first_row) return;
    int cur_s = -1, tcs = 0, tbase = 0;
    int64_t cur_grp = -1;
    uint4 ga = make_uint4(0, 0, 0, 0), gb = ga;
    float ri = B.R[i], cj = B.C[j];
    GradQuad qr(B.GR, B.capR, B.n), qc(B.GC, B.capC, B.m);
    while (true) {
        const float vv = __fsub_rn(ri, cj);
        float d = vv;
        if (W) d = __fmul_rn(w[i == 0 ? imax(j - 1, 0) : abs(i - j)], vv);
        gr = __fadd_rn(gr, d);
        gc = __fadd_rn(gc, d);
        if (i == 0 && j == 0) {
            qr.put(0, sc * gr);
            qc.put(0, -(sc * gc));
            qr.flush();
            qc.flush();
            done = true;
            return;
        }
        uint32_t move;
        if (i == 0) {
            move = 2;
        } else if (j == 0) {
            move = 1;
        } else {
            const int s = (i - 1) / kGradStrip;
            if (s != cur_s) {
                const int loc = s - g * K;
                tcs = tab_cs[loc];
                tbase = tab_base[loc];
                cur_s = s;
            }
            const int64_t widx = (int64_t)tbase + (j - tcs);
            if ((uint64_t)widx >= (uint64_t)dir_cap) {
                // a word outside this lane's directions (tables that do not
                // belong to this job): NaN gradients, no read
                const float qn = __int_as_float(0x7fc00000);
                qr.put(i, qn);
                qc.put(j, qn);
                qr.flush();
                qc.flush();
                done = true;
                return;
            }
            const int64_t grp = widx >> 3;
            if (grp != cur_grp) {
                const uint4 *src = reinterpret_cast<const uint4 *>(dirs + dir_index(grp << 3, gtid, nth));
                ga = src[0];
                gb = src[1];
                cur_grp = grp;
            }
            const int e = (int)(widx & 7);
            const uint4 h = (e & 4) ? gb : ga;
            const uint32_t lo2 = (e & 2) ? h.z : h.x;
            const uint32_t hi2 = (e & 2) ? h.w : h.y;
            const uint32_t word = (e & 1) ? hi2 : lo2;
            move = (word >> (2 * ((i - 1) - s * kGradStrip))) & 3u;
        }
        if (move != 2) {  // leaving row i
            qr.put(i, sc * gr);
            gr = 0.0f;
            i -= 1;
        }
        if (move != 1) {  // leaving column j
            qc.put(j, -(sc * gc));
            gc = 0.0f;
            j -= 1;
        }
        if (i < first_row) {
            qr.flush();
            qc.flush();
            return;
        }
        if (move != 2) ri = B.R[i];
        if (move != 1) cj = B.C[j];
    }
}

// The backward geometry of item t (nothing for t >= n_items, an empty series
// or a zero upstream gradient): dtw items transposed so that the rows are the
// shorter series; an item longer than the planned rows gets NaN gradients,
// never zeros.  g: the upstream gradient of the item.
__device__ __forceinline__ void bwd_setup(const Dtw32Job &J, int64_t t, BwdItem &B, double &g) {
    constexpr int S = kGradStrip;
    const float qnan = __int_as_float(0x7fc00000);
    g = 0.0;
    if (t >= J.n_items) return;
    Item it = load_item(J, t);
    int64_t cx, cy;
    if (J.item_x) {
        cx = J.item_x[t];
        cy = J.item_y[t];
    } else {
        cy = t / J.nx;
        cx = t - cy * J.nx;
    }
    float *gx = J.grad_x ? J.grad_x + cx * J.gx_stride : nullptr;
    float *gy = J.grad_y ? J.grad_y + cy * J.gy_stride : nullptr;
    g = J.grad_out ? J.grad_out[t] : 1.0;
    if (it.n < 1 || it.m < 1 || g == 0.0) return;
    if (it.m >= J.ring_cols || it.n >= J.ring_cols) {
        if (gx)
            for (int i = 0; i < it.n; i++) atomicAdd(gx + i, qnan);
        if (gy)
            for (int j = 0; j < it.m; j++) atomicAdd(gy + j, qnan);
        return;
    }
    if (!J.weights && it.n > it.m) {  // rows: the shorter series (dtw)
        B.R = it.Y;
        B.C = it.X;
        B.GR = gy;
        B.GC = gx;
        B.capR = J.y_len;
        B.capC = J.x_len;
        B.n = it.m;
        B.m = it.n;
    } else {
        B.R = it.X;
        B.C = it.Y;
        B.GR = gx;
        B.GC = gy;
        B.capR = J.x_len;
        B.capC = J.y_len;
        B.n = it.n;
        B.m = it.m;
    }
    B.r = it.r;
    B.mx = imax(0, B.m - B.n) + B.r;
    B.mn = imax(0, B.n - B.m);
    B.lo = -(B.mn + B.r - 1);
    B.width = (B.mx - 1) - B.lo + 1;
    B.nstrips = B.n > 1 ? (B.n - 2) / S + 1 : 0;
}

template <bool W>
__global__ void __launch_bounds__(kBwdBlock) dtw32_backward_kernel(const Dtw32Job J) {
    __shared__ int tab_cs_all[kBwdBlock / 32][kMaxSegStrips];
    __shared__ int tab_base_all[kBwdBlock / 32][kMaxSegStrips];
    // per lane 8 staged direction words, stride 33 words between slots so the
    // lanes of a warp hit different banks
    __shared__ uint32_t stage_all[kBwdBlock * 33 / 4 + 8 * 33];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    int *tab_cs = tab_cs_all[wid];
    int *tab_base = tab_base_all[wid];
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    float2 *ring = J.ring + gtid;
    float2 *ckpt = J.ckpt ? J.ckpt + gtid : nullptr;
    const int64_t slot = (int64_t)J.ring_cols * nth;  // elements per checkpoint row
    uint32_t *dirs = J.dirs;
    uint32_t *stage = stage_all + (threadIdx.x >> 5) * (32 * 8 + 8) + (threadIdx.x & 31);
    const int K = J.seg_strips;
    const float *__restrict__ w = J.weights;
    const float qnan = __int_as_float(0x7fc00000);
    for (;;) {
        const int64_t base = take_items(J.queue, lane);
        if (base >= J.n_items) break;
        const int64_t t = base + lane;
        BwdItem B;
        double g = 0.0;
        bwd_setup(J, t, B, g);
        const int nstr_w = __reduce_max_sync(FULL, B.nstrips);
        const int nseg_w = nstr_w > 0 ? (nstr_w + K - 1) / K : 1;
        const bool fits = nseg_w - 1 <= J.n_ckpt;
        HL result = hl_inf();
        bool ok = fits;
        // pass 1: checkpoints at the segment boundaries (multi-segment items)
        if (ok && nseg_w > 1) {
            HL dummy = hl_inf();
            bwd_row0<W>(B, w, ring, nth, dummy);
            for (int sg = 0; sg + 1 < nseg_w && ok; sg++) {
                const float2 *src = sg == 0 ? ring : ckpt + (int64_t)(sg - 1) * slot;
                ok = bwd_strips<W, false>(B, sg * K, (sg + 1) * K, src, ring,
                                          ckpt + (int64_t)sg * slot, nullptr, 0, tab_cs,
                                          tab_base, stage, gtid, nth, nth, w, dummy);
            }
        }
        // pass 2: segments from the last, each recomputed with its directions,
        // then the walk through its rows
        const int g_last = B.nstrips > 0 ? (B.nstrips - 1) / K : 0;
        int i = B.n - 1, j = B.m - 1;
        float gr = 0.0f, gcol = 0.0f, sc = 0.0f;
        bool done = B.n < 1;
        for (int sg = nseg_w - 1; sg >= 0 && ok; sg--) {
            if (sg == 0) bwd_row0<W>(B, w, ring, nth, result);
            const float2 *src = sg == 0 ? ring : ckpt + (int64_t)(sg - 1) * slot;
            ok = bwd_strips<W, true>(B, sg * K, imin((sg + 1) * K, nstr_w), src, ring, nullptr,
                                     dirs, J.dir_words, tab_cs, tab_base, stage, gtid, nth, nth,
                                     w, result);
            if (!ok) break;
            __syncwarp();
            if (!done && sg <= g_last) {
                if (sg == g_last) {
                    const double D = sqrt((double)result.h + (double)result.l);
                    sc = D > 0.0 ? (float)(g / D) : 0.0f;
                }
                bwd_walk<W>(B, sg, K, dirs, J.dir_words, tab_cs, tab_base, gtid, nth, w, sc, i,
                            j, gr, gcol, done);
            }
            __syncwarp();
        }
        if (!ok && B.n >= 1) {  // workspace too small for this warp's items
            for (int a = 0; a < B.n; a++) atomicAdd(B.GR + a, qnan);
            for (int b = 0; b < B.m; b++) atomicAdd(B.GC + b, qnan);
        }
    }
}

// ---------------------------------------------------------------------------
// Kept directions: when the direction words of every item fit the workspace
// budget, the forward of a differentiable call stores them (the backward's
// sweep, run once) and the backward only walks the paths.  One region per
// batch of 32 consecutive items (the items a warp takes together): the
// strip tables (cs_w, base) of the batch's sweep, then 32 lanes x cap words
// grouped 8 per lane as in the recompute path.

__device__ __forceinline__ void keep_region(const DirKeep &D, int64_t base, int *&tab_cs,
                                            int *&tab_base, uint32_t *&words) {
    unsigned char *reg = D.base + (base >> 5) * D.batch_bytes;
    tab_cs = reinterpret_cast<int *>(reg);
    tab_base = tab_cs + D.max_strips;
    words = reinterpret_cast<uint32_t *>(reg + D.tab_bytes);
}

// The sweep with directions of every item into its batch region, and the
// distance sqrt(hi + lo) of the same sweep (compensated predecessor choice).
template <bool W>
__global__ void __launch_bounds__(kBwdBlock) dtw32_keep_forward_kernel(const Dtw32Job J,
                                                                      const DirKeep D) {
    __shared__ uint32_t stage_all[kBwdBlock * 33 / 4 + 8 * 33];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    float2 *ring = J.ring + gtid;
    uint32_t *stage = stage_all + (threadIdx.x >> 5) * (32 * 8 + 8) + lane;
    const float *__restrict__ w = J.weights;
    for (;;) {
        const int64_t base = take_items(J.queue, lane);
        if (base >= J.n_items) break;
        const int64_t t = base + lane;
        BwdItem B;
        double g = 0.0;
        bwd_setup(J, t, B, g);
        int *tab_cs, *tab_base;
        uint32_t *words;
        keep_region(D, base, tab_cs, tab_base, words);
        const int nstr_w = __reduce_max_sync(FULL, B.nstrips);
        HL result = hl_inf();
        bwd_row0<W>(B, w, ring, nth, result);
        bool ok = true;
        if (nstr_w > 0)
            ok = bwd_strips<W, true>(B, 0, nstr_w, ring, ring, nullptr, words, D.cap, tab_cs,
                                     tab_base, stage, lane, 32, nth, w, result);
        if (t < J.n_items) {
            double res = __longlong_as_double(0x7ff8000000000000LL);  // NaN: empty or unplanned
            if (ok && B.n >= 1) {
                const double cost = (double)result.h + (double)result.l;
                if (J.out_cost) J.out_cost[t] = cost;
                res = sqrt(cost);
            } else if (J.out_cost) {
                J.out_cost[t] = res;
            }
            J.out[t] = res;
        }
    }
}

// The backward from kept directions: each lane walks its item's path with the
// distance of the kept forward (dist[t]) and adds the gradients as the
// recompute path does.
template <bool W>
__global__ void __launch_bounds__(kBwdBlock) dtw32_keep_walk_kernel(const Dtw32Job J,
                                                                   const DirKeep D,
                                                                   const double *dist) {
    const int lane = threadIdx.x & 31;
    const float *__restrict__ w = J.weights;
    for (;;) {
        const int64_t base = take_items(J.queue, lane);
        if (base >= J.n_items) break;
        const int64_t t = base + lane;
        BwdItem B;
        double g = 0.0;
        bwd_setup(J, t, B, g);
        int *tab_cs, *tab_base;
        uint32_t *words;
        keep_region(D, base, tab_cs, tab_base, words);
        int i = B.n - 1, j = B.m - 1;
        float gr = 0.0f, gcol = 0.0f, sc = 0.0f;
        bool done = B.n < 1;
        if (!done) {
            const double Dv = dist[t];
            // a NaN distance (an item the forward could not sweep) gives NaN
            // gradients, never zeros
            sc = (Dv > 0.0 || Dv != Dv) ? (float)(g / Dv) : 0.0f;
        }
        bwd_walk<W>(B, 0, 1, words, D.cap, tab_cs, tab_base, lane, 32, w, sc, i, j, gr, gcol,
                    done);
    }
}

int dtw32_keep_forward(const Dtw32Job &J, const DirKeep &D, cudaStream_t s) {
    if (J.n_items == 0) return WB_OK;
    WB_CUDA(cudaMemsetAsync(J.queue, 0, sizeof(unsigned long long), s));
    timer_begin("dtw32_keep_forward_kernel", s);
    if (J.weights) dtw32_keep_forward_kernel<true><<<J.grid, kBwdBlock, 0, s>>>(J, D);
    else dtw32_keep_forward_kernel<false><<<J.grid, kBwdBlock, 0, s>>>(J, D);
    timer_end(s);
    WB_LAUNCH_CHECK("dtw32_keep_forward_kernel");
    return WB_OK;
}

int dtw32_keep_walk(const Dtw32Job &J, const DirKeep &D, const double *dist, cudaStream_t s) {
    if (J.n_items == 0) return WB_OK;
    WB_CUDA(cudaMemsetAsync(J.queue, 0, sizeof(unsigned long long), s));
    timer_begin("dtw32_keep_walk_kernel", s);
    if (J.weights) dtw32_keep_walk_kernel<true><<<J.grid, kBwdBlock, 0, s>>>(J, D, dist);
    else dtw32_keep_walk_kernel<false><<<J.grid, kBwdBlock, 0, s>>>(J, D, dist);
    timer_end(s);
    WB_LAUNCH_CHECK("dtw32_keep_walk_kernel");
    return WB_OK;
}

int dtw32_keep_blocks_per_sm(bool walk, bool weighted) {
    int nb = 0;
    cudaError_t e;
    if (walk)
        e = weighted ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &nb, dtw32_keep_walk_kernel<true>, kBwdBlock, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &nb, dtw32_keep_walk_kernel<false>, kBwdBlock, 0);
    else
        e = weighted ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &nb, dtw32_keep_forward_kernel<true>, kBwdBlock, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &nb, dtw32_keep_forward_kernel<false>, kBwdBlock, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nb;
}

template <int S>
static int launch_fwd(const Dtw32Job &J, cudaStream_t s) {
    if (J.weights) dtw32_forward_kernel<S, true><<<J.grid, J.block, 0, s>>>(J);
    else dtw32_forward_kernel<S, false><<<J.grid, J.block, 0, s>>>(J);
    WB_LAUNCH_CHECK("dtw32_forward_kernel");
    return WB_OK;
}

int dtw32_forward(const Dtw32Job &J, int strip, cudaStream_t s) {
    if (J.n_items == 0) return WB_OK;
    WB_CUDA(cudaMemsetAsync(J.queue, 0, sizeof(unsigned long long), s));
    int st;
    timer_begin("dtw32_forward_kernel", s);
    switch (strip) {
        case 4: st = launch_fwd<4>(J, s); break;
        case 8: st = launch_fwd<8>(J, s); break;
        case 16: st = launch_fwd<16>(J, s); break;
        case 24: st = launch_fwd<24>(J, s); break;
        case 32: st = launch_fwd<32>(J, s); break;
        default: return fail(WB_EINVAL, "strip must be one of 4, 8, 16, 24, 32");
    }
    timer_end(s);
    return st;
}

int dtw32_backward(const Dtw32Job &J, cudaStream_t s) {
    if (J.n_items == 0) return WB_OK;
    WB_CUDA(cudaMemsetAsync(J.queue, 0, sizeof(unsigned long long), s));
    timer_begin("dtw32_backward_kernel", s);
    if (J.weights) dtw32_backward_kernel<true><<<J.grid, kBwdBlock, 0, s>>>(J);
    else dtw32_backward_kernel<false><<<J.grid, kBwdBlock, 0, s>>>(J);
    timer_end(s);
    WB_LAUNCH_CHECK("dtw32_backward_kernel");
    return WB_OK;
}

// resident blocks per SM of the kernel a job would launch (persistent grid)
int dtw32_blocks_per_sm(int strip, bool weighted, bool backward, int block) {
    int nb = 0;
    cudaError_t e = cudaSuccess;
    if (backward) {
        e = weighted ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &nb, dtw32_backward_kernel<true>, block, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &nb, dtw32_backward_kernel<false>, block, 0);
    } else {
#define WB_OCC(SS)                                                                    \
    case SS:                                                                          \
        e = weighted ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(                 \
                           &nb, dtw32_forward_kernel<SS, true>, block, 0)             \
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(                 \
                           &nb, dtw32_forward_kernel<SS, false>, block, 0);           \
        break;
        switch (strip) {
            WB_OCC(4)
            WB_OCC(8)
            WB_OCC(16)
            WB_OCC(24)
            WB_OCC(32)
            default: return 0;
        }
#undef WB_OCC
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nb;
}

// Item-order distances -> (nx, ny) row-major matrix.  Full grid: item
// t = j * nx + i holds (x_i, y_j).  Upper (singleton, nx == ny): item
// t = j (j - 1) / 2 + i holds the pair i < j; it is mirrored, the diagonal is 0.
__global__ void grid_to_matrix_kernel(const double *in, int64_t nx, int64_t ny, int upper,
                                      double *out) {
    const int64_t total = nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / ny, j = t - (t / ny) * ny;
        double v;
        if (!upper) {
            v = in[j * nx + i];
        } else if (i == j) {
            v = 0.0;
        } else {
            const int64_t a = i < j ? i : j, b = i < j ? j : i;
            v = in[b * (b - 1) / 2 + a];
        }
        out[t] = v;
    }
}

int launch_grid_to_matrix(const double *in, int64_t nx, int64_t ny, int upper, double *out,
                          cudaStream_t s) {
    if (nx == 0 || ny == 0) return WB_OK;
    int64_t g = (nx * ny + 255) / 256;
    int64_t cap = (int64_t)device_info().sm_count * 16;
    grid_to_matrix_kernel<<<(int)(g < cap ? g : cap), 256, 0, s>>>(in, nx, ny, upper, out);
    WB_LAUNCH_CHECK("grid_to_matrix_kernel");
    return WB_OK;
}

// items of the pairs i < j of n series, ordered by j then i
__global__ void upper_items_kernel(int64_t n, int32_t *ix, int32_t *iy) {
    const int64_t total = n * (n - 1) / 2;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t j = (int64_t)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
        while (j * (j - 1) / 2 > t) j--;
        while ((j + 1) * j / 2 <= t) j++;
        ix[t] = (int32_t)(t - j * (j - 1) / 2);
        iy[t] = (int32_t)j;
    }
}

int launch_upper_items(int64_t n, int32_t *item_x, int32_t *item_y, cudaStream_t s) {
    const int64_t total = n * (n - 1) / 2;
    if (total <= 0) return WB_OK;
    int64_t g = (total + 255) / 256;
    int64_t cap = (int64_t)device_info().sm_count * 16;
    upper_items_kernel<<<(int)(g < cap ? g : cap), 256, 0, s>>>(n, item_x, item_y);
    WB_LAUNCH_CHECK("upper_items_kernel");
    return WB_OK;
}

// valid length of each series: index of the first NaN (EoS or NaN padding)
__global__ void series_lengths_kernel(const float *x, int64_t n_series, int64_t stride, int L,
                                      int32_t *lengths) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = warp; s < n_series; s += nwarps) {
        const float *p = x + s * stride;
        int first = L;
        for (int b = 0; b < L; b += 32) {
            int i = b + lane;
            bool nan = (i < L) && isnan(p[i]);
            unsigned mask = __ballot_sync(0xffffffffu, nan);
            if (mask) {
                first = b + __ffs(mask) - 1;
                break;
            }
        }
        if (lane == 0) lengths[s] = first;
    }
}

int launch_series_lengths(const float *x, int64_t n_series, int64_t stride, int L,
                          int32_t *lengths, cudaStream_t s) {
    if (n_series == 0) return WB_OK;
    int64_t blocks = (n_series * 32 + 255) / 256;
    int64_t cap = (int64_t)device_info().sm_count * 16;
    if (blocks > cap) blocks = cap;
    series_lengths_kernel<<<(int)blocks, 256, 0, s>>>(x, n_series, stride, L, lengths);
    WB_LAUNCH_CHECK("series_lengths_kernel");
    return WB_OK;
}

}  // namespace wb
