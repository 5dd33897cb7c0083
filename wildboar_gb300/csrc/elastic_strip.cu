// elastic_strip.cu -- elastic recurrences swept in register strips.
//
// The pairwise / paired distance of every elastic metric, in FP64 with the
// reference's exact operations (bit-identical to the two-row recurrences of
// distance/_elastic.pyx) and in FP32 with compensated (hi, lo) accumulation.
//
// One thread per pair.  A thread sweeps its band in strips of S rows: for
// each column c the S cells (i0 + k, c) are updated top-down in registers
// (P[k] holds cell (i0 + k, c - 1) on entry and (i0 + k, c) on exit); the row
// above the strip comes from a global ring laid out [column][thread]
// (coalesced) into which the previous strip wrote its bottom row.  Ring
// traffic is one load and one store per S cells, so the arithmetic pipe, not
// memory, bounds the kernel even for full-width bands.
//
// What the reference reads outside the band (its two-row buffers) is
// reproduced per cell from the cell's position against the band of its row
// i, columns [js(i), je(i)), js = max(0, i - mn - r + 1), je = min(m, i + mx):
//   * right of the band (c >= je): the value the reference writes at je --
//     +inf for the dtw family (dtw, wdtw, adtw), 0 for the others;
//   * left of the band (c < js, read only at c = js - 1): +inf for the dtw
//     family, 0 for lcss / edr / erp / twe; msm reads stale buffer content,
//     the cell two rows up, (i - 2, js - 1);
//   * column -1 when js = 0 (column 0 for msm): the boundary column, +inf
//     (dtw family, twe), 0 (lcss, edr), the gap sum gx (erp), the cumulative
//     cost cy(i) (msm); the corner above row 0 is 0 for erp and twe.
// Row 0 of dtw / adtw / msm is the reference's cumulative first row; lcss,
// edr, erp and twe start from an initial row (0, 0, gy, +inf).

#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "argmin.cuh"

namespace wb {

#define WB_SINF64 __longlong_as_double(0x7ff0000000000000LL)
#define WB_SINF32 __int_as_float(0x7f800000)

// --------------------------------------------------------------------------
// arithmetic policies

struct ArF64 {
    using V = double;  // cumulative value
    using E = double;  // element / cost
    using R = double;  // ring entry
    __device__ static V inf() { return WB_SINF64; }
    __device__ static V zero() { return 0.0; }
    __device__ static V of(double v) { return v; }
    __device__ static E el(double v) { return v; }
    __device__ static V add(V a, E b) { return a + b; }
    __device__ static V vmin(V a, V b) { return nn_min(a, b); }
    __device__ static V vmin_any(V a, V b) { return cy_min(a, b); }
    __device__ static V vmax(V a, V b) { return nn_max(a, b); }
    __device__ static R pack(V v) { return v; }
    __device__ static V unpack(R r) { return r; }
    __device__ static double value(V v) { return v; }
    __device__ static E sub(E a, E b) { return a - b; }
    __device__ static E mul(E a, E b) { return a * b; }
    __device__ static E absv(E a) { return fabs(a); }
};

struct HLs {
    float h, l;
};

struct ArF32 {
    using V = HLs;
    using E = float;
    using R = float2;
    __device__ static V inf() { return HLs{WB_SINF32, 0.0f}; }
    __device__ static V zero() { return HLs{0.0f, 0.0f}; }
    __device__ static V of(double v) {
        const float h = (float)v;
        return HLs{h, (float)(v - (double)h)};
    }
    __device__ static E el(double v) { return (float)v; }
    // TwoSum: the rounding error of a.h + b joins the lo part
    __device__ static V add(V a, E b) {
        const float s = __fadd_rn(a.h, b);
        const float bb = __fsub_rn(s, a.h);
        const float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b, bb));
        return HLs{s, __fadd_rn(a.l, err)};
    }
    __device__ static V vmin(V a, V b) { return b.h < a.h ? b : a; }
    __device__ static V vmin_any(V a, V b) { return b.h < a.h ? b : a; }
    __device__ static V vmax(V a, V b) { return b.h > a.h ? b : a; }
    __device__ static R pack(V v) { return make_float2(v.h, v.l); }
    __device__ static V unpack(R r) { return HLs{r.x, r.y}; }
    __device__ static double value(V v) { return (double)v.h + (double)v.l; }
    __device__ static E sub(E a, E b) { return __fsub_rn(a, b); }
    __device__ static E mul(E a, E b) { return __fmul_rn(a, b); }
    __device__ static E absv(E a) { return fabsf(a); }
};

template <class A>
constexpr bool is_f64() {
    return std::is_same<A, ArF64>::value;
}

// _msm_cost, distance/_elastic.pyx:1583-1587: float arguments and float
// differences; the FP64 form adds them in double as the reference does.
template <class A>
__device__ __forceinline__ typename A::E msm_cost(float x, float y, float z, float c) {
    if ((y <= x && x <= z) || (y >= x && x >= z)) return (typename A::E)c;
    const float a = fabsf(__fsub_rn(x, y));
    const float b = fabsf(__fsub_rn(x, z));
    if constexpr (is_f64<A>()) return (double)c + f2d_nonneg(b < a ? b : a);  // exact widening
    else return __fadd_rn(c, b < a ? b : a);
}

template <class A>
__device__ __forceinline__ typename A::E weight(const void *w, int k) {
    if constexpr (is_f64<A>()) return __ldg(static_cast<const double *>(w) + k);
    else return __ldg(static_cast<const float *>(w) + k);
}

template <int KIND>
struct Kt {
    static constexpr bool dtwf =
        KIND == K_DTW || KIND == K_WDTW || KIND == K_ADTW || KIND == K_ADTW_ANY;
    static constexpr int first_row = (dtwf || KIND == K_MSM) ? 1 : 0;
    static constexpr int first_col = KIND == K_MSM ? 1 : 0;
};

// per-pair constants of a metric
template <class A>
struct PairCtx {
    typename A::E eps, g, pen, s2;
    long long eb;                  // eps_bits(eps) (FP64 lcss / edr comparisons)
    float c;                       // msm cost
    typename A::V gx_sum, gy_sum;  // erp gap sums
    const double *gY;              // erp: |y_j - g| of the column series
    const void *w;                 // weights (double for FP64, float for FP32)
    const double *stab;            // twe: (2 stiffness) k, FP64
};

// Per-row values of a strip (registers).
template <int S, class A>
struct Rows {
    typename A::E x[S];   // x_i
    typename A::E rx[S];  // erp |x_i - g|; twe |x_{i-1} - x_i|
    typename A::E px[S];  // twe x_{i-1}
    float xf[S];          // msm x_i as float
    float pxf[S];         // msm x_{i-1} as float
};

// One strip column.  Pin[k]: cell (i0 + k, c - 1); Pout[k]: cell (i0 + k, c);
// bup = cell (i0 - 1, c), bdiag = cell (i0 - 1, c - 1).  PP: Pin and Pout are
// two register sets that alternate between columns (no cell value is copied
// to free its register); otherwise they are the same array, updated in place.
// MASK: some rows of the strip are outside their band at this column or past
// the series end.
template <int KIND, int S, class A, bool MASK, bool KEY = false, bool PP = false>
__device__ __forceinline__ void column(const typename A::V (&Pin)[S], typename A::V (&Pout)[S],
                                       typename A::V bup, typename A::V bdiag,
                                       const Rows<S, A> &Rw, typename A::E yc,
                                       typename A::E yp, typename A::E colv, float ycf,
                                       float ypf, int c, int i0, int lo, int hi, int valid,
                                       const PairCtx<A> &C, typename A::V (&rmin)[S]) {
    using V = typename A::V;
    using E = typename A::E;
    constexpr bool DTWF = Kt<KIND>::dtwf;
    V dg = bdiag;
    V up = bup;
#pragma unroll
    for (int k = 0; k < S; k++) {
        if (PP && k > 0) {
            dg = Pin[k - 1];
            up = Pout[k - 1];
        }
        const V lf = Pin[k];
        const int d = c - (i0 + k);
        V nv;
        if constexpr (KIND == K_DTW || KIND == K_WDTW) {
            const E v = A::sub(Rw.x[k], yc);
            E cst = A::mul(v, v);
            if constexpr (KIND == K_WDTW)
                cst = A::mul(cst, weight<A>(C.w, (!MASK || k < valid) ? abs(d) : 0));
            nv = A::add(A::vmin(A::vmin(up, lf), dg), cst);
        } else if constexpr (KIND == K_ADTW || KIND == K_ADTW_ANY) {
            const E v = A::sub(Rw.x[k], yc);
            V mv;
            // min(up + p, left + p) == min(up, left) + p (monotone rounding, the
            // same operand): one (compensated) addition fewer per cell; exact in
            // FP64, within the compensated form's error in FP32
            if constexpr (KIND == K_ADTW) mv = A::vmin(A::add(A::vmin(up, lf), C.pen), dg);
            else mv = A::vmin_any(A::add(A::vmin_any(up, lf), C.pen), dg);
            nv = A::add(mv, A::mul(v, v));
        } else if constexpr (KIND == K_LCSS || KIND == K_WLCSS) {
            const E v = A::absv(A::sub(Rw.x[k], yc));
            E wt = A::el(1.0);
            if constexpr (KIND == K_WLCSS)
                wt = weight<A>(C.w, (!MASK || k < valid) ? abs(d) : 0);
            bool match;
            if constexpr (is_f64<A>()) match = abs_bits(A::sub(Rw.x[k], yc)) <= C.eb;  // integer pipe
            else match = v <= C.eps;
            nv = match ? A::add(dg, wt) : A::vmax(lf, up);
        } else if constexpr (KIND == K_EDR) {
            const E v = A::absv(A::sub(Rw.x[k], yc));
            if constexpr (is_f64<A>()) {
                // the comparison on the integer pipe; min(a + 1, b + 1) ==
                // min(a, b) + 1 exactly (monotone rounding): a match gives
                // min(dg, min(up, lf) + 1), a mismatch min(dg, up, lf) + 1
                const bool match = abs_bits(A::sub(Rw.x[k], yc)) < C.eb;
                const V mul = A::vmin(up, lf);
                const V r = A::add(match ? mul : A::vmin(dg, mul), 1.0);
                nv = match ? A::vmin(dg, r) : r;
            } else {
                // the same one-addition form (edit counts are small integers,
                // exact in FP32)
                const bool match = v < C.eps;
                const V mul = A::vmin(up, lf);
                const V r = A::add(match ? mul : A::vmin(dg, mul), A::el(1.0));
                nv = match ? A::vmin(dg, r) : r;
            }
        } else if constexpr (KIND == K_ERP) {
            const V a = A::add(dg, A::absv(A::sub(Rw.x[k], yc)));
            const V b = A::add(up, Rw.rx[k]);
            const V cc = A::add(lf, colv);
            nv = A::vmin(a, A::vmin(b, cc));
        } else if constexpr (KIND == K_MSM) {
            const V a = A::add(dg, A::absv(A::sub(Rw.x[k], yc)));
            const V b = A::add(up, msm_cost<A>(Rw.xf[k], Rw.pxf[k], ycf, C.c));
            const V e = A::add(lf, msm_cost<A>(ycf, Rw.xf[k], ypf, C.c));
            nv = A::vmin(A::vmin(a, b), e);
        } else {  // K_TWE
            // min((up + dx) + pen, (lf + dy) + pen) == min(up + dx, lf + dy) + pen
            // (monotone rounding, the same operand added last): exact in FP64
            const V del = A::add(A::vmin(A::add(up, Rw.rx[k]), A::add(lf, colv)), C.pen);
            E st;
            if constexpr (is_f64<A>())
                st = __ldg(C.stab + ((!MASK || k < valid) ? abs(d) : 0));
            else
                st = A::mul(C.s2, (float)abs(d));
            const V match = A::add(
                A::add(A::add(dg, A::absv(A::sub(Rw.x[k], yc))), A::absv(A::sub(Rw.px[k], yp))),
                st);
            nv = A::vmin(del, match);
        }
        if (MASK) {
            if (d > hi) {
                nv = DTWF ? A::inf() : A::zero();
            } else if (d < lo) {
                if constexpr (KIND == K_MSM) nv = (k < 2) ? bup : Pout[k >= 2 ? k - 2 : 0];
                else nv = DTWF ? A::inf() : A::zero();
            }
        }
        if constexpr (KEY) {
            // the row minimum of the two-row recurrences: in-band cells only
            if (!MASK || (d >= lo && d <= hi && k < valid))
                rmin[k] = KIND == K_ADTW_ANY ? A::vmin_any(rmin[k], nv) : A::vmin(rmin[k], nv);
        }
        if (!PP) {
            dg = lf;
            up = nv;
        }
        Pout[k] = nv;
    }
}

// The recurrence of one pair, resumable strip by strip: sweep_begin writes
// the row above the first strip into the ring, sweep_strip sweeps one strip
// (and with KEY the minimum of each of its rows over the row's band, the
// abandon key's terms); sweep_pair runs them all and returns cell
// (n - 1, m - 1).
template <class A>
struct SweepState {
    typename A::V result, cy, stale_next;
    typename A::E xprev;
    float xprevf;
    int i0, pstart, pend;
};

// true when the first row already completes the pair (st.result holds it)
template <int KIND, int S, class A>
__device__ __forceinline__ bool sweep_begin(const double *__restrict__ X, int n,
                                            const double *__restrict__ Y, int m, int r,
                                            const PairCtx<A> &C, typename A::R *__restrict__ ring,
                                            int64_t nth, SweepState<A> &st) {
    using V = typename A::V;
    using E = typename A::E;
    constexpr int FR = Kt<KIND>::first_row;
    const int mx = imax(0, m - n) + r;
    const int lim = imin(m, mx);
    const V INF = A::inf(), ZERO = A::zero();
    const double x0d = X[0];
    const E x0 = A::el(x0d);
    const float x0f = (float)x0d;
    const float y0f = (float)__ldg(Y);

    // msm: column 0 is the cumulative cost cy(i); with one column it is the result
    V cy = ZERO;
    if constexpr (KIND == K_MSM) {
        cy = A::add(ZERO, A::absv(A::sub(x0, A::el(__ldg(Y)))));
        if (m == 1) {
            float xpf = x0f;
            for (int i = 1; i < n; i++) {
                const float xif = (float)X[i];
                cy = A::add(cy, msm_cost<A>(xif, xpf, y0f, C.c));
                xpf = xif;
            }
            st.result = cy;
            return true;
        }
    }

    // ---- the row above the first strip
    V acc = ZERO;
    if constexpr (KIND == K_DTW || KIND == K_WDTW || KIND == K_ADTW || KIND == K_ADTW_ANY) {
        E v = A::sub(x0, A::el(__ldg(Y)));
        E c0 = A::mul(v, v);
        if constexpr (KIND == K_WDTW) c0 = A::mul(c0, weight<A>(C.w, 0));
        acc = A::add(ZERO, c0);
        ring[0] = A::pack(acc);
        for (int j = 1; j < lim; j++) {
            v = A::sub(x0, A::el(__ldg(Y + j)));
            E cj = A::mul(v, v);
            if constexpr (KIND == K_WDTW) cj = A::mul(cj, weight<A>(C.w, j - 1));
            acc = A::add(acc, cj);
            ring[(int64_t)j * nth] = A::pack(acc);
        }
        if (mx < m) ring[(int64_t)mx * nth] = A::pack(INF);
    } else if constexpr (KIND == K_MSM) {
        acc = cy;
        ring[0] = A::pack(acc);
        float yprev = y0f;
        for (int j = 1; j < lim; j++) {
            const float yj = (float)__ldg(Y + j);
            acc = A::add(acc, msm_cost<A>(yj, yprev, x0f, C.c));
            ring[(int64_t)j * nth] = A::pack(acc);
            yprev = yj;
        }
        if (mx < m) {
            acc = A::add(acc, msm_cost<A>((float)__ldg(Y + mx), (float)__ldg(Y + mx - 1), x0f,
                                          C.c));
            ring[(int64_t)mx * nth] = A::pack(acc);
        }
    } else {
        V init;
        if constexpr (KIND == K_ERP) init = C.gy_sum;
        else if constexpr (KIND == K_TWE) init = INF;
        else init = ZERO;
        for (int j = 0; j < lim; j++) ring[(int64_t)j * nth] = A::pack(init);
        if (mx < m) ring[(int64_t)mx * nth] = A::pack(init);
    }
    if (n == FR) {  // one row: lim == m, acc is cell (0, m - 1)
        st.result = acc;
        return true;
    }
    st.result = ZERO;
    st.cy = cy;
    st.stale_next = ZERO;  // msm: cell (i0 - 2, js(i0) - 1)
    st.xprev = FR == 1 ? x0 : A::el(0.0);  // x_{i0 - 1} (twe: 0 above row 0)
    st.xprevf = x0f;
    st.i0 = FR;
    st.pstart = 0;
    st.pend = mx < m ? mx + 1 : lim;
    return false;
}

// rows st.i0 .. st.i0 + rows - 1; returns rows
template <int KIND, int S, class A, bool KEY>
__device__ __forceinline__ int sweep_strip(const double *__restrict__ X, int n,
                                           const double *__restrict__ Y, int m, int r,
                                           const PairCtx<A> &C, typename A::R *__restrict__ ring,
                                           int64_t nth, SweepState<A> &st,
                                           typename A::V (&rmin)[S]) {
    using V = typename A::V;
    using E = typename A::E;
    constexpr bool DTWF = Kt<KIND>::dtwf;
    constexpr int FC = Kt<KIND>::first_col;
    const int mx = imax(0, m - n) + r, mn = imax(0, n - m);
    const int lo = -(mn + r - 1), hi = mx - 1;
    const V INF = A::inf(), ZERO = A::zero();
    const V ROOB = DTWF ? INF : ZERO;
    const float y0f = (float)__ldg(Y);
    const int i0 = st.i0;
    const int pstart = st.pstart, pend = st.pend;
    const int rows = imin(S, n - i0);
    Rows<S, A> Rw;
    V cyk[S];
    V cy = st.cy;
    const V cy_prev = cy;
#pragma unroll
    for (int k = 0; k < S; k++) {
        const double xd = (k < rows) ? X[i0 + k] : 0.0;
        Rw.x[k] = A::el(xd);
        if constexpr (KIND == K_ERP) Rw.rx[k] = A::absv(A::sub(Rw.x[k], C.g));
        if constexpr (KIND == K_TWE) {
            Rw.px[k] = (k == 0) ? st.xprev : Rw.x[k > 0 ? k - 1 : 0];
            Rw.rx[k] = A::absv(A::sub(Rw.px[k], Rw.x[k]));
        }
        if constexpr (KIND == K_MSM) {
            Rw.xf[k] = (float)xd;
            Rw.pxf[k] = (k == 0) ? st.xprevf : Rw.xf[k > 0 ? k - 1 : 0];
            cy = A::add(cy, msm_cost<A>(Rw.xf[k], Rw.pxf[k], y0f, C.c));
            cyk[k] = cy;
        }
        if constexpr (KEY) rmin[k] = KIND == K_MSM ? cyk[k] : INF;
    }
    st.cy = cy;
    const int cstart = imax(FC, i0 - mn - r + 1);
    const int cend = imin(m, i0 + rows - 1 + mx);
    int bstart = cend, bend = cend;
    if (rows == S) {
        bstart = imax(cstart, i0 + S - 1 + lo);
        bend = imin(cend, i0 + hi + 1);
        if (bstart >= bend) bstart = bend = cend;
    }
    const bool at_boundary = (cstart == FC);
    V P[S], Q[S];
#pragma unroll
    for (int k = 0; k < S; k++) {
        V v;
        if (at_boundary) {
            if constexpr (KIND == K_ERP) v = C.gx_sum;
            else if constexpr (KIND == K_MSM) v = cyk[k];
            else if constexpr (DTWF || KIND == K_TWE) v = INF;
            else v = ZERO;
        } else {
            if constexpr (KIND == K_MSM) v = st.stale_next;
            else v = DTWF ? INF : ZERO;
        }
        P[k] = v;
    }
    V bdiag;
    if (at_boundary) {
        if constexpr (KIND == K_ERP) bdiag = i0 == 0 ? ZERO : C.gx_sum;
        else if constexpr (KIND == K_TWE) bdiag = i0 == 0 ? ZERO : INF;
        else if constexpr (KIND == K_MSM) bdiag = cy_prev;
        else bdiag = DTWF ? INF : ZERO;
    } else {
        bdiag = A::unpack(ring[(int64_t)(cstart - 1) * nth]);
    }
    const bool last = (i0 + rows == n);
    const int cnext = imax(FC, i0 + S - mn - r + 1);  // msm: next strip's first column
    auto ld_up = [&](int c) -> V {
        return (c >= pstart && c < pend) ? A::unpack(ring[(int64_t)c * nth]) : ROOB;
    };
    auto ld_y = [&](int c) -> double { return c < cend ? __ldg(Y + c) : 0.0; };
    V nb0 = ld_up(cstart), nb1 = ld_up(cstart + 1);
    double ny0 = ld_y(cstart), ny1 = ld_y(cstart + 1);
    E yp = cstart > 0 ? A::el(__ldg(Y + cstart - 1)) : A::el(0.0);
    float ypf = cstart > 0 ? (float)__ldg(Y + cstart - 1) : 0.0f;
    // column c from the cells of column c - 1 (Pin) into Pout; the compensated
    // FP32 forms alternate two register sets (PP), FP64 and msm (whose masked
    // cells read the stale cell two rows up, and which measured slower that
    // way) update P in place
    constexpr bool PP = !is_f64<A>() && KIND != K_MSM;
    auto step = [&](int c, const V(&Pin)[S], V(&Pout)[S]) {
        const V bup = nb0;
        const double ycd = ny0;
        nb0 = nb1;
        ny0 = ny1;
        nb1 = ld_up(c + 2);
        ny1 = ld_y(c + 2);
        const E yc = A::el(ycd);
        const float ycf = (float)ycd;
        E colv = A::el(0.0);
        if constexpr (KIND == K_ERP) colv = A::el(__ldg(C.gY + c));
        if constexpr (KIND == K_TWE) colv = A::absv(A::sub(yp, yc));
        if (c >= bstart && c < bend)
            column<KIND, S, A, false, KEY, PP>(Pin, Pout, bup, bdiag, Rw, yc, yp, colv, ycf,
                                               ypf, c, i0, lo, hi, rows, C, rmin);
        else
            column<KIND, S, A, true, KEY, PP>(Pin, Pout, bup, bdiag, Rw, yc, yp, colv, ycf,
                                              ypf, c, i0, lo, hi, rows, C, rmin);
        if constexpr (KIND == K_MSM) {
            if (c == cnext - 1) st.stale_next = Pout[S - 2];
        }
        if (last && c == m - 1) {
#pragma unroll
            for (int k = 0; k < S; k++)
                if (k < rows) st.result = Pout[k];  // ends at Pout[rows - 1], no indexed P
        }
        ring[(int64_t)c * nth] = A::pack(Pout[S - 1]);
        bdiag = bup;
        yp = yc;
        ypf = ycf;
    };
    if constexpr (PP) {
        int c = cstart;
        for (; c + 1 < cend; c += 2) {
            step(c, P, Q);
            step(c + 1, Q, P);
        }
        if (c < cend) step(c, P, Q);
    } else {
        for (int c = cstart; c < cend; c++) step(c, P, P);
    }
    st.pstart = cstart;
    st.pend = cend;
    // carried into the next strip (only the last strip has rows < S)
    if constexpr (KIND == K_TWE) st.xprev = Rw.x[S - 1];
    if constexpr (KIND == K_MSM) st.xprevf = Rw.xf[S - 1];
    st.i0 = i0 + rows;
    return rows;
}

template <int KIND, int S, class A>
__device__ __forceinline__ typename A::V sweep_pair(const double *__restrict__ X, int n,
                                    const double *__restrict__ Y, int m, int r,
                                    const PairCtx<A> &C, typename A::R *__restrict__ ring,
                                    int64_t nth) {
    SweepState<A> st;
    if (sweep_begin<KIND, S, A>(X, n, Y, m, r, C, ring, nth, st)) return st.result;
    typename A::V unused[S];
    while (st.i0 < n) sweep_strip<KIND, S, A, false>(X, n, Y, m, r, C, ring, nth, st, unused);
    return st.result;
}

__device__ __forceinline__ double finish_value(const ElasticJob &J, double v) {
    switch (J.result) {
        case R_SQRT: return sqrt(v);
        case R_LCSS: return 1.0 - v / (double)imin(J.len_norm_rows, J.len_norm_cols);
        case R_EDR: return v / (double)imax(J.len_norm_rows, J.len_norm_cols);
        default: return v;
    }
}

constexpr int kStripThreads = 128;

template <int KIND, int S, class A>
__global__ void __launch_bounds__(kStripThreads)
    strip_pairs_kernel(const ElasticJob J, typename A::R *ring_base) {
    const int lane = threadIdx.x & 31;
    const int64_t gtid = (int64_t)blockIdx.x * kStripThreads + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * kStripThreads;
    const int64_t warp = gtid >> 5;
    const int64_t nwarps = nth >> 5;
    typename A::R *ring = ring_base + gtid;
    const int n = J.rows.len, m = J.cols.len;

    auto run = [&](int64_t rs, int64_t cs) -> double {
        if (J.all_zero) return 0.0;
        PairCtx<A> C;
        double epsd = J.eps;
        if constexpr (KIND == K_EDR) {
            if (J.std_rows) epsd = cy_max(J.std_rows[rs], J.std_cols[cs]) / 4.0;
        }
        C.eps = A::el(epsd);
        C.eb = eps_bits(epsd);
        C.g = A::el(J.g);
        C.pen = A::el(KIND == K_TWE ? J.penalty + J.stiffness : J.p);
        C.s2 = A::el(J.stiffness * 2.0);
        C.c = (float)J.c;
        C.gx_sum = A::zero();
        C.gy_sum = A::zero();
        C.gY = nullptr;
        if constexpr (KIND == K_ERP) {
            C.gx_sum = A::of(J.gsum_rows[rs]);
            C.gy_sum = A::of(J.gsum_cols[cs]);
            C.gY = J.gtab_cols + cs * (int64_t)m;
        }
        if constexpr (is_f64<A>()) C.w = J.weights;
        else C.w = J.weights32;
        C.stab = J.stab;
        const double *X = J.rows.base + rs * J.rows.stride;
        const double *Y = J.cols.base + cs * J.cols.stride;
        typename A::V v = sweep_pair<KIND, S, A>(X, n, Y, m, J.band, C, ring, nth);
        return finish_value(J, A::value(v));
    };

    if (J.mode == PM_PAIRED) {
        for (int64_t s = gtid; s < J.rows.count; s += nth) J.out[s] = run(s, s);
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
        const double d = run(rs, cs);
        J.out[rs * J.out_ld + cs] = d;
        if (J.mode == PM_UPPER) J.out[cs * J.out_ld + rs] = d;
    }
}

// --------------------------------------------------------------------------
// argmin chunks with early abandoning, one pair per lane at a time (the lane
// queue of argmin_ea.cu): after every strip the lane folds the strip's row
// minima into the pair's key and stops the pair once the key exceeds the
// threshold bound of the chunk (the reference abandons it then as well).
template <int KIND, int S>
__global__ void __launch_bounds__(kStripThreads)
    strip_ea_kernel(const ElasticJob J, const EaChunk Ch, double *ring_base, int64_t ring_ld) {
    using A = ArF64;
    using V = A::V;
    const int64_t gtid = (int64_t)blockIdx.x * kStripThreads + threadIdx.x;
    double *ring = ring_base + gtid * ring_ld;
    const int n = J.rows.len, m = J.cols.len;
    const double INF = WB_SINF64;
    const int64_t total = Ch.nq * Ch.nc;

    int64_t p = (int64_t)atomicAdd(Ch.counter, 1ULL);
    int64_t qi = 0, cj = 0;
    const double *X = nullptr, *Y = nullptr;
    double bound = INF, kmax = -INF;
    PairCtx<A> C;
    SweepState<A> st;
    bool finished = false;

    auto next_pair = [&]() {
        while (p < total) {
            qi = p / Ch.nc;
            cj = Ch.j0 + (p - qi * Ch.nc);
            const double d = Ch.cur_dist[qi];
            const int64_t o = qi * Ch.ny + cj;
            if (Ch.lower_bound && Ch.lower_bound[o] >= d) {
                // the replay skips it: lb >= D_a >= every later k-th distance
                J.out[o] = INF;
                J.key[o] = INF;
                p = (int64_t)atomicAdd(Ch.counter, 1ULL);
                continue;
            }
            bound = abandon_threshold(Ch.metric, d, Ch.xl, Ch.yl);
            C.eps = J.eps;
            if constexpr (KIND == K_EDR) {
                if (J.std_rows) C.eps = cy_max(J.std_rows[qi], J.std_cols[cj]) / 4.0;
            }
            C.eb = eps_bits(C.eps);
            C.g = J.g;
            C.pen = KIND == K_TWE ? J.penalty + J.stiffness : J.p;
            C.s2 = J.stiffness * 2.0;
            C.c = (float)J.c;
            C.gx_sum = 0.0;
            C.gy_sum = 0.0;
            C.gY = nullptr;
            if constexpr (KIND == K_ERP) {
                C.gx_sum = J.gsum_rows[qi];
                C.gy_sum = J.gsum_cols[cj];
                C.gY = J.gtab_cols + cj * (int64_t)m;
            }
            C.w = J.weights;
            C.stab = J.stab;
            X = J.rows.base + qi * J.rows.stride;
            Y = J.cols.base + cj * J.cols.stride;
            kmax = -INF;
            finished = sweep_begin<KIND, S, A>(X, n, Y, m, J.band, C, ring, 1, st);
            return;
        }
    };
    next_pair();

    while (p < total) {
        if (!finished) {
            V rmin[S];
            const int rows = sweep_strip<KIND, S, A, true>(X, n, Y, m, J.band, C, ring, 1, st,
                                                           rmin);
#pragma unroll
            for (int k = 0; k < S; k++)
                if (k < rows) kmax = fmax(kmax, rmin[k]);
            finished = st.i0 >= n;
        }
        if (finished || kmax > bound) {
            const int64_t o = qi * Ch.ny + cj;
            J.out[o] = finished ? finish_value(J, st.result) : INF;
            J.key[o] = kmax;
            p = (int64_t)atomicAdd(Ch.counter, 1ULL);
            next_pair();
        }
    }
}

constexpr int kStripEaRowsLight = 16;  // edr, lcss, wlcss, adtw
constexpr int kStripEaRowsHeavy = 8;   // erp, msm, twe

bool strip_ea_supported(const ElasticJob &J) {
    switch (J.kind) {
        case K_EDR:
        case K_ERP:
        case K_TWE:
        case K_LCSS:
        case K_WLCSS:
        case K_ADTW_ANY:
            break;
        case K_MSM:
            if (J.cols.len < 2) return false;  // one column: no strips, no key
            break;
        default:
            return false;
    }
    return !J.all_zero && J.mode == PM_ALL && J.key && J.rows.len >= 1 && J.cols.len >= 1;
}

template <int KIND, int S>
static int strip_ea_occupancy() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, strip_ea_kernel<KIND, S>, kStripThreads,
                                                  0);
    return nb;
}

int strip_ea_blocks_per_sm(const ElasticJob &J) {
    switch (J.kind) {
        case K_EDR: return strip_ea_occupancy<K_EDR, kStripEaRowsLight>();
        case K_LCSS: return strip_ea_occupancy<K_LCSS, kStripEaRowsLight>();
        case K_WLCSS: return strip_ea_occupancy<K_WLCSS, kStripEaRowsLight>();
        case K_ADTW_ANY: return strip_ea_occupancy<K_ADTW_ANY, kStripEaRowsLight>();
        case K_ERP: return strip_ea_occupancy<K_ERP, kStripEaRowsHeavy>();
        case K_MSM: return strip_ea_occupancy<K_MSM, kStripEaRowsHeavy>();
        case K_TWE: return strip_ea_occupancy<K_TWE, kStripEaRowsHeavy>();
    }
    return 0;
}

int launch_strip_ea(const ElasticJob &J, const EaChunk &Ch, double *ring, int64_t ring_ld,
                    int grid, cudaStream_t s) {
    if (Ch.nq * Ch.nc == 0) return WB_OK;
    auto run = [&](auto kfn) -> int {
        kfn<<<grid, kStripThreads, 0, s>>>(J, Ch, ring, ring_ld);
        WB_LAUNCH_CHECK("strip_ea_kernel");
        return WB_OK;
    };
    switch (J.kind) {
        case K_EDR: return run(strip_ea_kernel<K_EDR, kStripEaRowsLight>);
        case K_LCSS: return run(strip_ea_kernel<K_LCSS, kStripEaRowsLight>);
        case K_WLCSS: return run(strip_ea_kernel<K_WLCSS, kStripEaRowsLight>);
        case K_ADTW_ANY: return run(strip_ea_kernel<K_ADTW_ANY, kStripEaRowsLight>);
        case K_ERP: return run(strip_ea_kernel<K_ERP, kStripEaRowsHeavy>);
        case K_MSM: return run(strip_ea_kernel<K_MSM, kStripEaRowsHeavy>);
        case K_TWE: return run(strip_ea_kernel<K_TWE, kStripEaRowsHeavy>);
    }
    return fail(WB_EINVAL, "no strip early-abandoning kernel for this metric kind");
}

// --------------------------------------------------------------------------
// host side

template <int KIND, int S, class A>
static int strip_grid(const ElasticJob &J) {
    const DeviceInfo &dev = device_info();
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, strip_pairs_kernel<KIND, S, A>,
                                                  kStripThreads, 0);
    if (nb < 1) nb = 1;
    int64_t work;
    if (J.mode == PM_PAIRED) work = J.rows.count;
    else work = ((J.rows.count + 31) / 32) * 32 * J.cols.count;
    int64_t want = (work + kStripThreads - 1) / kStripThreads;
    int64_t cap = (int64_t)nb * dev.sm_count;
    int64_t g = want < cap ? want : cap;
    return (int)(g < 1 ? 1 : g);
}

template <int KIND, int S, class A>
static int strip_launch(const ElasticJob &J, Workspace *ws, size_t *bytes) {
    const int grid = strip_grid<KIND, S, A>(J);
    const size_t nring = (size_t)(J.cols.len + 1) * grid * kStripThreads;
    if (bytes) {
        *bytes = align256(nring * sizeof(typename A::R));
        return WB_OK;
    }
    typename A::R *ring = ws->take<typename A::R>(nring);
    if (!ring) return fail(WB_ENOMEM, "workspace reservation exceeded");
    cudaStream_t s = ws->stream();
    timer_begin(is_f64<A>() ? "strip_pairs_kernel<f64>" : "strip_pairs_kernel<f32>", s);
    strip_pairs_kernel<KIND, S, A><<<grid, kStripThreads, 0, s>>>(J, ring);
    timer_end(s);
    WB_LAUNCH_CHECK("strip_pairs_kernel");
    return WB_OK;
}

template <class A>
static int strip_dispatch(const ElasticJob &J, Workspace *ws, size_t *bytes) {
    constexpr int SL = is_f64<A>() ? 16 : 16;  // light recurrences
    constexpr int SH = 8;                      // erp, msm, twe (more per-row registers)
    switch (J.kind) {
        case K_DTW: return strip_launch<K_DTW, SL, A>(J, ws, bytes);
        case K_WDTW: return strip_launch<K_WDTW, SL, A>(J, ws, bytes);
        case K_ADTW: return strip_launch<K_ADTW, SL, A>(J, ws, bytes);
        case K_ADTW_ANY: return strip_launch<K_ADTW_ANY, SL, A>(J, ws, bytes);
        case K_LCSS: return strip_launch<K_LCSS, SL, A>(J, ws, bytes);
        case K_WLCSS: return strip_launch<K_WLCSS, SL, A>(J, ws, bytes);
        case K_EDR: return strip_launch<K_EDR, SL, A>(J, ws, bytes);
        case K_ERP: return strip_launch<K_ERP, SH, A>(J, ws, bytes);
        case K_MSM: return strip_launch<K_MSM, SH, A>(J, ws, bytes);
        case K_TWE: return strip_launch<K_TWE, SH, A>(J, ws, bytes);
    }
    return fail(WB_EINVAL, "no strip kernel for this metric kind");
}

// The strip kernel can serve every pairwise / paired job without an abandon
// key (argmin keeps the ring kernel, which also reports per-row minima).
// WB_GPU_ELASTIC=ring / =strip force the FP64 choice (comparisons); without
// it the FP64 path picks with `prefer_strip_f64`.
bool strip_supported(const ElasticJob &J) {
    if (J.kind == K_EUCLID || J.key != nullptr || J.rows.len < 1 || J.cols.len < 1) return false;
    const char *e = getenv("WB_GPU_ELASTIC");
    return !(e && strcmp(e, "ring") == 0);
}

bool strip_forced() {
    const char *e = getenv("WB_GPU_ELASTIC");
    return e && strcmp(e, "strip") == 0;
}

size_t strip_workspace_bytes(const ElasticJob &J, bool fp32) {
    size_t b = 0;
    if (fp32) strip_dispatch<ArF32>(J, nullptr, &b);
    else strip_dispatch<ArF64>(J, nullptr, &b);
    return b;
}

int launch_strip(const ElasticJob &J, Workspace &ws, bool fp32) {
    if (J.rows.count == 0 || J.cols.count == 0) return WB_OK;
    return fp32 ? strip_dispatch<ArF32>(J, &ws, nullptr) : strip_dispatch<ArF64>(J, &ws, nullptr);
}

// --------------------------------------------------------------------------
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
