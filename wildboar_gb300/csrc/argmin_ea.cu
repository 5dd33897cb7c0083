// argmin_ea.cu -- early-abandoned candidate distances for argmin_distance.
//
// The reference's k-nearest loop (_ArgMinBatch.__call__,
// distance/_cdistance.pyx:1302-1345) calls eadistance with the heap's current
// k-th distance; the dtw-family recurrences (dtw_distance with its threshold,
// distance/_elastic.pyx:869-940, and adtw_distance :943-1008) stop at the
// first row whose minimum exceeds the squared threshold.  That threshold only
// decreases while j advances, so after replaying candidates [0, a) the k-th
// distance D_a bounds every later threshold: a pair (i, j >= a) whose running
// largest row minimum exceeds D_a^2 is abandoned by the reference as well.
// The host therefore walks the candidates in chunks [a, b) of growing size;
// each chunk's pairs are computed here with the bound of the replayed prefix
// and stop as soon as they cross it, then the replay kernel advances the
// heap over the chunk with the exact thresholds.
//
// Work layout.  Abandoning makes the pair lengths unequal, so lanes do not
// share a pair schedule: every lane takes pairs one at a time from a global
// counter and advances its own pair one recurrence row per loop iteration;
// a lane whose pair finished or crossed the bound takes the next pair at
// once, and the warp keeps all lanes busy until the chunk's pairs run out.
// The live band of each lane's pair stays in a shared-memory ring
// [k][thread] (conflict-free for any mix of ring positions across lanes).
// Every cell performs the reference's IEEE double operations in its order
// (compiled with -fmad=false), so a pair that is not abandoned gets the
// same distance and key as the all-pairs kernel.
//
// Wide bands, whose ring does not fit in shared memory, run the strip form:
// the lane sweeps its pair in strips of S rows held in registers (row 0, the
// reference's cumulative first row, is the first strip's top row), keeps
// each strip's bottom row in a per-lane global ring (contiguous per lane, so
// a lane's consecutive columns share cache lines whatever the other lanes
// do) and checks the bound after each strip.

#include <stdlib.h>
#include <string.h>

#include "argmin.cuh"
#include "elastic_rec.cuh"

namespace wb {

constexpr int kEaThreads = 128;

// KIND: K_DTW (dtw, ddtw on slopes), K_WDTW (wdtw, wddtw), K_ADTW (penalty >= 0)
template <int KIND>
__global__ void __launch_bounds__(kEaThreads)
argmin_ea_kernel(const ElasticJob J, const EaChunk C, int P) {
    const RingS ring{(int)threadIdx.x, kEaThreads};
    const int n = J.rows.len, m = J.cols.len, r = J.band;
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const double INF = WB_INF;
    const int64_t total = C.nq * C.nc;

    int64_t p = (int64_t)atomicAdd(C.counter, 1ULL);
    int64_t qi = 0, cj = 0;
    const double *X = nullptr, *Y = nullptr;
    double bound = INF, kmax = -INF;
    int i = 0;

    // take pairs until one needs computing (lower-bound skips are settled here)
    auto next_pair = [&]() {
        while (p < total) {
            qi = p / C.nc;
            cj = C.j0 + (p - qi * C.nc);
            const double d = C.cur_dist[qi];
            if (C.lower_bound && C.lower_bound[qi * C.ny + cj] >= d) {
                // the replay skips it: lb >= D_a >= every later k-th distance
                J.out[qi * C.ny + cj] = INF;
                J.key[qi * C.ny + cj] = INF;
                p = (int64_t)atomicAdd(C.counter, 1ULL);
                continue;
            }
            bound = abandon_threshold(C.metric, d, C.xl, C.yl);
            X = J.rows.base + qi * J.rows.stride;
            Y = J.cols.base + cj * J.cols.stride;
            i = 0;
            kmax = -INF;
            return;
        }
    };
    next_pair();

    while (p < total) {
        // row i of the pair; row 0 is the cumulative first row of the
        // reference (its "previous row" reads as +inf, the first cell's
        // diagonal as 0: min(inf, inf, 0) + c = c exactly)
        const bool first = i == 0;
        const int js = first ? 0 : imax(0, i - mn - r + 1);
        const int je = imin(m, i + mx);
        const double xi = X[i];
        int q = js % P;
        double diag = first ? 0.0 : (js > 0 ? ring.ld(wrap_dec(q, P)) : INF);
        double left = INF;
        double rmin = INF;
        for (int j = js; j < je; j++) {
            const double up = first ? INF : ring.ld(q);
            const double d = xi - ldg(Y + j);
            double nv;
            if constexpr (KIND == K_DTW) {
                nv = nn_min(nn_min(up, left), diag) + d * d;
                left = nv;
            } else if constexpr (KIND == K_WDTW) {
                // the reference's first row weighs column j with w[j - 1]
                const int wi = first ? imax(j - 1, 0) : abs(i - j);
                nv = nn_min(nn_min(up, left), diag) + (d * d) * ldg(J.weights + wi);
                left = nv;
            } else {
                // left holds the previous cell; min(up + p, left + p) ==
                // min(up, left) + p exactly; row 0 moves left without p
                const double t = nn_min(up, left) + J.p;
                nv = nn_min(first ? left : t, diag) + d * d;
                left = nv;
            }
            ring.st(q, nv);
            rmin = nn_min(rmin, nv);
            diag = up;
            q = wrap_inc(q, P);
        }
        if (je < m) ring.st(q, INF);
        if (!first) kmax = fmax(kmax, rmin);
        i += 1;
        const bool done = i == n;
        if (done || kmax > bound) {
            const int64_t o = qi * C.ny + cj;
            J.out[o] = done ? sqrt(ring.ld((m - 1) % P)) : INF;
            J.key[o] = kmax;
            p = (int64_t)atomicAdd(C.counter, 1ULL);
            next_pair();
        }
    }
}

// Strip form (wide bands).  Cells outside their row's band are +inf, the
// value the reference's buffers hold there for the dtw family; row 0 reads
// +inf above it and a 0 diagonal at column 0, which reproduces its
// cumulative first row (and, for wdtw, its weight index j - 1; for adtw, its
// penalty-free left move).
template <int KIND, int S>
__global__ void __launch_bounds__(kEaThreads)
argmin_ea_strip_kernel(const ElasticJob J, const EaChunk C, double *ring_base, int64_t ring_ld) {
    const int64_t gtid = (int64_t)blockIdx.x * kEaThreads + threadIdx.x;
    double *ring = ring_base + gtid * ring_ld;
    const int n = J.rows.len, m = J.cols.len, r = J.band;
    const int mx = imax(0, m - n) + r;
    const int mn = imax(0, n - m);
    const int lo = -(mn + r - 1);                   // band: lo <= c - i <= mx - 1
    const unsigned span = (unsigned)(mx - 1 - lo);
    const double INF = WB_INF;
    const int64_t total = C.nq * C.nc;

    int64_t p = (int64_t)atomicAdd(C.counter, 1ULL);
    int64_t qi = 0, cj = 0;
    const double *X = nullptr, *Y = nullptr;
    double bound = INF, kmax = -INF;
    int i0 = 0, pstart = 0, pend = 0;

    auto next_pair = [&]() {
        while (p < total) {
            qi = p / C.nc;
            cj = C.j0 + (p - qi * C.nc);
            const double d = C.cur_dist[qi];
            if (C.lower_bound && C.lower_bound[qi * C.ny + cj] >= d) {
                J.out[qi * C.ny + cj] = INF;
                J.key[qi * C.ny + cj] = INF;
                p = (int64_t)atomicAdd(C.counter, 1ULL);
                continue;
            }
            bound = abandon_threshold(C.metric, d, C.xl, C.yl);
            X = J.rows.base + qi * J.rows.stride;
            Y = J.cols.base + cj * J.cols.stride;
            i0 = 0;
            pstart = pend = 0;
            kmax = -INF;
            return;
        }
    };
    next_pair();

    while (p < total) {
        const int rows = imin(S, n - i0);
        double x[S], P[S], rmin[S];
#pragma unroll
        for (int k = 0; k < S; k++) {
            x[k] = (k < rows) ? X[i0 + k] : 0.0;
            P[k] = INF;  // column cstart - 1: left of the band, or column -1
            rmin[k] = INF;
        }
        const int cstart = imax(0, i0 - mn - r + 1);
        const int cend = imin(m, i0 + rows - 1 + mx);
        // cell (i0 - 1, cstart - 1): written by the previous strip when
        // cstart > 0 (js grows by at most one per row)
        double bdiag = i0 == 0 ? 0.0 : (cstart > 0 ? ring[cstart - 1] : INF);
        for (int c = cstart; c < cend; c++) {
            const double bup = (i0 > 0 && c >= pstart && c < pend) ? ring[c] : INF;
            const double yc = ldg(Y + c);
            double dg = bdiag, up = bup;
#pragma unroll
            for (int k = 0; k < S; k++) {
                const double lf = P[k];
                const int d = c - (i0 + k);
                const bool in_band = (unsigned)(d - lo) <= span && k < rows;
                const double v = x[k] - yc;
                double nv;
                if constexpr (KIND == K_DTW) {
                    nv = nn_min(nn_min(up, lf), dg) + v * v;
                } else if constexpr (KIND == K_WDTW) {
                    int wi = (k == 0 && i0 == 0) ? imax(c - 1, 0) : abs(d);
                    wi = in_band ? wi : 0;
                    nv = nn_min(nn_min(up, lf), dg) + (v * v) * ldg(J.weights + wi);
                } else {
                    // min(up + p, lf + p) == min(up, lf) + p exactly; row 0
                    // (up = +inf) moves left without p
                    const double t = nn_min(up, lf) + J.p;
                    nv = nn_min((k == 0 && i0 == 0) ? lf : t, dg) + v * v;
                }
                nv = in_band ? nv : INF;
                rmin[k] = nn_min(rmin[k], nv);
                dg = lf;
                up = nv;
                P[k] = nv;
            }
            ring[c] = P[S - 1];
            bdiag = bup;
        }
        // the last strip ends at column m - 1 (cend = m for its last row);
        // the running assignment leaves P[rows - 1] without an indexed P
        double result = 0.0;
#pragma unroll
        for (int k = 0; k < S; k++) {
            if (k < rows && i0 + k >= 1) kmax = fmax(kmax, rmin[k]);
            if (k < rows) result = P[k];
        }
        pstart = cstart;
        pend = cend;
        i0 += rows;
        const bool done = i0 == n;
        if (done || kmax > bound) {
            const int64_t o = qi * C.ny + cj;
            J.out[o] = done ? sqrt(result) : INF;
            J.key[o] = kmax;
            p = (int64_t)atomicAdd(C.counter, 1ULL);
            next_pair();
        }
    }
}

constexpr int kEaStripRows = 16;

// Plan of the early-abandoning kernels: the shared-memory ring form when at
// least two blocks of rings fit per SM, else the strip form.
struct EaPlan {
    int form = 0;  // 0: not applicable, 1: shared-memory ring, 2: dtw strips, 3: generic strips
    int P = 0;
    int blocks_per_sm = 0;
    bool chunked = false;  // the metric's threshold grows with the k-th distance
};

template <int KIND>
static int strip_blocks_per_sm() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &nb, argmin_ea_strip_kernel<KIND, kEaStripRows>, kEaThreads, 0);
    return nb;
}

static EaPlan ea_plan(const ElasticJob &J) {
    EaPlan pl;
    if (J.all_zero || J.mode != PM_ALL || !J.key) return pl;
    if (J.rows.len < 1 || J.cols.len < 1) return pl;
    const DeviceInfo &dev = device_info();
    pl.P = imax(2, ring_len(J.rows.len, J.cols.len, J.band));
    const size_t per_block = (size_t)pl.P * kEaThreads * sizeof(double);
    int b = 0;
    if (per_block <= (size_t)dev.max_smem_optin && per_block + 2048 <= (size_t)dev.smem_per_sm)
        b = (int)(((size_t)dev.smem_per_sm - 1024) / (per_block + 1024));
    if (J.kind != K_DTW && J.kind != K_WDTW && J.kind != K_ADTW) {
        if (!strip_ea_supported(J)) return pl;
        pl.chunked = J.kind == K_EDR || J.kind == K_ERP || J.kind == K_MSM || J.kind == K_TWE;
        // lcss / wlcss / negative-penalty adtw cannot abandon out of order; the
        // strip sweep only replaces the all-pairs kernel's global ring
        if (!pl.chunked && b >= 1) return pl;
        pl.blocks_per_sm = strip_ea_blocks_per_sm(J);
        if (pl.blocks_per_sm >= 1) pl.form = 3;
        return pl;
    }
    pl.chunked = true;
    const char *force = getenv("WB_GPU_ARGMIN_FORM");
    const bool strip_forced = force && strcmp(force, "strip") == 0;
    if (b >= 2 && !strip_forced) {
        pl.form = 1;
        pl.blocks_per_sm = b > 4 ? 4 : b;
        return pl;
    }
    switch (J.kind) {
        case K_DTW: b = strip_blocks_per_sm<K_DTW>(); break;
        case K_WDTW: b = strip_blocks_per_sm<K_WDTW>(); break;
        default: b = strip_blocks_per_sm<K_ADTW>(); break;
    }
    if (b < 1) return pl;
    pl.form = 2;
    pl.blocks_per_sm = b;
    return pl;
}

bool argmin_ea_disabled() {
    const char *e = getenv("WB_GPU_ARGMIN");
    return e && strcmp(e, "all") == 0;
}

int64_t argmin_pair_budget() {
    const char *e = getenv("WB_GPU_ARGMIN_BATCH");
    const long long v = e ? atoll(e) : 0;
    return v > 0 ? (int64_t)v : ((int64_t)1 << 27);  // 2 GiB of distances and keys
}

int64_t argmin_ea_first_chunk() {
    const char *e = getenv("WB_GPU_ARGMIN");
    if (!e) return 0;
    long long c = atoll(e);
    return c > 0 ? (int64_t)c : 0;
}

bool argmin_ea_supported(const ElasticJob &J) { return ea_plan(J).form != 0; }

int64_t argmin_ea_lanes(const ElasticJob &J) {
    return (int64_t)ea_plan(J).blocks_per_sm * device_info().sm_count * kEaThreads;
}

bool argmin_ea_chunked(const ElasticJob &J) { return ea_plan(J).chunked; }

// per-lane ring of the strip forms: columns 0 .. m (the generic sweep may
// write column m's boundary value)
static int64_t ea_ring_ld(const ElasticJob &J) { return (int64_t)J.cols.len + 1; }

size_t argmin_ea_ring_bytes(const ElasticJob &J) {
    const EaPlan pl = ea_plan(J);
    if (pl.form < 2) return 0;
    return align256((size_t)argmin_ea_lanes(J) * (size_t)ea_ring_ld(J) * sizeof(double));
}

int launch_argmin_ea(const ElasticJob &J, int metric, int xl, int yl, int64_t j0, int64_t nc,
                     int64_t ny, const double *cur_dist, const double *lower_bound,
                     unsigned long long *counter, double *ring, cudaStream_t s) {
    const EaPlan pl = ea_plan(J);
    if (pl.form == 0) return fail(WB_EINVAL, "no early-abandoning argmin kernel for this job");
    if (pl.form >= 2 && !ring) return fail(WB_EINVAL, "strip ring missing");
    EaChunk C;
    C.j0 = j0;
    C.nc = nc;
    C.nq = J.rows.count;
    C.ny = ny;
    C.cur_dist = cur_dist;
    C.lower_bound = lower_bound;
    C.counter = counter;
    C.metric = metric;
    C.xl = xl;
    C.yl = yl;
    const int64_t total = C.nq * nc;
    if (total == 0) return WB_OK;
    // the grid is the resident one: every lane loops over the chunk's pairs
    // (the strip ring is sized for exactly these lanes)
    const int grid = pl.blocks_per_sm * device_info().sm_count;
    if (pl.form == 1) {
        const size_t smem = (size_t)pl.P * kEaThreads * sizeof(double);
        auto run = [&](auto kfn) -> int {
            WB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
            kfn<<<grid, kEaThreads, smem, s>>>(J, C, pl.P);
            WB_LAUNCH_CHECK("argmin_ea_kernel");
            return WB_OK;
        };
        switch (J.kind) {
            case K_DTW: return run(argmin_ea_kernel<K_DTW>);
            case K_WDTW: return run(argmin_ea_kernel<K_WDTW>);
            case K_ADTW: return run(argmin_ea_kernel<K_ADTW>);
        }
    } else if (pl.form == 3) {
        return launch_strip_ea(J, C, ring, ea_ring_ld(J), grid, s);
    } else {
        const int64_t ld = ea_ring_ld(J);
        auto run = [&](auto kfn) -> int {
            kfn<<<grid, kEaThreads, 0, s>>>(J, C, ring, ld);
            WB_LAUNCH_CHECK("argmin_ea_strip_kernel");
            return WB_OK;
        };
        switch (J.kind) {
            case K_DTW: return run(argmin_ea_strip_kernel<K_DTW, kEaStripRows>);
            case K_WDTW: return run(argmin_ea_strip_kernel<K_WDTW, kEaStripRows>);
            case K_ADTW: return run(argmin_ea_strip_kernel<K_ADTW, kEaStripRows>);
        }
    }
    return fail(WB_EINVAL, "unsupported early-abandoning kernel");
}

}  // namespace wb
