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

#include <stdlib.h>
#include <string.h>

#include "argmin.cuh"
#include "elastic_rec.cuh"

namespace wb {

constexpr int kEaThreads = 128;

struct EaChunk {
    int64_t j0 = 0, nc = 0;                 // candidates [j0, j0 + nc)
    int64_t nq = 0;                         // queries
    int64_t ny = 0;                         // row stride of out / key / lower_bound
    const double *cur_dist = nullptr;       // k-th distance after the replayed prefix
    const double *lower_bound = nullptr;    // (nq, ny) or null
    unsigned long long *counter = nullptr;  // next pair of the chunk
    int metric = WB_DTW;
    int xl = 0, yl = 0;
};

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
                const double a = up + J.p;
                nv = nn_min(nn_min(a, left), diag) + d * d;
                left = first ? nv : nv + J.p;
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

// Plan of the early-abandoning kernel: the ring must fit in shared memory
// with at least one block per SM (narrow bands); 0 blocks = not applicable.
static int ea_blocks_per_sm(const ElasticJob &J, int *P_out) {
    const DeviceInfo &dev = device_info();
    const int P = imax(2, ring_len(J.rows.len, J.cols.len, J.band));
    const size_t per_block = (size_t)P * kEaThreads * sizeof(double);
    if (P_out) *P_out = P;
    if (per_block > (size_t)dev.max_smem_optin || per_block + 2048 > (size_t)dev.smem_per_sm)
        return 0;
    int b = (int)(((size_t)dev.smem_per_sm - 1024) / (per_block + 1024));
    return b > 4 ? 4 : b;
}

bool argmin_ea_disabled() {
    const char *e = getenv("WB_GPU_ARGMIN");
    return e && strcmp(e, "all") == 0;
}

int64_t argmin_ea_first_chunk() {
    const char *e = getenv("WB_GPU_ARGMIN");
    if (!e) return 0;
    long long c = atoll(e);
    return c > 0 ? (int64_t)c : 0;
}

bool argmin_ea_supported(const ElasticJob &J) {
    if (J.kind != K_DTW && J.kind != K_WDTW && J.kind != K_ADTW) return false;
    if (J.all_zero || J.mode != PM_ALL || !J.key) return false;
    return ea_blocks_per_sm(J, nullptr) >= 1;
}

int64_t argmin_ea_lanes(const ElasticJob &J) {
    return (int64_t)ea_blocks_per_sm(J, nullptr) * device_info().sm_count * kEaThreads;
}

int launch_argmin_ea(const ElasticJob &J, int metric, int xl, int yl, int64_t j0, int64_t nc,
                     int64_t ny, const double *cur_dist, const double *lower_bound,
                     unsigned long long *counter, cudaStream_t s) {
    int P = 0;
    const int bps = ea_blocks_per_sm(J, &P);
    if (bps < 1) return fail(WB_EINVAL, "early-abandoning argmin needs a narrow band");
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
    int64_t want = (total + kEaThreads - 1) / kEaThreads;
    int64_t cap = (int64_t)bps * device_info().sm_count;
    const int grid = (int)(want < cap ? want : cap);
    const size_t smem = (size_t)P * kEaThreads * sizeof(double);
    auto run = [&](auto kfn) -> int {
        WB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        kfn<<<grid, kEaThreads, smem, s>>>(J, C, P);
        WB_LAUNCH_CHECK("argmin_ea_kernel");
        return WB_OK;
    };
    switch (J.kind) {
        case K_DTW: return run(argmin_ea_kernel<K_DTW>);
        case K_WDTW: return run(argmin_ea_kernel<K_WDTW>);
        case K_ADTW: return run(argmin_ea_kernel<K_ADTW>);
    }
    return fail(WB_EINVAL, "unsupported early-abandoning kernel");
}

}  // namespace wb
