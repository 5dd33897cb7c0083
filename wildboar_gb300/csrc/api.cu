// api.cu -- the extern "C" entry points declared in include/wbgpu.h.
//
// Each call: validates its arguments, stages host inputs into the stream's
// device workspace (one 2-D copy per series set gathers the requested dim),
// prepares per-metric tables on the device, launches the kernels and copies
// host outputs back.  Host-side work is limited to argument checks and the
// metric constructor's parameter tables (wdtw weights with libm exp, exactly
// as WeightedDtwMetric.reset computes them, distance/_elastic.pyx:3333-3341).

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <vector>

#include "dtw32.cuh"
#include "elastic.cuh"
#include "subseq.cuh"

namespace wb {

// --------------------------------------------------------------------------
// errors

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return WB_ENOMEM;
    return WB_ECUDA;
}

void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Armed fault: the site, and how many matching events pass before it fires
// (once).  WB_GPU_INJECT_FAULT="reserve|launch|wait[:skip]" arms it when the
// library is first used; wb_inject_fault arms or clears it at run time.
static std::mutex g_inject_mu;
static int g_inject_site = INJ_NONE;
static int64_t g_inject_skip = 0;
static bool g_inject_env_read = false;

static void inject_from_env() {
    if (g_inject_env_read) return;
    g_inject_env_read = true;
    const char *e = getenv("WB_GPU_INJECT_FAULT");
    if (!e || !*e) return;
    std::string v(e);
    std::string name = v.substr(0, v.find(':'));
    int64_t skip = 0;
    if (v.find(':') != std::string::npos) skip = atoll(v.c_str() + v.find(':') + 1);
    if (name == "reserve") g_inject_site = INJ_RESERVE;
    else if (name == "launch") g_inject_site = INJ_LAUNCH;
    else if (name == "wait") g_inject_site = INJ_WAIT;
    g_inject_skip = skip;
}

bool injected(int site) {
    std::lock_guard<std::mutex> g(g_inject_mu);
    inject_from_env();
    if (g_inject_site != site) return false;
    if (g_inject_skip > 0) {
        g_inject_skip--;
        return false;
    }
    g_inject_site = INJ_NONE;
    return true;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// --------------------------------------------------------------------------
// device info

const DeviceInfo &device_info() {
    static thread_local DeviceInfo cache[64];
    static thread_local bool have[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!have[dev]) {
        DeviceInfo d;
        d.device = dev;
        cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&d.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&d.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        if (d.sm_count <= 0) d.sm_count = 1;
        cache[dev] = d;
        have[dev] = true;
    }
    return cache[dev];
}

// --------------------------------------------------------------------------
// workspace

static std::mutex g_arena_mu;
static std::map<std::pair<int, cudaStream_t>, Arena *> g_arenas;

static Arena *arena_for(cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(g_arena_mu);
    auto key = std::make_pair(dev, s);
    auto it = g_arenas.find(key);
    if (it != g_arenas.end()) return it->second;
    Arena *a = new Arena();
    g_arenas[key] = a;
    return a;
}

Workspace::Workspace(cudaStream_t stream)
    : arena_(arena_for(stream)), stream_(stream), lock_(arena_->mu) {
    arena_->used = 0;
}

Workspace::~Workspace() { arena_->used = 0; }

int Workspace::reserve(size_t bytes) {
    if (injected(INJ_RESERVE))
        return fail(WB_ENOMEM, "cannot allocate device workspace (injected fault)");
    bytes = align256(bytes) + 4096;
    if (bytes > arena_->cap) {
        if (arena_->base) {
            // cudaFree waits for the device, so earlier work on this stream
            // that still reads the arena has finished
            cudaError_t e = cudaFree(arena_->base);
            arena_->base = nullptr;
            arena_->cap = 0;
            if (e != cudaSuccess) return cuda_fail(e, "cudaFree(workspace)");
        }
        size_t cap = bytes + bytes / 4;
        cudaError_t e = cudaMalloc((void **)&arena_->base, cap);
        if (e != cudaSuccess) {
            cudaGetLastError();
            arena_->base = nullptr;
            if (e != cudaErrorMemoryAllocation) return cuda_fail(e, "cudaMalloc(workspace)");
            return fail(WB_ENOMEM, "cannot allocate " + std::to_string(cap) +
                                       " bytes of device workspace");
        }
        arena_->cap = cap;
    }
    arena_->used = 0;
    return WB_OK;
}

// --------------------------------------------------------------------------
// argument handling

static int check_series(const wb_series *s, const char *name, bool allow_f32 = false) {
    if (!s) return fail(WB_EINVAL, std::string(name) + " is NULL");
    if (s->n < 0 || s->n_dims < 1 || s->n_timestep < 1)
        return fail(WB_EINVAL, std::string(name) + " has an invalid shape");
    if (s->n > 0 && !s->data) return fail(WB_EINVAL, std::string(name) + " data is NULL");
    if (s->dtype != WB_F64 && !(allow_f32 && s->dtype == WB_F32))
        return fail(WB_EINVAL, std::string(name) + " must be float64");
    if (s->n_timestep > (int64_t)1 << 28)
        return fail(WB_EINVAL, std::string(name) + " has too many timesteps");
    return WB_OK;
}

static bool is_elastic(int metric) {
    return metric >= WB_DTW && metric <= WB_TWE;
}

static bool weighted(int metric) {
    return metric == WB_WDTW || metric == WB_WDDTW || metric == WB_WLCSS;
}

static bool derivative(int metric) { return metric == WB_DDTW || metric == WB_WDDTW; }

// Bytes needed to stage one dim of a series set on the device.
static size_t stage_bytes(const wb_series *s) {
    return s->on_device ? 0 : align256((size_t)s->n * s->n_timestep * sizeof(double));
}

// Series set of one dim: device data used in place, host data gathered into
// the workspace with one strided copy.
static int stage(const wb_series *s, int64_t dim, Workspace &ws, SeriesSet &out) {
    out.count = s->n;
    out.len = (int)s->n_timestep;
    const double *base = static_cast<const double *>(s->data);
    if (s->on_device) {
        out.base = base + dim * s->n_timestep;
        out.stride = s->n_dims * s->n_timestep;
        return WB_OK;
    }
    WB_TAKE(d, double, ws, (size_t)s->n * s->n_timestep);
    if (s->n > 0) {
        WB_CUDA(cudaMemcpy2DAsync(d, s->n_timestep * sizeof(double),
                                  base + dim * s->n_timestep,
                                  s->n_dims * s->n_timestep * sizeof(double),
                                  s->n_timestep * sizeof(double), s->n,
                                  cudaMemcpyHostToDevice, ws.stream()));
    }
    out.base = d;
    out.stride = s->n_timestep;
    return WB_OK;
}

// logistic weights of WeightedDtwMetric.reset (distance/_elastic.pyx:3333-3341)
static std::vector<double> logistic_weights(int64_t n, double g) {
    std::vector<double> w((size_t)std::max<int64_t>(n, 1));
    for (int64_t i = 0; i < n; i++)
        w[i] = 1.0 / (1.0 + std::exp(-g * ((double)i - (double)n / 2.0)));
    return w;
}

// Everything a recurrence job needs beyond the two series sets.
struct MetricPrep {
    ElasticJob job;
    std::vector<double> weights;
    size_t bytes = 0;  // workspace bytes needed by `build`
};

// Fill the metric fields of `job` (kind, result, band, parameters) for the
// metric's distance (ea = false) or eadistance (ea = true) entry.
static int metric_fields(int metric, const wb_params *p, int xl, int yl, bool ea,
                         ElasticJob &J) {
    J.len_norm_rows = xl;
    J.len_norm_cols = yl;
    int rl = std::min(xl, yl);
    if (metric != WB_EUCLIDEAN && !(p->r >= 0.0 && p->r <= 1.0))
        return fail(WB_EINVAL, "r must be in [0, 1]");
    switch (metric) {
        case WB_EUCLIDEAN:
            J.kind = K_EUCLID;
            J.result = R_SQRT;
            J.band = 1;
            return WB_OK;
        case WB_DTW:
        case WB_WDTW:
            J.kind = metric == WB_DTW ? K_DTW : K_WDTW;
            J.result = R_SQRT;
            J.band = compute_r(rl, p->r);
            return WB_OK;
        case WB_DDTW:
        case WB_WDDTW:
            J.kind = metric == WB_DDTW ? K_DTW : K_WDTW;
            J.result = R_SQRT;
            // DerivativeDtwMetric: _distance uses the series lengths,
            // _eadistance the slope lengths (distance/_elastic.pyx:3280, 3308)
            J.band = compute_r(ea ? rl - 2 : rl, p->r);
            return WB_OK;
        case WB_ADTW:
            J.kind = p->p >= 0.0 ? K_ADTW : K_ADTW_ANY;
            J.result = R_SQRT;
            J.p = p->p;
            J.band = compute_r(rl, p->r);
            return WB_OK;
        case WB_LCSS:
        case WB_WLCSS:
            if (!(p->epsilon > 0.0)) return fail(WB_EINVAL, "epsilon must be > 0");
            J.kind = metric == WB_LCSS ? K_LCSS : K_WLCSS;
            J.result = R_LCSS;
            J.eps = p->epsilon;
            J.band = compute_r(rl, p->r);
            return WB_OK;
        case WB_EDR:
            J.kind = K_EDR;
            J.result = R_EDR;
            J.eps = p->epsilon;
            // EdrMetric.eadistance passes min(X.shape[2], X.shape[2])
            // (distance/_elastic.pyx:3833)
            J.band = compute_r(ea ? xl : rl, p->r);
            return WB_OK;
        case WB_ERP:
            J.kind = K_ERP;
            J.result = R_IDENT;
            J.g = p->g;
            J.band = compute_r(rl, p->r);
            return WB_OK;
        case WB_MSM:
            J.kind = K_MSM;
            J.result = R_IDENT;
            J.c = p->c;
            J.band = compute_r(rl, p->r);
            return WB_OK;
        case WB_TWE:
            J.kind = K_TWE;
            J.result = R_IDENT;
            J.penalty = p->penalty;
            J.stiffness = p->stiffness;
            J.band = compute_r(rl, p->r);
            return WB_OK;
    }
    return fail(WB_EUNSUPPORTED, "unsupported metric id " + std::to_string(metric));
}

// Workspace bytes of the per-metric tables for rows R and columns C.
static size_t table_bytes(int metric, const wb_params *p, const SeriesSet &R,
                          const SeriesSet &C, int64_t nR, int64_t nC, int lR, int lC) {
    size_t b = 0;
    if (derivative(metric))
        b += align256((size_t)nR * std::max(lR - 2, 0) * 8) +
             align256((size_t)nC * std::max(lC - 2, 0) * 8);
    if (weighted(metric)) b += align256((size_t)std::max(lR, lC) * 8);
    if (metric == WB_EDR && std::isnan(p->epsilon)) b += align256(nR * 8) + align256(nC * 8);
    if (metric == WB_ERP) b += align256(nR * 8) + align256(nC * 8) + align256((size_t)nC * lC * 8);
    if (metric == WB_TWE) b += align256((size_t)nC * lC * 8) + align256((size_t)std::max(lR, lC) * 8);
    return b;
}

// Build the device tables of a recurrence job whose row/column sets are
// already staged.  `same` marks the singleton path (rows and columns are the
// same array, reset(x, x)).  wlen_* are the widths that size the weights.
static int build_tables(int metric, const wb_params *p, ElasticJob &J, Workspace &ws,
                        bool same, int wlen_rows, int wlen_cols) {
    cudaStream_t s = ws.stream();
    if (derivative(metric)) {
        if (std::min(J.rows.len, J.cols.len) < 3) {
            J.all_zero = 1;
        } else {
            SeriesSet dr = J.rows, dc = J.cols;
            WB_TAKE(dR, double, ws, (size_t)J.rows.count * (J.rows.len - 2));
            WB_TRY(launch_slopes(J.rows, dR, s));
            dr.base = dR;
            dr.stride = J.rows.len - 2;
            dr.len = J.rows.len - 2;
            if (same) {
                dc = dr;
            } else {
                WB_TAKE(dC, double, ws, (size_t)J.cols.count * (J.cols.len - 2));
                WB_TRY(launch_slopes(J.cols, dC, s));
                dc.base = dC;
                dc.stride = J.cols.len - 2;
                dc.len = J.cols.len - 2;
            }
            J.rows = dr;
            J.cols = dc;
        }
    }
    if (weighted(metric)) {
        int64_t nw = metric == WB_WDDTW ? std::max(wlen_rows - 2, wlen_cols - 2)
                                        : std::max(wlen_rows, wlen_cols);
        std::vector<double> w = logistic_weights(nw, p->g);
        WB_TAKE(dw, double, ws, std::max<size_t>(w.size(), 1));
        WB_CUDA(cudaMemcpyAsync(dw, w.data(), w.size() * sizeof(double),
                                cudaMemcpyHostToDevice, s));
        // the host vector must outlive the copy
        WB_CUDA(cudaStreamSynchronize(s));
        J.weights = dw;
    }
    if (metric == WB_EDR && std::isnan(p->epsilon)) {
        WB_TAKE(sr, double, ws, J.rows.count);
        WB_TRY(launch_mean_std(J.rows, sr, s));
        double *sc = sr;
        if (!same) {
            sc = ws.take<double>(J.cols.count);
            if (!sc) return fail(WB_ENOMEM, "workspace reservation exceeded");
            WB_TRY(launch_mean_std(J.cols, sc, s));
        }
        J.std_rows = sr;
        J.std_cols = sc;
    }
    if (metric == WB_ERP) {
        WB_TAKE(gr, double, ws, J.rows.count);
        WB_TAKE(gc, double, ws, J.cols.count);
        WB_TAKE(gt, double, ws, (size_t)J.cols.count * J.cols.len);
        WB_TRY(launch_erp_tables(J.rows, p->g, nullptr, gr, s));
        WB_TRY(launch_erp_tables(J.cols, p->g, gt, gc, s));
        J.gsum_rows = gr;
        J.gsum_cols = gc;
        J.gtab_cols = gt;
    }
    if (metric == WB_TWE) {
        WB_TAKE(dt, double, ws, (size_t)J.cols.count * J.cols.len);
        WB_TRY(launch_twe_tables(J.cols, dt, s));
        int ns = std::max(J.rows.len, J.cols.len);
        WB_TAKE(st, double, ws, ns);
        WB_TRY(launch_fill_stab(p->stiffness * 2.0, ns, st, s));
        J.dtab_cols = dt;
        J.stab = st;
    }
    return WB_OK;
}

static int finish_host_copy(void *dst, const void *src, size_t bytes, bool out_on_device,
                            cudaStream_t s) {
    if (out_on_device) return WB_OK;
    if (bytes) WB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    WB_CUDA(cudaStreamSynchronize(s));
    return WB_OK;
}

static int check_dim(const wb_series *x, int64_t dim) {
    if (dim < 0 || dim >= x->n_dims) return fail(WB_EINVAL, "The parameter dim must be 0 <= dim < n_dims");
    return WB_OK;
}

}  // namespace wb

using namespace wb;

// ==========================================================================

extern "C" int wb_pairwise_distance(const wb_series *x, const wb_series *y, int64_t dim,
                                    int32_t metric, const wb_params *params, double *out,
                                    int32_t out_on_device, void *stream_) {
    WB_TRACE();
    WB_TRY(check_series(x, "x"));
    if (y) WB_TRY(check_series(y, "y"));
    if (!params) return fail(WB_EINVAL, "params is NULL");
    if (!out && x->n > 0) return fail(WB_EINVAL, "out is NULL");
    WB_TRY(check_dim(x, dim));
    if (y && y->n_dims != x->n_dims)
        return fail(WB_EINVAL, "x and y must have the same number of dimensions.");
    if (!is_elastic(metric) && metric != WB_EUCLIDEAN)
        return fail(WB_EUNSUPPORTED, "unsupported metric id " + std::to_string(metric));
    const bool same = (y == nullptr);
    const wb_series *yy = same ? x : y;
    if (metric == WB_EUCLIDEAN && x->n_timestep != yy->n_timestep)
        return fail(WB_EINVAL, "Illegal n_timestep for non-elastic distance measure");
    cudaStream_t s = (cudaStream_t)stream_;
    const int xl = (int)x->n_timestep, yl = (int)yy->n_timestep;
    ElasticJob J;
    WB_TRY(metric_fields(metric, params, xl, yl, false, J));
    if (x->n == 0 || yy->n == 0) return WB_OK;

    Workspace ws(s);
    const size_t out_elems = (size_t)x->n * yy->n;
    SeriesSet probeR{nullptr, 0, x->n, xl}, probeC{nullptr, 0, yy->n, yl};
    size_t need = stage_bytes(x) + (same ? 0 : stage_bytes(yy)) +
                  table_bytes(metric, params, probeR, probeC, x->n, yy->n, xl, yl) +
                  (out_on_device ? 0 : align256(out_elems * 8));
    // ring workspace depends on the band of the (possibly derivative) job
    ElasticJob probe = J;
    probe.rows = probeR;
    probe.cols = probeC;
    probe.mode = same ? PM_UPPER : PM_ALL;
    if (derivative(metric) && std::min(xl, yl) >= 3) {
        probe.rows.len -= 2;
        probe.cols.len -= 2;
    }
    need += elastic_workspace_bytes(probe);
    WB_TRY(ws.reserve(need));

    WB_TRY(stage(x, dim, ws, J.rows));
    if (same) J.cols = J.rows;
    else WB_TRY(stage(yy, dim, ws, J.cols));
    WB_TRY(build_tables(metric, params, J, ws, same, xl, yl));
    double *dout = out_on_device ? out : ws.take<double>(out_elems);
    if (!dout) return fail(WB_ENOMEM, "workspace reservation exceeded");
    J.out = dout;
    J.out_ld = yy->n;
    J.mode = same ? PM_UPPER : PM_ALL;
    if (same) {
        WB_CUDA(cudaMemsetAsync(dout, 0, out_elems * sizeof(double), s));
    }
    WB_TRY(launch_elastic(J, ws, nullptr));
    return finish_host_copy(out, dout, out_elems * sizeof(double), out_on_device, s);
}

extern "C" int wb_pairwise_distance_fp32(const wb_series *x, const wb_series *y, int64_t dim,
                                         int32_t metric, const wb_params *params, double *out,
                                         int32_t out_on_device, void *stream_) {
    WB_TRACE();
    WB_TRY(check_series(x, "x"));
    if (y) WB_TRY(check_series(y, "y"));
    if (!params) return fail(WB_EINVAL, "params is NULL");
    if (!out && x->n > 0) return fail(WB_EINVAL, "out is NULL");
    WB_TRY(check_dim(x, dim));
    if (y && y->n_dims != x->n_dims)
        return fail(WB_EINVAL, "x and y must have the same number of dimensions.");
    if (!is_elastic(metric))
        return fail(WB_EUNSUPPORTED, "no FP32 form of metric id " + std::to_string(metric));
    const bool same = (y == nullptr);
    const wb_series *yy = same ? x : y;
    cudaStream_t s = (cudaStream_t)stream_;
    const int xl = (int)x->n_timestep, yl = (int)yy->n_timestep;
    ElasticJob J;
    WB_TRY(metric_fields(metric, params, xl, yl, false, J));
    if (x->n == 0 || yy->n == 0) return WB_OK;
    if (same && x->n > ((int64_t)1 << 31) - 1) return fail(WB_EINVAL, "too many series");

    const size_t out_elems = (size_t)x->n * yy->n;
    const bool all_zero = derivative(metric) && std::min(xl, yl) < 3;
    const bool strips = (J.kind == K_DTW || J.kind == K_WDTW) && !all_zero;
    const int lr = derivative(metric) && !all_zero ? xl - 2 : xl;
    const int lc = derivative(metric) && !all_zero ? yl - 2 : yl;
    const int64_t nw = metric == WB_WDDTW ? std::max(xl - 2, yl - 2) : std::max(xl, yl);
    SeriesSet probeR{nullptr, 0, x->n, xl}, probeC{nullptr, 0, yy->n, yl};
    size_t need = stage_bytes(x) + (same ? 0 : stage_bytes(yy)) +
                  table_bytes(metric, params, probeR, probeC, x->n, yy->n, xl, yl) +
                  (out_on_device ? 0 : align256(out_elems * 8)) +
                  align256((size_t)std::max<int64_t>(nw, 1) * 4);
    Dtw32Job D;
    int strip = 16;
    const int64_t n_items = same ? x->n * (x->n - 1) / 2 : (int64_t)out_elems;
    if (strips) {
        // planning reads only whether the item and weight pointers are set;
        // the real ones are filled in below
        static const int32_t plan_mark = 0;
        wb_dtw32 q{};
        q.x_len = lr;
        q.y_len = lc;
        q.nx = x->n;
        q.ny = yy->n;
        q.item_x = same ? &plan_mark : nullptr;
        q.item_y = same ? &plan_mark : nullptr;
        q.n_items = n_items;
        q.r = params->r;
        q.weights = J.kind == K_WDTW ? reinterpret_cast<const float *>(&plan_mark) : nullptr;
        strip = lr >= 512 ? 32 : (lr >= 128 ? 16 : 8);
        q.strip = strip;
        size_t dbytes = 0;
        WB_TRY(dtw32_plan(&q, false, D, dbytes));
        need += dbytes + align256((size_t)x->n * lr * 4) + (same ? 0 : align256((size_t)yy->n * lc * 4)) +
                align256((size_t)std::max<int64_t>(n_items, 1) * 8) +
                (same ? 2 * align256((size_t)std::max<int64_t>(n_items, 1) * 4) : 0);
    } else {
        ElasticJob probe = J;
        probe.rows = probeR;
        probe.cols = probeC;
        probe.mode = same ? PM_UPPER : PM_ALL;
        need += std::max(strip_workspace_bytes(probe, true), elastic_workspace_bytes(probe));
    }
    Workspace ws(s);
    WB_TRY(ws.reserve(need));
    WB_TRY(stage(x, dim, ws, J.rows));
    if (same) J.cols = J.rows;
    else WB_TRY(stage(yy, dim, ws, J.cols));
    WB_TRY(build_tables(metric, params, J, ws, same, xl, yl));
    double *dout = out_on_device ? out : ws.take<double>(out_elems);
    if (!dout) return fail(WB_ENOMEM, "workspace reservation exceeded");
    float *w32 = nullptr;
    if (weighted(metric)) {
        w32 = ws.take<float>((size_t)std::max<int64_t>(nw, 1));
        if (!w32) return fail(WB_ENOMEM, "workspace reservation exceeded");
        WB_TRY(launch_weights_f32(J.weights, (int)nw, w32, s));
    }
    if (strips) {
        WB_TRY(dtw32_take(ws, D, false));
        WB_TAKE(fr, float, ws, (size_t)x->n * lr);
        WB_TRY(launch_to_f32(J.rows, fr, s));
        float *fc = fr;
        if (!same) {
            fc = ws.take<float>((size_t)yy->n * lc);
            if (!fc) return fail(WB_ENOMEM, "workspace reservation exceeded");
            WB_TRY(launch_to_f32(J.cols, fc, s));
        }
        WB_TAKE(item_out, double, ws, (size_t)std::max<int64_t>(n_items, 1));
        D.x = fr;
        D.x_stride = lr;
        D.y = fc;
        D.y_stride = lc;
        D.band_fixed = J.band;
        D.weights = w32;
        D.out = item_out;
        D.out_cost = nullptr;
        D.item_x = D.item_y = nullptr;
        if (same) {
            WB_TAKE(ix, int32_t, ws, (size_t)std::max<int64_t>(n_items, 1));
            WB_TAKE(iy, int32_t, ws, (size_t)std::max<int64_t>(n_items, 1));
            WB_TRY(launch_upper_items(x->n, ix, iy, s));
            D.item_x = ix;
            D.item_y = iy;
        }
        D.n_items = n_items;
        if (n_items > 0) WB_TRY(dtw32_forward(D, strip, s));
        WB_TRY(launch_grid_to_matrix(item_out, x->n, yy->n, same ? 1 : 0, dout, s));
    } else {
        J.weights32 = w32;
        J.out = dout;
        J.out_ld = yy->n;
        J.mode = same ? PM_UPPER : PM_ALL;
        if (same) WB_CUDA(cudaMemsetAsync(dout, 0, out_elems * sizeof(double), s));
        if (all_zero) WB_TRY(launch_elastic(J, ws, nullptr));
        else WB_TRY(launch_strip(J, ws, true));
    }
    return finish_host_copy(out, dout, out_elems * sizeof(double), out_on_device, s);
}

extern "C" int wb_paired_distance(const wb_series *x, const wb_series *y, int64_t dim,
                                  int32_t metric, const wb_params *params, double *out,
                                  int32_t out_on_device, void *stream_) {
    WB_TRACE();
    WB_TRY(check_series(x, "x"));
    WB_TRY(check_series(y, "y"));
    if (!params) return fail(WB_EINVAL, "params is NULL");
    WB_TRY(check_dim(x, dim));
    if (x->n != y->n) return fail(WB_EINVAL, "x and y must have the same number of samples.");
    if (y->n_dims != x->n_dims)
        return fail(WB_EINVAL, "x and y must have the same number of dimensions.");
    if (!is_elastic(metric) && metric != WB_EUCLIDEAN)
        return fail(WB_EUNSUPPORTED, "unsupported metric id " + std::to_string(metric));
    if (metric == WB_EUCLIDEAN && x->n_timestep != y->n_timestep)
        return fail(WB_EINVAL, "Illegal n_timestep for non-elastic distance measure");
    if (x->n == 0) return WB_OK;
    if (!out) return fail(WB_EINVAL, "out is NULL");
    cudaStream_t s = (cudaStream_t)stream_;
    // the metric sees (y, x): rows of the recurrence are y's series
    const int rl = (int)y->n_timestep, cl = (int)x->n_timestep;
    ElasticJob J;
    WB_TRY(metric_fields(metric, params, rl, cl, false, J));
    Workspace ws(s);
    SeriesSet probeR{nullptr, 0, y->n, rl}, probeC{nullptr, 0, x->n, cl};
    ElasticJob probe = J;
    probe.rows = probeR;
    probe.cols = probeC;
    probe.mode = PM_PAIRED;
    if (derivative(metric) && std::min(rl, cl) >= 3) {
        probe.rows.len -= 2;
        probe.cols.len -= 2;
    }
    size_t need = stage_bytes(x) + stage_bytes(y) +
                  table_bytes(metric, params, probeR, probeC, y->n, x->n, rl, cl) +
                  elastic_workspace_bytes(probe) +
                  (out_on_device ? 0 : align256((size_t)x->n * 8));
    WB_TRY(ws.reserve(need));
    WB_TRY(stage(y, dim, ws, J.rows));
    WB_TRY(stage(x, dim, ws, J.cols));
    WB_TRY(build_tables(metric, params, J, ws, false, rl, cl));
    double *dout = out_on_device ? out : ws.take<double>(x->n);
    if (!dout) return fail(WB_ENOMEM, "workspace reservation exceeded");
    J.out = dout;
    J.out_ld = 0;
    J.mode = PM_PAIRED;
    WB_TRY(launch_elastic(J, ws, nullptr));
    return finish_host_copy(out, dout, (size_t)x->n * sizeof(double), out_on_device, s);
}

extern "C" int wb_argmin_distance(const wb_series *x, const wb_series *y, int64_t dim,
                                  int32_t metric, const wb_params *params, int64_t k,
                                  const double *lower_bound, int64_t *indices,
                                  double *distances, int32_t out_on_device, void *stream_) {
    WB_TRACE();
    WB_TRY(check_series(x, "x"));
    WB_TRY(check_series(y, "y"));
    if (!params) return fail(WB_EINVAL, "params is NULL");
    WB_TRY(check_dim(x, dim));
    if (y->n_dims != x->n_dims)
        return fail(WB_EINVAL, "x and y must have the same number of dimensions.");
    if (!is_elastic(metric) && metric != WB_EUCLIDEAN)
        return fail(WB_EUNSUPPORTED, "unsupported metric id " + std::to_string(metric));
    if (metric == WB_EUCLIDEAN && x->n_timestep != y->n_timestep)
        return fail(WB_EINVAL, "Illegal n_timestep for non-elastic distance measure.");
    if (k < 1) return fail(WB_EINVAL, "k must be >= 1");
    if (k > y->n) k = y->n;
    if (x->n == 0 || y->n == 0) return WB_OK;
    if (!indices || !distances) return fail(WB_EINVAL, "outputs are NULL");
    cudaStream_t s = (cudaStream_t)stream_;
    const int xl = (int)x->n_timestep, yl = (int)y->n_timestep;
    ElasticJob J;
    WB_TRY(metric_fields(metric, params, xl, yl, true, J));
    Workspace ws(s);
    // Queries go in batches whose (distance, key) matrices stay within 2 GiB:
    // the reference keeps O(k) per query, so the whole (nx, ny) matrix is
    // never needed at once (every query's candidate loop is independent).
    const int64_t budget = argmin_pair_budget();
    const int64_t batch = std::max<int64_t>(1, std::min<int64_t>(x->n, budget / y->n));
    const size_t bpairs = (size_t)batch * y->n;
    SeriesSet probeR{nullptr, 0, batch, xl}, probeC{nullptr, 0, y->n, yl};
    ElasticJob probe = J;
    probe.rows = probeR;
    probe.cols = probeC;
    probe.mode = PM_ALL;
    // the recurrence also writes abandon keys: the kernel choice (and so its
    // workspace) depends on it
    double dummy_key = 0.0;
    probe.key = metric == WB_EUCLIDEAN ? nullptr : &dummy_key;
    if (derivative(metric) && std::min(xl, yl) >= 3) {
        probe.rows.len -= 2;
        probe.cols.len -= 2;
    }
    // early-abandoned chunks of candidates (argmin_ea.cu) where the metric
    // and band allow them: chunk sizes double from a first chunk that gives
    // every lane a few pairs, so the k-th distances tighten early
    ElasticJob ea = probe;
    ea.all_zero = derivative(metric) && std::min(xl, yl) < 3;
    const bool use_ea = !argmin_ea_disabled() && argmin_ea_supported(ea);
    const size_t ea_ring_bytes = use_ea ? argmin_ea_ring_bytes(ea) : 0;
    constexpr int kMaxChunks = 64;  // doubling chunks of at most 2^31 candidates
    auto schedule = [&](int64_t nq) {
        std::vector<int64_t> chunks;
        int64_t c = std::max<int64_t>(64, 4 * argmin_ea_lanes(ea) / nq);
        if (argmin_ea_first_chunk() > 0) c = argmin_ea_first_chunk();
        if (!argmin_ea_chunked(ea)) c = y->n;  // one chunk without a bound
        for (int64_t a = 0; a < y->n; c *= 2) {
            chunks.push_back(a);
            a = std::min<int64_t>(y->n, a + c);
        }
        chunks.push_back(y->n);
        return chunks;
    };
    const size_t fixed = stage_bytes(x) + stage_bytes(y) +
                         table_bytes(metric, params, SeriesSet{nullptr, 0, x->n, xl}, probeC,
                                     x->n, y->n, xl, yl) +
                         (out_on_device ? 0 : 2 * align256((size_t)x->n * k * 8));
    const size_t per_batch =
        (use_ea ? 0 : elastic_workspace_bytes(probe)) + 2 * align256(bpairs * 8) +
        2 * align256((size_t)batch * k * 8) +
        (lower_bound && !out_on_device ? align256(bpairs * 8) : 0) +
        (use_ea ? 2 * align256((size_t)batch * 8) + align256(kMaxChunks * 8) + ea_ring_bytes
                : 0);
    WB_TRY(ws.reserve(fixed + per_batch));
    WB_TRY(stage(x, dim, ws, J.rows));
    WB_TRY(stage(y, dim, ws, J.cols));
    WB_TRY(build_tables(metric, params, J, ws, false, xl, yl));
    int64_t *hidx_all = out_on_device ? indices : ws.take<int64_t>((size_t)x->n * k);
    double *hdist_all = out_on_device ? distances : ws.take<double>((size_t)x->n * k);
    if (!hidx_all || !hdist_all) return fail(WB_ENOMEM, "workspace reservation exceeded");
    int never_push = 0;
    if (derivative(metric) && std::min(xl, yl) < 3) never_push = 1;
    const size_t batch_mark = ws.mark();
    if (use_ea) timer_begin("argmin_ea_kernel", s);
    for (int64_t b0 = 0; b0 < x->n; b0 += batch) {
        const int64_t nb = std::min<int64_t>(batch, x->n - b0);
        const size_t pairs = (size_t)nb * y->n;
        ws.rewind(batch_mark);
        ElasticJob Jb = J;
        Jb.rows.base = J.rows.base + b0 * J.rows.stride;
        Jb.rows.count = nb;
        if (J.std_rows) Jb.std_rows = J.std_rows + b0;
        if (J.gsum_rows) Jb.gsum_rows = J.gsum_rows + b0;
        WB_TAKE(D, double, ws, pairs);
        WB_TAKE(K, double, ws, pairs);
        Jb.out = D;
        Jb.out_ld = y->n;
        Jb.key = metric == WB_EUCLIDEAN ? nullptr : K;
        Jb.mode = PM_ALL;
        if (!never_push && !use_ea) WB_TRY(launch_elastic(Jb, ws, nullptr));

        const double *lb = lower_bound ? lower_bound + (size_t)b0 * y->n : nullptr;
        if (lower_bound && !out_on_device) {
            WB_TAKE(dlb, double, ws, pairs);
            WB_CUDA(cudaMemcpyAsync(dlb, lb, pairs * 8, cudaMemcpyHostToDevice, s));
            lb = dlb;
        }
        ArgminJob A;
        A.metric = metric;
        A.nx = nb;
        A.ny = y->n;
        A.k = k;
        A.dist = D;
        A.key = Jb.key;
        A.lower_bound = lb;
        A.xl = xl;
        A.yl = yl;
        A.never_push = never_push;
        A.heap_idx = ws.take<int64_t>((size_t)nb * k);
        A.heap_val = ws.take<double>((size_t)nb * k);
        A.out_idx = hidx_all + (size_t)b0 * k;
        A.out_dist = hdist_all + (size_t)b0 * k;
        if (!A.heap_idx || !A.heap_val) return fail(WB_ENOMEM, "workspace reservation exceeded");
        if (use_ea && !never_push) {
            const std::vector<int64_t> chunks = schedule(nb);
            if ((int)chunks.size() > kMaxChunks + 1)
                return fail(WB_EINVAL, "too many candidate chunks");
            A.state_n = ws.take<int64_t>(nb);
            A.state_dist = ws.take<double>(nb);
            auto *counters = ws.take<unsigned long long>(kMaxChunks);
            double *ea_ring = ea_ring_bytes ? ws.take<double>(ea_ring_bytes / 8) : nullptr;
            if (!A.state_n || !A.state_dist || !counters || (ea_ring_bytes && !ea_ring))
                return fail(WB_ENOMEM, "workspace reservation exceeded");
            WB_CUDA(cudaMemsetAsync(counters, 0, kMaxChunks * 8, s));
            WB_TRY(launch_fill(A.state_dist, HUGE_VAL, nb, s));
            for (size_t c = 0; c + 1 < chunks.size(); c++) {
                const int64_t a = chunks[c], b = chunks[c + 1];
                WB_TRY(launch_argmin_ea(Jb, metric, xl, yl, a, b - a, y->n, A.state_dist, lb,
                                        counters + c, ea_ring, s));
                A.j0 = a;
                A.j1 = b;
                A.resume = c > 0;
                A.finish = c + 2 == chunks.size();
                WB_TRY(launch_argmin_replay(A, s));
            }
        } else {
            WB_TRY(launch_argmin_replay(A, s));
        }
    }
    if (use_ea) timer_end(s);
    if (!out_on_device) {
        WB_CUDA(cudaMemcpyAsync(indices, hidx_all, (size_t)x->n * k * 8,
                                cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaMemcpyAsync(distances, hdist_all, (size_t)x->n * k * 8,
                                cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaStreamSynchronize(s));
    }
    return WB_OK;
}

// elastic subsequence metrics: the *_subsequence_distance functions of
// distance/_elastic.pyx:622-1866 with the metric classes of :2206-3124
static int subseq_elastic(const double *shapelets, const int64_t *offsets,
                          const int64_t *lengths, const double *stds, int64_t m,
                          const wb_series *x, int64_t dim, int32_t metric,
                          const wb_params *p, double *out_dist, int64_t *out_idx,
                          int32_t out_on_device, cudaStream_t s,
                          const std::vector<int64_t> &hlen, int64_t total, bool paired,
                          double *prof_raw = nullptr, double *prof_key = nullptr,
                          int64_t prof_ld = 0, int std_as_given = 0) {
    if (!(p->r >= 0.0 && p->r <= 1.0)) return fail(WB_EINVAL, "r must be in [0, 1]");
    const bool dev_in = x->on_device != 0;
    const bool slopes = derivative(metric);
    const int T = (int)x->n_timestep;
    const bool profile = prof_raw != nullptr;
    const size_t n_out = profile ? (size_t)m * prof_ld * 2 : (paired ? (size_t)m : (size_t)x->n * m);
    SubseqElasticJob J;
    J.m = m;
    J.paired = paired ? 1 : 0;
    J.std_as_given = std_as_given;
    J.metric = metric;
    J.slopes = slopes ? 1 : 0;
    J.t_len_thr = T;
    J.eps = p->epsilon;
    J.p = p->p;
    J.g = p->g;
    J.c = p->c;
    J.penalty = p->penalty;
    J.stiffness = p->stiffness;
    int kind;
    switch (metric) {
        case WB_DTW: case WB_DDTW: kind = K_DTW; break;
        case WB_WDTW: case WB_WDDTW: kind = K_WDTW; break;
        case WB_ADTW: kind = p->p >= 0.0 ? K_ADTW : K_ADTW_ANY; break;
        case WB_LCSS:
            if (!(p->epsilon > 0.0)) return fail(WB_EINVAL, "epsilon must be > 0");
            kind = K_LCSS;
            break;
        case WB_EDR:
            if (std::isnan(p->epsilon) && !stds)
                return fail(WB_EINVAL, "edr with the default epsilon needs shapelet stds");
            kind = K_EDR;
            break;
        case WB_ERP: kind = K_ERP; break;
        case WB_MSM: kind = K_MSM; break;
        case WB_TWE: kind = K_TWE; break;
        default:
            return fail(WB_EUNSUPPORTED, "unsupported subsequence metric id " +
                                             std::to_string(metric));
    }
    // per-shapelet bands: _compute_r(s_len, r)
    std::vector<int32_t> band(m);
    int max_len = 1, max_band = 1, max_orig = 1;
    for (int64_t i = 0; i < m; i++) {
        band[i] = compute_r(hlen[i], p->r);
        int cl = (int)(slopes ? std::max<int64_t>(hlen[i] - 2, 1) : hlen[i]);
        max_len = std::max(max_len, cl);
        max_band = std::max(max_band, (int)band[i]);
        max_orig = std::max(max_orig, (int)hlen[i]);
    }
    const int xs_len = slopes ? std::max(T - 2, 1) : T;
    J.x.count = x->n;
    J.x.len = xs_len;
    J.t_len = xs_len;
    int P = 0, grid = 0;
    size_t ring = elastic_subseq_ring_bytes(J, max_len, max_band, &P, &grid);
    std::vector<double> w;
    if (metric == WB_WDTW) w = logistic_weights(T, p->g);
    if (metric == WB_WDDTW) w = logistic_weights(std::max(T - 2, 0), p->g);
    Workspace ws(s);
    size_t need = ring + stage_bytes(x) + align256(m * 4) + align256(w.size() * 8 + 8) +
                  (dev_in ? 0 : align256(total * 8) + 3 * align256(m * 8)) +
                  (slopes ? align256((size_t)x->n * xs_len * 8) + align256(total * 8) : 0) +
                  (metric == WB_ERP ? align256((size_t)x->n * T * 8) + align256(x->n * 8) : 0) +
                  (metric == WB_TWE ? align256((size_t)max_orig * 8 + 8) : 0) +
                  (out_on_device ? 0 : 2 * align256(n_out * 8));
    WB_TRY(ws.reserve(need));
    WB_TAKE(gring, double, ws, ring / sizeof(double));
    SeriesSet X;
    WB_TRY(stage(x, dim, ws, X));
    const double *dshp = shapelets;
    const int64_t *doff = offsets, *dlen = lengths;
    const double *dstd = stds;
    if (!dev_in) {
        WB_TAKE(hs, double, ws, total);
        WB_TAKE(ho, int64_t, ws, m);
        WB_TAKE(hl, int64_t, ws, m);
        WB_CUDA(cudaMemcpyAsync(hs, shapelets, total * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(ho, offsets, m * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(hl, lengths, m * 8, cudaMemcpyHostToDevice, s));
        dshp = hs;
        doff = ho;
        dlen = hl;
        if (stds) {
            WB_TAKE(hd, double, ws, m);
            WB_CUDA(cudaMemcpyAsync(hd, stds, m * 8, cudaMemcpyHostToDevice, s));
            dstd = hd;
        }
    }
    WB_TAKE(dband, int32_t, ws, m);
    WB_CUDA(cudaMemcpyAsync(dband, band.data(), m * 4, cudaMemcpyHostToDevice, s));
    if (!w.empty()) {
        WB_TAKE(dw, double, ws, w.size());
        WB_CUDA(cudaMemcpyAsync(dw, w.data(), w.size() * 8, cudaMemcpyHostToDevice, s));
        J.weights = dw;
    }
    J.x = X;
    J.x.len = xs_len;
    if (slopes) {
        WB_TAKE(xsl, double, ws, (size_t)x->n * xs_len);
        WB_TRY(launch_slopes(X, xsl, s));
        J.x.base = xsl;
        J.x.stride = xs_len;
        WB_TAKE(ssl, double, ws, total);
        WB_TRY(launch_shapelet_slopes(dshp, doff, dlen, m, ssl, s));
        dshp = ssl;
    }
    if (metric == WB_ERP) {
        WB_TAKE(gt, double, ws, (size_t)x->n * T);
        WB_TAKE(gs, double, ws, x->n);
        WB_TRY(launch_erp_tables(X, p->g, gt, gs, s));
        J.gtab = gt;
    }
    if (metric == WB_TWE) {
        WB_TAKE(st, double, ws, max_orig);
        WB_TRY(launch_fill_stab(p->stiffness * 2.0, max_orig, st, s));
        J.stab = st;
    }
    J.shp = dshp;
    J.off = doff;
    J.len = dlen;
    J.band_of_len = dband;
    J.shp_std = (metric == WB_EDR && std::isnan(p->epsilon)) ? dstd : nullptr;
    if (profile) {
        const size_t np = (size_t)m * prof_ld;
        double *rr = prof_raw, *kk = prof_key;
        if (!out_on_device) {
            rr = ws.take<double>(np);
            kk = ws.take<double>(np);
            if (!rr || !kk) return fail(WB_ENOMEM, "workspace reservation exceeded");
        }
        J.prof_raw = rr;
        J.prof_key = kk;
        J.prof_ld = prof_ld;
        WB_TRY(launch_elastic_subseq(J, kind, gring, P, grid, s));
        if (!out_on_device) {
            WB_CUDA(cudaMemcpyAsync(prof_raw, rr, np * 8, cudaMemcpyDeviceToHost, s));
            WB_CUDA(cudaMemcpyAsync(prof_key, kk, np * 8, cudaMemcpyDeviceToHost, s));
        }
        WB_CUDA(cudaStreamSynchronize(s));
        return WB_OK;
    }
    double *od = out_dist;
    int64_t *oi = out_idx;
    if (!out_on_device) {
        od = ws.take<double>(n_out);
        oi = ws.take<int64_t>(n_out);
        if (!od || !oi) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    J.out_dist = od;
    J.out_idx = oi;
    WB_TRY(launch_elastic_subseq(J, kind, gring, P, grid, s));
    if (!out_on_device) {
        WB_CUDA(cudaMemcpyAsync(out_dist, od, n_out * 8, cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaMemcpyAsync(out_idx, oi, n_out * 8, cudaMemcpyDeviceToHost, s));
    }
    // host vectors above feed asynchronous copies
    WB_CUDA(cudaStreamSynchronize(s));
    return WB_OK;
}

// scaled_dtw: staging and outputs around subseq_scaled_dtw (scaled_dtw.cu)
static int subseq_sdtw_entry(const double *shapelets, const int64_t *offsets,
                             const int64_t *lengths, const double *means, const double *stds,
                             int64_t m, const wb_series *x, int64_t dim, const wb_params *p,
                             double *out_dist, int64_t *out_idx, int32_t out_on_device,
                             cudaStream_t s, const std::vector<int64_t> &hlen, int64_t total,
                             bool paired, double *prof_raw, double *prof_key, int64_t prof_ld,
                             int std_as_given) {
    if (!(p->r >= 0.0 && p->r <= 1.0)) return fail(WB_EINVAL, "r must be in [0, 1]");
    const bool dev_in = x->on_device != 0;
    const bool profile = prof_raw != nullptr;
    const size_t n_out = profile ? (size_t)m * prof_ld : (paired ? (size_t)m : (size_t)x->n * m);
    Workspace ws(s);
    size_t need = subseq_scaled_dtw_bytes(m, total, x->n, (int)x->n_timestep, hlen, p->r,
                                          x->n_timestep, paired) +
                  stage_bytes(x) + (dev_in ? 0 : align256(total * 8) + 4 * align256(m * 8)) +
                  (out_on_device ? 0 : 2 * align256(n_out * 8));
    WB_TRY(ws.reserve(need));
    SeriesSet X;
    WB_TRY(stage(x, dim, ws, X));
    const double *dshp = shapelets, *dmean = means, *dstd = stds;
    const int64_t *doff = offsets, *dlen = lengths;
    if (!dev_in) {
        WB_TAKE(hs, double, ws, total);
        WB_TAKE(ho, int64_t, ws, m);
        WB_TAKE(hl, int64_t, ws, m);
        WB_TAKE(hm, double, ws, m);
        WB_TAKE(hd, double, ws, m);
        WB_CUDA(cudaMemcpyAsync(hs, shapelets, total * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(ho, offsets, m * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(hl, lengths, m * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(hm, means, m * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(hd, stds, m * 8, cudaMemcpyHostToDevice, s));
        dshp = hs;
        doff = ho;
        dlen = hl;
        dmean = hm;
        dstd = hd;
    }
    double *od = profile ? prof_raw : out_dist, *ok = prof_key;
    int64_t *oi = out_idx;
    if (!out_on_device) {
        od = ws.take<double>(n_out);
        if (profile)
            ok = ws.take<double>(n_out);
        else
            oi = ws.take<int64_t>(n_out);
        if (!od || (profile ? !ok : !oi)) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    WB_TRY(subseq_scaled_dtw(dshp, doff, dlen, dmean, dstd, m, hlen, total, X, x->n_timestep,
                             p->r, paired, std_as_given, profile ? nullptr : od,
                             profile ? nullptr : oi, profile ? od : nullptr,
                             profile ? ok : nullptr, prof_ld, ws, s));
    if (!out_on_device) {
        if (profile) {
            WB_CUDA(cudaMemcpyAsync(prof_raw, od, n_out * 8, cudaMemcpyDeviceToHost, s));
            WB_CUDA(cudaMemcpyAsync(prof_key, ok, n_out * 8, cudaMemcpyDeviceToHost, s));
        } else {
            WB_CUDA(cudaMemcpyAsync(out_dist, od, n_out * 8, cudaMemcpyDeviceToHost, s));
            WB_CUDA(cudaMemcpyAsync(out_idx, oi, n_out * 8, cudaMemcpyDeviceToHost, s));
        }
    }
    WB_CUDA(cudaStreamSynchronize(s));
    return WB_OK;
}

// Shared by the pairwise (every series against every shapelet) and paired
// (series i against shapelet i) subsequence entries.
static int subseq_entry(const double *shapelets, const int64_t *offsets, const int64_t *lengths,
                        const double *means, const double *stds, int64_t m, const wb_series *x,
                        int64_t dim, int32_t metric, const wb_params *params, double *out_dist,
                        int64_t *out_idx, int32_t out_on_device, void *stream_, bool paired,
                        double *prof_raw = nullptr, double *prof_key = nullptr,
                        int64_t prof_ld = 0, int std_as_given = 0,
                        const double *stop_sq = nullptr) {
    WB_TRY(check_series(x, "x"));
    const bool profile = prof_raw != nullptr;
    if (paired && m != x->n)
        return fail(WB_EINVAL, "The number of subsequences and samples must be the same, got " +
                                   std::to_string(m) + " subsequences and " +
                                   std::to_string(x->n) + " samples.");
    WB_TRY(check_dim(x, dim));
    const bool elastic = is_elastic(metric) && metric != WB_WLCSS;
    const bool sdtw = metric == WB_SCALED_DTW;
    if (metric != WB_EUCLIDEAN && metric != WB_SCALED_EUCLIDEAN && !elastic && !sdtw)
        return fail(WB_EUNSUPPORTED, "unsupported subsequence metric id " + std::to_string(metric));
    if ((elastic || sdtw) && !params) return fail(WB_EINVAL, "params is NULL");
    if (sdtw && (!means || !stds)) return fail(WB_EINVAL, "scaled metric needs means and stds");
    if (m < 0) return fail(WB_EINVAL, "negative number of shapelets");
    if (m == 0 || x->n == 0) return WB_OK;
    if (!shapelets || !offsets || !lengths || (!profile && (!out_dist || !out_idx)))
        return fail(WB_EINVAL, "NULL shapelet or output array");
    const bool scaled = metric == WB_SCALED_EUCLIDEAN;
    if (scaled && (!means || !stds)) return fail(WB_EINVAL, "scaled metric needs means and stds");
    cudaStream_t s = (cudaStream_t)stream_;
    const bool dev_in = x->on_device != 0;

    // Host copies of lengths/offsets drive the grouping by length.
    std::vector<int64_t> hlen(m), hoff(m);
    if (dev_in) {
        WB_CUDA(cudaMemcpy(hlen.data(), lengths, m * 8, cudaMemcpyDeviceToHost));
        WB_CUDA(cudaMemcpy(hoff.data(), offsets, m * 8, cudaMemcpyDeviceToHost));
    } else {
        std::memcpy(hlen.data(), lengths, m * 8);
        std::memcpy(hoff.data(), offsets, m * 8);
    }
    int64_t total = 0;
    for (int64_t i = 0; i < m; i++) {
        if (hlen[i] < 1 || hlen[i] > x->n_timestep)
            return fail(WB_EINVAL, "Invalid subsequnce shape (" + std::to_string(hlen[i]) +
                                       " > " + std::to_string(x->n_timestep) + ")");
        if (hoff[i] < 0) return fail(WB_EINVAL, "negative shapelet offset");
        total = std::max(total, hoff[i] + hlen[i]);
        if (profile && x->n_timestep - hlen[i] + 1 > prof_ld)
            return fail(WB_EINVAL, "ld is smaller than the number of windows");
    }
    if (elastic)
        return subseq_elastic(shapelets, offsets, lengths, stds, m, x, dim, metric, params,
                              out_dist, out_idx, out_on_device, s, hlen, total, paired,
                              prof_raw, prof_key, prof_ld, std_as_given);
    if (sdtw)
        return subseq_sdtw_entry(shapelets, offsets, lengths, means, stds, m, x, dim, params,
                                 out_dist, out_idx, out_on_device, s, hlen, total, paired,
                                 prof_raw, prof_key, prof_ld, std_as_given);
    const size_t n_out = profile ? (size_t)m * prof_ld : (paired ? (size_t)m : (size_t)x->n * m);
    std::vector<int64_t> order(m);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t b) { return hlen[a] < hlen[b]; });
    std::vector<int32_t> group_of(m), group_len;
    for (int64_t t = 0; t < m; t++) {
        int64_t i = order[t];
        if (group_len.empty() || group_len.back() != hlen[i]) group_len.push_back((int32_t)hlen[i]);
        group_of[i] = (int32_t)group_len.size() - 1;
    }

    // scaled metric: chunks of <= kScaledTileChunk shapelets of one length for
    // the tiled kernel (the z-normalised tiles are shared by a chunk)
    std::vector<int64_t> ch_first;
    std::vector<int32_t> ch_count, ch_group;
    int max_len = 0;
    for (int64_t i = 0; i < m; i++) max_len = std::max<int>(max_len, (int)hlen[i]);
    const bool tiled = scaled && !paired && max_len <= kScaledTileMaxLen;
    if (tiled) {
        for (int64_t t = 0; t < m;) {
            int64_t u = t;
            while (u < m && u - t < kScaledTileChunk && group_of[order[u]] == group_of[order[t]])
                u++;
            ch_first.push_back(t);
            ch_count.push_back((int32_t)(u - t));
            ch_group.push_back(group_of[order[t]]);
            t = u;
        }
    }

    SubseqJob J;
    J.m = m;
    J.n_groups = (int)group_len.size();
    J.max_len = max_len;
    J.paired = paired ? 1 : 0;
    J.std_as_given = std_as_given;
    J.total_values = total;
    if (stop_sq && !profile) return fail(WB_EINVAL, "stop values apply to profiles only");
    J.win_stride = (int)x->n_timestep;
    J.chunk = kScaledTileChunk;
    Workspace ws(s);
    size_t need = stage_bytes(x) + align256(m * 8) * 3 + align256(m * 4) +
                  align256(group_len.size() * 4) +
                  (dev_in ? 0 : align256(total * 8) + 2 * align256(m * 8) + 2 * align256(m * 8)) +
                  (out_on_device ? 0 : 2 * align256(n_out * 8)) +
                  align256(ch_first.size() * 8) + 2 * align256(ch_first.size() * 4) +
                  (stop_sq ? align256(m * 8) : 0);
    J.x.count = x->n;
    J.x.len = (int)x->n_timestep;
    need += subseq_workspace_bytes(J, scaled);
    WB_TRY(ws.reserve(need));
    WB_TRY(stage(x, dim, ws, J.x));
    if (stop_sq) {
        WB_TAKE(dstop, double, ws, m);
        WB_CUDA(cudaMemcpyAsync(dstop, stop_sq, m * 8, cudaMemcpyHostToDevice, s));
        J.stop_sq = dstop;
    }
    if (dev_in) {
        J.shapelets = shapelets;
        J.offsets = offsets;
        J.lengths = lengths;
        J.means = means;
        J.stds = stds;
    } else {
        WB_TAKE(dsh, double, ws, total);
        WB_TAKE(doff, int64_t, ws, m);
        WB_TAKE(dlen, int64_t, ws, m);
        WB_CUDA(cudaMemcpyAsync(dsh, shapelets, total * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(doff, offsets, m * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(dlen, lengths, m * 8, cudaMemcpyHostToDevice, s));
        J.shapelets = dsh;
        J.offsets = doff;
        J.lengths = dlen;
        if (scaled) {
            WB_TAKE(dm, double, ws, m);
            WB_TAKE(ds, double, ws, m);
            WB_CUDA(cudaMemcpyAsync(dm, means, m * 8, cudaMemcpyHostToDevice, s));
            WB_CUDA(cudaMemcpyAsync(ds, stds, m * 8, cudaMemcpyHostToDevice, s));
            J.means = dm;
            J.stds = ds;
        }
    }
    WB_TAKE(dorder, int64_t, ws, m);
    WB_TAKE(dgroup, int32_t, ws, m);
    WB_TAKE(dglen, int32_t, ws, group_len.size());
    WB_CUDA(cudaMemcpyAsync(dorder, order.data(), m * 8, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(dgroup, group_of.data(), m * 4, cudaMemcpyHostToDevice, s));
    WB_CUDA(cudaMemcpyAsync(dglen, group_len.data(), group_len.size() * 4,
                            cudaMemcpyHostToDevice, s));
    J.order = dorder;
    J.group_of = dgroup;
    J.group_len = dglen;
    if (tiled) {
        const size_t nc = ch_first.size();
        WB_TAKE(dcf, int64_t, ws, nc);
        WB_TAKE(dcc, int32_t, ws, nc);
        WB_TAKE(dcg, int32_t, ws, nc);
        WB_CUDA(cudaMemcpyAsync(dcf, ch_first.data(), nc * 8, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(dcc, ch_count.data(), nc * 4, cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaMemcpyAsync(dcg, ch_group.data(), nc * 4, cudaMemcpyHostToDevice, s));
        J.chunk_first = dcf;
        J.chunk_count = dcc;
        J.chunk_group = dcg;
        J.n_chunks = (int64_t)nc;
    }
    if (profile) {
        double *rr = out_on_device ? prof_raw : ws.take<double>(n_out);
        if (!rr) return fail(WB_ENOMEM, "workspace reservation exceeded");
        WB_TRY(launch_subseq_profile(J, scaled, ws, rr, prof_ld));
        if (prof_key) {
            // the euclidean sums have no abandoning rows: key -inf
            if (out_on_device) {
                WB_TRY(launch_fill(prof_key, -HUGE_VAL, (int64_t)n_out, s));
            } else {
                std::vector<double> kk(n_out, -HUGE_VAL);
                std::memcpy(prof_key, kk.data(), n_out * 8);
            }
        }
        if (!out_on_device)
            WB_CUDA(cudaMemcpyAsync(prof_raw, rr, n_out * 8, cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaStreamSynchronize(s));
        return WB_OK;
    }
    J.out_dist = out_on_device ? out_dist : ws.take<double>(n_out);
    J.out_idx = out_on_device ? out_idx : ws.take<int64_t>(n_out);
    if (!J.out_dist || !J.out_idx) return fail(WB_ENOMEM, "workspace reservation exceeded");
    WB_TRY(launch_subseq(J, scaled, ws));
    if (!out_on_device) {
        WB_CUDA(cudaMemcpyAsync(out_dist, J.out_dist, n_out * 8, cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaMemcpyAsync(out_idx, J.out_idx, n_out * 8, cudaMemcpyDeviceToHost, s));
    }
    // the host vectors above feed asynchronous copies
    WB_CUDA(cudaStreamSynchronize(s));
    return WB_OK;
}

extern "C" int wb_pairwise_subsequence_distance(
    const double *shapelets, const int64_t *offsets, const int64_t *lengths,
    const double *means, const double *stds, int64_t m, const wb_series *x, int64_t dim,
    int32_t metric, const wb_params *params, double *out_dist, int64_t *out_idx,
    int32_t out_on_device, void *stream_) {
    WB_TRACE();
    return subseq_entry(shapelets, offsets, lengths, means, stds, m, x, dim, metric, params,
                        out_dist, out_idx, out_on_device, stream_, false);
}

extern "C" int wb_subsequence_profile(const double *shapelets, const int64_t *offsets,
                                      const int64_t *lengths, const double *means,
                                      const double *stds, int64_t m, const wb_series *x,
                                      int64_t dim, int32_t metric, const wb_params *params,
                                      double *out_raw, double *out_key, int64_t ld,
                                      int32_t std_as_given, int32_t out_on_device,
                                      void *stream_) {
    WB_TRACE();
    if (!out_raw) return fail(WB_EINVAL, "out_raw is NULL");
    if (!out_key && metric != WB_EUCLIDEAN && metric != WB_SCALED_EUCLIDEAN)
        return fail(WB_EINVAL, "out_key is NULL");
    return subseq_entry(shapelets, offsets, lengths, means, stds, m, x, dim, metric, params,
                        nullptr, nullptr, out_on_device, stream_, true, out_raw, out_key, ld,
                        std_as_given ? 1 : 0);
}

extern "C" int wb_subsequence_profile_stop(const double *shapelets, const int64_t *offsets,
                                           const int64_t *lengths, const double *means,
                                           const double *stds, int64_t m, const wb_series *x,
                                           int64_t dim, const double *stop_sq,
                                           double *out_raw, int64_t ld, int32_t out_on_device,
                                           void *stream_) {
    WB_TRACE();
    if (!out_raw) return fail(WB_EINVAL, "out_raw is NULL");
    if (!stop_sq) return fail(WB_EINVAL, "stop_sq is NULL");
    wb_params p{};
    return subseq_entry(shapelets, offsets, lengths, means, stds, m, x, dim,
                        WB_SCALED_EUCLIDEAN, &p, nullptr, nullptr, out_on_device, stream_,
                        true, out_raw, nullptr, ld, 0, stop_sq);
}

extern "C" int wb_paired_subsequence_distance(
    const double *shapelets, const int64_t *offsets, const int64_t *lengths,
    const double *means, const double *stds, int64_t m, const wb_series *x, int64_t dim,
    int32_t metric, const wb_params *params, double *out_dist, int64_t *out_idx,
    int32_t out_on_device, void *stream_) {
    WB_TRACE();
    return subseq_entry(shapelets, offsets, lengths, means, stds, m, x, dim, metric, params,
                        out_dist, out_idx, out_on_device, stream_, true);
}

// ---------------------------------------------------------------------------
// distance profiles outside the subsequence scans

extern "C" int wb_dilated_profile(const wb_series *y, const wb_series *x, int64_t dim,
                                  int32_t metric, const wb_params *params, int64_t dilation,
                                  int64_t padding, int32_t scale, double *out,
                                  int32_t out_on_device, void *stream_) {
    WB_TRACE();
    WB_TRY(check_series(y, "y"));
    WB_TRY(check_series(x, "x"));
    if (!params) return fail(WB_EINVAL, "params is NULL");
    WB_TRY(check_dim(x, dim));
    if (!is_elastic(metric) && metric != WB_EUCLIDEAN)
        return fail(WB_EUNSUPPORTED, "unsupported metric id " + std::to_string(metric));
    if (dilation < 1) return fail(WB_EINVAL, "dilation must be >= 1");
    if (padding < 0) return fail(WB_EINVAL, "padding must be >= 0");
    if (y->n != x->n) return fail(WB_EINVAL, "y and x must have the same number of samples.");
    const int L = (int)y->n_timestep, T = (int)x->n_timestep;
    const int64_t ks = (int64_t)(L - 1) * dilation + 1;
    const int64_t input_size = T + 2 * padding;
    if (L < 1 || ks > input_size)
        return fail(WB_EINVAL, "subsequence in y is larger than input in x.");
    const int64_t n = x->n;
    const int out_size = (int)(input_size - ks + 1);
    if (n == 0) return WB_OK;
    if (!out) return fail(WB_EINVAL, "out is NULL");
    cudaStream_t s = (cudaStream_t)stream_;
    // window size k of every output position (_cdistance.pyx:832-852);
    // positions of equal k form runs
    std::vector<int> kk(out_size);
    for (int p = 0; p < out_size; p++) {
        const int64_t po = padding - p;
        int64_t ko = 0, io;
        if (po > 0) {
            ko = po % dilation == 0 ? po : po + dilation - po % dilation;
            io = ko - po;
        } else {
            io = -po;
        }
        const int64_t conv = std::min<int64_t>(T, io + ks - std::max<int64_t>(0, po)) - io;
        kk[p] = conv > 0 ? (int)((conv + dilation - 1) / dilation) : 0;
    }
    // workspace: staged inputs, the largest run's windows and distances, the
    // metric tables at the largest k, the output
    int64_t max_run = 0;
    for (int p = 0; p < out_size;) {
        int q = p;
        while (q < out_size && kk[q] == kk[p]) q++;
        max_run = std::max<int64_t>(max_run, q - p);
        p = q;
    }
    const int64_t rows_max = n * max_run;
    ElasticJob J0;
    WB_TRY(metric_fields(metric, params, L, L, true, J0));
    SeriesSet probeR{nullptr, 0, rows_max, L}, probeC{nullptr, 0, rows_max, L};
    ElasticJob probe = J0;
    probe.rows = probeR;
    probe.cols = probeC;
    probe.mode = PM_PAIRED;
    size_t need = stage_bytes(x) + stage_bytes(y) + 2 * align256((size_t)rows_max * L * 8) +
                  align256((size_t)rows_max * 8) +
                  table_bytes(metric, params, probeR, probeC, rows_max, rows_max, L, L) +
                  align256((size_t)std::max(T, 1) * 8) + elastic_workspace_bytes(probe) +
                  align256((size_t)n * out_size * 8);
    Workspace ws(s);
    WB_TRY(ws.reserve(need));
    SeriesSet sx, sy;
    WB_TRY(stage(x, dim, ws, sx));
    // the subsequences have one dim (the reference reads y[i, dim], past the
    // end of y for dim > 0)
    WB_TRY(stage(y, 0, ws, sy));
    double *dout = out_on_device ? out : ws.take<double>((size_t)n * out_size);
    WB_TAKE(xw, double, ws, (size_t)rows_max * L);
    WB_TAKE(kw, double, ws, (size_t)rows_max * L);
    WB_TAKE(dist, double, ws, (size_t)rows_max);
    if (!dout) return fail(WB_ENOMEM, "workspace reservation exceeded");
    const size_t mark = ws.mark();
    for (int p = 0; p < out_size;) {
        int q = p;
        while (q < out_size && kk[q] == kk[p]) q++;
        const int k = kk[p], np = q - p;
        const int64_t rows = n * np;
        ws.rewind(mark);
        WB_TRY(launch_dilated_gather(sx.base, n, sx.stride, T, sy.base, sy.stride, L,
                                     (int)dilation, (int)padding, p, np, k, scale, xw, kw, s));
        // metric._eadistance(x window, k, kernel, k): the window is the
        // recurrence's rows; weights sized from the series length T as in
        // Metric.reset(X, X)
        ElasticJob J;
        WB_TRY(metric_fields(metric, params, k, k, true, J));
        J.rows = SeriesSet{xw, k, rows, k};
        J.cols = SeriesSet{kw, k, rows, k};
        WB_TRY(build_tables(metric, params, J, ws, false, T, T));
        J.out = dist;
        J.out_ld = 0;
        J.mode = PM_PAIRED;
        WB_TRY(launch_elastic(J, ws, nullptr));
        WB_TRY(launch_dilated_scatter(dist, n, p, np, k, L, dout, out_size, s));
        p = q;
    }
    return finish_host_copy(out, dout, (size_t)n * out_size * sizeof(double), out_on_device, s);
}

extern "C" int wb_mass_profile(const wb_series *y, const wb_series *x, double *out,
                               int32_t out_on_device, void *stream_) {
    WB_TRACE();
    WB_TRY(check_series(y, "y"));
    WB_TRY(check_series(x, "x"));
    if (y->n != x->n) return fail(WB_EINVAL, "y and x must have the same number of samples.");
    const int L = (int)y->n_timestep, T = (int)x->n_timestep;
    if (L < 1 || L > T) return fail(WB_EINVAL, "subsequence in y is larger than input in x.");
    const int64_t n = x->n;
    const int nwin = T - L + 1;
    if (n == 0) return WB_OK;
    if (!out) return fail(WB_EINVAL, "out is NULL");
    cudaStream_t s = (cudaStream_t)stream_;
    Workspace ws(s);
    WB_TRY(ws.reserve(stage_bytes(x) + stage_bytes(y) + 3 * align256((size_t)n * nwin * 8)));
    SeriesSet sx, sy;
    // _DistanceProfile reads x[i, 0] and y[i, 0] (distance/_cdistance.pyx:1680-1699)
    WB_TRY(stage(x, 0, ws, sx));
    WB_TRY(stage(y, 0, ws, sy));
    WB_TAKE(mt, double, ws, (size_t)n * nwin);
    WB_TAKE(st, double, ws, (size_t)n * nwin);
    double *dout = out_on_device ? out : ws.take<double>((size_t)n * nwin);
    if (!dout) return fail(WB_ENOMEM, "workspace reservation exceeded");
    WB_TRY(launch_mass_profile(sx.base, n, sx.stride, T, sy.base, sy.stride, L, mt, st, dout, s));
    return finish_host_copy(out, dout, (size_t)n * nwin * sizeof(double), out_on_device, s);
}

extern "C" int wb_inject_fault(int32_t site, int64_t skip) {
    WB_TRACE();
    if (site < INJ_NONE || site > INJ_WAIT) return fail(WB_EINVAL, "unknown fault site");
    if (skip < 0) return fail(WB_EINVAL, "skip must be >= 0");
    std::lock_guard<std::mutex> g(g_inject_mu);
    g_inject_env_read = true;  // an explicit setting replaces the environment's
    g_inject_site = site;
    g_inject_skip = skip;
    return WB_OK;
}

extern "C" const char *wb_last_error(void) { return g_last_error.c_str(); }

extern "C" int32_t wb_version(void) { return 1; }

extern "C" int64_t wb_launch_count(void) { return g_launches.load(); }

extern "C" int wb_release_workspace(void *stream_) {
    WB_TRACE();
    std::lock_guard<std::mutex> g(g_arena_mu);
    for (auto it = g_arenas.begin(); it != g_arenas.end();) {
        if (stream_ == nullptr || it->first.second == (cudaStream_t)stream_) {
            Arena *a = it->second;
            std::lock_guard<std::mutex> ga(a->mu);
            if (a->base) cudaFree(a->base);
            a->base = nullptr;
            a->cap = 0;
            it = g_arenas.erase(it);
            // the arena object itself is kept alive: a concurrent Workspace
            // may still hold a pointer to it
        } else {
            ++it;
        }
    }
    return WB_OK;
}
