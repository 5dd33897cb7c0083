// noalloc.cu -- pairwise distance without any device allocation.
//
// Some callers cannot let a library call cudaMalloc / cudaFree: services that
// reserve all device memory up front and account for every byte (a
// cudaMalloc there can fail under fragmentation or silently push the process
// past its budget), and hosts whose hot loop must not synchronise the device
// (cudaFree waits for the whole device).  wb_pairwise_distance_noalloc serves
// them: the caller passes device-resident inputs and output, and the only
// scratch the recurrence needs -- the per-thread band rings of the global-ring
// variant of elastic_pairs_kernel, plus the wdtw/wlcss weight table -- lives in
// the file-scope array below, sized once at load time.
//
// The array is kStaticScratchBytes (64 MiB) of device memory that every GPU
// which loads this library keeps until the process exits.  All calls share
// it and it keeps the previous call's contents; nothing in it needs to start
// at zero (every ring slot is written before it is read, the weight table is
// rewritten by each call that uses it).  Calls that overlap on the GPU -- two
// streams, or two host threads -- race on the array: serialise them.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address with cudaGetSymbolAddress and caches it per device;
// make that first call before any stream capture begins.  The cached address
// belongs to the device context the library first saw: a cudaDeviceReset after
// that call is not supported (a new context may place the array elsewhere).
//
// A band ring that fits in shared memory runs on the shared-memory kernel and
// touches no scratch at all; only wider bands use the static array.  wdtw and
// wlcss upload their weight table from pageable host memory, a copy the CUDA
// driver orders with the stream's earlier work before it returns: those two
// metrics wait for the stream on every call and are refused while the stream
// is being captured.

#include <algorithm>
#include <mutex>
#include <vector>

#include "elastic.cuh"

namespace wb {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static std::mutex g_scratch_mu;
static void *g_scratch_addr[64] = {nullptr};

// Device address of g_static_scratch on the current device (the host-side
// name is only a stand-in and must never reach a kernel).
static int static_scratch(void **out) {
    int dev = 0;
    WB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(WB_EINVAL, "device ordinal out of range");
    std::lock_guard<std::mutex> g(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return WB_OK;
}

static int check_device_series(const wb_series *s, const char *name) {
    if (!s) return fail(WB_EINVAL, std::string(name) + " is NULL");
    if (s->n < 0 || s->n_dims < 1 || s->n_timestep < 1)
        return fail(WB_EINVAL, std::string(name) + " has an invalid shape");
    if (s->dtype != WB_F64) return fail(WB_EINVAL, std::string(name) + " must be float64");
    if (!s->on_device)
        return fail(WB_EINVAL, std::string(name) +
                                   " must be device memory: the no-allocation entry point "
                                   "does not stage host inputs");
    if (s->n > 0 && !s->data) return fail(WB_EINVAL, std::string(name) + " data is NULL");
    if (s->n_timestep > (int64_t)1 << 28)
        return fail(WB_EINVAL, std::string(name) + " has too many timesteps");
    return WB_OK;
}

}  // namespace wb

using namespace wb;

extern "C" int wb_pairwise_distance_noalloc(const wb_series *x, const wb_series *y,
                                            int64_t dim, int32_t metric,
                                            const wb_params *params, double *out,
                                            void *stream_) {
    WB_TRACE();
    WB_TRY(check_device_series(x, "x"));
    if (y) WB_TRY(check_device_series(y, "y"));
    if (!params) return fail(WB_EINVAL, "params is NULL");
    if (dim < 0 || dim >= x->n_dims)
        return fail(WB_EINVAL, "The parameter dim must be 0 <= dim < n_dims");
    if (y && y->n_dims != x->n_dims)
        return fail(WB_EINVAL, "x and y must have the same number of dimensions.");
    const wb_series *yy = y ? y : x;
    const int xl = (int)x->n_timestep, yl = (int)yy->n_timestep;
    if (metric == WB_EUCLIDEAN && xl != yl)
        return fail(WB_EINVAL, "Illegal n_timestep for non-elastic distance measure");
    const double r = params->r;
    if (metric != WB_EUCLIDEAN && !(r >= 0.0 && r <= 1.0))
        return fail(WB_EINVAL, "r must be in [0, 1]");

    ElasticJob J;
    J.len_norm_rows = xl;
    J.len_norm_cols = yl;
    J.band = compute_r(std::min(xl, yl), r);
    bool weights = false;
    switch (metric) {
        case WB_EUCLIDEAN: J.kind = K_EUCLID; J.result = R_SQRT; J.band = 1; break;
        case WB_DTW: J.kind = K_DTW; J.result = R_SQRT; break;
        case WB_WDTW: J.kind = K_WDTW; J.result = R_SQRT; weights = true; break;
        case WB_ADTW:
            J.kind = params->p >= 0.0 ? K_ADTW : K_ADTW_ANY;
            J.result = R_SQRT;
            J.p = params->p;
            break;
        case WB_LCSS:
        case WB_WLCSS:
            if (!(params->epsilon > 0.0)) return fail(WB_EINVAL, "epsilon must be > 0");
            J.kind = metric == WB_LCSS ? K_LCSS : K_WLCSS;
            J.result = R_LCSS;
            J.eps = params->epsilon;
            weights = metric == WB_WLCSS;
            break;
        case WB_EDR:
            if (!(params->epsilon > 0.0))
                return fail(WB_EINVAL, "the no-allocation entry point needs an explicit "
                                       "edr epsilon > 0 (the per-pair default needs a "
                                       "std table)");
            J.kind = K_EDR;
            J.result = R_EDR;
            J.eps = params->epsilon;
            break;
        case WB_MSM: J.kind = K_MSM; J.result = R_IDENT; J.c = params->c; break;
        default:
            return fail(WB_EUNSUPPORTED,
                        "metric id " + std::to_string(metric) +
                            " needs per-call tables and is not provided without allocation "
                            "(supported: euclidean, dtw, wdtw, adtw, lcss, wlcss, edr with "
                            "epsilon, msm)");
    }
    if (x->n == 0 || yy->n == 0) return WB_OK;
    if (!out) return fail(WB_EINVAL, "out is NULL");
    cudaStream_t s = (cudaStream_t)stream_;

    void *base = nullptr;
    WB_TRY(static_scratch(&base));
    char *scratch = static_cast<char *>(base);
    size_t avail = kStaticScratchBytes;
    if (weights) {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        WB_CUDA(cudaStreamIsCapturing(s, &cap));
        if (cap != cudaStreamCaptureStatusNone)
            return fail(WB_EUNSUPPORTED, "wdtw / wlcss upload a weight table from host "
                                         "memory and cannot run while the stream is "
                                         "captured");
        // WeightedDtwMetric.reset: w[i] = 1 / (1 + exp(-g (i - n/2))), n = max width
        const int64_t nw = std::max(xl, yl);
        const size_t wbytes = align256((size_t)nw * sizeof(double));
        if (wbytes >= avail)
            return fail(WB_EINVAL, "weight table exceeds the static scratch of " +
                                       std::to_string(kStaticScratchBytes) + " bytes");
        std::vector<double> w((size_t)nw);
        for (int64_t i = 0; i < nw; i++)
            w[i] = 1.0 / (1.0 + std::exp(-params->g * ((double)i - (double)nw / 2.0)));
        // a copy from pageable memory returns once the driver holds the data,
        // so the vector may go out of scope afterwards
        WB_CUDA(cudaMemcpyAsync(scratch, w.data(), nw * sizeof(double),
                                cudaMemcpyHostToDevice, s));
        J.weights = reinterpret_cast<const double *>(scratch);
        scratch += wbytes;
        avail -= wbytes;
    }

    const double *xb = static_cast<const double *>(x->data);
    const double *yb = static_cast<const double *>(yy->data);
    J.rows.base = xb + dim * x->n_timestep;
    J.rows.stride = x->n_dims * x->n_timestep;
    J.rows.count = x->n;
    J.rows.len = xl;
    J.cols.base = yb + dim * yy->n_timestep;
    J.cols.stride = yy->n_dims * yy->n_timestep;
    J.cols.count = yy->n;
    J.cols.len = yl;
    J.out = out;
    J.out_ld = yy->n;
    J.mode = y ? PM_ALL : PM_UPPER;
    if (!y) WB_CUDA(cudaMemsetAsync(out, 0, (size_t)x->n * x->n * sizeof(double), s));
    const int st = launch_elastic_shared_ring(J, s);
    if (st != WB_EUNSUPPORTED) return st;
    return launch_elastic_external_ring(J, reinterpret_cast<double *>(scratch), avail, s);
}

extern "C" int64_t wb_noalloc_scratch_bytes(void) { return (int64_t)kStaticScratchBytes; }
