// common.cuh -- shared host/device helpers of the wbgpu library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <mutex>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "../../include/wbgpu.h"

namespace wb {

// An NVTX range named after the C-ABI entry for the duration of the call, so
// profiler timelines (nsys, ncu --nvtx) show which entry launched which
// kernels; without an attached tool it costs one pointer test.
struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};
#define WB_TRACE() ::wb::TraceRange wb_trace_range_(__func__)

// ---------------------------------------------------------------------------
// errors

void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
void count_launch(int64_t n = 1);
// optional device timing of the main kernel of a call (wb_profile_enable)
void timer_begin(const char *name, cudaStream_t s);
void timer_end(cudaStream_t s);

#define WB_CUDA(call)                                       \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return ::wb::cuda_fail(e_, #call); \
    } while (0)

// Host-side fault injection (wb_inject_fault, WB_GPU_INJECT_FAULT): a
// matching site returns its error as if the CUDA call or the wait had failed;
// nothing on the device faults.
enum InjectSite { INJ_NONE = 0, INJ_RESERVE = 1, INJ_LAUNCH = 2, INJ_WAIT = 3 };
bool injected(int site);

#define WB_LAUNCH_CHECK(what)                               \
    do {                                                    \
        ::wb::count_launch();                               \
        cudaError_t e_ = cudaGetLastError();                \
        if (e_ != cudaSuccess) return ::wb::cuda_fail(e_, what); \
        if (::wb::injected(::wb::INJ_LAUNCH))               \
            return ::wb::fail(WB_ECUDA, std::string(what) + ": injected launch failure"); \
    } while (0)

#define WB_TAKE(var, T, ws, count)                                           \
    T *var = (ws).take<T>(count);                                            \
    if (!var) return ::wb::fail(WB_ENOMEM, "workspace reservation exceeded");

#define WB_TRY(call)                 \
    do {                             \
        int s_ = (call);             \
        if (s_ != WB_OK) return s_;  \
    } while (0)

// ---------------------------------------------------------------------------
// device workspace: one grow-only arena per stream, bump-allocated per call

struct Arena {
    char *base = nullptr;
    size_t cap = 0;
    size_t used = 0;
    std::mutex mu;
};

// Holds the arena of `stream` for the duration of one API call.
class Workspace {
  public:
    explicit Workspace(cudaStream_t stream);
    ~Workspace();
    // reserve `bytes` (256-byte aligned) for this call; grows the arena when
    // the call's total exceeds it.  Must be called before any pointer from
    // this call is used (all requests are made up front by `plan`).
    int reserve(size_t bytes);
    // nullptr when the call's reservation is exhausted (see WB_TAKE)
    template <class T>
    T *take(size_t count) {
        size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        if (!arena_->base || arena_->used + bytes > arena_->cap) return nullptr;
        char *p = arena_->base + arena_->used;
        arena_->used += bytes;
        return reinterpret_cast<T *>(p);
    }
    cudaStream_t stream() const { return stream_; }
    // rewind to an earlier position: later takes reuse the memory, which is
    // safe for work enqueued on this call's stream (it runs in order)
    size_t mark() const { return arena_->used; }
    void rewind(size_t m) { arena_->used = m; }

  private:
    Arena *arena_;
    cudaStream_t stream_;
    std::unique_lock<std::mutex> lock_;
};

size_t align256(size_t b);

// ---------------------------------------------------------------------------
// device properties

struct DeviceInfo {
    int device = 0;
    int sm_count = 0;
    int max_smem_optin = 0;   // per block
    int smem_per_sm = 0;
};
const DeviceInfo &device_info();

// ---------------------------------------------------------------------------
// device helpers

__host__ __device__ inline int imin(int a, int b) { return a < b ? a : b; }
__host__ __device__ inline int imax(int a, int b) { return a > b ? a : b; }

// band half-width: _compute_r (distance/_elastic.pyx:1924-1925)
inline int compute_r(int64_t length, double r) {
    double v = std::floor((double)length * r);
    return (int)(v > 1.0 ? v : 1.0);
}

#ifdef __CUDACC__
// min / max of non-negative doubles (including +inf) through their bit
// patterns: for x, y >= +0 the IEEE order equals the signed 64-bit order, so
// the comparison runs on the integer pipe instead of the FP64 pipe.  Equal
// values have equal bits, so the result is the value Cython's
// "b < a ? b : a" would give.
// Bit pattern of an epsilon compared with v = |x - y| (non-negative, never
// NaN) on the integer pipe: v <= eps iff bits(v) <= eps_bits(eps), and the
// same for <.  Negative doubles have negative patterns (never reached by v);
// NaN, which no comparison satisfies, maps to -1.0 and -0.0 to +0.0 (equal
// as doubles, different patterns).
__device__ __forceinline__ long long eps_bits(double eps) {
    if (isnan(eps)) eps = -1.0;
    if (eps == 0.0) eps = 0.0;
    return __double_as_longlong(eps);
}
__device__ __forceinline__ long long dbits_of(double v) { return __double_as_longlong(v); }
// bit pattern of |d|: clearing the sign bit is an integer operation, where a
// stand-alone fabs could take an FP64 instruction
__device__ __forceinline__ long long abs_bits(double d) {
    return __double_as_longlong(d) & 0x7fffffffffffffffLL;
}

// (double)m for a non-negative float, exact, on the integer pipe for zero and
// normal floats (sign 0, exponent field e in 1..254: the double has exponent
// field e + 1023 - 127 and the 23 mantissa bits shifted up by 29); subnormal,
// infinite and NaN values go through the conversion instruction.
__device__ __forceinline__ double f2d_nonneg(float m) {
    const unsigned int u = __float_as_uint(m);
    if (u - 0x00800000u >= 0x7f000000u && u != 0u) return (double)m;
    const unsigned long long b = u ? ((unsigned long long)u << 29) + (896ull << 52) : 0ull;
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ double nn_min(double a, double b) {
    long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    return __longlong_as_double(ib < ia ? ib : ia);
}
__device__ __forceinline__ double nn_max(double a, double b) {
    long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    return __longlong_as_double(ib > ia ? ib : ia);
}
// Cython's lowering of builtin min/max on C doubles
__device__ __forceinline__ double cy_min(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double cy_max(double a, double b) { return b > a ? b : a; }
#endif

}  // namespace wb
