// diag.cu -- measurement helpers: device timing of the main kernel of the
// last call, and an FP64 / FP32 throughput probe used as the roofline peak of
// the ALU-bound recurrence kernels.

#include "common.cuh"

namespace wb {

struct KernelTimer {
    bool enabled = false;
    cudaEvent_t start = nullptr, stop = nullptr;
    std::string name;
    bool pending = false;
};
static thread_local KernelTimer g_timer;

void timer_begin(const char *name, cudaStream_t s) {
    if (!g_timer.enabled) return;
    if (!g_timer.start) {
        cudaEventCreate(&g_timer.start);
        cudaEventCreate(&g_timer.stop);
    }
    g_timer.name = name;
    cudaEventRecord(g_timer.start, s);
}

void timer_end(cudaStream_t s) {
    if (!g_timer.enabled || !g_timer.start) return;
    cudaEventRecord(g_timer.stop, s);
    g_timer.pending = true;
}

// independent add/mul chains (no contraction: this file is built with
// -fmad=false), 8 per thread so the pipe, not latency, is the limit
template <typename T>
__global__ void alu_probe_kernel(T *out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int i = 0; i < iters; i++) {
        x0 = x0 * a; x1 = x1 * a; x2 = x2 * a; x3 = x3 * a;
        x4 = x4 * a; x5 = x5 * a; x6 = x6 * a; x7 = x7 * a;
        x0 = x0 + b; x1 = x1 + b; x2 = x2 + b; x3 = x3 + b;
        x4 = x4 + b; x5 = x5 + b; x6 = x6 + b; x7 = x7 + b;
    }
    T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-12345) out[0] = s;  // keep the chains alive
}

}  // namespace wb

using namespace wb;

extern "C" int wb_profile_enable(int32_t on) {
    WB_TRACE();
    g_timer.enabled = on != 0;
    g_timer.pending = false;
    return WB_OK;
}

extern "C" int wb_profile_last(double *ms) {
    WB_TRACE();
    if (!ms) return fail(WB_EINVAL, "ms is NULL");
    *ms = -1.0;
    if (!g_timer.pending) return WB_OK;
    WB_CUDA(cudaEventSynchronize(g_timer.stop));
    float f = 0;
    WB_CUDA(cudaEventElapsedTime(&f, g_timer.start, g_timer.stop));
    *ms = f;
    g_timer.pending = false;
    return WB_OK;
}

extern "C" int wb_alu_probe(int32_t dtype, int32_t iters, double *ops_per_s) {
    WB_TRACE();
    if (!ops_per_s) return fail(WB_EINVAL, "ops_per_s is NULL");
    const DeviceInfo &dev = device_info();
    int grid = dev.sm_count * 8, block = 256;
    void *scratch = nullptr;
    WB_CUDA(cudaMalloc(&scratch, 64));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    auto run = [&](int it) {
        if (dtype == WB_F64)
            alu_probe_kernel<double><<<grid, block>>>((double *)scratch, it, 0.999999, 1e-6);
        else
            alu_probe_kernel<float><<<grid, block>>>((float *)scratch, it, 0.999999f, 1e-6f);
    };
    run(16);  // warm-up
    cudaEventRecord(a);
    run(iters);
    cudaEventRecord(b);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(scratch);
    if (e != cudaSuccess) return cuda_fail(e, "alu probe");
    count_launch(2);
    double ops = 16.0 * (double)iters * grid * block;
    *ops_per_s = ops / (ms * 1e-3);
    return WB_OK;
}
