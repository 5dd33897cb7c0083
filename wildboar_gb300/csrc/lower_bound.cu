// lower_bound.cu -- the dtw lower-bound producers of distance/lb.py:
// DtwKeoghLowerBound (:314-432) and DtwKimLowerBound (:198-311), FP64, the
// reference's values.
//
//  * lb_envelope_kernel: one thread per series runs find_min_max with the
//    reference's deques (capacity 2 r + 2, as _dtw_envelop allocates them,
//    distance/_elastic.pyx:1076-1092); envelopes are written k-major so that
//    a warp of consecutive series writes consecutive addresses.
//  * lb_keogh_kernel: out[i, j] = max(left, right), left = sqrt(sum_k
//    term(q_i[k], env x_j)), right = sqrt(sum_k term(x_j[k], env q_i)) with
//    term the excursion of cumulative_bound (:240-270) at mean 0, std 1; the
//    sum runs over k in order.  A thread owns one database series j and four
//    queries; database values and envelopes are k-major (coalesced across the
//    warp), query values are broadcast.  Bound: FP64 (five operations per
//    term), the loads hit L2.
//  * lb_kim_kernel: the six-term constant-time bound of DtwKimLowerBound, one
//    thread per (query, database) pair, the reference's numpy operations in
//    its order.

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "envelope.cuh"

namespace wb {

namespace {

__global__ void lb_envelope_kernel(const double *x, int64_t n, int L, int r, int *dq,
                                   double *lowerT, double *upperT) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int cap = 2 * r + 2;
    DevDeque dl{dq + j * 2 * cap, cap, 0, 0, 0}, du{dq + j * 2 * cap + cap, cap, 0, 0, 0};
    sdtw_envelope(x + j * L, L, r, lowerT + j, upperT + j, dl, du, n);
}

__global__ void lb_transpose_kernel(const double *x, int64_t n, int L, double *xT) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * (int64_t)L) return;
    const int64_t k = t / n, j = t - (t / n) * n;
    xT[t] = x[j * L + k];
}

// excursion of x outside [lo, up]: cumulative_bound's term at mean 0, std 1
__device__ __forceinline__ double lb_term(double x, double up, double lo) {
    if (x > up) {
        const double d = x - up;
        return d * d;
    }
    if (x < lo) {
        const double d = x - lo;
        return d * d;
    }
    return 0.0;
}

constexpr int kLbQ = 4;  // queries per thread

// kind: 0 both, 1 left (query vs database envelope), 2 right (database vs
// query envelope)
__global__ void lb_keogh_kernel(const double *q, const double *ql, const double *qu,
                                int64_t nq, const double *xT, const double *xlT,
                                const double *xuT, int64_t nx, int L, int kind, double *out) {
    const double NINF = -__longlong_as_double(0x7ff0000000000000LL);
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t i0 = (int64_t)blockIdx.y * kLbQ;
    if (j >= nx) return;
    const bool left = kind != 2, right = kind != 1;
    double sl[kLbQ], sr[kLbQ];
#pragma unroll
    for (int a = 0; a < kLbQ; a++) {
        sl[a] = 0.0;
        sr[a] = 0.0;
    }
    for (int k = 0; k < L; k++) {
        const int64_t o = (int64_t)k * nx + j;
        const double xv = right ? xT[o] : 0.0;
        const double xl = left ? xlT[o] : 0.0;
        const double xu = left ? xuT[o] : 0.0;
#pragma unroll
        for (int a = 0; a < kLbQ; a++) {
            const int64_t i = i0 + a;
            if (i < nq) {
                const int64_t p = i * L + k;
                if (left) sl[a] = sl[a] + lb_term(q[p], xu, xl);
                if (right) sr[a] = sr[a] + lb_term(xv, qu[p], ql[p]);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < kLbQ; a++) {
        const int64_t i = i0 + a;
        if (i < nq) {
            const double d1 = left ? sqrt(sl[a]) : NINF;
            const double d2 = right ? sqrt(sr[a]) : NINF;
            // max(dist1, dist2) of Python: the first unless the second is larger
            out[i * nx + j] = d2 > d1 ? d2 : d1;
        }
    }
}

__device__ __forceinline__ double kd(double a, double b) {
    const double v = a - b;
    return v * v;
}
// np.minimum of two non-NaN values
__device__ __forceinline__ double kmin(double a, double b) { return b < a ? b : a; }

// DtwKimLowerBound.transform (distance/lb.py:224-311): x rows are the
// fitted series, y rows the queries; out is (ny, nx)
__global__ void lb_kim_kernel(const double *y, int64_t ny, const double *x, int64_t nx, int L,
                              double *out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ny * nx) return;
    const int64_t i = t / nx, j = t - (t / nx) * nx;
    const double *X = x + j * L, *Y = y + i * L;
    const double x0 = X[0], x0_ = X[L - 1], y0 = Y[0], y0_ = Y[L - 1];
    double d = kd(x0, y0) + kd(x0_, y0_);
    if (L > 1) {
        const double x1 = X[1], x1_ = X[L - 2], y1 = Y[1], y1_ = Y[L - 2];
        d = d + kmin(kd(x1, y0), kmin(kd(x0, y1), kd(x1, y1)));
        d = d + kmin(kd(x1_, y1), kmin(kd(x0_, y1_), kd(x1_, y1_)));
        if (L > 2) {
            const double x2 = X[2], x2_ = X[L - 3], y2 = Y[2], y2_ = Y[L - 3];
            d = d + kmin(kd(x0, y2),
                         kmin(kd(x1, y2), kmin(kd(x2, y2), kmin(kd(x2, y1), kd(x2, y0)))));
            d = d + kmin(kd(x0_, y2_), kmin(kd(x1_, y2_),
                                            kmin(kd(x2_, y2_), kmin(kd(x2_, y1_), kd(x2_, y0_)))));
        }
    }
    out[t] = d;
}

// _dtw_lb_keogh (distance/_elastic.pyx:1095-1115) of one series: the terms
// cb[k] and sqrt of their sum in order (one thread: the sum is sequential)
__global__ void lb_terms_kernel(const double *x, const double *lo, const double *up, int L,
                                double *cb, double *dist) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double s = 0.0;
    for (int k = 0; k < L; k++) {
        const double d = lb_term(x[k], up[k], lo[k]);
        cb[k] = d;
        s = s + d;
    }
    dist[0] = sqrt(s);
}

int dev_in(const double *src, size_t count, int on_device, Workspace &ws, const double **dst) {
    if (on_device) {
        *dst = src;
        return WB_OK;
    }
    double *d = ws.take<double>(count);
    if (!d) return fail(WB_ENOMEM, "workspace reservation exceeded");
    WB_CUDA(cudaMemcpyAsync(d, src, count * 8, cudaMemcpyHostToDevice, ws.stream()));
    *dst = d;
    return WB_OK;
}

}  // namespace

}  // namespace wb

using namespace wb;

extern "C" int wb_dtw_envelope(const double *x, int64_t n, int64_t n_timestep, int64_t warp,
                               double *lower, double *upper, int32_t on_device, void *stream) {
    WB_TRACE();
    const cudaStream_t s = (cudaStream_t)stream;
    if (n < 0 || n_timestep < 1 || n_timestep > INT32_MAX / 4)
        return fail(WB_EINVAL, "invalid sizes");
    if (!(0 <= warp && warp < n_timestep)) return fail(WB_EINVAL, "invalid r");
    if (n == 0) return WB_OK;
    if (!x || !lower || !upper) return fail(WB_EINVAL, "NULL array");
    const int L = (int)n_timestep, r = (int)warp;
    const size_t cnt = (size_t)n * L;
    Workspace ws(s);
    WB_TRY(ws.reserve((on_device ? 0 : align256(cnt * 8)) + 3 * align256(cnt * 8) +
                      align256((size_t)n * 2 * (2 * r + 2) * 4) + 1024));
    const double *dx;
    WB_TRY(dev_in(x, cnt, on_device, ws, &dx));
    WB_TAKE(lT, double, ws, cnt);
    WB_TAKE(uT, double, ws, cnt);
    WB_TAKE(dq, int, ws, (size_t)n * 2 * (2 * r + 2));
    lb_envelope_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(dx, n, L, r, dq, lT, uT);
    WB_LAUNCH_CHECK("lb_envelope_kernel");
    // back to row-major
    WB_TAKE(tmp, double, ws, cnt);
    const int64_t nt = (int64_t)cnt;
    // lT is (L, n): its transpose with "rows" L and length n
    for (int which = 0; which < 2; which++) {
        const double *src = which == 0 ? lT : uT;
        double *dst = which == 0 ? lower : upper;
        double *o = on_device ? dst : tmp;
        lb_transpose_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(src, L, (int)n, o);
        WB_LAUNCH_CHECK("lb_transpose_kernel");
        if (!on_device)
            WB_CUDA(cudaMemcpyAsync(dst, tmp, cnt * 8, cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaStreamSynchronize(s));
    }
    return WB_OK;
}

extern "C" int wb_lb_keogh(const double *q, int64_t nq, const double *x, int64_t nx,
                           int64_t n_timestep, int64_t warp, int32_t kind, double *out,
                           int32_t on_device, void *stream) {
    WB_TRACE();
    const cudaStream_t s = (cudaStream_t)stream;
    if (nq < 0 || nx < 0 || n_timestep < 1 || n_timestep > INT32_MAX / 4)
        return fail(WB_EINVAL, "invalid sizes");
    if (!(0 <= warp && warp < n_timestep)) return fail(WB_EINVAL, "invalid r");
    if (kind < 0 || kind > 2) return fail(WB_EINVAL, "kind must be 0 (both), 1 (left), 2 (right)");
    if (nq == 0 || nx == 0) return WB_OK;
    if (!q || !x || !out) return fail(WB_EINVAL, "NULL array");
    const int L = (int)n_timestep, r = (int)warp;
    const size_t cq = (size_t)nq * L, cx = (size_t)nx * L, co = (size_t)nq * nx;
    const int cap = 2 * r + 2;
    Workspace ws(s);
    WB_TRY(ws.reserve((on_device ? 0 : align256(cq * 8) + align256(cx * 8) + align256(co * 8)) +
                      3 * align256(cx * 8) + 4 * align256(cq * 8) +
                      align256((size_t)std::max(nq, nx) * 2 * cap * 4) + 2048));
    const double *dq_, *dx_;
    WB_TRY(dev_in(q, cq, on_device, ws, &dq_));
    WB_TRY(dev_in(x, cx, on_device, ws, &dx_));
    WB_TAKE(xT, double, ws, cx);
    WB_TAKE(xlT, double, ws, cx);
    WB_TAKE(xuT, double, ws, cx);
    WB_TAKE(qlT, double, ws, cq);
    WB_TAKE(quT, double, ws, cq);
    WB_TAKE(ql, double, ws, cq);
    WB_TAKE(qu, double, ws, cq);
    WB_TAKE(dqs, int, ws, (size_t)std::max(nq, nx) * 2 * cap);
    double *o = out;
    if (!on_device) {
        o = ws.take<double>(co);
        if (!o) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    // database values and envelopes k-major; query envelopes row-major
    lb_transpose_kernel<<<(unsigned)(((int64_t)cx + 255) / 256), 256, 0, s>>>(dx_, nx, L, xT);
    WB_LAUNCH_CHECK("lb_transpose_kernel");
    if (kind != 2) {
        lb_envelope_kernel<<<(unsigned)((nx + 127) / 128), 128, 0, s>>>(dx_, nx, L, r, dqs, xlT,
                                                                         xuT);
        WB_LAUNCH_CHECK("lb_envelope_kernel");
    }
    if (kind != 1) {
        lb_envelope_kernel<<<(unsigned)((nq + 127) / 128), 128, 0, s>>>(dq_, nq, L, r, dqs, qlT,
                                                                         quT);
        WB_LAUNCH_CHECK("lb_envelope_kernel");
        // (L, nq) k-major -> (nq, L)
        lb_transpose_kernel<<<(unsigned)(((int64_t)cq + 255) / 256), 256, 0, s>>>(qlT, L,
                                                                                  (int)nq, ql);
        lb_transpose_kernel<<<(unsigned)(((int64_t)cq + 255) / 256), 256, 0, s>>>(quT, L,
                                                                                  (int)nq, qu);
        WB_LAUNCH_CHECK("lb_transpose_kernel");
    }
    dim3 grid((unsigned)((nx + 127) / 128), (unsigned)((nq + kLbQ - 1) / kLbQ));
    timer_begin("lb_keogh_kernel", s);
    lb_keogh_kernel<<<grid, 128, 0, s>>>(dq_, ql, qu, nq, xT, xlT, xuT, nx, L, (int)kind, o);
    timer_end(s);
    WB_LAUNCH_CHECK("lb_keogh_kernel");
    if (!on_device) WB_CUDA(cudaMemcpyAsync(out, o, co * 8, cudaMemcpyDeviceToHost, s));
    WB_CUDA(cudaStreamSynchronize(s));
    return WB_OK;
}

extern "C" int wb_lb_kim(const double *y, int64_t ny, const double *x, int64_t nx,
                         int64_t n_timestep, double *out, int32_t on_device, void *stream) {
    WB_TRACE();
    const cudaStream_t s = (cudaStream_t)stream;
    if (ny < 0 || nx < 0 || n_timestep < 1 || n_timestep > INT32_MAX / 4)
        return fail(WB_EINVAL, "invalid sizes");
    if (ny == 0 || nx == 0) return WB_OK;
    if (!y || !x || !out) return fail(WB_EINVAL, "NULL array");
    const int L = (int)n_timestep;
    const size_t cy = (size_t)ny * L, cx = (size_t)nx * L, co = (size_t)ny * nx;
    Workspace ws(s);
    WB_TRY(ws.reserve((on_device ? 0 : align256(cy * 8) + align256(cx * 8) + align256(co * 8)) +
                      1024));
    const double *dy, *dx;
    WB_TRY(dev_in(y, cy, on_device, ws, &dy));
    WB_TRY(dev_in(x, cx, on_device, ws, &dx));
    double *o = out;
    if (!on_device) {
        o = ws.take<double>(co);
        if (!o) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    const int64_t t = (int64_t)co;
    lb_kim_kernel<<<(unsigned)((t + 255) / 256), 256, 0, s>>>(dy, ny, dx, nx, L, o);
    WB_LAUNCH_CHECK("lb_kim_kernel");
    if (!on_device) WB_CUDA(cudaMemcpyAsync(out, o, co * 8, cudaMemcpyDeviceToHost, s));
    WB_CUDA(cudaStreamSynchronize(s));
    return WB_OK;
}

extern "C" int wb_lb_keogh_terms(const double *x, const double *lower, const double *upper,
                                 int64_t n_timestep, double *cb, double *dist,
                                 int32_t on_device, void *stream) {
    WB_TRACE();
    const cudaStream_t s = (cudaStream_t)stream;
    if (n_timestep < 1 || n_timestep > INT32_MAX / 4) return fail(WB_EINVAL, "invalid sizes");
    if (!x || !lower || !upper || !cb || !dist) return fail(WB_EINVAL, "NULL array");
    const size_t L = (size_t)n_timestep;
    Workspace ws(s);
    WB_TRY(ws.reserve((on_device ? 0 : 4 * align256(L * 8) + align256(8)) + 1024));
    const double *dx, *dl, *du;
    WB_TRY(dev_in(x, L, on_device, ws, &dx));
    WB_TRY(dev_in(lower, L, on_device, ws, &dl));
    WB_TRY(dev_in(upper, L, on_device, ws, &du));
    double *dcb = cb, *dd = dist;
    if (!on_device) {
        dcb = ws.take<double>(L);
        dd = ws.take<double>(1);
        if (!dcb || !dd) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    lb_terms_kernel<<<1, 32, 0, s>>>(dx, dl, du, (int)L, dcb, dd);
    WB_LAUNCH_CHECK("lb_terms_kernel");
    if (!on_device) {
        WB_CUDA(cudaMemcpyAsync(cb, dcb, L * 8, cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaMemcpyAsync(dist, dd, 8, cudaMemcpyDeviceToHost, s));
    }
    WB_CUDA(cudaStreamSynchronize(s));
    return WB_OK;
}
