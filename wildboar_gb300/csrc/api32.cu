// api32.cu -- C ABI of the FP32 (compensated) dtw forms: batched / ragged
// distances and the backward pass.  Device pointers only; no host
// synchronisation and no allocation once the stream's workspace has grown to
// the job's size, so a call can be captured in a CUDA graph after a warm-up.

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "dtw32.cuh"

namespace wb {

// Validate a job and fill `J` (everything but the scratch pointers); `bytes`
// is the workspace the scratch needs.
int dtw32_plan(const wb_dtw32 *q, bool backward, Dtw32Job &J, size_t &bytes) {
    if (!q) return fail(WB_EINVAL, "job is NULL");
    if (q->x_len < 1 || q->y_len < 1) return fail(WB_EINVAL, "x_len and y_len must be >= 1");
    if (!(q->r >= 0.0 && q->r <= 1.0)) return fail(WB_EINVAL, "r must be in [0, 1]");
    if (q->n_items < 0) return fail(WB_EINVAL, "negative number of items");
    const bool items = q->item_x != nullptr;
    if (items != (q->item_y != nullptr)) return fail(WB_EINVAL, "item_x and item_y go together");
    if (!items && q->n_items != q->nx * q->ny)
        return fail(WB_EINVAL, "without item arrays n_items must be nx * ny");
    const int strip = backward ? 16 : (q->strip ? q->strip : 16);
    if (strip != 4 && strip != 8 && strip != 16 && strip != 24 && strip != 32)
        return fail(WB_EINVAL, "strip must be one of 4, 8, 16, 24, 32");
    int block = q->block ? q->block : 128;
    if (block % 32 || block < 32 || block > 256)
        return fail(WB_EINVAL, "block must be a multiple of 32 in [32, 256]");
    const DeviceInfo &dev = device_info();
    // the longer series of a dtw item goes on the columns, the shorter on the
    // rows; wdtw keeps x on the rows
    const int cols_max = std::max(q->x_len, q->y_len);
    const int rows_max = q->weights ? q->x_len : std::min(q->x_len, q->y_len);
    J.ring_cols = cols_max + 1;
    // backward geometry: strips of 16 rows cut into segments of K strips; the
    // direction words of one segment (K strips x at most cols_max columns) and
    // one checkpoint row per segment boundary per resident thread
    size_t per_thread = (size_t)J.ring_cols * sizeof(float2);
    if (backward) {
        const int64_t strips = rows_max > 1 ? (rows_max - 2) / 16 + 1 : 0;
        int64_t K = std::max<int64_t>(strips, 1);
        if (K > 64 || K * cols_max * 4 > (64 << 10)) {
            K = (int64_t)std::ceil(std::sqrt(2.0 * (double)strips));
            K = std::min<int64_t>(std::max<int64_t>(K, 1), 64);
        }
        J.seg_strips = (int)K;
        J.n_ckpt = strips > 0 ? (int)((strips + K - 1) / K - 1) : 0;
        J.dir_words = (K * cols_max + 7) / 8 * 8;  // whole 8-word groups
        per_thread += (size_t)J.dir_words * sizeof(uint32_t) +
                      (size_t)J.n_ckpt * J.ring_cols * sizeof(float2);
        block = 128;  // the backward kernel's block size
    }
    int grid = q->grid;
    if (grid <= 0) {
        int nb = dtw32_blocks_per_sm(strip, q->weights != nullptr, backward, block);
        if (nb < 1) nb = 1;
        grid = nb * dev.sm_count;
        if (backward) {
            // resident threads bounded by the backward workspace budget
            const char *env = getenv("WB_GPU_BWD_WORKSPACE_MB");
            const double mb = env ? atof(env) : 8192.0;
            const int64_t cap = (int64_t)(mb * 1048576.0 / ((double)per_thread * block));
            grid = (int)std::max<int64_t>(1, std::min<int64_t>(grid, cap));
        }
        int64_t need = (q->n_items + block - 1) / block;
        if (need < grid) grid = (int)std::max<int64_t>(need, 1);
    }
    J.x = q->x;
    J.x_stride = q->x_stride;
    J.xlen = q->x_lengths;
    J.x_len = q->x_len;
    J.nx = q->nx;
    J.y = q->y;
    J.y_stride = q->y_stride;
    J.ylen = q->y_lengths;
    J.y_len = q->y_len;
    J.ny = q->ny;
    J.item_x = q->item_x;
    J.item_y = q->item_y;
    J.n_items = q->n_items;
    J.r = q->r;
    J.weights = q->weights;
    J.grid = grid;
    J.block = block;
    const int64_t nth = (int64_t)grid * block;
    size_t ring_bytes = align256((size_t)J.ring_cols * nth * sizeof(float2));
    size_t dir_bytes = 0;
    if (backward) {
        dir_bytes = align256((size_t)J.dir_words * nth * sizeof(uint32_t)) +
                    align256((size_t)std::max(J.n_ckpt, 1) * J.ring_cols * nth * sizeof(float2));
    }
    bytes = ring_bytes + dir_bytes + 256;
    return WB_OK;
}

// Take the scratch of a planned job from a reserved workspace.
int dtw32_take(Workspace &ws, Dtw32Job &J, bool backward) {
    const int64_t nth = (int64_t)J.grid * J.block;
    J.ring = ws.take<float2>((size_t)J.ring_cols * nth);
    J.queue = ws.take<unsigned long long>(1);
    if (!J.ring || !J.queue) return fail(WB_ENOMEM, "workspace reservation exceeded");
    if (backward) {
        J.dirs = ws.take<uint32_t>((size_t)J.dir_words * nth);
        J.ckpt = ws.take<float2>((size_t)std::max(J.n_ckpt, 1) * J.ring_cols * nth);
        if (!J.dirs || !J.ckpt) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    return WB_OK;
}

// Geometry of the kept directions of a job: per batch of 32 items the two
// strip tables and 32 lanes x cap words, cap = every strip of the longest
// rows over the longest columns (whole groups of 8).
static int keep_geometry(const wb_dtw32 *q, DirKeep &D, int64_t &total) {
    if (!q) return fail(WB_EINVAL, "job is NULL");
    if (q->x_len < 1 || q->y_len < 1) return fail(WB_EINVAL, "x_len and y_len must be >= 1");
    if (q->n_items < 0) return fail(WB_EINVAL, "negative number of items");
    const int64_t cols_max = std::max(q->x_len, q->y_len);
    const int64_t rows_max = q->weights ? q->x_len : std::min(q->x_len, q->y_len);
    const int64_t strips = rows_max > 1 ? (rows_max - 2) / 16 + 1 : 0;
    D.max_strips = (int)std::max<int64_t>(strips, 1);
    D.cap = (std::max<int64_t>(strips * cols_max, 8) + 7) / 8 * 8;
    D.tab_bytes = (int64_t)align256((size_t)2 * D.max_strips * sizeof(int));
    D.batch_bytes = D.tab_bytes + 32 * D.cap * (int64_t)sizeof(uint32_t);
    total = (q->n_items + 31) / 32 * D.batch_bytes;
    return WB_OK;
}

// A planned job for the kept-direction kernels (128-thread blocks, grid by
// their occupancy); the ring only for the forward.
static int prepare_keep(const wb_dtw32 *q, bool walk, void *keep, int64_t keep_bytes,
                        Workspace &ws, Dtw32Job &J, DirKeep &D) {
    if (q && (!q->x || !q->y)) return fail(WB_EINVAL, "x and y must be device pointers");
    int64_t total = 0;
    WB_TRY(keep_geometry(q, D, total));
    if (!keep || keep_bytes < total) return fail(WB_EINVAL, "kept-direction buffer too small");
    D.base = static_cast<unsigned char *>(keep);
    size_t bytes = 0;
    WB_TRY(dtw32_plan(q, false, J, bytes));
    J.block = 128;
    int nb = dtw32_keep_blocks_per_sm(walk, q->weights != nullptr);
    if (nb < 1) nb = 1;
    int grid = nb * device_info().sm_count;
    const int64_t need = (q->n_items + J.block - 1) / J.block;
    if (need < grid) grid = (int)std::max<int64_t>(need, 1);
    J.grid = grid;
    const int64_t nth = (int64_t)grid * J.block;
    const size_t ring_bytes = walk ? 0 : align256((size_t)J.ring_cols * nth * sizeof(float2));
    WB_TRY(ws.reserve(ring_bytes + 512));
    if (!walk) {
        J.ring = ws.take<float2>((size_t)J.ring_cols * nth);
        if (!J.ring) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    J.queue = ws.take<unsigned long long>(1);
    if (!J.queue) return fail(WB_ENOMEM, "workspace reservation exceeded");
    return WB_OK;
}

static int prepare32(const wb_dtw32 *q, bool backward, Workspace &ws, Dtw32Job &J) {
    if (q && (!q->x || !q->y)) return fail(WB_EINVAL, "x and y must be device pointers");
    size_t bytes = 0;
    WB_TRY(dtw32_plan(q, backward, J, bytes));
    WB_TRY(ws.reserve(bytes));
    return dtw32_take(ws, J, backward);
}

}  // namespace wb

using namespace wb;

extern "C" int wb_dtw32_distance(const wb_dtw32 *q, double *out, double *out_cost,
                                 void *stream_) {
    WB_TRACE();
    if (!out) return fail(WB_EINVAL, "out is NULL");
    cudaStream_t s = (cudaStream_t)stream_;
    Workspace ws(s);
    Dtw32Job J;
    WB_TRY(prepare32(q, false, ws, J));
    J.out = out;
    J.out_cost = out_cost;
    return dtw32_forward(J, q->strip ? q->strip : 16, s);
}

extern "C" int wb_dtw32_backward(const wb_dtw32 *q, const double *grad_out, float *grad_x,
                                 int64_t gx_stride, float *grad_y, int64_t gy_stride,
                                 void *stream_) {
    WB_TRACE();
    if (!q) return fail(WB_EINVAL, "job is NULL");
    if (!grad_x || !grad_y) return fail(WB_EINVAL, "gradient outputs are NULL");
    if (gx_stride < q->x_len || gy_stride < q->y_len)
        return fail(WB_EINVAL, "gradient strides must cover x_len / y_len");
    cudaStream_t s = (cudaStream_t)stream_;
    Workspace ws(s);
    Dtw32Job J;
    WB_TRY(prepare32(q, true, ws, J));
    J.grad_out = grad_out;
    J.grad_x = grad_x;
    J.gx_stride = gx_stride;
    J.grad_y = grad_y;
    J.gy_stride = gy_stride;
    return dtw32_backward(J, s);
}

extern "C" int64_t wb_dtw32_keep_bytes(const wb_dtw32 *q) {
    WB_TRACE();
    DirKeep D;
    int64_t total = 0;
    if (keep_geometry(q, D, total) != WB_OK) return -1;
    return total;
}

extern "C" int wb_dtw32_distance_keep(const wb_dtw32 *q, double *out, double *out_cost,
                                      void *keep, int64_t keep_bytes, void *stream_) {
    WB_TRACE();
    if (!out) return fail(WB_EINVAL, "out is NULL");
    cudaStream_t s = (cudaStream_t)stream_;
    Workspace ws(s);
    Dtw32Job J;
    DirKeep D;
    WB_TRY(prepare_keep(q, false, keep, keep_bytes, ws, J, D));
    J.out = out;
    J.out_cost = out_cost;
    return dtw32_keep_forward(J, D, s);
}

extern "C" int wb_dtw32_backward_keep(const wb_dtw32 *q, const double *dist,
                                      const double *grad_out, float *grad_x, int64_t gx_stride,
                                      float *grad_y, int64_t gy_stride, const void *keep,
                                      int64_t keep_bytes, void *stream_) {
    WB_TRACE();
    if (!q) return fail(WB_EINVAL, "job is NULL");
    if (!dist) return fail(WB_EINVAL, "dist is NULL");
    if (!grad_x || !grad_y) return fail(WB_EINVAL, "gradient outputs are NULL");
    if (gx_stride < q->x_len || gy_stride < q->y_len)
        return fail(WB_EINVAL, "gradient strides must cover x_len / y_len");
    cudaStream_t s = (cudaStream_t)stream_;
    Workspace ws(s);
    Dtw32Job J;
    DirKeep D;
    WB_TRY(prepare_keep(q, true, const_cast<void *>(keep), keep_bytes, ws, J, D));
    J.grad_out = grad_out;
    J.grad_x = grad_x;
    J.gx_stride = gx_stride;
    J.grad_y = grad_y;
    J.gy_stride = gy_stride;
    return dtw32_keep_walk(J, D, dist, s);
}

extern "C" int wb_series_lengths_f32(const float *x, int64_t n_series, int64_t stride,
                                     int32_t L, int32_t *lengths, void *stream_) {
    WB_TRACE();
    if (n_series < 0 || L < 0) return fail(WB_EINVAL, "negative size");
    if (n_series > 0 && (!x || !lengths)) return fail(WB_EINVAL, "NULL pointer");
    return launch_series_lengths(x, n_series, stride, L, lengths, (cudaStream_t)stream_);
}
