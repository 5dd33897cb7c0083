// dtw32.cuh -- job description of the FP32 (compensated) dtw / wdtw kernels.
#pragma once

#include "common.cuh"

namespace wb {

// A batch of (x series, y series) dtw problems in float32.  Series s of x
// starts at x + s * x_stride; its valid length is xlen[s] (NaN padding cut
// off) or x_len when xlen is null.  Item t pairs x series item_x[t] with y
// series item_y[t]; without item arrays the items are the full grid
// t = cy * nx + cx (32 consecutive items share one y series).
struct Dtw32Job {
    const float *x = nullptr;
    int64_t x_stride = 0;
    const int32_t *xlen = nullptr;
    int x_len = 0;
    int64_t nx = 0;
    const float *y = nullptr;
    int64_t y_stride = 0;
    const int32_t *ylen = nullptr;
    int y_len = 0;
    int64_t ny = 0;
    const int32_t *item_x = nullptr;
    const int32_t *item_y = nullptr;
    int64_t n_items = 0;
    double r = 1.0;               // band fraction; per item band = max(floor(min(n,m) r), 1)
    int band_fixed = 0;           // > 0: this band for every item (ddtw: band of the series)
    const float *weights = nullptr;  // wdtw weights (device) or null
    double *out = nullptr;        // per item: sqrt(hi + lo) in double
    double *out_cost = nullptr;   // optional per item: hi + lo (squared distance)
    // backward
    const double *grad_out = nullptr;  // per item upstream gradient of the distance
    float *grad_x = nullptr;      // per x series (series s at s * gx_stride), accumulated
    int64_t gx_stride = 0;
    float *grad_y = nullptr;      // per y series, accumulated
    int64_t gy_stride = 0;
    // scratch
    float2 *ring = nullptr;       // [column][thread] (hi, lo) boundary rows
    int ring_cols = 0;            // columns per thread (longest series + 1)
    uint32_t *dirs = nullptr;     // [word][thread] direction words (backward)
    int64_t dir_words = 0;        // words per thread
    float2 *ckpt = nullptr;       // [slot][column][thread] segment checkpoints (backward)
    int n_ckpt = 0;               // checkpoint rows per thread
    int seg_strips = 1;           // strips per segment (backward)
    unsigned long long *queue = nullptr;  // work counter (persistent kernel)
    int grid = 0, block = 0;
};

// Kept directions of a differentiable call (see dtw32.cu): one region of
// batch_bytes per batch of 32 consecutive items, the two strip tables
// (max_strips ints each, tab_bytes in all) first, then 32 lanes x cap words.
struct DirKeep {
    unsigned char *base = nullptr;
    int64_t batch_bytes = 0;
    int64_t tab_bytes = 0;
    int64_t cap = 0;       // direction words per lane (multiple of 8)
    int max_strips = 0;
};

int dtw32_forward(const Dtw32Job &J, int strip, cudaStream_t s);
int dtw32_keep_forward(const Dtw32Job &J, const DirKeep &D, cudaStream_t s);
int dtw32_keep_walk(const Dtw32Job &J, const DirKeep &D, const double *dist, cudaStream_t s);
int dtw32_keep_blocks_per_sm(bool walk, bool weighted);
int dtw32_backward(const Dtw32Job &J, cudaStream_t s);
int dtw32_blocks_per_sm(int strip, bool weighted, bool backward, int block);
int launch_grid_to_matrix(const double *in, int64_t nx, int64_t ny, int upper, double *out,
                          cudaStream_t s);
int dtw32_plan(const wb_dtw32 *q, bool backward, Dtw32Job &J, size_t &bytes);
int dtw32_take(Workspace &ws, Dtw32Job &J, bool backward);
int launch_upper_items(int64_t n, int32_t *item_x, int32_t *item_y, cudaStream_t s);
int launch_series_lengths(const float *x, int64_t n_series, int64_t stride, int L,
                          int32_t *lengths, cudaStream_t s);

}  // namespace wb
