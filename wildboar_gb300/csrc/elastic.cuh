// elastic.cuh -- job description of the FP64 elastic-distance kernels.
#pragma once

#include <vector>

#include "common.cuh"

namespace wb {

// A set of equally long series: series s starts at base + s * stride.
struct SeriesSet {
    const double *base = nullptr;
    int64_t stride = 0;
    int64_t count = 0;
    int len = 0;
};

enum PairMode {
    PM_ALL = 0,     // every (row series, column series) pair
    PM_UPPER = 1,   // rows == cols, pairs i < j, mirrored output
    PM_PAIRED = 2,  // row series s with column series s
};

// kernel variants (one recurrence each)
enum ElasticKind {
    K_DTW = 0,      // dtw / ddtw (on slopes)
    K_WDTW = 1,     // wdtw / wddtw
    K_ADTW = 2,     // adtw, penalty >= 0
    K_ADTW_ANY = 3, // adtw, negative penalty (IEEE min instead of integer min)
    K_LCSS = 4,
    K_WLCSS = 5,
    K_EDR = 6,
    K_ERP = 7,
    K_MSM = 8,
    K_TWE = 9,
    K_EUCLID = 10,  // pairwise euclidean (EuclideanMetric), no recurrence
};

// final transform of the recurrence value
enum ResultKind {
    R_SQRT = 0,      // dtw family
    R_LCSS = 1,      // 1 - v / min(n, m)
    R_EDR = 2,       // v / max(n, m)
    R_IDENT = 3,     // erp, msm, twe
};

struct ElasticJob {
    int kind = K_DTW;
    int result = R_SQRT;
    int mode = PM_ALL;
    SeriesSet rows;          // rows of the recurrence (the metric's X)
    SeriesSet cols;          // columns of the recurrence (the metric's Y)
    int band = 1;            // r of the recurrence
    int len_norm_rows = 0;   // lengths used by the LCSS / EDR normalisation
    int len_norm_cols = 0;
    double eps = 0, p = 0, g = 0, c = 0, penalty = 0, stiffness = 0;
    const double *weights = nullptr;    // wdtw / wlcss weights (device)
    const float *weights32 = nullptr;   // the same weights in float32 (FP32 kernels)
    const double *std_rows = nullptr;   // edr default epsilon tables (device)
    const double *std_cols = nullptr;
    const double *gsum_rows = nullptr;  // erp: sum_i |x_i - g| per series
    const double *gsum_cols = nullptr;
    const double *gtab_cols = nullptr;  // erp: |y_j - g|, (cols.count, cols.len)
    const double *dtab_cols = nullptr;  // twe: |y_{j-1} - y_j|, (cols.count, cols.len)
    const double *stab = nullptr;       // twe: (2 * stiffness) * k
    double *out = nullptr;              // distances
    int64_t out_ld = 0;                 // row stride of out (PM_ALL / PM_UPPER)
    double *key = nullptr;              // early-abandon keys (argmin), or null
    int all_zero = 0;                   // ddtw on series shorter than 3
};

// Ring length (in elements) needed for a band recurrence of an (n x m)
// problem with half-width r: the live window spans columns js-1 .. je.
inline int ring_len(int n, int m, int r) {
    int64_t w = (int64_t)(m > n ? m - n : n - m) + 2 * (int64_t)r + 2;
    int64_t full = (int64_t)m + 1;
    return (int)(w < full ? w : full);
}

int launch_elastic(const ElasticJob &job, Workspace &ws, size_t *ring_bytes_query);
// Same kernels with the per-thread rings in a caller-provided device buffer of
// `ring_bytes` (always the global-ring variant); the grid is the largest that
// fits.  WB_EINVAL when not even one block's rings fit.
int launch_elastic_external_ring(const ElasticJob &job, double *ring, size_t ring_bytes,
                                 cudaStream_t s);
// The shared-memory ring kernels (and the tiled euclidean kernel) without any
// workspace; WB_EUNSUPPORTED when the band ring does not fit in shared memory.
int launch_elastic_shared_ring(const ElasticJob &job, cudaStream_t s);
size_t elastic_workspace_bytes(const ElasticJob &job);

// elastic subsequence distance (one warp per (series, shapelet), one lane per
// window); rows are the shapelet (or its slopes), columns the window.
struct SubseqElasticJob {
    SeriesSet x;                  // series scanned (slopes for ddtw / wddtw)
    int t_len = 0;                // row stride of gtab (erp) = x.len
    int t_len_thr = 0;            // the series length the reference's thresholds use
    const double *shp = nullptr;  // packed shapelets (slopes for ddtw / wddtw)
    const int64_t *off = nullptr;
    const int64_t *len = nullptr; // original shapelet lengths
    const int32_t *band_of_len = nullptr;  // band of each shapelet
    const double *shp_std = nullptr;       // edr default epsilon (NaN epsilon)
    int64_t m = 0;
    int metric = WB_DTW;
    int slopes = 0;
    double eps = 0, p = 0, g = 0, c = 0, penalty = 0, stiffness = 0;
    const double *weights = nullptr;
    const double *gtab = nullptr;  // erp: |x - g| per series, (x.count, t_len)
    const double *stab = nullptr;  // twe: (2 stiffness) k
    double *out_dist = nullptr;
    int64_t *out_idx = nullptr;
    int paired = 0;  // series i against shapelet i only (x.count == m), outputs (m,)
    // profile (paired only): every window's final recurrence value and abandon
    // key at [pair * prof_ld + window] instead of the minimum
    double *prof_raw = nullptr;
    double *prof_key = nullptr;
    int64_t prof_ld = 0;
    int std_as_given = 0;  // a zero shapelet std gives epsilon 0 (distance profile)
};
size_t elastic_subseq_ring_bytes(const SubseqElasticJob &J, int max_len, int max_band,
                                 int *P_out, int *grid_out);
int launch_elastic_subseq(const SubseqElasticJob &J, int kind, double *gring, int P, int grid,
                          cudaStream_t s);
int launch_shapelet_slopes(const double *shp, const int64_t *off, const int64_t *len,
                           int64_t m, double *out, cudaStream_t s);

// scaled_dtw subsequence metric (scaled_dtw.cu); shapelet arrays on the device
int subseq_scaled_dtw(const double *shp, const int64_t *off, const int64_t *len,
                      const double *means, const double *stds, int64_t m,
                      const std::vector<int64_t> &hlen, int64_t total, const SeriesSet &X,
                      int64_t n_timestep, double r, bool paired, int std_as_given,
                      double *out_dist, int64_t *out_idx, double *prof_raw, double *prof_key,
                      int64_t prof_ld, Workspace &ws, cudaStream_t s);
size_t subseq_scaled_dtw_bytes(int64_t m, int64_t total, int64_t n_series, int n,
                               const std::vector<int64_t> &hlen, double r, int64_t n_timestep,
                               bool paired);

// argmin_subsequence_distance (argmin_subseq.cu)
struct ArgminSubseqJob;
int wb_argmin_subsequence_impl(const double *s, const int64_t *s_len, int64_t s_stride,
                               int64_t n, const double *s_mean, const double *s_std,
                               const wb_series *x, int64_t dim, int32_t metric,
                               const wb_params *params, int32_t scaled, int64_t k,
                               int64_t *indices, double *distances, int32_t out_on_device,
                               cudaStream_t stream);

// register-strip kernels of every elastic metric, FP64 (exact) or FP32
// (compensated) (elastic_strip.cu)
bool strip_supported(const ElasticJob &J);
bool strip_forced();
// WB_GPU_ARGMIN=all: argmin evaluates every candidate pair in full (no
// early-abandoned chunks; argmin_subsequence: every window in full);
// WB_GPU_ARGMIN=<c>: first chunk of c candidates
// (default: enough pairs for every lane); WB_GPU_ARGMIN_FORM=strip: the
// strip form of the chunks for any band.  All forms give the same results.
bool argmin_ea_disabled();
int64_t argmin_ea_first_chunk();
// pairs of one query batch of argmin_distance (WB_GPU_ARGMIN_BATCH=<pairs>
// overrides the 2^27 default, for tests of the batching)
int64_t argmin_pair_budget();
size_t strip_workspace_bytes(const ElasticJob &J, bool fp32);
int launch_strip(const ElasticJob &J, Workspace &ws, bool fp32);

// float64 -> float32 conversions for the FP32 dtw strip kernel (elastic_strip.cu)
int launch_to_f32(const SeriesSet &in, float *out, cudaStream_t s);
int launch_weights_f32(const double *w, int n, float *out, cudaStream_t s);

// per-series preparation kernels
int launch_slopes(const SeriesSet &in, double *out, cudaStream_t s);
int launch_mean_std(const SeriesSet &in, double *std_out, cudaStream_t s);
int launch_erp_tables(const SeriesSet &in, double g, double *tab, double *sums,
                      cudaStream_t s);
int launch_twe_tables(const SeriesSet &in, double *tab, cudaStream_t s);
int launch_fill_stab(double s2, int n, double *stab, cudaStream_t s);
int launch_fill(double *p, double v, int64_t n, cudaStream_t s);

// argmin heap replay
struct ArgminJob {
    int metric = WB_DTW;
    int64_t nx = 0, ny = 0, k = 1;
    const double *dist = nullptr;   // (nx, ny)
    const double *key = nullptr;    // (nx, ny) or null
    const double *lower_bound = nullptr;
    int xl = 0, yl = 0;             // series lengths (threshold transforms)
    int never_push = 0;             // ddtw / wddtw with series shorter than 3
    int64_t *out_idx = nullptr;
    double *out_dist = nullptr;
    int64_t *heap_idx = nullptr;    // (nx, k) scratch
    double *heap_val = nullptr;     // (nx, k) scratch
    // replay of candidates [j0, j1) only (j1 < 0: all), resuming the heaps
    // and k-th distances left by the previous range when `resume` is set;
    // outputs written when `finish` is set
    int64_t j0 = 0, j1 = -1;
    int resume = 0, finish = 1;
    int64_t *state_n = nullptr;     // (nx,) heap sizes between ranges
    double *state_dist = nullptr;   // (nx,) k-th distance (inf until the heap is full)
};
int launch_argmin_replay(const ArgminJob &job, cudaStream_t s);

// One chunk of argmin candidates for the early-abandoning kernels.
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

// Generic strip form (elastic_strip.cu) of the early-abandoning kernels:
// edr / erp / msm / twe (chunked: their thresholds grow with the k-th
// distance) and, with one chunk and no bound, the keyed all-pairs sweep of
// lcss / wlcss / adtw with a negative penalty for wide bands.  The ring is
// per lane [lane][column] (ring_ld >= cols.len).
bool strip_ea_supported(const ElasticJob &job);
int strip_ea_blocks_per_sm(const ElasticJob &job);
int launch_strip_ea(const ElasticJob &job, const EaChunk &chunk, double *ring, int64_t ring_ld,
                    int grid, cudaStream_t s);

// early-abandoned candidate chunks (argmin_ea.cu): dtw / wdtw / ddtw / wddtw
// / adtw with a non-negative penalty, and through the generic strip form
// edr / erp / msm / twe (and unchunked lcss / wlcss / adtw for wide bands).  Writes out / key of pairs (i, j in
// [j0, j0 + nc)) with row stride ny; an abandoned pair gets distance inf and
// its partial key, which exceeds the threshold the replay compares it with.
// Wide bands need a device ring of argmin_ea_ring_bytes (0 for narrow ones).
bool argmin_ea_supported(const ElasticJob &job);
// candidates may be split in chunks with bounds (else one chunk, no bound)
bool argmin_ea_chunked(const ElasticJob &job);
int64_t argmin_ea_lanes(const ElasticJob &job);
size_t argmin_ea_ring_bytes(const ElasticJob &job);
int launch_argmin_ea(const ElasticJob &job, int metric, int xl, int yl, int64_t j0, int64_t nc,
                     int64_t ny, const double *cur_dist, const double *lower_bound,
                     unsigned long long *counter, double *ring, cudaStream_t s);

}  // namespace wb
