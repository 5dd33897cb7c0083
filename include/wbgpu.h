/*
 * wbgpu.h -- C ABI of the GB300 (sm_103a) distance library.
 *
 * Drop-in boundary for wildboar's distance hot path.  Each entry point
 * replaces one Cython driver of the reference (wildboar src/wildboar/distance/
 * _cdistance.pyx) and is reached from Python through ctypes
 * (wildboar_gb300/_lib.py).  Plain pointers and sizes only.
 *
 * Conventions
 *  - Every function returns an int status (WB_OK = 0); the message of the
 *    last failure on the calling thread is wb_last_error().
 *  - Series are (n, n_dims, n_timestep) row-major arrays, as produced by the
 *    reference's _check_ts_array (utils/validation.py:594-620).  `on_device`
 *    says whether `data` is a host pointer (copied in by the library) or a
 *    CUDA device pointer (used in place).
 *  - Outputs follow `out_on_device` the same way.  Host outputs are complete
 *    when the call returns; device outputs are ordered on `stream`.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).
 *  - The caller owns every buffer it passes.  The library owns a per-stream
 *    device workspace that grows on demand and is released by
 *    wb_release_workspace().
 */
#ifndef WBGPU_H
#define WBGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define WB_OK 0
#define WB_EINVAL 1      /* bad argument: maps to ValueError */
#define WB_ENOMEM 2      /* device allocation failed: maps to MemoryError */
#define WB_ECUDA 3       /* CUDA runtime error: maps to RuntimeError */
#define WB_ETIMEOUT 4    /* a bounded device wait gave up */
#define WB_EUNSUPPORTED 5

/* metric ids (same numbering as the oracle) */
#define WB_EUCLIDEAN 0
#define WB_DTW 1
#define WB_WDTW 2
#define WB_DDTW 3
#define WB_WDDTW 4
#define WB_ADTW 5
#define WB_LCSS 6
#define WB_WLCSS 7
#define WB_EDR 8
#define WB_ERP 9
#define WB_MSM 10
#define WB_TWE 11
#define WB_SCALED_EUCLIDEAN 32
#define WB_SCALED_DTW 33     /* subsequence metric only (the UCR-suite scan) */

/* dtypes */
#define WB_F64 0
#define WB_F32 1

typedef struct wb_series {
    const void *data;   /* (n, n_dims, n_timestep) row-major */
    int64_t n;
    int64_t n_dims;
    int64_t n_timestep;
    int32_t dtype;      /* WB_F64 (the drop-in) or WB_F32 (batched forms) */
    int32_t on_device;  /* 0: host pointer, 1: device pointer */
} wb_series;

/* Union of the reference metric constructor arguments
 * (distance/_elastic.pyx:3133-4006).  Unused fields are ignored. */
typedef struct wb_params {
    double r;          /* band as a fraction of the shorter length, [0, 1] */
    double g;          /* wdtw/wddtw/wlcss weight steepness; erp gap value */
    double p;          /* adtw penalty */
    double epsilon;    /* lcss/edr match threshold; NaN = edr per-pair default */
    double c;          /* msm split/merge cost */
    double penalty;    /* twe penalty (lambda) */
    double stiffness;  /* twe stiffness (nu) */
} wb_params;

/*
 * pairwise distance of every x[i, dim] and y[j, dim]: out is (x.n, y.n).
 * y == NULL is the reference's singleton path (x is y): strict upper
 * triangle computed, mirrored, zero diagonal.
 * Replaces _pairwise_distance / _singleton_pairwise_distance
 * (distance/_cdistance.pyx:1184-1267) and the per-pair Metric.distance calls
 * of the elastic metric classes (distance/_elastic.pyx:3126-4082) and
 * EuclideanMetric (distance/_metric.pyx:381-409).
 */
int wb_pairwise_distance(const wb_series *x, const wb_series *y, int64_t dim,
                         int32_t metric, const wb_params *params, double *out,
                         int32_t out_on_device, void *stream);

/*
 * paired distance of x[i, dim] and y[i, dim]: out is (x.n,).  As in the
 * reference the metric receives (y[i], x[i]): the rows of the recurrence come
 * from the second argument.  Replaces _paired_distance
 * (distance/_cdistance.pyx:1597-1652).
 */
int wb_paired_distance(const wb_series *x, const wb_series *y, int64_t dim,
                       int32_t metric, const wb_params *params, double *out,
                       int32_t out_on_device, void *stream);

/*
 * k nearest y rows of every x row (dim must be 0 in the public API; any dim is
 * accepted here).  indices/distances are (x.n, k) in the reference's heap
 * order, including its early-abandoning decisions.  lower_bound is NULL or a
 * (x.n, y.n) matrix on the same side as the outputs.  Replaces
 * _argmin_distance (distance/_cdistance.pyx:1270-1378) and the Heap of
 * utils/_misc.pyx:18-107.
 */
int wb_argmin_distance(const wb_series *x, const wb_series *y, int64_t dim,
                       int32_t metric, const wb_params *params, int64_t k,
                       const double *lower_bound, int64_t *indices, double *distances,
                       int32_t out_on_device, void *stream);

/*
 * minimum subsequence distance and first argmin window of every shapelet
 * against every x[i, dim]: out_dist / out_idx are (x.n, m).  Shapelets are
 * packed float64 values; offsets/lengths index them.  means/stds are the
 * np.mean / np.std of each shapelet (std <= 1e-13 given as 0): the scaled
 * metric uses both, edr with a NaN epsilon uses stds (epsilon = std / 4).
 * metric is WB_EUCLIDEAN, WB_SCALED_EUCLIDEAN, WB_SCALED_DTW (params->r;
 * means and stds required) or an elastic id (dtw, wdtw, ddtw, wddtw, adtw,
 * lcss, edr, erp, msm, twe) with `params` (NULL allowed for the euclidean
 * ones).  Shapelet arrays live on the same side as x.  Replaces
 * _pairwise_subsequence_distance (distance/_cdistance.pyx:956-1037) with
 * euclidean_distance / scaled_euclidean_distance (distance/_metric.pyx:561-682),
 * the elastic *_subsequence_distance functions (distance/_elastic.pyx:
 * 622-1866), including their early abandoning at the running minimum, and
 * the UCR-suite scaled_dtw_subsequence_distance (distance/_elastic.pyx:
 * 159-465) with its LB_Kim / LB_Keogh pruning decisions.
 */
int wb_pairwise_subsequence_distance(const double *shapelets, const int64_t *offsets,
                                     const int64_t *lengths, const double *means,
                                     const double *stds, int64_t m, const wb_series *x,
                                     int64_t dim, int32_t metric, const wb_params *params,
                                     double *out_dist, int64_t *out_idx,
                                     int32_t out_on_device, void *stream);

/*
 * shapelet i against x[i, dim] only (m == x.n): out_dist / out_idx are (m,).
 * Arguments as wb_pairwise_subsequence_distance.  Replaces
 * _paired_subsequence_distance (distance/_cdistance.pyx:1040-1062).
 */
int wb_paired_subsequence_distance(const double *shapelets, const int64_t *offsets,
                                   const int64_t *lengths, const double *means,
                                   const double *stds, int64_t m, const wb_series *x,
                                   int64_t dim, int32_t metric, const wb_params *params,
                                   double *out_dist, int64_t *out_idx,
                                   int32_t out_on_device, void *stream);

/*
 * every window of shapelet i against x[i, dim] (m == x.n), no minimum:
 * out_raw[i * ld + w] is the final value of the metric's recurrence for
 * window w (squared sum for euclidean / scaled_euclidean, squared cost for
 * the dtw family, match count for lcss, edit count for edr, the cost for
 * erp / msm / twe; NaN past the pair's last window) and out_key[i * ld + w]
 * the largest per-row minimum of the recurrence (the value the reference's
 * early abandoning compares with its threshold; -inf for the euclidean
 * metrics, whose key may be NULL).  For WB_SCALED_DTW out_raw is the squared
 * dtw cost and out_key the largest of LB_Kim, the two LB_Keogh bounds and
 * the per-row "row minimum + cumulative bound" (scaled_dtw_matches,
 * distance/_elastic.pyx:468-620): a window matches threshold t iff
 * key < t^2 and raw <= t^2.  ld >= x.n_timestep - min length + 1.
 * Shapelets may share storage (equal offsets).  stds of 0 are taken as 1
 * (persistent subsequences, _cdistance.pyx:283-343) unless std_as_given
 * (the distance profile's transient statistics, _cdistance.pyx:1680-1699,
 * divide by them as they are).  With these two numbers the
 * caller reproduces the distances and the match sets of
 * SubsequenceMetric._matches (distance/_cdistance.pyx:301-432) for any
 * threshold: distance_profile, subsequence_match and paired_subsequence_match
 * (distance/_distance.py:732-1080, 1477-1620).
 */
int wb_subsequence_profile(const double *shapelets, const int64_t *offsets,
                           const int64_t *lengths, const double *means, const double *stds,
                           int64_t m, const wb_series *x, int64_t dim, int32_t metric,
                           const wb_params *params, double *out_raw, double *out_key,
                           int64_t ld, int32_t std_as_given, int32_t out_on_device,
                           void *stream);

/*
 * the k closest windows of subsequence i in x[i, dim] (argmin_subsequence_
 * distance, distance/_distance.py:1636-1761): s is (n, s_stride) float64
 * on the host (row i holds s_len[i] values), x.n == n.  metric is a pairwise
 * metric id (euclidean or elastic) evaluated through its eadistance with the
 * reference's early abandoning; scaled z-normalises the subsequence with
 * s_mean / s_std (fast_mean_std of the row; host arrays) and every window
 * with the IncStats sequence of its series.  indices / distances are (n, k)
 * in the reference's heap order.  Replaces _argmin_subsequence_distance
 * (distance/_cdistance.pyx:1381-1594).
 */
int wb_argmin_subsequence_distance(const double *s, const int64_t *s_len, int64_t s_stride,
                                   int64_t n, const double *s_mean, const double *s_std,
                                   const wb_series *x, int64_t dim, int32_t metric,
                                   const wb_params *params, int32_t scaled, int64_t k,
                                   int64_t *indices, double *distances, int32_t out_on_device,
                                   void *stream);

/* ------------------------------------------------------------------------
 * FP32 forms (batched, ragged, differentiable).  No counterpart in the
 * reference, which computes every distance in FP64 on the CPU; they follow
 * dtw_distance (distance/_elastic.pyx:869-940) with FP32 costs and
 * compensated (TwoSum) accumulation, the final sqrt in FP64.  All pointers are
 * device pointers; calls neither synchronise nor allocate once the stream's
 * workspace has grown to the job, so they can be captured in CUDA graphs
 * after a warm-up call.
 * ------------------------------------------------------------------------ */
typedef struct wb_dtw32 {
    const float *x;            /* x series s starts at x + s * x_stride */
    int64_t x_stride;
    const int32_t *x_lengths;  /* valid length of each x series, or NULL (x_len) */
    int32_t x_len;             /* padded (maximum) x length */
    int64_t nx;
    const float *y;
    int64_t y_stride;
    const int32_t *y_lengths;
    int32_t y_len;
    int64_t ny;
    const int32_t *item_x;     /* item t pairs x series item_x[t] with y series */
    const int32_t *item_y;     /* item_y[t]; both NULL: the nx*ny grid, t = j*nx + i */
    int64_t n_items;
    double r;                  /* band fraction in [0, 1] */
    const float *weights;      /* wdtw weights (length >= max length) or NULL */
    int32_t strip;             /* rows per register strip: 4, 8, 16, 24, 32 (0 = 16) */
    int32_t block;             /* threads per block (0 = 128) */
    int32_t grid;              /* persistent grid (0 = occupancy x SMs) */
} wb_dtw32;

/* dtw distance of every item: out[t] = sqrt(cost), out_cost[t] = cost (or NULL) */
int wb_dtw32_distance(const wb_dtw32 *job, double *out, double *out_cost, void *stream);

/* d distance[t] / d x and d distance[t] / d y of every item, scaled by
 * grad_out[t] (NULL = 1): grad_x row t at grad_x + t * gx_stride (x_len
 * floats), grad_y likewise.  Recomputes the forward with a direction bitmap
 * and walks the optimal path back (dtw_mapping tie order: diag, up, left). */
int wb_dtw32_backward(const wb_dtw32 *job, const double *grad_out, float *grad_x,
                      int64_t gx_stride, float *grad_y, int64_t gy_stride, void *stream);

/*
 * Kept directions (no counterpart in the reference): the forward of a
 * differentiable call may store the 2-bit traceback directions of every item
 * (the sweep the backward would otherwise recompute), so that the backward
 * only walks the paths.  wb_dtw32_keep_bytes gives the buffer size for a job
 * (-1 for an invalid job); wb_dtw32_distance_keep computes out / out_cost like
 * wb_dtw32_distance (predecessors chosen by compensated comparison, as in the
 * backward) and fills the buffer; wb_dtw32_backward_keep adds the gradients
 * of wb_dtw32_backward from that buffer and the distances `dist` of the same
 * forward.  The job must be the same in both calls.
 */
int64_t wb_dtw32_keep_bytes(const wb_dtw32 *job);
int wb_dtw32_distance_keep(const wb_dtw32 *job, double *out, double *out_cost, void *keep,
                           int64_t keep_bytes, void *stream);
int wb_dtw32_backward_keep(const wb_dtw32 *job, const double *dist, const double *grad_out,
                           float *grad_x, int64_t gx_stride, float *grad_y, int64_t gy_stride,
                           const void *keep, int64_t keep_bytes, void *stream);

/* Full-series euclidean distance matrix on the tensor cores (precision form,
 * no counterpart in the reference, whose EuclideanMetric sums in FP64 on the
 * CPU, distance/_metric.pyx:381-409): out[i, j] = sqrt(|x_i|^2 + |y_j|^2 -
 * 2 x_i . y_j) with the dot products from a tcgen05 kind::tf32 GEMM over the
 * 3xTF32 split of the float32-rounded series (FP32 accumulation), norms and
 * the combination in FP64.  x, y: device float64 series of equal length;
 * out (x.n, y.n) float64 on the device or host. */
int wb_euclidean_tc(const wb_series *x, const wb_series *y, int64_t dim, double *out,
                    int32_t out_on_device, void *stream);

/* Pairwise distance of the elastic metrics in FP32 (precision form, no
 * counterpart in the reference, which computes in FP64: the arguments and
 * the output are those of wb_pairwise_distance, ref distance/_distance.py:
 * 644-748).  Series are rounded to float32; every cumulative cost is a
 * compensated (hi, lo) float pair (TwoSum on each addition, minima on hi);
 * the final normalisation and sqrt are FP64.  dtw, wdtw, ddtw and wddtw run
 * on the dtw strip kernel (slopes and weights formed in FP64 first), the
 * other elastic metrics on a thread-per-pair kernel.  euclidean is not
 * accepted here (wb_euclidean_tc is its precision form). */
int wb_pairwise_distance_fp32(const wb_series *x, const wb_series *y, int64_t dim,
                              int32_t metric, const wb_params *params, double *out,
                              int32_t out_on_device, void *stream);

/*
 * wb_subsequence_profile for WB_SCALED_EUCLIDEAN with the reference's
 * threshold stop: the sum of window w of pair i stops before the first term
 * at which it is >= stop_sq[i] (host array of m values), as
 * inner_scaled_euclidean_distance breaks on the squared threshold inside
 * scaled_euclidean_distance_matches (distance/_metric.pyx:625-651, 798-860).
 * A window then matches threshold t iff out_raw <= t^2 with distance
 * sqrt(out_raw): a partial sum equal to t^2 matches with that distance, and
 * t = 0 matches every window with distance 0, as in the reference.
 */
int wb_subsequence_profile_stop(const double *shapelets, const int64_t *offsets,
                                const int64_t *lengths, const double *means,
                                const double *stds, int64_t m, const wb_series *x, int64_t dim,
                                const double *stop_sq, double *out_raw, int64_t ld,
                                int32_t out_on_device, void *stream);

/*
 * Distance profile with dilation and / or padding (distance_profile,
 * distance/_distance.py:1560-1619; _dilated_distance_profile,
 * distance/_cdistance.pyx:804-933, 1809-1841): out (x.n, T + 2 padding -
 * (L - 1) dilation) where output position p compares the samples of x[i, dim]
 * at a dilation stride with the values of y[i] (one dim, L values) by the
 * pairwise metric's early-abandoning distance with an infinite threshold,
 * divided by (float) k / (float) L when padding leaves only k < L samples.
 * scale != 0 z-normalises every window by its own mean and variance over L
 * (variance <= 1e-13 -> std 1); y is given already scaled.
 */
int wb_dilated_profile(const wb_series *y, const wb_series *x, int64_t dim, int32_t metric,
                       const wb_params *params, int64_t dilation, int64_t padding,
                       int32_t scale, double *out, int32_t out_on_device, void *stream);

/*
 * The "mass" distance profile (ScaledMassSubsequenceMetric,
 * distance/_mass.pyx:35-240): z-normalised euclidean distance of y[i, 0] at
 * every window of x[i, 0] by the MASS formula, with the windows' IncStats
 * mean / std and the exact dot products in place of the reference's
 * pocketfft cross-correlation (equal up to that rounding).  out (x.n, T - L + 1).
 */
int wb_mass_profile(const wb_series *y, const wb_series *x, double *out, int32_t out_on_device,
                    void *stream);

/*
 * Host-side fault injection for testing the error paths (no counterpart in
 * the reference, whose metrics report failures only as -1 from reset,
 * distance/_elastic.pyx:2224-2225).  Arms one fault that fires once:
 * site 1 = the next device-workspace reservation returns WB_ENOMEM, 2 = the
 * next kernel launch check returns WB_ECUDA (the kernel itself runs), 3 =
 * the next bounded-wait status read (tensor-core euclidean) returns
 * WB_ETIMEOUT; skip = matching events let through first; site 0 disarms.
 * The environment variable WB_GPU_INJECT_FAULT=reserve|launch|wait[:skip]
 * arms the same fault when the library is first used.  No device code is
 * made to fail: the host takes the error path the real failure would take,
 * and the library stays usable for the next call.
 */
int wb_inject_fault(int32_t site, int64_t skip);

/* valid length of each float32 series: index of its first NaN (padding or
 * end-of-series marker, utils/variable_len.py:66-115), else L */
int wb_series_lengths_f32(const float *x, int64_t n_series, int64_t stride, int32_t L,
                          int32_t *lengths, void *stream);

/*
 * wb_pairwise_distance_noalloc -- no counterpart in the reference.
 * wb_pairwise_distance for callers that cannot have the library allocate
 * device memory (memory budgeted up front, or no device-synchronising
 * cudaMalloc/cudaFree allowed in their loop): x, y (or NULL for the singleton
 * path) and out must be device memory; nothing is allocated.  Bands whose ring
 * fits in shared memory run on the shared-memory kernel with no scratch; wider
 * ones keep their rings in a static 64 MiB device array
 * (wb_noalloc_scratch_bytes()) that every GPU loading the library keeps until
 * exit; a band ring that does not fit in it is rejected with WB_EINVAL.
 * Metrics: euclidean, dtw, wdtw, adtw, lcss, wlcss, edr (explicit epsilon),
 * msm; others give WB_EUNSUPPORTED.  All calls share the array: calls that
 * overlap on the GPU race.  The first call on a device looks the array up;
 * make it before any stream capture, and do not reset the device afterwards.
 * wdtw and wlcss copy their weight table from pageable host memory, which
 * waits for the stream, on every call, and are refused (WB_EUNSUPPORTED)
 * while the stream is being captured.
 */
int wb_pairwise_distance_noalloc(const wb_series *x, const wb_series *y, int64_t dim,
                                 int32_t metric, const wb_params *params, double *out,
                                 void *stream);

/* size in bytes of the static scratch of wb_pairwise_distance_noalloc */
int64_t wb_noalloc_scratch_bytes(void);

/*
 * wb_dtw_average_mm_step -- one epoch of the majorize-minimize DTW barycenter
 * for a batch of groups; replaces the per-sample loop of _mm_dtw_average
 * (distance/dtw.py:661-690): dtw_alignment (distance/dtw.py:246-290,
 * _elastic.pyx:1011-1073; wdtw_alignment :293-327 when `weights` is given),
 * the traceback of dtw_mapping (distance/dtw.py:362-426) and the z / V sums.
 * Every pointer is device memory.  Pair q aligns the mean in row
 * pair_group[q] of `means` (mean_len values per row) with sample member[q]
 * (row member[q] of x, stride x_stride, n_timestep values).  The pairs of
 * group gi are group_start[gi] .. group_start[gi + 1] - 1, in sample order;
 * its new mean (the reference's z / V) goes to row groups[gi] of new_means
 * (row gi when groups is NULL; new_means may be means).  `r` is the window
 * fraction (warp max(floor(max(mean_len, n_timestep) r), 1)); `weights`
 * (length >= max(mean_len, n_timestep)) weighs cell (i, j) by
 * weights[|i - j|], NULL for dtw; sample_weight[q] weighs pair q (NULL: 1).
 * last[q] (optional) receives the final alignment cell of pair q.
 * new_means NULL: alignment and `last` only.
 */
int wb_dtw_average_mm_step(const double *x, int64_t x_stride, int64_t n_timestep,
                           const double *means, int64_t mean_len, const int64_t *member,
                           const int32_t *pair_group, const int64_t *group_start,
                           const int32_t *groups, int64_t n_groups, int64_t n_pairs, double r,
                           const double *weights, const double *sample_weight,
                           double *new_means, double *last, void *stream);

/*
 * wb_dtw_envelope -- _dtw_envelop (distance/_elastic.pyx:1076-1092, the
 * streaming find_min_max of :98-151 with deques of capacity 2 warp + 2) of
 * every row of x (n, n_timestep): lower / upper are (n, n_timestep).
 * 0 <= warp < n_timestep.  All arrays on the side `on_device` says.
 */
int wb_dtw_envelope(const double *x, int64_t n, int64_t n_timestep, int64_t warp,
                    double *lower, double *upper, int32_t on_device, void *stream);

/*
 * wb_lb_keogh -- DtwKeoghLowerBound.transform (distance/lb.py:390-432):
 * out[i, j] = max(left, right) for query q[i] and fitted series x[j] (both
 * (., n_timestep) rows), left = sqrt(LB_Keogh of q[i] against the envelope
 * of x[j]) and right = sqrt(LB_Keogh of x[j] against the envelope of q[i])
 * (_dtw_lb_keogh, distance/_elastic.pyx:1095-1115), warp as the caller
 * computes it (distance/lb.py:372-376).  kind: 0 both, 1 left only,
 * 2 right only (the other side is -inf).  out is (nq, nx).
 */
int wb_lb_keogh(const double *q, int64_t nq, const double *x, int64_t nx, int64_t n_timestep,
                int64_t warp, int32_t kind, double *out, int32_t on_device, void *stream);

/*
 * wb_lb_kim -- DtwKimLowerBound.transform (distance/lb.py:224-311): the
 * constant-time bound of every query y[i] against every fitted x[j];
 * out is (ny, nx).
 */
int wb_lb_kim(const double *y, int64_t ny, const double *x, int64_t nx, int64_t n_timestep,
              double *out, int32_t on_device, void *stream);

/*
 * wb_nearest_pivot -- batched nearest-pivot assignment for proximity trees
 * (_partition_pivots, tree/_cptree.pyx:869-894, find_min_branch :273-290).
 * Group g holds samples[sample_ptr[g] .. sample_ptr[g + 1]) and pivots
 * pivots[pivot_ptr[g] .. pivot_ptr[g + 1]) (row indices of x, dim `dim`) and
 * uses metric slot group_slot[g] (slot_metric[slot], slot_params[slot]).
 * out_branch / out_dist, aligned with `samples`, receive the position within
 * the group's pivots of the first pivot at the strictly smallest (full, not
 * early-abandoned) distance and that distance; a sample without a finite
 * distance keeps the previous sample's branch (-1 for a group's first), as
 * the running pivot of _partition_pivots does.  Index arrays and outputs are
 * host arrays; x may be on either side.
 */
int wb_nearest_pivot(const wb_series *x, int64_t dim, int64_t n_groups, const int64_t *sample_ptr,
                     const int64_t *samples, const int64_t *pivot_ptr, const int64_t *pivots,
                     const int32_t *group_slot, const int32_t *slot_metric,
                     const wb_params *slot_params, int32_t n_slots, int64_t *out_branch,
                     double *out_dist, void *stream);

/*
 * wb_subsequence_distance_views -- the shapelet transform's attribute values
 * (transient_distance / persistent_distance, distance/_cdistance.pyx:265-299)
 * for subsequence views of x: view v is x[view_sample[v], view_dim[v],
 * view_start[v] : view_start[v] + view_length[v]] with the statistics its
 * SubsequenceView holds (view_mean, view_std from _ts_view_update_statistics,
 * :167-185; a zero std is used as 1).  Every view against every series of
 * `target` at `dim`: out_dist / out_idx are (target.n, m) on the target's
 * side.  View arrays are host arrays.
 */
int wb_subsequence_distance_views(const wb_series *x, const int64_t *view_sample,
                                  const int64_t *view_dim, const int64_t *view_start,
                                  const int64_t *view_length, const double *view_mean,
                                  const double *view_std, int64_t m, const wb_series *target,
                                  int64_t dim, int32_t metric, const wb_params *params,
                                  double *out_dist, int64_t *out_idx, void *stream);

/*
 * wb_dtw_average_ssg_epoch -- the sample loop of one epoch of the stochastic
 * subgradient DTW mean (_ssg_dtw_average, distance/dtw.py:597-658): for
 * step i, the path of (mean, x[order[i]]) (dtw_alignment / wdtw_alignment and
 * dtw_mapping as wb_dtw_average_mm_step), z[m] = sum over its cells (m, x)
 * of (mean[m] - x[order[i], x] w), mean -= lr[i] z, with
 * w = sample_weight[order[i]] (NULL: 1).  x, mean and weights are device
 * pointers (mean updated in place); order, lr and sample_weight are host
 * arrays of n_steps (order, lr) and n samples (sample_weight).
 */
int wb_dtw_average_ssg_epoch(const double *x, int64_t x_stride, int64_t n_timestep,
                             double *mean, int64_t mean_len, const int64_t *order,
                             const double *lr, int64_t n_steps, double r, const double *weights,
                             const double *sample_weight, void *stream);

/*
 * wb_dtw_alignment -- the cumulative cost matrix of dtw_alignment /
 * wdtw_alignment (distance/dtw.py:246-327, _elastic.pyx:1011-1073): out is
 * (n, m) with the band's cells and +inf elsewhere (the reference leaves the
 * cells off the band and its boundary markers unset).  r is the window
 * fraction (warp max(floor(max(n, m) r), 1)); weights (length >= max(n, m))
 * weigh cell (i, j) by weights[|i - j|], NULL for dtw.
 */
int wb_dtw_alignment(const double *x, int64_t n, const double *y, int64_t m, double r,
                     const double *weights, double *out, int32_t on_device, void *stream);

/*
 * wb_lb_keogh_terms -- _dtw_lb_keogh (distance/_elastic.pyx:1095-1115) of one
 * series against an envelope: cb[k] the excursion of x[k] outside
 * [lower[k], upper[k]] squared, *dist the square root of their sum.
 */
int wb_lb_keogh_terms(const double *x, const double *lower, const double *upper,
                      int64_t n_timestep, double *cb, double *dist, int32_t on_device,
                      void *stream);

/*
 * wb_group_mean -- x[group].mean(axis=0) of the euclidean KMeans update
 * (_EuclideanCluster._update_centroid, distance/_neighbors.py:364-369):
 * the rows member[group_start[gi] .. group_start[gi + 1] - 1] summed in that
 * order, divided by their count, into row groups[gi] (or gi) of out.
 * Device pointers.
 */
int wb_group_mean(const double *x, int64_t x_stride, int64_t n_timestep,
                  const int64_t *member, const int64_t *group_start, const int32_t *groups,
                  int64_t n_groups, double *out, void *stream);

/* message of the last failed call on this thread ("" if none) */
const char *wb_last_error(void);

/* library ABI version */
int32_t wb_version(void);

/* free the workspace the library holds for `stream` (NULL: all streams) */
int wb_release_workspace(void *stream);

/* number of kernel launches issued by this process (diagnostics) */
int64_t wb_launch_count(void);

/* Diagnostics (no counterpart in the reference): when enabled, the main
 * kernel of each call is bracketed by CUDA events on the call's stream and
 * wb_profile_last() returns its device time in ms (-1 if none). */
int wb_profile_enable(int32_t on);
int wb_profile_last(double *ms);

/* Diagnostics: sustained add+mul throughput of the FP64 (dtype WB_F64) or
 * FP32 (WB_F32) pipes of the current device, in operations per second; the
 * roofline peak of the ALU-bound recurrence kernels. */
int wb_alu_probe(int32_t dtype, int32_t iters, double *ops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* WBGPU_H */
