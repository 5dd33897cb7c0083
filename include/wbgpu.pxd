# wbgpu.pxd -- Cython declarations of the whole wbgpu C ABI (wbgpu.h) for
# compiled callers: the proximity trees (tree/_cptree.pyx:254-290, 869-894)
# and the shapelet transforms (transform/_cshapelet.pyx:50-131) call the
# reference's cdef metrics per pair; with these declarations they hand whole
# nodes or attribute columns to the batched entries instead.  Link with
# libwbgpu.so.

from libc.stdint cimport int32_t, int64_t

cdef extern from "wbgpu.h" nogil:
    enum:
        WB_OK
        WB_EINVAL
        WB_ENOMEM
        WB_ECUDA
        WB_ETIMEOUT
        WB_EUNSUPPORTED
        WB_EUCLIDEAN
        WB_DTW
        WB_WDTW
        WB_DDTW
        WB_WDDTW
        WB_ADTW
        WB_LCSS
        WB_WLCSS
        WB_EDR
        WB_ERP
        WB_MSM
        WB_TWE
        WB_SCALED_EUCLIDEAN
        WB_SCALED_DTW
        WB_F64
        WB_F32

    ctypedef struct wb_series:
        const void *data
        int64_t n
        int64_t n_dims
        int64_t n_timestep
        int32_t dtype
        int32_t on_device

    ctypedef struct wb_params:
        double r
        double g
        double p
        double epsilon
        double c
        double penalty
        double stiffness

    const char *wb_last_error()
    int32_t wb_version()

    int wb_pairwise_distance(const wb_series *x, const wb_series *y, int64_t dim,
                             int32_t metric, const wb_params *params, double *out,
                             int32_t out_on_device, void *stream)
    int wb_paired_distance(const wb_series *x, const wb_series *y, int64_t dim,
                           int32_t metric, const wb_params *params, double *out,
                           int32_t out_on_device, void *stream)
    int wb_nearest_pivot(const wb_series *x, int64_t dim, int64_t n_groups,
                         const int64_t *sample_ptr, const int64_t *samples,
                         const int64_t *pivot_ptr, const int64_t *pivots,
                         const int32_t *group_slot, const int32_t *slot_metric,
                         const wb_params *slot_params, int32_t n_slots,
                         int64_t *out_branch, double *out_dist, void *stream)
    int wb_subsequence_distance_views(const wb_series *x, const int64_t *view_sample,
                                      const int64_t *view_dim, const int64_t *view_start,
                                      const int64_t *view_length, const double *view_mean,
                                      const double *view_std, int64_t m,
                                      const wb_series *target, int64_t dim, int32_t metric,
                                      const wb_params *params, double *out_dist,
                                      int64_t *out_idx, void *stream)

    # the rest of the C ABI (include/wbgpu.h), in its order
    ctypedef struct wb_dtw32:
        const float *x
        int64_t x_stride
        const int32_t *x_lengths
        int32_t x_len
        int64_t nx
        const float *y
        int64_t y_stride
        const int32_t *y_lengths
        int32_t y_len
        int64_t ny
        const int32_t *item_x
        const int32_t *item_y
        int64_t n_items
        double r
        const float *weights
        int32_t strip
        int32_t block
        int32_t grid

    int wb_argmin_distance(const wb_series *x, const wb_series *y, int64_t dim,
                           int32_t metric, const wb_params *params, int64_t k,
                           const double *lower_bound, int64_t *indices, double *distances,
                           int32_t out_on_device, void *stream)
    int wb_pairwise_subsequence_distance(const double *shapelets, const int64_t *offsets,
                                         const int64_t *lengths, const double *means,
                                         const double *stds, int64_t m, const wb_series *x,
                                         int64_t dim, int32_t metric,
                                         const wb_params *params, double *out_dist,
                                         int64_t *out_idx, int32_t out_on_device,
                                         void *stream)
    int wb_paired_subsequence_distance(const double *shapelets, const int64_t *offsets,
                                       const int64_t *lengths, const double *means,
                                       const double *stds, int64_t m, const wb_series *x,
                                       int64_t dim, int32_t metric, const wb_params *params,
                                       double *out_dist, int64_t *out_idx,
                                       int32_t out_on_device, void *stream)
    int wb_subsequence_profile(const double *shapelets, const int64_t *offsets,
                               const int64_t *lengths, const double *means,
                               const double *stds, int64_t m, const wb_series *x,
                               int64_t dim, int32_t metric, const wb_params *params,
                               double *out_raw, double *out_key, int64_t ld,
                               int32_t std_as_given, int32_t out_on_device, void *stream)
    int wb_argmin_subsequence_distance(const double *s, const int64_t *s_len,
                                       int64_t s_stride, int64_t n, const double *s_mean,
                                       const double *s_std, const wb_series *x, int64_t dim,
                                       int32_t metric, const wb_params *params,
                                       int32_t scaled, int64_t k, int64_t *indices,
                                       double *distances, int32_t out_on_device,
                                       void *stream)
    int wb_dtw32_distance(const wb_dtw32 *job, double *out, double *out_cost, void *stream)
    int wb_dtw32_backward(const wb_dtw32 *job, const double *grad_out, float *grad_x,
                          int64_t gx_stride, float *grad_y, int64_t gy_stride, void *stream)
    int64_t wb_dtw32_keep_bytes(const wb_dtw32 *job)
    int wb_dtw32_distance_keep(const wb_dtw32 *job, double *out, double *out_cost,
                               void *keep, int64_t keep_bytes, void *stream)
    int wb_dtw32_backward_keep(const wb_dtw32 *job, const double *dist,
                               const double *grad_out, float *grad_x, int64_t gx_stride,
                               float *grad_y, int64_t gy_stride, const void *keep,
                               int64_t keep_bytes, void *stream)
    int wb_euclidean_tc(const wb_series *x, const wb_series *y, int64_t dim, double *out,
                        int32_t out_on_device, void *stream)
    int wb_pairwise_distance_fp32(const wb_series *x, const wb_series *y, int64_t dim,
                                  int32_t metric, const wb_params *params, double *out,
                                  int32_t out_on_device, void *stream)
    int wb_subsequence_profile_stop(const double *shapelets, const int64_t *offsets,
                                    const int64_t *lengths, const double *means,
                                    const double *stds, int64_t m, const wb_series *x,
                                    int64_t dim, const double *stop_sq, double *out_raw,
                                    int64_t ld, int32_t out_on_device, void *stream)
    int wb_dilated_profile(const wb_series *y, const wb_series *x, int64_t dim,
                           int32_t metric, const wb_params *params, int64_t dilation,
                           int64_t padding, int32_t scale, double *out,
                           int32_t out_on_device, void *stream)
    int wb_mass_profile(const wb_series *y, const wb_series *x, double *out,
                        int32_t out_on_device, void *stream)
    int wb_inject_fault(int32_t site, int64_t skip)
    int wb_series_lengths_f32(const float *x, int64_t n_series, int64_t stride, int32_t L,
                              int32_t *lengths, void *stream)
    int wb_pairwise_distance_noalloc(const wb_series *x, const wb_series *y, int64_t dim,
                                     int32_t metric, const wb_params *params, double *out,
                                     void *stream)
    int64_t wb_noalloc_scratch_bytes()
    int wb_dtw_average_mm_step(const double *x, int64_t x_stride, int64_t n_timestep,
                               const double *means, int64_t mean_len, const int64_t *member,
                               const int32_t *pair_group, const int64_t *group_start,
                               const int32_t *groups, int64_t n_groups, int64_t n_pairs,
                               double r, const double *weights, const double *sample_weight,
                               double *new_means, double *last, void *stream)
    int wb_dtw_envelope(const double *x, int64_t n, int64_t n_timestep, int64_t warp,
                        double *lower, double *upper, int32_t on_device, void *stream)
    int wb_lb_keogh(const double *q, int64_t nq, const double *x, int64_t nx,
                    int64_t n_timestep, int64_t warp, int32_t kind, double *out,
                    int32_t on_device, void *stream)
    int wb_lb_kim(const double *y, int64_t ny, const double *x, int64_t nx,
                  int64_t n_timestep, double *out, int32_t on_device, void *stream)
    int wb_dtw_average_ssg_epoch(const double *x, int64_t x_stride, int64_t n_timestep,
                                 double *mean, int64_t mean_len, const int64_t *order,
                                 const double *lr, int64_t n_steps, double r,
                                 const double *weights, const double *sample_weight,
                                 void *stream)
    int wb_dtw_alignment(const double *x, int64_t n, const double *y, int64_t m, double r,
                         const double *weights, double *out, int32_t on_device,
                         void *stream)
    int wb_lb_keogh_terms(const double *x, const double *lower, const double *upper,
                          int64_t n_timestep, double *cb, double *dist, int32_t on_device,
                          void *stream)
    int wb_group_mean(const double *x, int64_t x_stride, int64_t n_timestep,
                      const int64_t *member, const int64_t *group_start,
                      const int32_t *groups, int64_t n_groups, double *out, void *stream)
    int wb_release_workspace(void *stream)
    int64_t wb_launch_count()
    int wb_profile_enable(int32_t on)
    int wb_profile_last(double *ms)
    int wb_alu_probe(int32_t dtype, int32_t iters, double *ops_per_s)
