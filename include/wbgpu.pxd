# wbgpu.pxd -- Cython declarations of the wbgpu C ABI (wbgpu.h) for compiled
# callers: the proximity trees (tree/_cptree.pyx:254-290, 869-894) and the
# shapelet transforms (transform/_cshapelet.pyx:50-131) call the reference's
# cdef metrics per pair; with these declarations they hand whole nodes or
# attribute columns to the batched entries instead.  Link with libwbgpu.so.

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
