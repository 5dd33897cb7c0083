# cython: language_level=3
# A compiled caller of the batched pivot partition, written as a proximity
# tree's builder would call it through include/wbgpu.pxd: every open node of
# a depth (its samples and pivots as rows of x, its sampled metric) goes to
# one wb_nearest_pivot call instead of _partition_pivots' per-sample
# metric.distance calls (tree/_cptree.pyx:869-894).

import numpy as np

from wbgpu cimport (WB_F64, WB_OK, wb_last_error, wb_nearest_pivot, wb_params, wb_series,
                    wb_version)
from libc.stdint cimport int32_t, int64_t


def version():
    return wb_version()


def partition_nodes(double[:, :, ::1] x, int64_t[::1] sample_ptr, int64_t[::1] samples,
                    int64_t[::1] pivot_ptr, int64_t[::1] pivots, int32_t[::1] group_slot,
                    int32_t[::1] slot_metric, double[::1] slot_r, int64_t dim=0):
    """(status, message, branch, dist) of one batched partition (host arrays)."""
    cdef wb_series sx
    sx.data = &x[0, 0, 0]
    sx.n = x.shape[0]
    sx.n_dims = x.shape[1]
    sx.n_timestep = x.shape[2]
    sx.dtype = WB_F64
    sx.on_device = 0
    cdef int32_t n_slots = slot_metric.shape[0]
    params = np.zeros((n_slots, 7))
    cdef double[:, ::1] pv = params
    cdef int32_t k
    for k in range(n_slots):
        pv[k, 0] = slot_r[k]          # r
        pv[k, 1] = 0.05               # g
        pv[k, 2] = 1.0                # p
        pv[k, 3] = 1.0                # epsilon
        pv[k, 4] = 1.0                # c
        pv[k, 5] = 1.0                # penalty
        pv[k, 6] = 0.001              # stiffness
    branch = np.empty(samples.shape[0], dtype=np.int64)
    dist = np.empty(samples.shape[0])
    cdef int64_t[::1] bv = branch
    cdef double[::1] dv = dist
    cdef int st
    with nogil:
        st = wb_nearest_pivot(&sx, dim, sample_ptr.shape[0] - 1, &sample_ptr[0], &samples[0],
                              &pivot_ptr[0], &pivots[0], &group_slot[0], &slot_metric[0],
                              <const wb_params *> &pv[0, 0], n_slots, &bv[0], &dv[0], NULL)
    msg = wb_last_error().decode() if st != WB_OK else ""
    return st, msg, branch, dist
