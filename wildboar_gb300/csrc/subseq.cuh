// subseq.cuh -- job description of the subsequence scan kernels.
#pragma once

#include "elastic.cuh"

namespace wb {

struct SubseqJob {
    SeriesSet x;                     // the series scanned (one dim)
    const double *shapelets = nullptr;   // packed values (device)
    const int64_t *offsets = nullptr;    // (m,)
    const int64_t *lengths = nullptr;    // (m,)
    const double *means = nullptr;       // (m,) np.mean of each shapelet
    const double *stds = nullptr;        // (m,) np.std (<= 1e-13 given as 0)
    const int64_t *order = nullptr;      // processing order (by length) or null
    const int32_t *group_of = nullptr;   // (m,) index of the shapelet's length group
    const int32_t *group_len = nullptr;  // (n_groups,) distinct lengths
    int n_groups = 0;
    int64_t m = 0;
    int64_t total_values = 0;
    int win_stride = 0;                  // row stride of the window-stat tables
    int chunk = 64;                      // shapelets per block
    double *out_dist = nullptr;          // (x.count, m)
    int64_t *out_idx = nullptr;          // (x.count, m)
};

size_t subseq_workspace_bytes(const SubseqJob &J, bool scaled);
int launch_subseq(const SubseqJob &J, bool scaled, Workspace &ws);

}  // namespace wb
