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
    // scaled metric, tiled kernel: chunks of <= chunk shapelets of one length
    // (positions [chunk_first, chunk_first + chunk_count) of `order`)
    const int64_t *chunk_first = nullptr;
    const int32_t *chunk_count = nullptr;
    const int32_t *chunk_group = nullptr;
    int64_t n_chunks = 0;
    int max_len = 0;
    // paired: series i against shapelet i only (x.count == m); outputs (m,),
    // window-stat tables one row per series at its shapelet's length
    int paired = 0;
    int std_as_given = 0;  // a zero std divides as is (distance profile's transient stats)
    // scaled profile only: per pair, stop a window's sum once it reaches this
    // value (checked before each term, as scaled_euclidean_distance_matches
    // does with the squared threshold, distance/_metric.pyx:625-651, 798-860)
    const double *stop_sq = nullptr;
    // FP32 pre-filter of the minimum scans (set by launch_subseq)
    const float *shp_f32 = nullptr;      // packed shapelets (z-normalised when scaled)
    const float *shp_absmax = nullptr;   // (m,) max |value| of each shapelet, rounded up
    double *out_dist = nullptr;          // (x.count, m)
    int64_t *out_idx = nullptr;          // (x.count, m)
};

size_t subseq_workspace_bytes(const SubseqJob &J, bool scaled);
// longest shapelet the tiled scaled kernel takes (its z-normalised window
// tile is L x 32 doubles of shared memory)
constexpr int kScaledTileMaxLen = 384;
// shapelets of one length sharing the z-normalised window tiles of a block
constexpr int kScaledTileChunk = 256;
int launch_subseq(const SubseqJob &J, bool scaled, Workspace &ws);
// paired jobs: every window's full sum at raw[pair * ld + window]
int launch_subseq_profile(const SubseqJob &J, bool scaled, Workspace &ws, double *raw,
                          int64_t ld);

// profile.cu: dilated / padded distance profile windows and the MASS profile
int launch_dilated_gather(const double *x, int64_t n, int64_t x_stride, int T, const double *y,
                          int64_t y_stride, int L, int dilation, int padding, int p0, int np,
                          int k, int scale, double *xw, double *kw, cudaStream_t s);
int launch_dilated_scatter(const double *d, int64_t n, int p0, int np, int k, int L,
                           double *out, int64_t out_ld, cudaStream_t s);
int launch_mass_profile(const double *x, int64_t n, int64_t x_stride, int T, const double *y,
                        int64_t y_stride, int L, double *mean_tab, double *std_tab,
                        double *out, cudaStream_t s);

}  // namespace wb
