// euclid_gemm.cu -- full-series euclidean distance matrix on the tensor cores.
//
// d(x_i, y_j)^2 = |x_i - y_j|^2.  Every series is rounded to float32 and
// centred on its own float32 mean m, X = fl(fl(x) - m); then
//   |x - y|^2 = |X|^2 + |Y|^2 - 2 X.Y + dm (K dm + 2 (sX - sY)),
// dm = m_x - m_y, sX = sum_k X_k (the rounding residue of the centring),
// up to the float32 rounding of the inputs.  The dot products X.Y
// come from a tcgen05 GEMM of kind::tf32 with the 3xTF32 split: every
// float32 value v = hi + lo with hi = tf32(v) and lo = v - hi, and
// X.Y ~ hi_x.hi_y + hi_x.lo_y + lo_x.hi_y (the lo.lo term is below FP32
// resolution), accumulated in FP32 in tensor memory.  Centring keeps the
// accumulated partial sums, and with them the accumulation error, small for
// series that share an offset or drift.  |X|^2 is summed with error-free
// FP32 transformations and kept as a float pair; the epilogue forms the expression above with
// compensated FP32 arithmetic (TwoSum, error terms carried in a lo part); the
// square root is the FP32 approximation (relative error ~2^-22, far below
// that of d^2) and the float -> double widening of the result is done
// with integer operations (the FP64 pipe stays free); rows are stored as
// float64 through a shared-memory transpose (coalesced).
//
// Kernel: persistent, one CTA per SM over 128 x 256 output tiles, 320
// threads: a TMA producer warp (64-byte swizzled K-major tiles of 16 floats
// into a 4-stage ring of 48 KB stages), an MMA warp (M=128, N=256, K=8, six
// MMAs per stage, tcgen05.commit frees a stage) and eight epilogue warps (two
// per TMEM lane quarter) that read the accumulator back with tcgen05.ld while
// the next tile accumulates into the second TMEM buffer.  A 128 x 256 tile
// reads 3 operand bytes per 256 MACs where a 128 x 128 tile reads 4.  Every
// mbarrier wait is bounded: a wait that runs out sets an error flag, the CTA
// still releases its TMEM.

#include <cuda.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace wb {

constexpr int kBM = 128, kBN = 256, kBK = 16;  // kBK floats = 64 bytes (one swizzle row)
constexpr int kStages = 4;
constexpr int kTileA = kBM * kBK * 4;          // 8 KB per A tile (hi or lo)
constexpr int kTileB = kBN * kBK * 4;          // 16 KB per B tile
constexpr int kStageBytes = 2 * kTileA + 2 * kTileB;  // A hi, A lo, B hi, B lo
constexpr int kEpiWarps = 8;      // two per TMEM lane quarter, each half of the columns
constexpr int kGemmThreads = 64 + 32 * kEpiWarps;  // producer warp, MMA warp, epilogue
// two accumulator buffers of kBN columns fill the 512 TMEM columns
constexpr int kTmemCols = 2 * kBN;
constexpr long long kWaitLimit = 1ll << 26;

// TwoSum (Knuth): returns s = fl(a + b) and sets e so that s + e == a + b exactly
__device__ __forceinline__ float two_sum(float a, float b, float &e) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}

// bounded wait on the phase `parity` of an mbarrier; false when it gave up
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long long i = 0; i < kWaitLimit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0,
                                            int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

// shared-memory matrix descriptor: K-major, 64-byte swizzle, 8-row groups
// 512 bytes apart (SBO), descriptor version 1
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;    // stride byte offset
    d |= (uint64_t)1 << 46;             // version
    d |= (uint64_t)4 << 61;             // layout: SWIZZLE_64B
    return d;
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, N = 256, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                            ((uint32_t)(kBM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            bar)
        : "memory");
}

// Persistent, warp-specialised: one CTA per SM walks the output tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...  Warp 0 (one lane) streams the
// operand tiles with TMA into a kStages-deep ring; warp 1 owns the tensor
// memory and (one lane) issues the MMAs; warps 2-9 run the epilogue, warp w
// reading TMEM lanes 32 (w % 4) .. +31 and columns 128 ((w - 2) / 4) .. +127.  Two accumulator buffers of kBN
// columns let the epilogue of tile t overlap the MMAs of tile t + 1.
//   full[s]  : TMA bytes of stage s landed        (producer -> MMA)
//   empty[s] : MMAs reading stage s completed     (MMA -> producer)
//   accf[b]  : all MMAs of buffer b's tile done   (MMA -> epilogue)
//   acce[b]  : epilogue finished reading buffer b (epilogue -> MMA, one arrival
//              per epilogue warp)
// Every wait is bounded; one that runs out raises a shared abort flag that
// the other roles poll, the error word is set, and the CTA still waits for its
// issued MMAs before releasing the tensor memory.
__device__ __forceinline__ bool bwait(uint32_t bar, uint32_t parity, volatile int *abort_flag) {
    for (long long i = 0; i < kWaitLimit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((i & 1023) == 1023 && *abort_flag) return false;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// float -> double of a non-negative normal float or +0 by its bit pattern:
// the exponent is re-biased (127 -> 1023) and the mantissa shifted into
// place, +0 stays 0 (the square root below flushes subnormal results to zero)
__device__ __forceinline__ double widen_nonneg(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t hi = (b >> 3) + (b ? 0x38000000u : 0u);
    return __hiloint2double((int)hi, (int)(b << 29));
}

__device__ __forceinline__ float sqrt_approx(float v) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}

__global__ void __launch_bounds__(kGemmThreads, 1)
euclid_tc_kernel(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
                 const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo,
                 // per series: {|X|^2 hi, |X|^2 lo, m, 0} and sX
                 const float4 *__restrict__ stx, const float *__restrict__ sumx,
                 const float4 *__restrict__ sty, const float *__restrict__ sumy, int M, int N,
                 int K, int Kp, double *out, int64_t ld_out, int *err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem =
        (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *stage_out = reinterpret_cast<float *>(smem + kStages * kStageBytes);
    __shared__ __align__(8) uint64_t full_bar[kStages];
    __shared__ __align__(8) uint64_t empty_bar[kStages];
    __shared__ __align__(8) uint64_t accf_bar[2];
    __shared__ __align__(8) uint64_t acce_bar[2];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int KT = Kp / kBK;
    const int tiles_n = (N + kBN - 1) / kBN;
    const int ntiles = ((M + kBM - 1) / kBM) * tiles_n;

    if (tid == 0) {
        for (int s = 0; s < kStages; s++) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&accf_bar[b]), 1);
            mbar_init(smem_u32(&acce_bar[b]), kEpiWarps);
        }
        mbar_init(smem_u32(&done_bar), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    // stage layout: A hi | A lo | B hi | B lo
    auto a_hi = [&](int st) { return smem + st * kStageBytes; };
    auto a_lo = [&](int st) { return smem + st * kStageBytes + kTileA; };
    auto b_hi = [&](int st) { return smem + st * kStageBytes + 2 * kTileA; };
    auto b_lo = [&](int st) { return smem + st * kStageBytes + 2 * kTileA + kTileB; };

    if (warp == 0) {
        // ---------------- producer
        if (lane == 0) {
            int st = 0;
            uint32_t ph = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                const int m0 = (tile / tiles_n) * kBM, n0 = (tile % tiles_n) * kBN;
                for (int kt = 0; kt < KT; kt++) {
                    ok = bwait(smem_u32(&empty_bar[st]), ph ^ 1u, &abort_flag);
                    if (!ok) break;
                    const uint32_t bar = smem_u32(&full_bar[st]);
                    mbar_expect_tx(bar, kStageBytes);
                    const int kc = kt * kBK;
                    tma_load_2d(smem_u32(a_hi(st)), &mAhi, kc, m0, bar);
                    tma_load_2d(smem_u32(a_lo(st)), &mAlo, kc, m0, bar);
                    tma_load_2d(smem_u32(b_hi(st)), &mBhi, kc, n0, bar);
                    tma_load_2d(smem_u32(b_lo(st)), &mBlo, kc, n0, bar);
                    if (++st == kStages) {
                        st = 0;
                        ph ^= 1u;
                    }
                }
            }
            if (!ok) {
                abort_flag = 1;
                atomicExch(err, 1);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            int st = 0;
            uint32_t ph = 0;
            bool ok = true;
            int it = 0;
            for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, it++) {
                const int b = it & 1;
                const uint32_t bph = (uint32_t)(it >> 1) & 1u;
                ok = bwait(smem_u32(&acce_bar[b]), bph ^ 1u, &abort_flag);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t dtm = tmem + (uint32_t)(b * kBN);
                for (int kt = 0; kt < KT; kt++) {
                    ok = bwait(smem_u32(&full_bar[st]), ph, &abort_flag);
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t ahi = smem_u32(a_hi(st)), alo = smem_u32(a_lo(st));
                    const uint32_t bhi = smem_u32(b_hi(st)), blo = smem_u32(b_lo(st));
#pragma unroll
                    for (int kk = 0; kk < kBK / 8; kk++) {
                        const uint32_t off = kk * 32;  // 8 tf32 = 32 bytes along K
                        const uint64_t dAh = smem_desc_sw64(ahi + off), dAl = smem_desc_sw64(alo + off);
                        const uint64_t dBh = smem_desc_sw64(bhi + off), dBl = smem_desc_sw64(blo + off);
                        mma_tf32(dtm, dAh, dBh, (kt > 0 || kk > 0) ? 1u : 0u);
                        mma_tf32(dtm, dAh, dBl, 1u);
                        mma_tf32(dtm, dAl, dBh, 1u);
                    }
                    mma_commit(smem_u32(&empty_bar[st]));
                    if (++st == kStages) {
                        st = 0;
                        ph ^= 1u;
                    }
                }
                if (!ok) break;
                mma_commit(smem_u32(&accf_bar[b]));
            }
            if (!ok) {
                abort_flag = 1;
                atomicExch(err, 1);
            }
            // no MMA may still be running when the tensor memory is released
            mma_commit(smem_u32(&done_bar));
            if (!mbar_wait(smem_u32(&done_bar), 0u)) atomicExch(err, 1);
        }
    } else {
        // ---------------- epilogue (warps 2..9)
        const int q = warp & 3;                  // TMEM lane quarter this warp may read
        const int ch = ((warp - 2) >> 2) * (kBN / 2);  // its half of the columns
        float *tile_s = stage_out + (warp - 2) * (32 * 17);
        const float Kf = (float)K;
        int it = 0;
        bool ok = true;
        for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, it++) {
            const int m0 = (tile / tiles_n) * kBM, n0 = (tile % tiles_n) * kBN;
            const int b = it & 1;
            const uint32_t bph = (uint32_t)(it >> 1) & 1u;
            ok = bwait(smem_u32(&accf_bar[b]), bph, &abort_flag);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int row = q * 32 + lane;
            const int gi = m0 + row;
            const float4 sxi = gi < M ? stx[gi] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float smx = gi < M ? sumx[gi] : 0.0f;
#pragma unroll 1
            for (int c0 = ch; c0 < ch + kBN / 2; c0 += 16) {
                uint32_t v[16];
                const uint32_t taddr =
                    tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kBN + c0);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                      "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]),
                      "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int gj = n0 + c0 + j;
                    const float4 syj = gj < N ? __ldg(&sty[gj]) : make_float4(0.f, 0.f, 0.f, 0.f);
                    const float smy = gj < N ? __ldg(&sumy[gj]) : 0.0f;
                    // t = |X|^2 + |Y|^2 - 2 X.Y with its rounding errors carried
                    float e1, e2;
                    const float s1 = two_sum(sxi.x, syj.x, e1);
                    const float t = two_sum(s1, -2.0f * __uint_as_float(v[j]), e2);
                    // delta = dm (K dm + 2 (sX - sY)) >= ~0 adds to t >= ~0 without
                    // cancellation, so plain FP32 (relative error ~u of d^2) suffices
                    const float dm = __fsub_rn(sxi.z, syj.z);
                    const float delta =
                        __fmul_rn(dm, __fmaf_rn(Kf, dm, 2.0f * __fsub_rn(smx, smy)));
                    const float corr = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(sxi.y, syj.y));
                    const float d2 = __fadd_rn(__fadd_rn(t, delta), corr);
                    tile_s[lane * 17 + j] = sqrt_approx(fmaxf(d2, 0.0f));
                }
                __syncwarp();
                // 32 rows x 16 columns: each half-warp writes one row's 16 values
#pragma unroll 4
                for (int r2 = 0; r2 < 32; r2 += 2) {
                    const int r = r2 + (lane >> 4);
                    const int gr = m0 + q * 32 + r;
                    const int gj = n0 + c0 + (lane & 15);
                    if (gr < M && gj < N)
                        out[(int64_t)gr * ld_out + gj] = widen_nonneg(tile_s[r * 17 + (lane & 15)]);
                }
                __syncwarp();
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&acce_bar[b]));
        }
        if (!ok && lane == 0) {
            abort_flag = 1;
            atomicExch(err, 1);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
}

// float64 rows -> centred float32 X = fl(fl(x) - m) with its hi / lo tf32
// split (zero padded to (rows_p, Kp)) and the row statistics.  One warp per
// row, FP32 only (GB300's FP64 rate is a small fraction of its FP32 rate):
// m is the float32 mean of fl(x) (any centre serves, the expansion is exact
// for the m it is given); |X|^2 is summed with error-free transformations
// (the exact square p + e by an FMA, TwoSum into (S, E)) and kept as a
// (hi, lo) pair, so it carries ~2^-44 relative error; sX = sum_k X_k is
// plain FP32 (it only enters multiplied by dm next to K dm^2).  KR > 0: each
// lane keeps its KR values of fl(x) in registers between the two passes
// (Kp <= 32 KR); KR == 0: the first pass leaves fl(x) in the hi row, which
// the same lane reads back.
struct SplitAcc {
    float S = 0.0f, E = 0.0f, s1 = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float p = __fmul_rn(v, v);
        const float e = __fmaf_rn(v, v, -p);
        float err;
        S = two_sum(S, p, err);
        E = __fadd_rn(E, __fadd_rn(err, e));
        s1 = __fadd_rn(s1, v);
    }
};

__device__ __forceinline__ void split_store(float v, float *hr, float *lr, int k) {
    uint32_t hb;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hb) : "f"(v));
    const float h = __uint_as_float(hb);
    hr[k] = h;
    lr[k] = __fsub_rn(v, h);
}

// one operand of the split: rows_p rows of Kp floats, rows live ones
struct SplitSide {
    const double *x;
    int64_t stride;
    int rows, rows_p;
    float *hi, *lo;
    float4 *stat;
    float *sum;
};

// rows 0 .. A.rows_p - 1 of the launch are A's, the next B.rows_p are B's;
// the first thread also clears the GEMM's wait-status word
template <int KR>
__global__ void tf32_split_kernel(SplitSide A, SplitSide B, int K, int Kp, int *err) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *err = 0;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t total = (int64_t)A.rows_p + B.rows_p;
    for (int64_t t = warp; t < total; t += nwarps) {
        const bool second = t >= A.rows_p;
        const SplitSide &P = second ? B : A;
        const int64_t r = second ? t - A.rows_p : t;
        const double *x = P.x;
        const int64_t stride = P.stride;
        float *hr = P.hi + r * (int64_t)Kp;
        float *lr = P.lo + r * (int64_t)Kp;
        const bool live = r < P.rows;
        float xv[KR > 0 ? KR : 1];
        float s = 0.0f;
        if (KR > 0) {
#pragma unroll
            for (int i = 0; i < KR; i++) {
                const int k = lane + 32 * i;
                xv[i] = (live && k < K) ? (float)x[r * stride + k] : 0.0f;
                s += xv[i];
            }
        } else if (live) {
            for (int k = lane; k < K; k += 32) {
                const float xf = (float)x[r * stride + k];
                hr[k] = xf;
                s += xf;
            }
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const float m = live ? s / (float)K : 0.0f;
        SplitAcc acc;
        if (KR > 0) {
#pragma unroll
            for (int i = 0; i < KR; i++) {
                const int k = lane + 32 * i;
                if (k < Kp) {
                    const float v = (live && k < K) ? __fsub_rn(xv[i], m) : 0.0f;
                    split_store(v, hr, lr, k);
                    acc.add(v);
                }
            }
        } else {
            for (int k = lane; k < Kp; k += 32) {
                const float v = (live && k < K) ? __fsub_rn(hr[k], m) : 0.0f;
                split_store(v, hr, lr, k);
                acc.add(v);
            }
        }
        float S = acc.S, E = acc.E, s1 = acc.s1;
        for (int o = 16; o > 0; o >>= 1) {
            const float S2 = __shfl_xor_sync(0xffffffffu, S, o);
            const float E2 = __shfl_xor_sync(0xffffffffu, E, o);
            float err;
            S = two_sum(S, S2, err);
            E = __fadd_rn(E, __fadd_rn(E2, err));
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (lane == 0 && live) {
            float nl;
            const float nh = two_sum(S, E, nl);
            P.stat[r] = make_float4(nh, nl, m, 0.0f);
            P.sum[r] = s1;
        }
    }
}

static void launch_split(const SplitSide &A, const SplitSide &B, int K, int Kp, int *err,
                         cudaStream_t s) {
    const int64_t rows = (int64_t)A.rows_p + B.rows_p;
    const int grid = (int)std::min<int64_t>((int64_t)device_info().sm_count * 8, (rows + 7) / 8);
    if (Kp <= 32 * 32)
        tf32_split_kernel<32><<<grid, 256, 0, s>>>(A, B, K, Kp, err);
    else
        tf32_split_kernel<0><<<grid, 256, 0, s>>>(A, B, K, Kp, err);
}

// a pinned host word per thread for the status read-back (allocated once)
static int *pinned_status() {
    thread_local int *p = nullptr;
    if (!p && cudaMallocHost(&p, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
    }
    return p;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

static int make_map(CUtensorMap *map, float *base, int rows_p, int Kp, int box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return fail(WB_ECUDA, "cuTensorMapEncodeTiled is unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows_p};
    cuuint64_t strides[1] = {(cuuint64_t)Kp * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(WB_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return WB_OK;
}

static int round_up(int v, int m) { return (v + m - 1) / m * m; }

// x: (M, K) float64 rows with row stride sx; y: (N, K); out (M, N) float64
int euclid_tc(const double *x, int64_t sx, int M, const double *y, int64_t sy, int N, int K,
              double *out, int64_t ld_out, Workspace &ws, bool reserve_only, size_t *bytes) {
    const int Mp = round_up(std::max(M, 1), kBM), Np = round_up(std::max(N, 1), kBN);
    const int Kp = round_up(std::max(K, 1), kBK);
    const size_t need = 2 * align256((size_t)Mp * Kp * 4) + 2 * align256((size_t)Np * Kp * 4) +
                        align256((size_t)M * 16) + align256((size_t)N * 16) +
                        align256((size_t)M * 4) + align256((size_t)N * 4) + 256;
    if (reserve_only) {
        *bytes = need;
        return WB_OK;
    }
    cudaStream_t s = ws.stream();
    WB_TAKE(ahi, float, ws, (size_t)Mp * Kp);
    WB_TAKE(alo, float, ws, (size_t)Mp * Kp);
    WB_TAKE(bhi, float, ws, (size_t)Np * Kp);
    WB_TAKE(blo, float, ws, (size_t)Np * Kp);
    WB_TAKE(stx, float4, ws, M);
    WB_TAKE(sty, float4, ws, N);
    WB_TAKE(smx, float, ws, M);
    WB_TAKE(smy, float, ws, N);
    WB_TAKE(err, int, ws, 1);
    launch_split(SplitSide{x, sx, M, Mp, ahi, alo, stx, smx},
                 SplitSide{y, sy, N, Np, bhi, blo, sty, smy}, K, Kp, err, s);
    WB_LAUNCH_CHECK("tf32_split_kernel");
    CUtensorMap mAh, mAl, mBh, mBl;
    WB_TRY(make_map(&mAh, ahi, Mp, Kp, kBM));
    WB_TRY(make_map(&mAl, alo, Mp, Kp, kBM));
    WB_TRY(make_map(&mBh, bhi, Np, Kp, kBN));
    WB_TRY(make_map(&mBl, blo, Np, Kp, kBN));
    // stage ring + one staging block of 32 x 17 floats per epilogue warp + alignment slack
    const int smem = kStages * kStageBytes + kEpiWarps * 32 * 17 * 4 + 1024;
    static bool smem_set[64] = {};  // per device ordinal
    int devno = 0;
    WB_CUDA(cudaGetDevice(&devno));
    if (devno < 0 || devno >= 64 || !smem_set[devno]) {
        WB_CUDA(cudaFuncSetAttribute(euclid_tc_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        if (devno >= 0 && devno < 64) smem_set[devno] = true;
    }
    const int ntiles = (Mp / kBM) * (Np / kBN);
    const int grid = std::min(ntiles, device_info().sm_count);
    timer_begin("euclid_tc_kernel", s);
    euclid_tc_kernel<<<grid, kGemmThreads, smem, s>>>(mAh, mAl, mBh, mBl, stx, smx, sty, smy, M,
                                                      N, K, Kp, out, ld_out, err);
    timer_end(s);
    WB_LAUNCH_CHECK("euclid_tc_kernel");
    int herr = 0;
    int *ph = pinned_status();
    WB_CUDA(cudaMemcpyAsync(ph ? ph : &herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    WB_CUDA(cudaStreamSynchronize(s));
    if (ph) herr = *ph;
    if (herr || injected(INJ_WAIT))
        return fail(WB_ETIMEOUT, "euclid_tc_kernel: a pipeline wait gave up");
    return WB_OK;
}

}  // namespace wb

using namespace wb;

extern "C" int wb_euclidean_tc(const wb_series *x, const wb_series *y, int64_t dim, double *out,
                               int32_t out_on_device, void *stream_) {
    WB_TRACE();
    if (!x || !y) return fail(WB_EINVAL, "x and y are required");
    if (x->dtype != WB_F64 || y->dtype != WB_F64) return fail(WB_EINVAL, "float64 series expected");
    if (!x->on_device || !y->on_device)
        return fail(WB_EINVAL, "the tensor-core euclidean path takes device series");
    if (x->n_timestep != y->n_timestep)
        return fail(WB_EINVAL, "Illegal n_timestep for non-elastic distance measure");
    if (dim < 0 || dim >= x->n_dims || y->n_dims != x->n_dims)
        return fail(WB_EINVAL, "The parameter dim must be 0 <= dim < n_dims");
    if (x->n > (1 << 30) || y->n > (1 << 30) || x->n_timestep > (1 << 28))
        return fail(WB_EINVAL, "problem too large");
    if (x->n == 0 || y->n == 0) return WB_OK;
    if (!out) return fail(WB_EINVAL, "out is NULL");
    cudaStream_t s = (cudaStream_t)stream_;
    const int M = (int)x->n, N = (int)y->n, K = (int)x->n_timestep;
    Workspace ws(s);
    size_t need = 0;
    euclid_tc(nullptr, 0, M, nullptr, 0, N, K, nullptr, 0, ws, true, &need);
    size_t out_bytes = out_on_device ? 0 : align256((size_t)M * N * 8);
    WB_TRY(ws.reserve(need + out_bytes));
    double *dout = out;
    if (!out_on_device) {
        dout = ws.take<double>((size_t)M * N);
        if (!dout) return fail(WB_ENOMEM, "workspace reservation exceeded");
    }
    const double *xb = static_cast<const double *>(x->data) + dim * x->n_timestep;
    const double *yb = static_cast<const double *>(y->data) + dim * y->n_timestep;
    WB_TRY(euclid_tc(xb, x->n_dims * x->n_timestep, M, yb, y->n_dims * y->n_timestep, N, K,
                     dout, N, ws, false, nullptr));
    if (!out_on_device) {
        WB_CUDA(cudaMemcpyAsync(out, dout, (size_t)M * N * 8, cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaStreamSynchronize(s));
    }
    return WB_OK;
}
