// bf16 tensor-core screening of the distance sweeps, with exact f32 re-evaluation.
//
// The kNN sweep and every Borůvka round first run a screening pass on the 5th-generation tensor
// cores: the points are rounded to bf16 once, in a pre-swizzled tiled copy, and one persistent
// CTA per SM computes 128 x 256 tiles of dot products with tcgen05.mma (fp32 accumulators in
// TMEM, operands streamed into shared memory by bulk async copies). From each dot product the
// epilogue forms a proven LOWER bound of the reference's f32 squared distance,
//
//     L_ij = (1 - C_B)(p_i + p_j) - 2 dot_ij - C_A m_i m_j  <=  d2_ij (sequential-FMA f32),
//
// where p = ||x||^2 (f32), m >= ||x||, C_A bounds the bf16 rounding of both operands and the
// tensor-core accumulation, and C_B the f32 rounding of norms, of the reference sum and of the
// epilogue arithmetic (see error_coefficients below). Per query row the M smallest bounds (for
// Borůvka: max(L, core_i, core_j) over other components) stay in registers. A second kernel
// re-evaluates those M candidates with the exact f32 direct-difference arithmetic and checks the
// result against the M-th bound: every pair outside the list has a lower bound >= that bound, so
// when it is larger than the selected exact value no outside pair can change the result. Rows
// that fail the check are re-run by the exact f32 kernels. The outputs are therefore bit
// identical to the plain path.
//
// Operand formats: bf16 of x; fp16 of x * 2^k (a power-of-two scale that brings the largest
// |x| into [2^14, 2^15)); and split bf16, x = hi + lo with hi = bf16(x) and lo = bf16(x - hi),
// whose dot product hi.hi' + hi.lo' + lo.hi' (three K blocks per 64 features) misses x.y by
// about 3 * 2^-16 |x||y| instead of 2^-7. A bf16-refined fit whose plain bf16 screen leaves too
// many kNN rows inconclusive screens again with split bf16 (d <= 64, where a tile of hi and lo
// blocks fits two pipeline stages) or with scaled fp16 operands (wider rows), and keeps that
// format for its Borůvka rounds.
#include <cuda_bf16.h>

#include <cmath>

#include "common.cuh"
#include "forest.cuh"

namespace cuscan {

namespace {

constexpr int BM = 128;            // query rows per block = TMEM lanes
constexpr int BN = 256;            // reference rows per tile = MMA N
constexpr int EPI_WARPS = 8;            // two per TMEM lane quadrant
constexpr int HALF = 128;                // columns of a tile per epilogue warp
constexpr int THREADS = (2 + EPI_WARPS) * 32;
constexpr uint32_t KBLOCK_A = BM * 128;   // bytes of one 64-element K block of A (16 KiB)
constexpr uint32_t KBLOCK_B = BN * 128;   // bytes of one 64-element K block of B (32 KiB)
constexpr uint64_t WAIT_NS = 2000000000ull;  // bounded mbarrier waits: 2 s of wall time
constexpr uint32_t WAIT_POLLS = 1u << 22;      // poll bound of the abort-path drains
constexpr int VSTRIDE = 36;               // floats per lane in the hit staging area
constexpr int PB_STRIDE = 4 * HALF;       // kNN modes, per epilogue warp: [2][HALF] pb, [2][HALF] m
constexpr int BORUVKA_CAP = 32;           // Borůvka candidate slots per row half

struct Params {
    const uint8_t *xt;        // 16-bit tiles, pre-swizzled (see tile_16bit_kernel)
    int nbk;                  // K blocks per tile row of the copy: kblocks, or 2 kblocks (split)
    int split;                // split bf16: blocks [0, kblocks) hold hi, [kblocks, 2 kblocks) lo
    // kNN sweeps: [0] tiles issued by all CTAs so far (see knn_tile), [1] query blocks taken
    unsigned long long *cursor;
    const float *pnorm;       // [n_pad] f32 squared norms (+inf on padding rows)
    const float *mnorm;       // [n_pad] norms rounded up (0 on padding rows)
    // column terms of this launch (screen_columns_kernel): (1 - C_B) p, cores in screen units
    // (Borůvka; 0 past n) and (min, min) of both over every 32-column chunk
    const float *colp;
    const float *colc;
    const float4 *cmin;       // [n_pad / 64]: two chunks per entry
    const float *core;        // [n] core distances (Borůvka)
    const int32_t *label;     // [n] component labels (Borůvka)
    const float *tile_mmax;   // [n_tiles] max m over each 256-row tile
    const int32_t *chunk_lo;  // [ceil(n/32)] label range of 32-row chunks (Borůvka)
    const int32_t *chunk_hi;
    const int32_t *tile_lo;   // [n_tiles] label range of 256-row tiles (Borůvka)
    const int32_t *tile_hi;
    int64_t n, n_tiles, n_qblocks, n_chunks;
    int kblocks, stages;
    // one-sided Borůvka with fewer query blocks than SMs: CTAs per query block, each running one
    // contiguous part of the block's tile order (work item qi = block qi / splits, part qi %
    // splits; appends then take their slots with atomics and the row bounds are min-reduced)
    int splits;
    float c_a, one_minus_cb;
    int32_t *cand_ids;        // [n][M]
    float *cand_lb;           // [n][M]
    int *error;               // [0]: error flag; bytes 8..15: (qb, tile) pairs the MMA ran (u64)
    float *debug_tile;        // when set: the raw 128 x 256 accumulator of query block 0 x tile 0
    float *debug_chunk;       // with debug_tile: [128][8] the phase-1 maxima of its 32-column chunks
    float c_b;                // norm coefficient of the bound (upper bounds use it)
    uint32_t *cbound;         // Borůvka: per-component upper bound of the cheapest edge (f32 bits)
    int32_t *rowcnt;          // Borůvka: candidates appended per row half ([n][2])
    int cap;                  // Borůvka: candidate slots per row half
    uint32_t idesc;           // MMA instruction descriptor (bf16 or fp16 operands)
    float s2, inv_s2;         // operand scale squared (a power of two) and its inverse: the
                              // screen works in scaled units, inputs and outputs are raw
    float abs_c;              // absolute error term of the bound (fp16 subnormal rounding)
    // query rows (the A operand): the reference set itself, or a gathered subset
    const uint8_t *xq;        // 16-bit tiles of the query rows, same layout as xt
    const float *pq, *mq;     // their squared norms and rounded-up norms
    int64_t nq;               // query rows
    const int32_t *qpos;      // position of each query row in the reference order (null: same)
    const float *qthr;        // threshold mode: per-query upper bound of the k-th distance (raw)
    // symmetric Borůvka: per-row upper bounds of the cheapest cross edge (raw f32 bits) and the
    // per-row buffers that other query blocks append column-side pairs to
    uint32_t *urow;
    int32_t *colcnt;
    int32_t *colbuf;
    int capc;
    // one-sided Borůvka: per query row and column half, a lower bound of every cross-component
    // pair weight the row has (raw f32, rounded down)
    float *rowlb;
};

// Screen modes: kNN lists, Borůvka thresholds with shared component bounds, kNN thresholds.
constexpr int MODE_KNN_LIST = 0;
constexpr int MODE_BORUVKA = 1;
constexpr int MODE_KNN_THRESHOLD = 2;
// Borůvka over each unordered pair once: a query block visits its own tile (both halves see
// every pair inside it) and the tiles after it, testing each pair for its row and, through
// the column-side buffers, for its column.
constexpr int MODE_BORUVKA_SYM = 3;
constexpr int BORUVKA_COL_CAP = 64;  // column-side candidate slots per row
constexpr double SYM_UNBOUNDED_MAX = 0.25;  // largest share of unbounded rows for the symmetric screen
constexpr int64_t SYM_MIN_ROWS = 131072;     // smallest point set for the symmetric screen
constexpr double SYM_ACTIVE_MIN = 0.9;  // smallest share of screened rows for the symmetric screen
constexpr int KNN_CAP = 512;  // threshold-mode candidate slots per row half
constexpr int KNN_LIST = 22;  // kNN list entries per row half
constexpr int RESCREEN_MIN_ROWS = 256;  // fewer inconclusive kNN rows go straight to exact f32
// A bf16-refined fit whose first kNN screen leaves more than this share of rows inconclusive
// screens again with tighter operands (split bf16, or scaled fp16 for rows too wide to split).
constexpr double TIGHTEN_TRIGGER = 0.15;
// Operand formats of the 16-bit copy.
constexpr int FMT_BF16 = 0;
constexpr int FMT_FP16 = 1;
constexpr int FMT_SPLIT = 2;

// ---- PTX wrappers ----
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait: returns false (and raises the CTA abort flag and the error word) when the
// barrier does not flip within WAIT_NS nanoseconds, or as soon as another role has aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort,
                                          int *error) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 0u) {
            if (*abort) return false;
            if (global_ns() - t0 > WAIT_NS) break;
        }
    }
    *abort = 1;
    atomicExch(error, 1);
    return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
    d |= (uint64_t)1 << 46;            // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;            // SWIZZLE_128B
    return d;
}
// Instruction descriptors of kind::f16: D f32, A and B both bf16 (format 1 in bits 7-9 and
// 10-12) or both fp16 (format 0), both K-major, M=128, N=256.
constexpr uint32_t IDESC_F16 = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
constexpr uint32_t IDESC_BF16 = IDESC_F16 | (1u << 7) | (1u << 10);

__device__ __forceinline__ void mma_16bit(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}
// Issue a 32-column TMEM load (no wait): the registers are valid only after tmem_ld_wait.
__device__ __forceinline__ void tmem_ld32_issue(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
}
// Issue a 32-column TMEM load that also returns the largest of the 32 values (tcgen05.ld.red,
// sm_103a): the reduction rides on the load, so the chunk maxima of the screens cost no ALU
// work. mx and r are valid only after tmem_ld_wait_max. The maximum is exact (no rounding), the
// same value as a max.f32 tree over r.
__device__ __forceinline__ void tmem_ld32_max_issue(uint32_t taddr, uint32_t (&r)[32], float &mx) {
    asm volatile(
        "tcgen05.ld.red.sync.aligned.32x32b.x32.max.f32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
        "%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, %32, "
        "[%33];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31]), "=f"(mx)
        : "r"(taddr));
}
// Wait for every issued TMEM load; the register operands tie r to the wait so the compiler
// cannot read them earlier.
__device__ __forceinline__ void tmem_ld_wait(uint32_t (&r)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    asm volatile(""
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                   "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                   "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]),
                   "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]),
                   "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31]));
}

// Byte offset of element (row r, column f < d_eff) in the tiled 16-bit copy: 256-row tiles, each
// split into 64-column K blocks of 256 rows x 128 bytes whose 16-byte chunks are XOR-swizzled
// by the row (the SWIZZLE_128B K-major layout), so one bulk copy lands a block ready for the
// MMA. d_eff is d_pad, or 2 d_pad for split copies (the lo parts in columns d_pad + f).
__host__ __device__ __forceinline__ uint64_t tiled_offset(int64_t r, int f, int d_eff) {
    const int64_t t = r >> 8;
    const int rr = (int)(r & 255);
    const int kb = f >> 6, c = f & 63;
    const int chunk = (c >> 3) ^ (rr & 7);
    return (uint64_t)t * (uint64_t)(BN * d_eff * 2) + (uint64_t)kb * KBLOCK_B +
           (uint64_t)rr * 128 + (uint64_t)chunk * 16 + (uint64_t)(c & 7) * 2;
}

// 16-bit tiled copy of the (scaled) rows: bf16, fp16 of x * scale (scale a power of two), or
// split bf16 (hi in columns [0, d_pad), lo = bf16(x - hi) in [d_pad, 2 d_pad)).
// Row r of the copy is row rowmap[r] of x (r itself when rowmap is null); rows >= n are zero.
template <int FMT>
__global__ void tile_16bit_kernel(const float *__restrict__ x, int64_t n, int d, int d_pad,
                                  int64_t n_pad, float scale, const int32_t *__restrict__ rowmap,
                                  uint8_t *__restrict__ xt) {
    // one thread per (row, group of 8 features): 16 bytes out (32 for split)
    const int groups = d_pad >> 3;
    const int d_eff = FMT == FMT_SPLIT ? 2 * d_pad : d_pad;
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_pad * groups) return;
    int64_t r = e / groups;
    int g = (int)(e - r * groups);
    const int64_t src = r < n ? (rowmap ? (int64_t)rowmap[r] : r) : 0;
    __align__(16) uint16_t h[8];
    __align__(16) uint16_t l[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        int f = g * 8 + q;
        float v = (r < n && f < d) ? x[src * d + f] : 0.0f;
        if constexpr (FMT == FMT_FP16) {
            h[q] = __half_as_ushort(__float2half_rn(v * scale));
        } else {
            const __nv_bfloat16 hi = __float2bfloat16_rn(v);
            h[q] = __bfloat16_as_ushort(hi);
            // v - hi is exact in f32 (hi is within a factor of two of v)
            if constexpr (FMT == FMT_SPLIT)
                l[q] = __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(hi)));
        }
    }
    *reinterpret_cast<uint4 *>(xt + tiled_offset(r, g * 8, d_eff)) =
        *reinterpret_cast<const uint4 *>(h);
    if constexpr (FMT == FMT_SPLIT)
        *reinterpret_cast<uint4 *>(xt + tiled_offset(r, d_pad + g * 8, d_eff)) =
            *reinterpret_cast<const uint4 *>(l);
}

// Squared norms and rounded-up norms of the scaled rows (x * scale, exact for a power of two);
// row r is row rowmap[r] of x when rowmap is given.
__global__ void norms_kernel(const float *__restrict__ x, int64_t n, int d, int64_t n_pad,
                             float scale, const int32_t *__restrict__ rowmap,
                             float *__restrict__ pnorm, float *__restrict__ mnorm) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_pad) return;
    if (r >= n) {
        pnorm[r] = CUSCAN_INF;
        mnorm[r] = 0.0f;
        return;
    }
    const int64_t src = rowmap ? (int64_t)rowmap[r] : r;
    float acc = 0.0f;
    for (int f = 0; f < d; ++f) {
        float v = x[src * d + f] * scale;
        acc = __fmaf_rn(v, v, acc);
    }
    pnorm[r] = acc;
    // rounded-up norm, widened by 2^-20 so it bounds the true norm despite the f32 sum
    mnorm[r] = __fmul_ru(__fsqrt_ru(acc), 1.0f + 0x1p-20f);
}

// Largest |x| over all coordinates (non-negative floats order like their bit patterns).
__global__ void absmax_kernel(const float *__restrict__ x, int64_t count,
                              unsigned int *__restrict__ out) {
    float m = 0.0f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// Column terms of one screen launch, computed once instead of by every epilogue warp that
// reads the columns: colp = (1 - C_B) p (+inf on padding rows), colc = core * s2 (Borůvka; 0
// past n), and for every 32-column chunk (min colp, min colc) (0 for colc in the kNN modes).
// One thread per padded row; n_pad is a multiple of the 256-thread block.
__global__ void screen_columns_kernel(const float *__restrict__ pnorm,
                                      const float *__restrict__ core, int64_t n,
                                      float one_minus_cb, float s2, float *__restrict__ colp,
                                      float *__restrict__ colc, float2 *__restrict__ cmin) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const float p = pnorm[j] * one_minus_cb;
    colp[j] = p;
    float c = 0.0f;
    if (core) {
        c = j < n ? core[j] * s2 : 0.0f;
        colc[j] = c;
    }
    float pm = p, cm = c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pm = fminf(pm, __shfl_xor_sync(0xffffffffu, pm, o));
        cm = fminf(cm, __shfl_xor_sync(0xffffffffu, cm, o));
    }
    if ((threadIdx.x & 31) == 0) cmin[j >> 5] = make_float2(pm, cm);
}

__global__ void tile_stats_kernel(const float *__restrict__ mnorm, const int32_t *__restrict__ chunk_lo,
                                  const int32_t *__restrict__ chunk_hi, int64_t n_tiles,
                                  int64_t n_chunks, float *__restrict__ tile_mmax,
                                  int32_t *__restrict__ tile_lo, int32_t *__restrict__ tile_hi) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tiles) return;
    float mx = 0.0f;
    for (int r = 0; r < BN; ++r) mx = fmaxf(mx, mnorm[t * BN + r]);
    tile_mmax[t] = mx;
    if (chunk_lo) {
        int32_t lo = INT32_MAX, hi = INT32_MIN;
        for (int64_t c = t * 8; c < t * 8 + 8 && c < n_chunks; ++c) {
            lo = min(lo, chunk_lo[c]);
            hi = max(hi, chunk_hi[c]);
        }
        tile_lo[t] = lo;
        tile_hi[t] = hi;
    }
}

// Order in which query block qb visits the reference tiles. Every order starts with a window of
// WARM tiles around the block's own tile: in cell-sorted data these hold the block's nearest
// neighbours, so the per-row thresholds tighten at once.
//
// Borůvka rounds (tile_order) go on cyclically from the window. Their blocks skip different
// tiles, and the tiles they run stay in L2 anyway (one to two GB of DRAM reads per round at
// 500,000 points), so the cheapest order wins there.
//
// The kNN sweeps (knn_tile) run every tile for every block. After the window a block enters one
// cyclic order of the other tiles that all CTAs share, at the rotation `rot` the producer takes
// from the tile cursor when the block starts: the average position of the CTAs. Blocks started
// at different times then stream the same tiles and share them in L2. Without the rotation the
// CTAs drift apart over the waves of the persistent loop and the sweep reads the copy from
// DRAM about a thousand times over.
constexpr int64_t WARM = 4;

// Order-preserving map of f32 values to u32 (for integer warp reductions) and back.
__device__ __forceinline__ uint32_t f2ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
__device__ __forceinline__ float warp_max_f(float v) {
    return ord2f(__reduce_max_sync(0xffffffffu, f2ord(v)));
}
__device__ __forceinline__ float warp_min_f(float v) {
    return ord2f(__reduce_min_sync(0xffffffffu, f2ord(v)));
}

__device__ __forceinline__ int64_t window_start(const Params &P, int64_t qb) {
    const int64_t w = P.n_tiles < WARM ? P.n_tiles : WARM;
    const int64_t first = P.qpos ? (int64_t)P.qpos[qb * BM] : qb * BM;
    int64_t a = first / BN - w / 2;
    if (a < 0) a = 0;
    if (a > P.n_tiles - w) a = P.n_tiles - w;
    return a;
}
__device__ __forceinline__ int64_t tile_order(const Params &P, int64_t a, int64_t i) {
    const int64_t t = a + i;
    return t < P.n_tiles ? t : t - P.n_tiles;
}
// n tiles, window [a, a + w), rotation r < n - w (r = 0 when n <= WARM).
__device__ __forceinline__ int32_t knn_tile(int32_t n, int32_t a, int32_t r, int32_t i) {
    const int32_t w = n < (int32_t)WARM ? n : (int32_t)WARM;
    if (i < w) return a + i;
    int32_t j = i - w + r;
    if (j >= n - w) j -= n - w;
    return j < a ? j : j + w;
}

// Tiles query block qb visits and the i-th of them. The symmetric Borůvka mode visits the
// block's own tile and then every later tile in order; the other modes visit every tile
// (tile_order).
template <bool SYM>
__device__ __forceinline__ int64_t vis_count(const Params &P, int64_t qb) {
    return SYM ? P.n_tiles - (qb >> 1) : P.n_tiles;
}
template <bool SYM>
__device__ __forceinline__ int64_t vis_tile(const Params &P, int64_t qb, int64_t wa, int64_t i) {
    return SYM ? (qb >> 1) + i : tile_order(P, wa, i);
}

// The query block a CTA takes at its qi-th step (blocks in order, strided over the CTAs).
template <bool SYM>
__device__ __forceinline__ int64_t block_at(const Params &P, int64_t qi) {
    return qi;
}

// Label range of query block qb (4 chunks of 32 rows).
__device__ __forceinline__ void qblock_range(const Params &P, int64_t qb, int32_t &lo,
                                             int32_t &hi) {
    if (P.qpos) {  // gathered query rows: no label range (no tile is skipped)
        lo = INT32_MIN;
        hi = INT32_MAX;
        return;
    }
    lo = INT32_MAX;
    hi = INT32_MIN;
    for (int64_t c = qb * 4; c < qb * 4 + 4 && c < P.n_chunks; ++c) {
        lo = min(lo, P.chunk_lo[c]);
        hi = max(hi, P.chunk_hi[c]);
    }
}

template <bool BORUVKA>
__device__ __forceinline__ bool tile_skipped(const Params &P, int64_t t, int32_t qlo, int32_t qhi) {
    if (!BORUVKA) return false;
    return qlo == qhi && P.tile_lo[t] == qlo && P.tile_hi[t] == qlo;
}

template <int M>
__device__ __forceinline__ void list_insert(float (&L)[M], int (&J)[M], float x, int j) {
#pragma unroll
    for (int s = M - 1; s >= 0; --s) {
        const bool here = x < L[s];
        const bool prev = (s > 0) ? (x < L[s > 0 ? s - 1 : 0]) : false;
        if (here) {
            if (prev) {
                L[s] = L[s > 0 ? s - 1 : 0];
                J[s] = J[s > 0 ? s - 1 : 0];
            } else {
                L[s] = x;
                J[s] = j;
            }
        }
    }
}

template <int M, int MODE>
__global__ void __launch_bounds__(THREADS, 1) screen_kernel(const Params P) {
    constexpr bool BORUVKA = MODE == MODE_BORUVKA || MODE == MODE_BORUVKA_SYM;
    constexpr bool SYM = MODE == MODE_BORUVKA_SYM;
    constexpr bool THRESH = MODE == MODE_KNN_THRESHOLD;
    constexpr bool APPEND = BORUVKA || THRESH;  // threshold modes append to per-row buffers
    constexpr bool ROT = !BORUVKA;              // kNN sweeps: rotated shared tile order
    // kNN sweeps: the column terms of each tile are copied into the warp's shared slots, where
    // the list insertions read them (Borůvka screens read them from global memory)
    constexpr bool STAGE = !BORUVKA;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t a_bytes = (uint32_t)P.nbk * KBLOCK_A;
    const uint32_t b_bytes = (uint32_t)P.nbk * KBLOCK_B;
    uint8_t *sA = smem;
    uint8_t *sB = smem + a_bytes;
    float *pbuf = (float *)(sB + (size_t)P.stages * b_bytes);      // [EPI_WARPS][PB_STRIDE]
    float *vstage = pbuf + EPI_WARPS * PB_STRIDE;                    // [EPI_WARPS][32][VSTRIDE]
    uint64_t *bars = (uint64_t *)(vstage + EPI_WARPS * 32 * VSTRIDE);
    uint64_t *full = bars;
    uint64_t *empty = bars + P.stages;
    uint64_t *a_full = bars + 2 * P.stages;
    uint64_t *a_empty = a_full + 1;
    uint64_t *t_full = a_full + 2;   // [2]
    uint64_t *t_empty = a_full + 4;  // [2]
    uint64_t *done = a_full + 6;     // MMA drain on the abort path
    // kNN sweeps: ring of the blocks the producer took and their rotations
    uint64_t *rot_full = a_full + 7;    // [4] the producer published a block
    uint64_t *rot_empty = a_full + 11;  // [4] the MMA warp and every epilogue warp have read it
    uint32_t *tmem_slot = (uint32_t *)(a_full + 15);
    volatile int *abort = (volatile int *)(tmem_slot + 1);
    int32_t *rot_val = (int32_t *)(tmem_slot + 2);  // [4] rotations
    int64_t *rot_blk = (int64_t *)(tmem_slot + 6);  // [4] query blocks (n_qblocks: none left)

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < P.stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(a_full, 1);
        mbar_init(a_empty, 1);
        mbar_init(done, 1);
        for (int b = 0; b < 2; ++b) {
            mbar_init(&t_full[b], 1);
            mbar_init(&t_empty[b], EPI_WARPS);
        }
        for (int r = 0; r < 4; ++r) {
            mbar_init(&rot_full[r], 1);
            mbar_init(&rot_empty[r], EPI_WARPS + 1);
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                         smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        // ---------------- producer: bulk copies of A (per query block) and B tiles ----------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0, a_phase = 0;
            // parity of the last fill of each stage (bit 1 set = a fill was issued)
            uint32_t issued[4] = {0, 0, 0, 0};
            uint32_t a_issued = 0;
            for (uint32_t li = 0; !*abort; ++li) {  // li: this CTA's query step
                int64_t qi = blockIdx.x + (int64_t)li * gridDim.x;
                int32_t rot = 0;
                if (ROT) {
                    // kNN sweeps: blocks come from a global counter, so that CTAs that run faster
                    // take more of them. The block and its rotation of the shared order (the
                    // CTAs' average position: tiles issued so far over the grid) go to the MMA
                    // and epilogue warps through the ring; n_qblocks there ends their loops.
                    qi = (int64_t)atomicAdd(P.cursor + 1, 1ull);
                    if (qi > P.n_qblocks) qi = P.n_qblocks;
                    if (P.n_tiles > WARM && qi < P.n_qblocks) {
                        const unsigned long long all = *(volatile unsigned long long *)P.cursor;
                        rot = (int32_t)((all / gridDim.x) % (unsigned long long)(P.n_tiles - WARM));
                    }
                    const uint32_t rs = li & 3;
                    if (!mbar_wait(&rot_empty[rs], ((li >> 2) & 1) ^ 1, abort, P.error)) break;
                    rot_blk[rs] = qi;
                    rot_val[rs] = rot;
                    mbar_arrive(&rot_full[rs]);
                }
                if (qi >= P.n_qblocks * P.splits) break;
                const int64_t qb = block_at<SYM>(P, qi / P.splits);
                const int64_t part = qi % P.splits;
                if (!mbar_wait(a_empty, a_phase ^ 1, abort, P.error)) break;
                a_issued = 2u | a_phase;
                a_phase ^= 1;
                mbar_expect_tx(a_full, a_bytes);
                const uint8_t *asrc = P.xq + (uint64_t)(qb >> 1) * (uint64_t)b_bytes +
                                      (uint64_t)(qb & 1) * KBLOCK_A;
                for (int kb = 0; kb < P.nbk; ++kb)
                    bulk_g2s(sA + kb * KBLOCK_A, asrc + (uint64_t)kb * KBLOCK_B, KBLOCK_A, a_full);
                int32_t qlo = 0, qhi = 0;
                if (BORUVKA) qblock_range(P, qb, qlo, qhi);
                const int64_t wa = window_start(P, qb);
                const int64_t nvis = vis_count<SYM>(P, qb);
                const int64_t i_hi = (part + 1) * nvis / P.splits;
                for (int64_t i = part * nvis / P.splits; i < i_hi; ++i) {
                    const int64_t t = ROT ? (int64_t)knn_tile((int32_t)P.n_tiles, (int32_t)wa, rot, (int32_t)i)
                                          : vis_tile<SYM>(P, qb, wa, i);
                    if (tile_skipped<BORUVKA>(P, t, qlo, qhi)) continue;
                    if (!mbar_wait(&empty[stage], phase ^ 1, abort, P.error)) break;
                    issued[stage] = 2u | phase;
                    mbar_expect_tx(&full[stage], b_bytes);
                    const uint8_t *bsrc = P.xt + (uint64_t)t * (uint64_t)b_bytes;
                    uint8_t *bdst = sB + (size_t)stage * b_bytes;
                    for (int kb = 0; kb < P.nbk; ++kb)
                        bulk_g2s(bdst + kb * KBLOCK_B, bsrc + (uint64_t)kb * KBLOCK_B, KBLOCK_B,
                                 &full[stage]);
                    if (++stage == P.stages) {
                        stage = 0;
                        phase ^= 1;
                    }
                    if (ROT) atomicAdd(P.cursor, 1ull);
                }
            }
            if (*abort) {
                // let every copy this thread issued land before the CTA exits
                for (int s2 = 0; s2 < P.stages; ++s2)
                    if (issued[s2]) {
                        for (uint32_t it = 0; it < WAIT_POLLS; ++it)
                            if (mbar_try_wait(&full[s2], issued[s2] & 1u)) break;
                    }
                if (a_issued)
                    for (uint32_t it = 0; it < WAIT_POLLS; ++it)
                        if (mbar_try_wait(a_full, a_issued & 1u)) break;
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer: one thread -------------------------------------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0, a_phase = 0;
            uint32_t tcount = 0, a_commits = 0;
            const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
            for (uint32_t li = 0; !*abort; ++li) {
                int64_t qi = blockIdx.x + (int64_t)li * gridDim.x;
                if (ROT) {  // kNN sweeps: the block the producer took
                    const uint32_t rs = li & 3;
                    if (!mbar_wait(&rot_full[rs], (li >> 2) & 1, abort, P.error)) break;
                    qi = *(volatile int64_t *)&rot_blk[rs];
                    mbar_arrive(&rot_empty[rs]);
                }
                if (qi >= P.n_qblocks * P.splits) break;
                const int64_t qb = block_at<SYM>(P, qi / P.splits);
                const int64_t part = qi % P.splits;
                if (!mbar_wait(a_full, a_phase, abort, P.error)) break;
                a_phase ^= 1;
                fence_after();
                int32_t qlo = 0, qhi = 0;
                if (BORUVKA) qblock_range(P, qb, qlo, qhi);
                const int64_t wa = window_start(P, qb);
                const int64_t nvis = vis_count<SYM>(P, qb);
                const int64_t i_hi = (part + 1) * nvis / P.splits;
                bool ok = true;
                for (int64_t i = part * nvis / P.splits; i < i_hi; ++i) {
                    const int64_t t = vis_tile<SYM>(P, qb, wa, i);
                    if (tile_skipped<BORUVKA>(P, t, qlo, qhi)) continue;
                    const uint32_t b = tcount & 1, tp = (tcount >> 1) & 1;
                    if (!mbar_wait(&t_empty[b], tp ^ 1, abort, P.error)) { ok = false; break; }
                    fence_after();
                    if (!mbar_wait(&full[stage], phase, abort, P.error)) { ok = false; break; }
                    fence_after();
                    const uint32_t d_tmem = tmem_base + b * BN;
                    const uint32_t bstage = b_base + (uint32_t)stage * b_bytes;
                    for (int kb = 0; kb < P.kblocks; ++kb) {
#pragma unroll
                        for (int ks = 0; ks < 4; ++ks) {
                            const uint64_t ad = desc_sw128(a_base + kb * KBLOCK_A + ks * 32);
                            const uint64_t bd = desc_sw128(bstage + kb * KBLOCK_B + ks * 32);
                            mma_16bit(d_tmem, ad, bd, P.idesc, (kb | ks) != 0);
                        }
                        if (P.split) {
                            // lo x hi and hi x lo (blocks kblocks + kb hold the lo parts)
                            const uint32_t lo = (uint32_t)(P.kblocks + kb);
#pragma unroll
                            for (int ks = 0; ks < 4; ++ks) {
                                mma_16bit(d_tmem, desc_sw128(a_base + lo * KBLOCK_A + ks * 32),
                                          desc_sw128(bstage + kb * KBLOCK_B + ks * 32), P.idesc, 1u);
                                mma_16bit(d_tmem, desc_sw128(a_base + kb * KBLOCK_A + ks * 32),
                                          desc_sw128(bstage + lo * KBLOCK_B + ks * 32), P.idesc, 1u);
                            }
                        }
                    }
                    mma_commit(&empty[stage]);
                    mma_commit(&t_full[b]);
                    if (++stage == P.stages) {
                        stage = 0;
                        phase ^= 1;
                    }
                    ++tcount;
                }
                mma_commit(a_empty);
                ++a_commits;
                if (!ok) break;
            }
            atomicAdd(reinterpret_cast<unsigned long long *>(P.error + 2),
                      (unsigned long long)tcount);
            // wait until every issued MMA has completed before TMEM can be released
            mma_commit(done);
            for (uint32_t it = 0; it < WAIT_POLLS; ++it)
                if (mbar_try_wait(done, 0)) break;
            if (a_commits)
                for (uint32_t it = 0; it < WAIT_POLLS; ++it)
                    if (mbar_try_wait(a_empty, (a_commits - 1) & 1u)) break;
        }
    } else {
        // ---------------- epilogue: two threads per query row ---------------------------------
        // Warps 2..9: warp w reads TMEM lane quadrant w % 4 (hardware rule) and handles one half
        // of every 256-column tile; the two threads of a row keep separate top-M lists.
        const int ew = warp - 2;              // 0..7
        const int quad = warp & 3;            // TMEM lane quadrant of this warp
        const int half = ew >> 2;             // column half of each tile
        const int row_local = quad * 32 + lane;
        float *my_v = vstage + (ew * 32 + lane) * VSTRIDE;
        float *my_pb = pbuf + ew * PB_STRIDE;
        uint32_t tcount = 0;
        for (uint32_t li = 0; !*abort; ++li) {
            int64_t qi = blockIdx.x + (int64_t)li * gridDim.x;
            int32_t rot = 0;
            if (ROT) {  // kNN sweeps: the block the producer took and its rotation
                const uint32_t rs = li & 3;
                if (!mbar_wait(&rot_full[rs], (li >> 2) & 1, abort, P.error)) break;
                qi = *(volatile int64_t *)&rot_blk[rs];
                rot = *(volatile int32_t *)&rot_val[rs];
                __syncwarp();
                if (lane == 0) mbar_arrive(&rot_empty[rs]);
            }
            if (qi >= P.n_qblocks * P.splits) break;
            const int64_t qb = block_at<SYM>(P, qi / P.splits);
            const int64_t part = qi % P.splits;
            // the debug entry point dumps query block 0 against tile 0 (its first tile)
            const bool debug = P.debug_tile != nullptr && qb == 0;
            const int64_t row = qb * BM + row_local;  // query row
            const bool valid = row < P.nq;
            const int64_t self = valid && P.qpos ? (int64_t)P.qpos[row] : row;
            const float p_i = valid ? P.pq[row] : 0.0f;
            const float m_i = valid ? P.mq[row] : 0.0f;
            const float ps_i = P.one_minus_cb * p_i - P.abs_c;
            const float cm_i = P.c_a * m_i;
            float core_i = 0.0f;
            int32_t lab_i = -1;
            if (BORUVKA && valid) {
                core_i = P.core[self] * P.s2;
                lab_i = P.label[self];
            }
            // kNN threshold mode: a fixed upper bound of the row's k-th distance (scaled); a row
            // without one overflows its buffer at once and is resolved exactly
            const float tau = THRESH && valid ? P.qthr[row] * P.s2 : CUSCAN_INF;
            const bool tau_ok = !THRESH || tau < CUSCAN_INF;
            // kNN: the row's M smallest lower bounds. Borůvka: an upper bound U on the row's
            // cheapest cross-component edge plus the shared bound of its component; pairs whose
            // lower bound does not exceed min(U, component bound) are appended for re-ranking.
            // kNN threshold: every pair whose lower bound does not exceed tau is appended.
            constexpr int LM = APPEND ? 1 : M;
            float L[LM];
            int J[LM];
#pragma unroll
            for (int s2 = 0; s2 < LM; ++s2) {
                L[s2] = CUSCAN_INF;
                J[s2] = -1;
            }
            float U = CUSCAN_INF, published = CUSCAN_INF;
            float lb_all = CUSCAN_INF;  // one-sided Borůvka: min chunk bound over cross chunks
            int cnt = 0;
            int32_t qlo = 0, qhi = 0;
            if (BORUVKA) qblock_range(P, qb, qlo, qhi);
            const int64_t wa = window_start(P, qb);
            const int64_t nvis = vis_count<SYM>(P, qb);
            // this work item's part [i_lo, i_hi) of the block's tile order
            const int64_t i_lo = part * nvis / P.splits, i_hi = (part + 1) * nvis / P.splits;
            // symmetric mode: the warp's 32 rows summarised for the column-side block test
            float psmin_w = CUSCAN_INF, cmmax_w = 0.0f, coremin_w = CUSCAN_INF;
            if (SYM) {
                psmin_w = warp_min_f(valid ? ps_i : CUSCAN_INF);
                cmmax_w = warp_max_f(valid ? cm_i : 0.0f);
                coremin_w = warp_min_f(valid ? core_i : CUSCAN_INF);
            }
            auto tile_at = [&](int64_t i) -> int64_t {
                return ROT ? (int64_t)knn_tile((int32_t)P.n_tiles, (int32_t)wa, rot, (int32_t)i)
                           : vis_tile<SYM>(P, qb, wa, i);
            };
            // next visited position i (>= i0) in this block's tile order, and its tile t_at
            int64_t t_at = 0;
            auto next_index = [&](int64_t i) -> int64_t {
                for (; i < i_hi; ++i) {
                    t_at = tile_at(i);
                    if (!tile_skipped<BORUVKA>(P, t_at, qlo, qhi)) break;
                }
                return i;
            };
            // per-tile column data, fetched one tile ahead: the chunk minima of this warp's four
            // chunks (the per-column terms are read where a chunk is tested pair by pair)
            float4 pre_k01 = make_float4(0, 0, 0, 0), pre_k23 = make_float4(0, 0, 0, 0);
            int32_t pre_ch = -2;
            float pre_mt = 0.0f, pre_cb = CUSCAN_INF;
            float4 pre_t = make_float4(0, 0, 0, 0);  // symmetric mode: column row bounds (raw)
            auto prefetch = [&](int64_t t, uint32_t slot) {
                const int64_t col = t * BN + half * HALF + lane * 4;
                pre_k01 = P.cmin[t * 4 + half * 2];
                pre_k23 = P.cmin[t * 4 + half * 2 + 1];
                pre_mt = P.tile_mmax[t];
                if (STAGE) {  // straight into the tile's shared slots (no registers)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                                     smem_u32(my_pb + slot * HALF + lane * 4)),
                                 "l"(P.colp + col)
                                 : "memory");
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                                     smem_u32(my_pb + (2 + slot) * HALF + lane * 4)),
                                 "l"(P.mnorm + col)
                                 : "memory");
                }
                if (BORUVKA) {
                    const int64_t ch = t * 8 + half * 4 + (lane & 3);
                    pre_ch = -2;
                    if (lane < 8 && ch < P.n_chunks) pre_ch = lane < 4 ? P.chunk_lo[ch] : P.chunk_hi[ch];
                    pre_cb = valid ? __uint_as_float(*(volatile uint32_t *)&P.cbound[lab_i])
                                   : CUSCAN_INF;
                    if (SYM) {
                        const volatile uint32_t *ur = P.urow;
                        pre_t.x = col + 0 < P.n ? __uint_as_float(ur[col + 0]) : -CUSCAN_INF;
                        pre_t.y = col + 1 < P.n ? __uint_as_float(ur[col + 1]) : -CUSCAN_INF;
                        pre_t.z = col + 2 < P.n ? __uint_as_float(ur[col + 2]) : -CUSCAN_INF;
                        pre_t.w = col + 3 < P.n ? __uint_as_float(ur[col + 3]) : -CUSCAN_INF;
                    }
                }
            };
            int64_t ti = next_index(i_lo);
            if (ti < i_hi) prefetch(t_at, tcount & 1);
            bool ok = true;
            while (ti < i_hi) {
                const int64_t t = t_at;
                const int64_t ti_next = next_index(ti + 1);
                const uint32_t b = tcount & 1, tp = (tcount >> 1) & 1;
                // this warp's columns: scaled norms pb, norms mb and (Borůvka) scaled cores cb,
                // and (min pb, min cb) of each 32-column chunk
                const int64_t col0 = t * BN + half * HALF;
                const float *pb = STAGE ? my_pb + b * HALF : P.colp + col0;
                const float *mb = STAGE ? my_pb + (2 + b) * HALF : P.mnorm + col0;
                const float *cb = BORUVKA ? P.colc + col0 : nullptr;
                if (STAGE) {  // this tile's column terms, copied one tile ahead
                    asm volatile("cp.async.wait_all;" ::: "memory");
                    __syncwarp();
                }
                const float2 chunk_min[4] = {make_float2(pre_k01.x, pre_k01.y),
                                             make_float2(pre_k01.z, pre_k01.w),
                                             make_float2(pre_k23.x, pre_k23.y),
                                             make_float2(pre_k23.z, pre_k23.w)};
                // symmetric mode: the largest column row bound of each chunk (scaled)
                float chunk_tmax[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                if (SYM) {
                    float tm = fmaxf(fmaxf(pre_t.x, pre_t.y), fmaxf(pre_t.z, pre_t.w)) * P.s2;
#pragma unroll
                    for (int o = 1; o < 8; o <<= 1)
                        tm = fmaxf(tm, __shfl_xor_sync(0xffffffffu, tm, o));
#pragma unroll
                    for (int c = 0; c < 4; ++c) chunk_tmax[c] = __shfl_sync(0xffffffffu, tm, 8 * c);
                }
                const float mt = pre_mt;
                const int32_t ch_word = pre_ch;
                const float comp_bound = pre_cb * P.s2;
                __syncwarp();
                if (ti_next < i_hi) prefetch(t_at, b ^ 1);
                if (!mbar_wait(&t_full[b], tp, abort, P.error)) { ok = false; break; }
                fence_after();
                const uint32_t taddr =
                    tmem_base + ((uint32_t)(quad * 32) << 16) + b * BN + half * HALF;
                // Phase 1: the largest dot product of each 32-column chunk, from the TMEM loads
                // themselves (tcgen05.ld.red); two chunks per wait, as the kNN lists leave room
                // for two 32-column loads in flight.
                // Phase 2: one coarse test per chunk against this tile's thresholds and one warp
                // vote per tile; the chunks that pass are read again from TMEM (the buffer is
                // released only after this tile) and tested element by element.
                float vmax[HALF / 32];
#pragma unroll
                for (int c = 0; c < HALF / 32; c += 2) {
                    uint32_t rA[32], rB[32];
                    tmem_ld32_max_issue(taddr + c * 32, rA, vmax[c]);
                    tmem_ld32_max_issue(taddr + (c + 1) * 32, rB, vmax[c + 1]);
                    tmem_ld_wait(rA);
                    tmem_ld_wait(rB);
                    asm volatile("" : "+f"(vmax[c]), "+f"(vmax[c + 1]));
                    if (debug && t == 0) {
#pragma unroll
                        for (int e = 0; e < 32; ++e) {
                            P.debug_tile[row_local * BN + half * HALF + c * 32 + e] = __uint_as_float(rA[e]);
                            P.debug_tile[row_local * BN + half * HALF + (c + 1) * 32 + e] = __uint_as_float(rB[e]);
                        }
                        if (P.debug_chunk) {
                            P.debug_chunk[row_local * 8 + half * 4 + c] = vmax[c];
                            P.debug_chunk[row_local * 8 + half * 4 + c + 1] = vmax[c + 1];
                        }
                    }
                }
                // Thresholds moved to the scale of F = (1 - C_B) p_j - 2 dot with the tile's
                // largest norm, then widened by a few ulps so that no pair whose exact-path
                // bound would pass is filtered out. For Borůvka the core condition
                // core_j < T rides along as max(F, core_j + (thr2 - T)). The element path
                // recomputes them after it lowers U or the list bound; a stale (larger)
                // threshold only admits more pairs to the exact test.
                float T = 0.0f, dlt = 0.0f, thr_fast = 0.0f;
                auto thresholds = [&]() {
                    T = BORUVKA ? fminf(U, comp_bound) : THRESH ? tau : L[LM - 1];
                    const float base = T - ps_i + cm_i * mt;
                    const float thr2 = base + 0x1p-21f * (fabsf(T) + ps_i + cm_i * mt);
                    dlt = thr2 - T;
                    thr_fast = thr2 + 0x1p-20f * (fabsf(thr2) + fabsf(T));
                };
                thresholds();
                // Coarse test of each chunk: with the chunk's smallest scaled norm and core,
                // fmaf(-2, max v, min pb) is below (or equal to) every element's
                // fmaf(-2, v_j, pb_j) and min core + dlt bounds the core term, because rounding
                // is monotonic.
                unsigned hitbits = 0, mixbits = 0;
                {
                    const bool row_on = valid && tau_ok && (!BORUVKA || core_i <= T);
#pragma unroll
                    for (int c = 0; c < HALF / 32; ++c) {
                        int32_t clo = 0, chi = 0;
                        if (BORUVKA) {
                            clo = __shfl_sync(0xffffffffu, ch_word, c);
                            chi = __shfl_sync(0xffffffffu, ch_word, 4 + c);
                        }
                        const bool cross = !BORUVKA || (clo != -2 && !(clo == lab_i && chi == lab_i));
                        const bool on = row_on && cross;
                        const float2 cmin = chunk_min[c];
                        float flb = fmaf(-2.0f, vmax[c], cmin.x);
                        if (MODE == MODE_BORUVKA && cross) {
                            if (clo <= lab_i && lab_i <= chi) {
                                // the chunk also holds rows of the row's own component: its
                                // bound may come from those, so it is taken pair by pair below
                                mixbits |= 1u << c;
                            } else {
                                // below every pair of the chunk: mb <= mt, dot <= vmax,
                                // pb >= min pb, core_j >= min core, and fmaf/add rounding is
                                // monotonic
                                const float lbc = fmaf(-cm_i, mt, flb + ps_i);
                                lb_all = fminf(lb_all, fmaxf(fmaxf(lbc, core_i), cmin.y));
                            }
                        }
                        if (BORUVKA) flb = fmaxf(flb, cmin.y + dlt);
                        if (on && flb < thr_fast) hitbits |= 1u << c;
                    }
                }
                const unsigned warp_bits = __reduce_or_sync(0xffffffffu, hitbits);
                // Symmetric mode, tiles after the block's own: the pairs of this block are also
                // the pairs of the tile's rows. Block test: with the warp's smallest scaled norm
                // and core and largest C_A m, the chunk's smallest scaled norm and core and the
                // block's largest dot product, fmaf/add rounding being monotonic, wl is below
                // every pair's exact-path bound max(lb, core_i, core_j); only blocks where it
                // reaches a column's row bound are tested pair by pair.
                unsigned colbits = 0;
                if (SYM && t > (qb >> 1)) {
#pragma unroll
                    for (int c = 0; c < HALF / 32; ++c) {
                        const float vb = warp_max_f(vmax[c]);
                        const float2 cmn = chunk_min[c];
                        const float lbb = fmaf(-cmmax_w, mt, fmaf(-2.0f, vb, cmn.x) + psmin_w);
                        const float wl = fmaxf(fmaxf(lbb, coremin_w), cmn.y);
                        if (wl <= chunk_tmax[c]) colbits |= 1u << c;
                    }
                }
                for (int c = 0; colbits != 0 && c < HALF / 32; ++c) {
                    if (!((colbits >> c) & 1u)) continue;
                    uint32_t rc2[32];
                    tmem_ld32_issue(taddr + c * 32, rc2);
                    // lane e refreshes column e's row bound with its component's current bound
                    // (rows of components that found edges elsewhere get tight at once)
                    const int64_t j0 = t * BN + half * HALF + c * 32;
                    int32_t lab_l = -1;
                    float t_l = -CUSCAN_INF;
                    if (j0 + lane < P.n) {
                        lab_l = P.label[j0 + lane];
                        const uint32_t cbv = *(volatile uint32_t *)&P.cbound[lab_l];
                        const uint32_t old = atomicMin(&P.urow[j0 + lane], cbv);
                        t_l = __uint_as_float(old < cbv ? old : cbv) * P.s2;
                    }
                    tmem_ld_wait(rc2);
#pragma unroll
                    for (int e = 0; e < 32; ++e) {
                        const float tj = __shfl_sync(0xffffffffu, t_l, e);
                        const int32_t lab_j = __shfl_sync(0xffffffffu, lab_l, e);
                        const int col = c * 32 + e;
                        const int64_t j = j0 + e;
                        if (j >= P.n) break;  // the same for every lane
                        const float lb = fmaf(-cm_i, mb[col],
                                              fmaf(-2.0f, __uint_as_float(rc2[e]), pb[col]) + ps_i);
                        const float cj = cb[col];
                        const float lbw = fmaxf(fmaxf(lb, core_i), cj);
                        const bool pv = valid && lab_j != lab_i && lbw <= tj;
                        const float eps2 =
                            2.0f * fmaf(cm_i, mb[col], P.c_b * (ps_i + pb[col]) * 1.001f) +
                            4.0f * P.abs_c;
                        const float ubr = lb + eps2;
                        const float ub =
                            fmaxf(fmaxf(ubr + 0x1p-20f * (fabsf(ubr) + eps2), core_i), cj);
                        // the block's best upper bound for this column's row: a pair above
                        // it cannot be the row's cheapest edge
                        const float tmin = warp_min_f(pv ? ub : CUSCAN_INF);
                        if (pv && lbw <= tmin) {
                            const int slot = atomicAdd(&P.colcnt[j], 1);
                            if (slot < P.capc) P.colbuf[j * P.capc + slot] = (int32_t)row;
                        }
                        if (lane == 0 && tmin < CUSCAN_INF) {
                            const uint32_t ub_raw = __float_as_uint(__fmul_ru(tmin, P.inv_s2));
                            atomicMin(&P.urow[j], ub_raw);
                            atomicMin(&P.cbound[lab_j], ub_raw);
                        }
                    }
                    __syncwarp();
                }
                for (int c = 0; warp_bits != 0 && c < HALF / 32; ++c) {
                    if (!((warp_bits >> c) & 1u)) continue;
                    uint32_t rc_[32];
                    tmem_ld32_issue(taddr + c * 32, rc_);
                    tmem_ld_wait(rc_);
                    float v[32];
#pragma unroll
                    for (int e = 0; e < 32; ++e) v[e] = __uint_as_float(rc_[e]);
                    const bool any_hit = (hitbits >> c) & 1u;
                    {

                        unsigned hits = 0;
                        if (any_hit) {
                            const float4 *pc = reinterpret_cast<const float4 *>(pb + c * 32);
                            const float4 *cc = reinterpret_cast<const float4 *>(cb + c * 32);
#pragma unroll
                            for (int q = 0; q < 8; ++q) {
                                const float4 pq = pc[q];
                                float f0 = fmaf(-2.0f, v[4 * q + 0], pq.x);
                                float f1 = fmaf(-2.0f, v[4 * q + 1], pq.y);
                                float f2 = fmaf(-2.0f, v[4 * q + 2], pq.z);
                                float f3 = fmaf(-2.0f, v[4 * q + 3], pq.w);
                                if (BORUVKA) {
                                    // core_j <= T is necessary for an append
                                    const float4 cq = cc[q];
                                    f0 = fmaxf(f0, cq.x + dlt);
                                    f1 = fmaxf(f1, cq.y + dlt);
                                    f2 = fmaxf(f2, cq.z + dlt);
                                    f3 = fmaxf(f3, cq.w + dlt);
                                }
                                hits |= (f0 < thr_fast ? 1u : 0u) << (4 * q + 0);
                                hits |= (f1 < thr_fast ? 1u : 0u) << (4 * q + 1);
                                hits |= (f2 < thr_fast ? 1u : 0u) << (4 * q + 2);
                                hits |= (f3 < thr_fast ? 1u : 0u) << (4 * q + 3);
                            }
#pragma unroll
                            for (int q = 0; q < 8; ++q)
                                reinterpret_cast<float4 *>(my_v)[q] =
                                    make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                        }
                        int32_t clo = 0, chi = 0;
                        if (BORUVKA) {
                            clo = __shfl_sync(0xffffffffu, ch_word, c);
                            chi = __shfl_sync(0xffffffffu, ch_word, 4 + c);
                        }
                        const bool uniform_other = BORUVKA && clo == chi && clo != lab_i;
                        while (hits) {
                            const int e = __ffs(hits) - 1;
                            hits &= hits - 1;
                            const int col = c * 32 + e;
                            const int64_t j = t * BN + half * HALF + col;
                            if (j >= P.n) continue;
                            if (!BORUVKA && j == self) continue;
                            const float dot = my_v[e];
                            // exact lower bound for this pair (per-column norm instead of the
                            // tile maximum); pb holds (1 - C_B) p_j
                            float lb = fmaf(-cm_i, mb[col], fmaf(-2.0f, dot, pb[col]) + ps_i);
                            if constexpr (BORUVKA) {
                                if (!uniform_other && P.label[j] == lab_i) continue;
                                const float cj = cb[col];
                                const float lbw = fmaxf(fmaxf(lb, core_i), cj);
                                const float Tn = fminf(U, comp_bound);
                                if (lbw <= Tn) {
                                    // split work items share the row's slots
                                    const int slot = P.splits > 1
                                        ? atomicAdd(&P.rowcnt[row * 2 + half], 1) : cnt;
                                    if (slot < P.cap) P.cand_ids[(row * 2 + half) * P.cap + slot] = (int32_t)j;
                                    ++cnt;
                                    // upper bound of this pair's weight: D + eps = L + 2 eps
                                    const float eps2 =
                                        2.0f * fmaf(cm_i, mb[col], P.c_b * (ps_i + pb[col]) * 1.001f) +
                                        4.0f * P.abs_c;
                                    const float ubr = lb + eps2;
                                    const float ub = fmaxf(fmaxf(ubr + 0x1p-20f * (fabsf(ubr) + eps2), core_i), cj);
                                    U = fminf(U, ub);
                                }
                            } else if constexpr (THRESH) {
                                if (lb <= tau) {
                                    if (cnt < P.cap) P.cand_ids[(row * 2 + half) * P.cap + cnt] = (int32_t)j;
                                    ++cnt;
                                }
                            } else {
                                if (lb < L[LM - 1]) list_insert<LM>(L, J, lb, (int)j);
                            }
                        }
                        __syncwarp();
                        thresholds();
                    }
                }
                // one-sided Borůvka: row bounds over the chunks shared with the own component,
                // other components' pairs only (at most a couple of chunks per component)
                if (MODE == MODE_BORUVKA) {
                    const unsigned wmix = __reduce_or_sync(0xffffffffu, mixbits);
                    for (int c = 0; wmix != 0 && c < HALF / 32; ++c) {
                        if (!((wmix >> c) & 1u)) continue;
                        uint32_t rm[32];
                        tmem_ld32_issue(taddr + c * 32, rm);
                        tmem_ld_wait(rm);
                        if ((mixbits >> c) & 1u) {
                            const int64_t j0 = t * BN + half * HALF + c * 32;
                            // fully unrolled: rm stays in registers
#pragma unroll
                            for (int e = 0; e < 32; ++e) {
                                const int col = c * 32 + e;
                                if (j0 + e >= P.n || P.label[j0 + e] == lab_i) continue;
                                const float lb = fmaf(-cm_i, mb[col],
                                                      fmaf(-2.0f, __uint_as_float(rm[e]), pb[col]) + ps_i);
                                lb_all = fminf(lb_all, fmaxf(fmaxf(lb, core_i), cb[col]));
                            }
                        }
                        __syncwarp();
                    }
                }
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&t_empty[b]);
                if (BORUVKA && valid && U < published) {
                    // raw units, rounded up so that the bound stays an upper bound
                    const uint32_t u_raw = __float_as_uint(__fmul_ru(U, P.inv_s2));
                    atomicMin(&P.cbound[lab_i], u_raw);
                    if (SYM) atomicMin(&P.urow[row], u_raw);
                    published = U;
                }
                ++tcount;
                ti = ti_next;
            }
            if (!ok) break;
            if (APPEND) {
                // each half of a row appends into its own slot range [(2 row + half) * cap, +cap)
                if (valid && P.splits == 1) P.rowcnt[row * 2 + half] = tau_ok ? cnt : P.cap + 1;
                if (MODE == MODE_BORUVKA && valid && P.rowlb) {
                    const float lbr = __fmul_rd(lb_all, P.inv_s2);
                    if (P.splits == 1) {
                        P.rowlb[row * 2 + half] = lbr;
                    } else {
                        // the least over the block's parts; pair weights are >= 0, so a bound
                        // below 0 is worth 0 and the bounds compare as unsigned bit patterns
                        atomicMin(reinterpret_cast<unsigned int *>(P.rowlb) + row * 2 + half,
                                  __float_as_uint(lbr > 0.0f ? lbr : 0.0f));
                    }
                }
            } else if (valid) {
                const int64_t base_at = row * (2 * M) + half * M;
#pragma unroll
                for (int s2 = 0; s2 < LM; ++s2) {
                    P.cand_ids[base_at + s2] = J[s2];
                    // raw units, rounded down so that the bound stays a lower bound
                    P.cand_lb[base_at + s2] = __fmul_rd(L[s2], P.inv_s2);
                }
            }
        }
        // copies of column terms still in flight (a loop left early) land before the CTA exits
        if (STAGE) asm volatile("cp.async.wait_all;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem_base)
                     : "memory");
    }
}

// Exact squared distance (the reference's order) from the warp's query row q_s (shared) to the
// candidate row j held by this lane (j < 0: none, returns +inf). The warp first copies the 32
// candidate rows into its shared staging area row by row, each row read with consecutive
// addresses, then every lane sums its own row sequentially; the row stride d + 1 keeps the
// lanes on distinct banks.
__device__ __forceinline__ float staged_d2(const float *__restrict__ x, int d,
                                           const float *q_s, int32_t j, float *rows_s,
                                           int lane) {
    // asynchronous 4-byte copies: every row's loads are in flight at once
    for (int r = 0; r < 32; ++r) {
        const int32_t jr = __shfl_sync(0xffffffffu, j, r);
        if (jr < 0) continue;
        const float *src = x + (int64_t)jr * d;
        float *dst = rows_s + r * (d + 1);
        for (int f = lane; f < d; f += 32)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst + f)),
                         "l"(src + f)
                         : "memory");
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
    float acc = CUSCAN_INF;
    if (j >= 0) {
        const float *row = rows_s + lane * (d + 1);
        acc = 0.0f;
        for (int f = 0; f < d; ++f) {
            const float t = q_s[f] - row[f];
            acc = __fmaf_rn(t, t, acc);
        }
    }
    __syncwarp();
    return acc;
}

// Shared floats one warp of a re-rank kernel stages: 32 candidate rows and the query row.
__host__ __device__ constexpr int64_t rerank_warp_floats(int d) { return 32 * (d + 1) + d; }
constexpr int RERANK_WARPS = 4;

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u < v ? u : v;
    }
    return v;
}

// Lower bound of every pair a row's two lists left out: a full list rejected or evicted only
// pairs whose bound is >= its M-th entry; a list that is not full kept every pair it saw.
template <int M>
__device__ __forceinline__ float unseen_bound(const int32_t *ids, const float *lb) {
    float b = CUSCAN_INF;
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (ids[h * M + M - 1] >= 0) b = fminf(b, lb[h * M + M - 1]);
    return b;
}

// kNN re-rank: one warp per row, exact distances of the 2M candidates, top-k by (d, id).
// x and the candidates are in sorted positions; perm maps a position to its original row, which
// is the id the reference orders ties by and the row the output goes to.
template <int M>
__global__ void rerank_knn_kernel(const float *__restrict__ x, const int32_t *__restrict__ perm,
                                  int64_t n, int d, int k, const int32_t *__restrict__ cand_ids,
                                  const float *__restrict__ cand_lb, int32_t *__restrict__ ids,
                                  float *__restrict__ dist, int32_t *__restrict__ fallback,
                                  float *__restrict__ fallback_thr,
                                  int *__restrict__ fallback_count) {
    extern __shared__ float rerank_smem[];
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    float *q_s = rerank_smem + (threadIdx.x >> 5) * rerank_warp_floats(d);
    float *rows_s = q_s + d;
    for (int f = lane; f < d; f += 32) q_s[f] = x[row * d + f];
    __syncwarp();
    constexpr int W = 2 * M;  // two lists of M per row (one per column half)
    // Each half's list is sorted by lower bound. The first round takes the F smallest bounds of
    // both lists (lanes 0..15: half 0, lanes 16..31: half 1); the rest, R per half, run in a
    // second round only when the smaller of their two first bounds does not exceed the k-th
    // distance of the first round, an upper bound of the final k-th distance: a candidate whose
    // lower bound exceeds it cannot be among the row's k nearest.
    constexpr int F = M < 16 ? M : 16;
    constexpr int R = M - F;
    static_assert(R <= 16, "two rounds of at most 16 candidates per half");
    constexpr int PER = 2;
    unsigned long long key[PER] = {~0ull, ~0ull};
    auto round_key = [&](int first, int count) -> unsigned long long {
        const int h = lane >> 4, o = lane & 15;
        const int32_t j = o < count ? cand_ids[row * W + h * M + first + o] : -1;
        const float dd = staged_d2(x, d, q_s, j, rows_s, lane);
        return j < 0 ? ~0ull : ((unsigned long long)__float_as_uint(dd) << 32) | (uint32_t)perm[j];
    };
    key[0] = round_key(0, F);
    if (R > 0) {
        // k-th smallest key of the first round (all keys distinct: the halves hold disjoint
        // columns)
        unsigned long long a = key[0], kth = ~0ull;
        for (int r = 0; r < k; ++r) {
            kth = warp_min_u64(a);
            if (kth == ~0ull) break;
            if (a == kth) a = ~0ull;
        }
        const float dk0 = kth == ~0ull ? CUSCAN_INF : __uint_as_float((uint32_t)(kth >> 32));
        float lb_rest = CUSCAN_INF;
#pragma unroll
        for (int h = 0; h < 2; ++h)
            if (cand_ids[row * W + h * M + F] >= 0) lb_rest = fminf(lb_rest, cand_lb[row * W + h * M + F]);
        if (!(lb_rest > dk0)) key[1] = round_key(F, R);
    }
    const int64_t orow = perm[row];
    float dk = CUSCAN_INF;
    for (int r = 0; r < k; ++r) {
        unsigned long long mine = key[0];
#pragma unroll
        for (int q = 1; q < PER; ++q) mine = key[q] < mine ? key[q] : mine;
        const unsigned long long best = warp_min_u64(mine);
#pragma unroll
        for (int q = 0; q < PER; ++q)
            if (key[q] == best) key[q] = ~0ull;
        if (best == ~0ull) {
            if (lane == 0) {
                ids[orow * k + r] = (int32_t)n;
                dist[orow * k + r] = CUSCAN_INF;
            }
            dk = CUSCAN_INF;
        } else {
            dk = __uint_as_float((uint32_t)(best >> 32));
            if (lane == 0) {
                ids[orow * k + r] = (int32_t)(uint32_t)best;
                dist[orow * k + r] = dk;
            }
        }
    }
    // every pair outside a full list has a lower bound >= that list's M-th bound; an
    // inconclusive row is listed by position with dk, an upper bound of its k-th distance
    const float bound = unseen_bound<M>(cand_ids + row * W, cand_lb + row * W);
    if (lane == 0 && !(bound > dk)) {
        const int at = atomicAdd(fallback_count, 1);
        fallback[at] = (int32_t)row;
        fallback_thr[at] = dk;
    }
}

// kNN re-rank of the threshold screen: query q (position qpos[q]) holds every pair whose lower
// bound does not exceed an upper bound of its k-th distance, so the exact top k of its appended
// candidates by (d, original id) is its exact kNN row. A buffer that overflowed (or a row with
// fewer than k candidates) sends the row's original index to the exact f32 sweep.
__global__ void rerank_knn_threshold_kernel(const float *__restrict__ x,
                                            const int32_t *__restrict__ perm,
                                            const int32_t *__restrict__ qpos, int64_t nq, int d,
                                            int k, const int32_t *__restrict__ cand_ids,
                                            const int32_t *__restrict__ rowcnt, int cap,
                                            int32_t *__restrict__ ids, float *__restrict__ dist,
                                            int32_t *__restrict__ fallback,
                                            int *__restrict__ fallback_count) {
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= nq) return;
    constexpr int PER = 2 * KNN_CAP / 32;
    const int64_t pos = qpos[q];
    const int64_t orow = perm[pos];
    const int c0 = rowcnt[q * 2], c1 = rowcnt[q * 2 + 1];
    if (c0 > cap || c1 > cap || c0 + c1 < k) {
        if (lane == 0) fallback[atomicAdd(fallback_count, 1)] = (int32_t)orow;
        return;
    }
    extern __shared__ float rerank_smem[];
    float *q_s = rerank_smem + (threadIdx.x >> 5) * rerank_warp_floats(d);
    float *rows_s = q_s + d;
    for (int f = lane; f < d; f += 32) q_s[f] = x[pos * d + f];
    __syncwarp();
    unsigned long long key[PER];
#pragma unroll
    for (int t = 0; t < PER; ++t) {
        const int s = lane + 32 * t;
        int32_t j = -1;
        if (s < c0 + c1)
            j = s < c0 ? cand_ids[(q * 2) * cap + s] : cand_ids[(q * 2 + 1) * cap + (s - c0)];
        // every lane joins the staging (it is warp-wide), the rounds are uniform per warp
        const float dd = t * 32 < c0 + c1 ? staged_d2(x, d, q_s, j, rows_s, lane) : CUSCAN_INF;
        key[t] = j < 0 ? ~0ull : ((unsigned long long)__float_as_uint(dd) << 32) | (uint32_t)perm[j];
    }
    for (int r = 0; r < k; ++r) {
        unsigned long long mine = key[0];
#pragma unroll
        for (int t = 1; t < PER; ++t) mine = key[t] < mine ? key[t] : mine;
        const unsigned long long best = warp_min_u64(mine);
#pragma unroll
        for (int t = 0; t < PER; ++t)
            if (key[t] == best) key[t] = ~0ull;
        if (lane == 0) {
            ids[orow * k + r] = (int32_t)(uint32_t)best;
            dist[orow * k + r] = __uint_as_float((uint32_t)(best >> 32));
        }
    }
}

// Original row of each listed position (in place).
__global__ void positions_to_rows_kernel(int32_t *__restrict__ list, int64_t count,
                                         const int32_t *__restrict__ perm) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) list[i] = perm[list[i]];
}

// Borůvka re-rank over component-sorted positions: exact weight of every appended candidate of
// both row halves, row minimum (w, original j) into row_keys[original row]. Rows whose buffer
// overflowed are re-run exactly; rows without candidates keep an empty key (they cannot hold
// their component's cheapest edge: every pair reaching it is appended).
__global__ void rerank_boruvka_kernel(const float *__restrict__ xp, const float *__restrict__ corep,
                                      const int32_t *__restrict__ labp,
                                      const int32_t *__restrict__ perm, int64_t nq,
                                      const int32_t *__restrict__ qpos, int d,
                                      const int32_t *__restrict__ cand_ids,
                                      const int32_t *__restrict__ rowcnt, int cap,
                                      const int32_t *__restrict__ colcnt,
                                      const int32_t *__restrict__ colbuf, int capc,
                                      unsigned long long *__restrict__ row_keys,
                                      int32_t *__restrict__ fallback,
                                      int *__restrict__ fallback_count) {
    // q indexes the screened rows (all positions, or the gathered positions qpos)
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= nq) return;
    const int64_t pos = qpos ? (int64_t)qpos[q] : q;
    const int c0 = rowcnt[q * 2], c1 = rowcnt[q * 2 + 1];
    const int c2 = colcnt ? colcnt[pos] : 0;  // pairs other blocks appended for this row
    if (c0 > cap || c1 > cap || c2 > capc) {
        if (lane == 0) {
            const int at = atomicAdd(fallback_count, 1);
            fallback[at] = (int32_t)pos;
        }
        return;
    }
    const int total = c0 + c1 + c2;
    if (total == 0) return;  // no candidate: the row keeps an empty key
    extern __shared__ float rerank_smem[];
    float *q_s = rerank_smem + (threadIdx.x >> 5) * rerank_warp_floats(d);
    float *rows_s = q_s + d;
    for (int f = lane; f < d; f += 32) q_s[f] = xp[pos * d + f];
    __syncwarp();
    const float ci = corep[pos];
    const int32_t li = labp[pos];
    unsigned long long mine = ~0ull;
    for (int base = 0; base < total; base += 32) {
        const int s = base + lane;
        int32_t j = -1;
        if (s < total) {
            j = s < c0        ? cand_ids[(q * 2) * cap + s]
                : s < c0 + c1 ? cand_ids[(q * 2 + 1) * cap + (s - c0)]
                              : colbuf[pos * capc + (s - c0 - c1)];
            if (labp[j] == li) j = -1;
        }
        const float d2 = staged_d2(xp, d, q_s, j, rows_s, lane);
        if (j < 0) continue;
        const float w = fmaxf(fmaxf(d2, ci), corep[j]);
        if (w != w) continue;
        const unsigned long long key =
            ((unsigned long long)weight_key_bits(w) << 32) | (uint32_t)perm[j];
        mine = key < mine ? key : mine;
    }
    const unsigned long long best = warp_min_u64(mine);
    if (lane == 0 && best != ~0ull) row_keys[perm[pos]] = best;
}

// Upper bounds of each component's cheapest edge from the exact kNN rows: a neighbour in another
// component is an edge of known exact weight max(d2, core_i, core_j).
__global__ void seed_bounds_kernel(const int32_t *__restrict__ knn_ids,
                                   const float *__restrict__ knn_sq, int k,
                                   const float *__restrict__ core, const int32_t *__restrict__ label,
                                   int64_t n, uint32_t *__restrict__ cbound) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t li = label[i];
    const float ci = core[i];
    float best = CUSCAN_INF;
    for (int s = 0; s < k; ++s) {
        const int32_t j = knn_ids[i * k + s];
        if (j < 0 || (int64_t)j >= n || label[j] == li) continue;
        best = fminf(best, fmaxf(fmaxf(knn_sq[i * k + s], ci), core[j]));
    }
    if (best < CUSCAN_INF) atomicMin(&cbound[li], __float_as_uint(best));
}

// Evenly spaced rows as cell pivots.
__global__ void pick_pivots_kernel(const float *__restrict__ x, int64_t n, int d, int npiv,
                                   float *__restrict__ piv) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)npiv * d) return;
    const int64_t p = e / d;
    const int f = (int)(e - p * d);
    const int64_t r = (p * n) / npiv;
    piv[e] = x[r * d + f];
}

// Per-row bounds of the symmetric screen: the bound of the row's component.
// Also counts the rows whose component has no bound yet.
// Row bounds of the symmetric screen (the component bounds), the count of rows without one, and
// the rows that can hold their component's cheapest edge. Every edge of row i weighs at least
// core_i and at least the row's lower bound from earlier rounds (its component has only grown
// since, so it has fewer cross edges); a row where either exceeds its component's upper bound
// cannot hold the cheapest edge, ties included.
__global__ void init_row_bounds_kernel(const uint32_t *__restrict__ cbound,
                                       const int32_t *__restrict__ labp,
                                       const float *__restrict__ corep,
                                       const float *__restrict__ rowlb,
                                       const int32_t *__restrict__ perm, int64_t n,
                                       uint32_t *__restrict__ urow, int *__restrict__ unbounded,
                                       int32_t *__restrict__ active) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool inf = false;
    if (i < n) {
        const uint32_t b = cbound[labp[i]];
        urow[i] = b;
        inf = b >= 0x7f800000u;
        const float ub = __uint_as_float(b);
        active[i] = !(corep[i] > ub) && !(rowlb[perm[i]] > ub) ? 1 : 0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, inf);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(unbounded, __popc(m));
}

// Fold the one-sided screen's bounds (two column halves per query row) into the per-row lower
// bounds, kept in original row order across rounds.
__global__ void update_row_lb_kernel(const float *__restrict__ lbtmp,
                                     const int32_t *__restrict__ qpos,
                                     const int32_t *__restrict__ perm, int64_t nq,
                                     float *__restrict__ rowlb) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int64_t pos = qpos ? (int64_t)qpos[q] : q;
    const int32_t orow = perm[pos];
    rowlb[orow] = fmaxf(rowlb[orow], fminf(lbtmp[2 * q], lbtmp[2 * q + 1]));
}

// Exact rounds: the weight of each scanned row's cheapest cross-component edge (the top half of
// its candidate key) is a lower bound of its cheapest cross edge in every later round, because
// merging components only removes cross edges. A row without a candidate keeps ~0: +inf.
__global__ void row_lb_from_keys_kernel(const unsigned long long *__restrict__ row_keys,
                                        const int32_t *__restrict__ qpos,
                                        const int32_t *__restrict__ perm, int64_t nq,
                                        float *__restrict__ rowlb) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int64_t pos = qpos ? (int64_t)qpos[q] : q;
    const int32_t orow = perm[pos];
    const unsigned long long key = row_keys[orow];  // keys are kept by original row
    const float w = key == ~0ull ? CUSCAN_INF : __uint_as_float((uint32_t)(key >> 32));
    rowlb[orow] = fmaxf(rowlb[orow], w);
}

// Positions of the flagged rows, in order (idx is the exclusive scan of the flags).
__global__ void compact_positions_kernel(const int32_t *__restrict__ flag,
                                         const int32_t *__restrict__ idx, int64_t n,
                                         int32_t *__restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) out[idx[i]] = (int32_t)i;
}

__global__ void fill_u32_kernel(uint32_t *p, int64_t n, uint32_t v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// Error bound coefficients of one operand format (fmt) at d features, K blocks of 64 (d_pad).
//  * Operands: unit roundoff u = 2^-8 (bf16) or 2^-11 (fp16 of the scaled values; |x * scale|
//    <= 2^15, so nothing overflows). Split bf16 represents x = hi + lo + e with |e| <= u^2 |x|,
//    so hi.hi' + hi.lo' + lo.hi' misses x.y by at most u^2 (3 + 4u) |x||y| per feature instead
//    of (2u + u^2) |x||y|.
//  * Accumulation: the K products of an entry (d_pad, or 3 d_pad for split operands) are
//    assumed to come out of the tensor core's f32 accumulation within K 2^-23 of the sum of
//    their magnitudes, two f32 units in the last place per product where f32 sequential
//    summation needs one. tests/test_gpu_accumulation.py drives the accumulator with
//    adversarial operands and requires the observed worst case to stay within a quarter of it.
//  * C_B: norms and the reference sum each carry at most (d + 2) f32 roundings; the epilogue
//    adds a few more; everything is taken three times over.
//  * abs_c: scaled fp16 values below 2^-14 round in the subnormal range with an absolute error
//    of at most 2^-25, which adds at most 2 [2^-25 (1 + u) sqrt(d) (m_i + m_j) + d 2^-50] to the
//    distance; with every scaled norm at most sqrt(d) 2^15 this is a constant. bf16 values (hi,
//    lo) in the subnormal range, or flushed to zero, err by at most 2^-126 each.
void error_coefficients(int d, int d_pad, int fmt, float absmax, float &c_a, float &c_b,
                        float &abs_c) {
    const bool fp16 = fmt == FMT_FP16;
    const double u = std::ldexp(1.0, fp16 ? -11 : -8);  // unit roundoff (round to nearest)
    const double u32 = std::ldexp(1.0, -24);            // f32 unit roundoff
    const double K = fmt == FMT_SPLIT ? 3.0 * d_pad : (double)d_pad;
    double rnd, mag;
    if (fmt == FMT_SPLIT) {
        rnd = u * u * (3.0 + 4.0 * u);
        mag = (1 + u) * (1 + u) * (1 + 2 * u * (1 + u));
    } else {
        rnd = 2.0 * u + u * u;
        mag = (1 + u) * (1 + u);
    }
    const double a1 = rnd + K * std::ldexp(1.0, -23) * mag;
    const double b = 3.5 * (double)(d + 4) * u32 + 1e-7;
    c_a = (float)(2.0 * a1 * (1.0 + 1e-4));
    c_b = (float)b;
    const double dd = (double)d;
    if (fp16) {
        const double eta = std::ldexp(1.0, -25);
        const double m_max = std::sqrt(dd) * std::ldexp(1.0, 15);
        abs_c = (float)(2.0 * (eta * (1 + u) * std::sqrt(dd) * 2.0 * m_max + dd * eta * eta) * 1.01);
    } else {
        abs_c = (float)(std::ldexp(1.0, -126) * (8.0 * dd * (double)absmax * 1.01 + 2.0 * K));
    }
}

// Power-of-two scale that brings the largest |x| into [2^14, 2^15) for fp16 operands; 0 when
// no such scale keeps scale^2 and the scaled sums inside the f32 range (bf16 is used then).
float fp16_scale(float absmax) {
    if (absmax == 0.0f) return 1.0f;
    if (!(absmax > 0.0f) || !std::isfinite(absmax)) return 0.0f;
    int e = 0;
    std::frexp((double)absmax, &e);  // absmax in [2^(e-1), 2^e)
    const int k = 15 - e;            // absmax * 2^k in [2^14, 2^15)
    if (k > 60 || k < -60) return 0.0f;
    return (float)std::ldexp(1.0, k);
}

}  // namespace

int refined_available() { return 1; }

struct Layout {
    int d_pad, kblocks, stages;
    int nbk, split;  // K blocks per tile row of the copy; split bf16 copy
    int64_t n_pad, n_tiles, n_qblocks;
    size_t smem;
};

// Tiling of n rows of d features; split copies hold hi and lo blocks, so a tile (the unit of a
// pipeline stage) is twice as large and fits two stages only for d <= 64.
static bool refined_layout(int64_t n, int d, Layout &L, bool split = false) {
    L.d_pad = (int)ceil_div(d, 64) * 64;
    if (L.d_pad > 128) return false;
    L.kblocks = L.d_pad / 64;
    L.split = split ? 1 : 0;
    L.nbk = split ? 2 * L.kblocks : L.kblocks;
    L.n_tiles = ceil_div(n, BN);
    L.n_pad = L.n_tiles * BN;
    L.n_qblocks = ceil_div(n, BM);
    const size_t a = (size_t)L.nbk * KBLOCK_A, b = (size_t)L.nbk * KBLOCK_B;
    const size_t fixed = a + (size_t)EPI_WARPS * (PB_STRIDE + 32 * VSTRIDE) * 4 +
                         256 + 1024;
    int st = (int)((227 * 1024 - fixed) / b);
    if (st > 4) st = 4;
    if (st < 2) return false;
    L.stages = st;
    L.smem = fixed + (size_t)st * b;
    return true;
}

static bool refined_shape_ok(int64_t n, int d, int k) {
    Layout L;
    return n >= 2048 && k <= 32 && refined_layout(n, d, L);
}

size_t refined_workspace_bytes(int64_t n, int d, int k) {
    Layout L;
    if (!refined_shape_ok(n, d, k) || !refined_layout(n, d, L)) return 0;
    constexpr size_t M = 32;
    // a bf16-refined fit may switch to split copies (twice the columns) when d <= 64
    const size_t copy_cols = (size_t)L.d_pad * (L.d_pad <= 64 ? 2 : 1);
    size_t b = (size_t)L.n_pad * copy_cols * 2 + 2 * sizeof(float) * (size_t)L.n_pad;  // xt, norms
    b += 3 * sizeof(float) * (size_t)L.n_tiles + 64;          // tile stats, flags, cursor
    b += 2 * sizeof(float) * (size_t)L.n_pad + sizeof(float) * (size_t)L.n_pad / 16;  // column terms
    b += sizeof(int32_t) * (size_t)n;                                                 // fallback
    b += 2 * 4 * (size_t)n * 2 * M;                  // candidate ids and bounds (two lists of M)
    b += sizeof(uint32_t) * (size_t)n + 2 * sizeof(int32_t) * (size_t)n;  // cbound, rowcnt
    b += 256 * sizeof(float) * (size_t)d + 8 * (size_t)n;                 // pivots, cells
    // threshold re-screen of inconclusive kNN rows (at most all n): thresholds, tiles, norms,
    // candidates, counts, fallback list
    b += 4 * (size_t)n + (size_t)L.n_pad * copy_cols * 2 + 2 * sizeof(float) * (size_t)L.n_pad;
    b += 4 * (size_t)n * 2 * KNN_CAP + 8 * (size_t)n + 4 * (size_t)n;
    // symmetric Borůvka: row bounds, column-side counts and candidates; subset rounds: flags,
    // their scan and the gathered positions
    b += 8 * (size_t)n + 4 * (size_t)n * BORUVKA_COL_CAP + 12 * (size_t)n;
    b += 12 * (size_t)n;  // row lower bounds (original order) and per-half screen bounds
    return b;
}

// 16-bit tiled copy and norms of n rows (row r = rowmap[r] of x, or r), padded to n_pad rows.
static int tile_rows(cuscan_ctx *ctx, const RefinedBuffers &R, const float *x, int64_t n, int d,
                     int d_pad, int64_t n_pad, const int32_t *rowmap, uint8_t *xt, float *pnorm,
                     float *mnorm, cudaStream_t s) {
    const int64_t groups = n_pad * (d_pad / 8);
    const unsigned gb = (unsigned)ceil_div(groups, 256);
    if (R.fp16)
        CUSCAN_KERNEL(tile_16bit_kernel<FMT_FP16>, gb, 256, 0, s, x, n, d, d_pad, n_pad, R.scale,
                      rowmap, xt);
    else if (R.split)
        CUSCAN_KERNEL(tile_16bit_kernel<FMT_SPLIT>, gb, 256, 0, s, x, n, d, d_pad, n_pad, 1.0f,
                      rowmap, xt);
    else
        CUSCAN_KERNEL(tile_16bit_kernel<FMT_BF16>, gb, 256, 0, s, x, n, d, d_pad, n_pad, 1.0f,
                      rowmap, xt);
    CUSCAN_KERNEL(norms_kernel, (unsigned)ceil_div(n_pad, 256), 256, 0, s, x, n, d, n_pad,
                  R.fp16 ? R.scale : 1.0f, rowmap, pnorm, mnorm);
    CUSCAN_LAUNCH(ctx, "16-bit tiles");
    return CUSCAN_OK;
}

static int prep(cuscan_ctx *ctx, RefinedBuffers &R, const Layout &L, const float *x, int64_t n,
                int d, const int32_t *chunk_lo, const int32_t *chunk_hi, cudaStream_t s) {
    int rc = ensure(ctx, R.xt, (size_t)L.n_tiles * L.nbk * KBLOCK_B, "16-bit tiles");
    if (!rc) rc = ensure(ctx, R.pnorm, sizeof(float) * L.n_pad, "norms");
    if (!rc) rc = ensure(ctx, R.mnorm, sizeof(float) * L.n_pad, "norms");
    if (!rc) rc = ensure(ctx, R.tile_mmax, sizeof(float) * L.n_tiles, "tile norms");
    if (!rc) rc = ensure(ctx, R.tile_lo, sizeof(int32_t) * L.n_tiles, "tile labels");
    if (!rc) rc = ensure(ctx, R.tile_hi, sizeof(int32_t) * L.n_tiles, "tile labels");
    if (!rc) rc = ensure(ctx, R.error, 16, "error flag");
    if (!rc) rc = ensure(ctx, R.count, 16, "fallback count");
    if (!rc) rc = ensure(ctx, R.cursor, 16, "tile cursor");
    if (!rc) rc = ensure(ctx, R.fallback, sizeof(int32_t) * n, "fallback rows");
    if (!rc) rc = ensure(ctx, R.qthr, sizeof(float) * n, "fallback thresholds");
    if (rc) return rc;
    if ((rc = tile_rows(ctx, R, x, n, d, L.d_pad, L.n_pad, nullptr, as<uint8_t>(R.xt),
                        as<float>(R.pnorm), as<float>(R.mnorm), s)))
        return rc;
    CUSCAN_KERNEL(tile_stats_kernel, (unsigned)ceil_div(L.n_tiles, 128), 128, 0, s,
                  as<float>(R.mnorm), chunk_lo, chunk_hi, L.n_tiles, ceil_div(n, 32),
                  as<float>(R.tile_mmax), as<int32_t>(R.tile_lo), as<int32_t>(R.tile_hi));
    CUSCAN_LAUNCH(ctx, "refined prep");
    return CUSCAN_OK;
}

// Operand format of this fit's screens: fp16 of x * scale when the caller asked for it and the
// data's range admits a power-of-two scale, else bf16. One reduction and one host read per fit.
// Largest d * max|x|^2 for which the screens stay exact: squared norms, dot products, bounds
// and every exact squared distance (at most 4 d max|x|^2) then stay below FLT_MAX / 4. Above it
// an f32 quantity may overflow: a bound may become NaN, and exact weights may tie at +inf,
// where the reference breaks the ties among ALL overflowing pairs, which bounds cannot narrow.
constexpr double kScreenRangeMax = 3.4028234663852886e38 / 16.0;

// Per fit: the largest |x| (one reduction and one host read) decides whether the screens may run
// (range_ok) and, when fp16 operands are wanted, their power-of-two scale.
static int choose_operands(cuscan_ctx *ctx, RefinedBuffers &R, const float *x, int64_t n, int d,
                           cudaStream_t s) {
    if (R.have_scale) return CUSCAN_OK;
    R.fp16 = false;
    R.split = false;
    R.scale = 1.0f;
    R.range_ok = true;
    int rc = ensure(ctx, R.absmax, 16, "range reduction");
    if (rc) return rc;
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.absmax.ptr, 0, sizeof(unsigned int), s));
    const int64_t count = n * (int64_t)d;
    int64_t blocks = ceil_div(count, 256);
    if (blocks > 8 * (int64_t)ctx->sm_count) blocks = 8 * (int64_t)ctx->sm_count;
    CUSCAN_KERNEL(absmax_kernel, (unsigned)blocks, 256, 0, s, x, count,
                  as<unsigned int>(R.absmax));
    CUSCAN_LAUNCH(ctx, "absmax_kernel");
    unsigned int bits = 0;
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(&bits, R.absmax.ptr, sizeof(bits), cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
    float amax;
    memcpy(&amax, &bits, sizeof(amax));
    R.range_ok = std::isfinite(amax) && (double)d * (double)amax * (double)amax <= kScreenRangeMax;
    R.amax_value = std::isfinite(amax) ? amax : 0.0f;
    if (R.want_fp16) {
        const float sc = fp16_scale(amax);
        if (sc > 0.0f) {
            R.fp16 = true;
            R.scale = sc;
        }
    }
    R.have_scale = true;
    return CUSCAN_OK;
}

// Operand format of the current fit's screens.
static int operand_format(const RefinedBuffers &R) {
    return R.split ? FMT_SPLIT : R.fp16 ? FMT_FP16 : FMT_BF16;
}

// Operand format a refined fit ended with: 0 bf16, 1 fp16, 2 split bf16 (-1: no screen ran).
int refined_operand_format(const ForestBuffers &b) {
    return b.refined.tile_pairs == 0 ? -1 : operand_format(b.refined);
}

// A operand of a screen and the outputs of the kNN threshold mode; the defaults mean the
// reference rows themselves.
struct QuerySet {
    const uint8_t *xq = nullptr;
    const float *pq = nullptr, *mq = nullptr;
    int64_t nq = -1;
    const int32_t *qpos = nullptr;
    const float *qthr = nullptr;
    int32_t *cand_ids = nullptr;
    int32_t *rowcnt = nullptr;
    float *rowlb = nullptr;  // one-sided Borůvka: per query row and half, the pair lower bound
};

template <int M, int MODE>
static int run_screen(cuscan_ctx *ctx, RefinedBuffers &R, const Layout &L, int64_t n, int d,
                      const float *core, const int32_t *label, const int32_t *chunk_lo,
                      const int32_t *chunk_hi, cudaStream_t s, float *debug_tile = nullptr,
                      float *debug_chunk = nullptr,
                      const QuerySet &Q = QuerySet()) {
    constexpr bool BORUVKA = MODE == MODE_BORUVKA || MODE == MODE_BORUVKA_SYM;
    int rc = ensure(ctx, R.cand_ids, sizeof(int32_t) * n * 2 * M, "screen candidates");
    if (!rc) rc = ensure(ctx, R.cand_lb, sizeof(float) * n * 2 * M, "screen bounds");
    if (rc) return rc;
    Params P{};
    P.xt = as<uint8_t>(R.xt);
    P.pnorm = as<float>(R.pnorm);
    P.mnorm = as<float>(R.mnorm);
    P.xq = Q.xq ? Q.xq : P.xt;
    P.pq = Q.pq ? Q.pq : P.pnorm;
    P.mq = Q.mq ? Q.mq : P.mnorm;
    P.nq = Q.nq >= 0 ? Q.nq : n;
    P.qpos = Q.qpos;
    P.qthr = Q.qthr;
    P.core = core;
    P.label = label;
    P.tile_mmax = as<float>(R.tile_mmax);
    P.chunk_lo = chunk_lo;
    P.chunk_hi = chunk_hi;
    P.tile_lo = as<int32_t>(R.tile_lo);
    P.tile_hi = as<int32_t>(R.tile_hi);
    P.n = n;
    P.n_tiles = L.n_tiles;
    P.n_qblocks = ceil_div(P.nq, (int64_t)BM);
    P.n_chunks = ceil_div(n, 32);
    P.kblocks = L.kblocks;
    P.nbk = L.nbk;
    P.split = L.split;
    P.stages = L.stages;
    P.cursor = as<unsigned long long>(R.cursor);
    // parts of at least 128 tiles: the start of a work item (A tile, pipeline fill) stays small
    // against its tiles, and the fits of a serving stream (under 32,768 rows) keep one CTA per
    // block, leaving the other SMs to the fits running beside them
    P.splits = 1;
    if (MODE == MODE_BORUVKA && P.n_qblocks > 0 && P.n_qblocks < ctx->sm_count && !debug_tile) {
        int64_t per = ctx->sm_count / P.n_qblocks;
        if (per > P.n_tiles / 128) per = P.n_tiles / 128;
        P.splits = (int)(per < 1 ? 1 : per < 16 ? per : 16);
    }
    float ca, cb, abs_c;
    error_coefficients(d, L.d_pad, operand_format(R), R.fp16 ? R.amax_value * R.scale : R.amax_value, ca, cb, abs_c);
    P.c_a = ca;
    P.one_minus_cb = 1.0f - cb;
    P.abs_c = abs_c;
    P.idesc = R.fp16 ? IDESC_F16 : IDESC_BF16;
    const float sc = R.fp16 ? R.scale : 1.0f;
    P.s2 = sc * sc;
    P.inv_s2 = 1.0f / (sc * sc);
    P.cand_ids = as<int32_t>(R.cand_ids);
    P.cand_lb = as<float>(R.cand_lb);
    P.error = as<int>(R.error);
    P.debug_tile = debug_tile;
    P.debug_chunk = debug_chunk;
    P.c_b = cb;
    P.cap = BORUVKA_CAP;
    if (BORUVKA) {
        rc = ensure(ctx, R.cbound, sizeof(uint32_t) * n, "component bounds");
        if (!rc) rc = ensure(ctx, R.rowcnt, sizeof(int32_t) * 2 * n, "row candidate counts");
        if (rc) return rc;
        P.cbound = as<uint32_t>(R.cbound);
        P.rowcnt = as<int32_t>(R.rowcnt);
        CUSCAN_CUDA(ctx, cudaMemsetAsync(R.rowcnt.ptr, 0, sizeof(int32_t) * 2 * n, s));
    }
    if (MODE == MODE_BORUVKA_SYM) {
        P.urow = as<uint32_t>(R.urow);
        P.colcnt = as<int32_t>(R.colcnt);
        P.colbuf = as<int32_t>(R.colbuf);
        P.capc = BORUVKA_COL_CAP;
    }
    if (MODE == MODE_BORUVKA) P.rowlb = Q.rowlb;
    if (MODE == MODE_BORUVKA && P.splits > 1 && P.rowlb && P.nq > 0)
        if (int rc = launch_fill_u64(ctx, reinterpret_cast<unsigned long long *>(P.rowlb), P.nq,
                                     0x7f8000007f800000ull, s))  // +inf in both halves
            return rc;
    if (MODE == MODE_KNN_THRESHOLD) {
        P.cap = KNN_CAP;
        P.cand_ids = Q.cand_ids;
        P.rowcnt = Q.rowcnt;
    }
    if (P.n_qblocks == 0) return CUSCAN_OK;
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.error.ptr, 0, 16, s));
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.cursor.ptr, 0, 16, s));
    // the column terms of this launch (its C_B and, for Borůvka, the core scale)
    if (int rc = ensure(ctx, R.colp, sizeof(float) * L.n_pad, "screen column norms")) return rc;
    if (BORUVKA)
        if (int rc = ensure(ctx, R.colc, sizeof(float) * L.n_pad, "screen column cores")) return rc;
    if (int rc = ensure(ctx, R.cmin, sizeof(float) * L.n_pad / 16, "screen chunk minima")) return rc;
    P.colp = as<float>(R.colp);
    P.colc = BORUVKA ? as<float>(R.colc) : nullptr;
    P.cmin = as<float4>(R.cmin);
    CUSCAN_KERNEL(screen_columns_kernel, (unsigned)(L.n_pad / 256), 256, 0, s, P.pnorm,
                  BORUVKA ? core : nullptr, n, P.one_minus_cb, P.s2, as<float>(R.colp),
                  BORUVKA ? as<float>(R.colc) : nullptr, as<float2>(R.cmin));
    CUSCAN_LAUNCH(ctx, "screen_columns_kernel");
    auto kernel = screen_kernel<M, MODE>;
    if (int rc = allow_dynamic_smem(ctx, kernel, L.smem)) return rc;
    const int64_t items = P.n_qblocks * P.splits;
    int64_t grid = items < ctx->sm_count ? items : ctx->sm_count;
    CUSCAN_KERNEL(kernel, (unsigned)grid, THREADS, L.smem, s, P);
    CUSCAN_LAUNCH(ctx, "screen_kernel");
    return CUSCAN_OK;
}

static int read_screen_status(cuscan_ctx *ctx, RefinedBuffers &R, cudaStream_t s, int &fallbacks) {
    unsigned long long status[2] = {0, 0};  // error flag, tile pairs
    int count = 0;
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(status, R.error.ptr, 16, cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(&count, R.count.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
    if ((int)(status[0] & 0xffffffffu))
        return fail(ctx, CUSCAN_BACKEND_UNAVAILABLE,
                    "tensor-core screening timed out waiting on a pipeline barrier");
    R.tile_pairs += (int64_t)status[1];
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.error.ptr, 0, 16, s));
    fallbacks = count;
    return CUSCAN_OK;
}

// The kNN list screen over every row in sorted positions and its exact re-rank. Rows whose
// lists are inconclusive are listed by position in R.fallback, with the k-th exact distance
// among their candidates in R.qthr; returns their count.
static int knn_list_pass(cuscan_ctx *ctx, RefinedBuffers &R, const Layout &L, const float *xs,
                         const int32_t *perm, int64_t n, int d, int k, int32_t *ids, float *dist,
                         cudaStream_t s, int &fallbacks) {
    // 22 bounds per row half: enough that nearly every row's unseen bound clears its k-th
    // exact distance at k <= 32 for bf16 screens (the rest go to the threshold re-screen), and
    // each insertion shifts 22 registers; 20 and 24 entries measured slower
    constexpr int M = KNN_LIST;
    if (int rc = prep(ctx, R, L, xs, n, d, nullptr, nullptr, s)) return rc;
    for (cudaEvent_t &e : R.screen_ev)
        if (!e) CUSCAN_CUDA(ctx, cudaEventCreate(&e));
    CUSCAN_CUDA(ctx, cudaEventRecord(R.screen_ev[0], s));
    if (int rc = run_screen<M, MODE_KNN_LIST>(ctx, R, L, n, d, nullptr, nullptr, nullptr, nullptr, s))
        return rc;
    CUSCAN_CUDA(ctx, cudaEventRecord(R.screen_ev[1], s));
    R.screen_timed = true;
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.count.ptr, 0, sizeof(int), s));
    const size_t rr_smem = sizeof(float) * RERANK_WARPS * (size_t)rerank_warp_floats(d);
    if (int rc = allow_dynamic_smem(ctx, rerank_knn_kernel<M>, rr_smem)) return rc;
    CUSCAN_KERNEL(rerank_knn_kernel<M>, (unsigned)ceil_div(n, (int64_t)RERANK_WARPS),
                  32 * RERANK_WARPS, rr_smem, s, xs, perm, n, d,
                  k, as<int32_t>(R.cand_ids), as<float>(R.cand_lb), ids, dist,
                  as<int32_t>(R.fallback), as<float>(R.qthr), as<int>(R.count));
    CUSCAN_LAUNCH(ctx, "rerank_knn_kernel");
    return read_screen_status(ctx, R, s, fallbacks);
}

int launch_knn_refined(cuscan_ctx *ctx, ForestBuffers &b, const float *x, int64_t n, int d, int k,
                       int32_t *ids, float *dist, cudaStream_t s, int64_t *refined_rows,
                       int64_t *fallback_rows, int64_t *rescreened_rows) {
    if (!refined_shape_ok(n, d, k)) {
        // shapes outside the tensor-core tiling run the exact f32 sweep
        return launch_exact_knn_fp32(ctx, x, n, x, n, d, k, 1, 0, 1, ids, dist, s, b.knn_ids_tmp,
                                     b.knn_dist_tmp);
    }
    RefinedBuffers &R = b.refined;
    Layout L;
    refined_layout(n, d, L);
    int rc = choose_operands(ctx, R, x, n, d, s);
    if (rc) return rc;
    if (!R.range_ok)  // values large enough to overflow f32: the exact sweep decides alone
        return launch_exact_knn_fp32(ctx, x, n, x, n, d, k, 1, 0, 1, ids, dist, s, b.knn_ids_tmp,
                                     b.knn_dist_tmp);
    // 1. cells: nearest of npiv evenly spaced pivot rows (exact f32, k = 1)
    const int npiv = (int)(n / 256 < 256 ? (n / 256 < 1 ? 1 : n / 256) : 256);
    rc = ensure(ctx, R.pivots, sizeof(float) * npiv * d, "cell pivots");
    if (!rc) rc = ensure(ctx, R.cells, sizeof(int32_t) * n, "cells");
    if (!rc) rc = ensure(ctx, R.cell_d, sizeof(float) * n, "cell distances");
    if (rc) return rc;
    CUSCAN_KERNEL(pick_pivots_kernel, (unsigned)ceil_div((int64_t)npiv * d, 256), 256, 0, s, x, n,
                  d, npiv, as<float>(R.pivots));
    CUSCAN_LAUNCH(ctx, "pick_pivots_kernel");
    if ((rc = launch_exact_knn_fp32(ctx, x, n, as<float>(R.pivots), npiv, d, 1, 0, 0, 1,
                                    as<int32_t>(R.cells), as<float>(R.cell_d), s, b.knn_ids_tmp,
                                    b.knn_dist_tmp)))
        return rc;
    // 2. rows sorted by cell (b.perm, b.xp)
    if ((rc = forest_sort_by_component(ctx, b, x, nullptr, as<int32_t>(R.cells), n, d, s)))
        return rc;
    const float *xs = as<float>(b.xp);
    const int32_t *perm = as<int32_t>(b.perm);
    // 3. screen + exact re-rank in sorted positions, outputs in original rows
    int fallbacks = 0;
    if ((rc = knn_list_pass(ctx, R, L, xs, perm, n, d, k, ids, dist, s, fallbacks))) return rc;
    if (refined_rows) *refined_rows += n;
    if (!R.fp16 && !R.split && (double)fallbacks > TIGHTEN_TRIGGER * (double)n) {
        // the bf16 bound is too loose for this data (norms large against the neighbour
        // distances): screen again, and run the Borůvka rounds, with split-bf16 operands, or
        // with scaled fp16 operands where a split tile does not fit the pipeline
        Layout Ls;
        const float sc = fp16_scale(R.amax_value);
        if (refined_layout(n, d, Ls, true)) {
            R.split = true;
            L = Ls;
        } else if (sc > 0.0f) {
            R.fp16 = true;
            R.scale = sc;
        }
        if (R.split || R.fp16)
            if ((rc = knn_list_pass(ctx, R, L, xs, perm, n, d, k, ids, dist, s, fallbacks)))
                return rc;
    }
    if (fallbacks == 0) return CUSCAN_OK;
    constexpr int M = KNN_LIST;
    const size_t rr_smem = sizeof(float) * RERANK_WARPS * (size_t)rerank_warp_floats(d);
    int32_t *exact_rows = as<int32_t>(R.fallback);
    int exact = fallbacks;
    if (fallbacks >= RESCREEN_MIN_ROWS && k <= 2 * KNN_CAP) {
        // 4. inconclusive rows, screened again in threshold mode: every pair whose bound does
        // not exceed the row's k-th distance among its candidates is appended and re-ranked
        const int64_t nq = fallbacks;
        const int64_t nq_pad = ceil_div(nq, (int64_t)BN) * BN;
        rc = ensure(ctx, R.xq, (size_t)(nq_pad / BN) * L.nbk * KBLOCK_B, "re-screen tiles");
        if (!rc) rc = ensure(ctx, R.pq, sizeof(float) * nq_pad, "re-screen norms");
        if (!rc) rc = ensure(ctx, R.mq, sizeof(float) * nq_pad, "re-screen norms");
        if (!rc) rc = ensure(ctx, R.cand2, sizeof(int32_t) * nq * 2 * KNN_CAP, "re-screen candidates");
        if (!rc) rc = ensure(ctx, R.rowcnt2, sizeof(int32_t) * nq * 2, "re-screen counts");
        if (!rc) rc = ensure(ctx, R.fallback2, sizeof(int32_t) * nq, "re-screen fallbacks");
        if (!rc) rc = tile_rows(ctx, R, xs, nq, d, L.d_pad, nq_pad, as<int32_t>(R.fallback),
                                as<uint8_t>(R.xq), as<float>(R.pq), as<float>(R.mq), s);
        if (rc) return rc;
        QuerySet Q;
        Q.xq = as<uint8_t>(R.xq);
        Q.pq = as<float>(R.pq);
        Q.mq = as<float>(R.mq);
        Q.nq = nq;
        Q.qpos = as<int32_t>(R.fallback);
        Q.qthr = as<float>(R.qthr);
        Q.cand_ids = as<int32_t>(R.cand2);
        Q.rowcnt = as<int32_t>(R.rowcnt2);
        if ((rc = run_screen<M, MODE_KNN_THRESHOLD>(ctx, R, L, n, d, nullptr, nullptr, nullptr,
                                                   nullptr, s, nullptr, nullptr, Q)))
            return rc;
        CUSCAN_CUDA(ctx, cudaMemsetAsync(R.count.ptr, 0, sizeof(int), s));
        if ((rc = allow_dynamic_smem(ctx, rerank_knn_threshold_kernel, rr_smem))) return rc;
        CUSCAN_KERNEL(rerank_knn_threshold_kernel, (unsigned)ceil_div(nq, (int64_t)RERANK_WARPS),
                      32 * RERANK_WARPS, rr_smem, s, xs,
                      perm, as<int32_t>(R.fallback), nq, d, k, as<int32_t>(R.cand2),
                      as<int32_t>(R.rowcnt2), KNN_CAP, ids, dist, as<int32_t>(R.fallback2),
                      as<int>(R.count));
        CUSCAN_LAUNCH(ctx, "rerank_knn_threshold_kernel");
        if ((rc = read_screen_status(ctx, R, s, exact))) return rc;
        if (rescreened_rows) *rescreened_rows += fallbacks;
        exact_rows = as<int32_t>(R.fallback2);
    } else {
        CUSCAN_KERNEL(positions_to_rows_kernel, (unsigned)ceil_div((int64_t)fallbacks, 256), 256, 0,
                      s, exact_rows, (int64_t)fallbacks, perm);
        CUSCAN_LAUNCH(ctx, "positions_to_rows_kernel");
    }
    if (fallback_rows) *fallback_rows += exact;
    // 5. rows still inconclusive (original indices): exact f32 sweep
    if (exact > 0)
        return launch_exact_knn_fp32(ctx, x, exact, x, n, d, k, 1, 0, 1, ids, dist, s,
                                     b.knn_ids_tmp, b.knn_dist_tmp, exact_rows);
    return CUSCAN_OK;
}

int launch_candidates_refined(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int d,
                              const int32_t *knn_ids, const float *knn_sq, int k,
                              const float *core, const int32_t *label, cudaStream_t s,
                              int64_t *fallback_rows) {
    const float *xp = as<float>(b.xp);
    const float *corep = as<float>(b.corep);
    const int32_t *labp = as<int32_t>(b.labp);
    const int32_t *perm = as<int32_t>(b.perm);
    unsigned long long *row_keys = as<unsigned long long>(b.row_keys);
    int32_t *clo = as<int32_t>(b.tile_lo), *chi = as<int32_t>(b.tile_hi);
    if (!refined_shape_ok(n, d, 1))
        return launch_candidates_fp32(ctx, xp, corep, labp, perm, n, d, row_keys, clo, chi, s);
    RefinedBuffers &R = b.refined;
    Layout L;
    refined_layout(n, d, L, R.split != 0);
    int rc = choose_operands(ctx, R, xp, n, d, s);
    if (rc) return rc;
    if (!R.range_ok)  // values large enough to overflow f32: the exact round decides alone
        return launch_candidates_fp32(ctx, xp, corep, labp, perm, n, d, row_keys, clo, chi, s);
    rc = launch_tile_ranges(ctx, labp, n, clo, chi, s);
    if (!rc) rc = prep(ctx, R, L, xp, n, d, clo, chi, s);
    if (rc) return rc;
    // component bounds: +inf, then the exact cross-component edges of the kNN rows
    if ((rc = ensure(ctx, R.cbound, sizeof(uint32_t) * n, "component bounds"))) return rc;
    CUSCAN_KERNEL(fill_u32_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, as<uint32_t>(R.cbound), n,
                  0x7f800000u);
    CUSCAN_KERNEL(seed_bounds_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, knn_ids, knn_sq, k,
                  core, label, n, as<uint32_t>(R.cbound));
    // symmetric screen: per-row bounds start at the component bounds; empty column buffers
    if ((rc = ensure(ctx, R.urow, sizeof(uint32_t) * n, "row bounds"))) return rc;
    if ((rc = ensure(ctx, R.colcnt, sizeof(int32_t) * n, "column-side counts"))) return rc;
    if ((rc = ensure(ctx, R.colbuf, sizeof(int32_t) * n * BORUVKA_COL_CAP, "column-side candidates")))
        return rc;
    rc = ensure(ctx, R.act_flag, sizeof(int32_t) * n, "active rows");
    if (!rc) rc = ensure(ctx, R.act_idx, sizeof(int32_t) * n, "active rows");
    if (!rc) rc = ensure(ctx, R.act_pos, sizeof(int32_t) * n, "active rows");
    if (!rc) rc = ensure(ctx, R.rowlb, sizeof(float) * n, "row lower bounds");
    if (!rc) rc = ensure(ctx, R.lbtmp, sizeof(float) * 2 * n, "row lower bounds");
    if (rc) return rc;
    if (!R.lb_valid) {  // first round of the fit: no bounds yet
        CUSCAN_CUDA(ctx, cudaMemsetAsync(R.rowlb.ptr, 0, sizeof(float) * n, s));
        R.lb_valid = true;
    }
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.colcnt.ptr, 0, sizeof(int32_t) * n, s));
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.count.ptr, 0, 2 * sizeof(int), s));
    CUSCAN_KERNEL(init_row_bounds_kernel, (unsigned)ceil_div(n, 256), 256, 0, s,
                  as<uint32_t>(R.cbound), labp, corep, as<float>(R.rowlb), perm, n,
                  as<uint32_t>(R.urow), as<int>(R.count), as<int32_t>(R.act_flag));
    CUSCAN_LAUNCH(ctx, "init_row_bounds_kernel");
    if ((rc = scan_exclusive(ctx, as<int32_t>(R.act_flag), as<int32_t>(R.act_idx), n,
                             as<int32_t>(R.count) + 1, b.scan_tmp, s)))
        return rc;
    int counts[2] = {0, 0};  // rows without a component bound, rows that can hold an edge
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(counts, R.count.ptr, sizeof(counts), cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
    const int64_t active = counts[1];
    // Forms of the round:
    //  * one-sided over the rows that can hold their component's cheapest edge (all rows, or a
    //    gathered subset): it also leaves each screened row a lower bound of its cheapest cross
    //    edge, which lets most rows skip the later rounds. After the kNN seed most components
    //    have a bound from a neighbour in another component and few rows are that close to the
    //    boundary; later rounds skip the rows whose earlier bound already exceeds the bound.
    //  * symmetric: each unordered pair once. It halves the tensor-core and epilogue work but
    //    leaves no row bounds and tests a pair for its column's row only against that row's
    //    known bound (rows of components without a bound draw many appends there); it is used
    //    only when nearly every row is screened.
    const bool sym = n >= SYM_MIN_ROWS &&
                     (double)counts[0] <= SYM_UNBOUNDED_MAX * (double)n &&
                     (double)active > SYM_ACTIVE_MIN * (double)n;
    const bool subset = !sym && active < n;
    CUSCAN_LAUNCH(ctx, "component bounds");
    constexpr int M = 32;
    const int32_t *qpos = nullptr;
    int64_t nq = n;
    if (subset) {
        nq = active;
        const int64_t nq_pad = ceil_div(nq > 0 ? nq : 1, (int64_t)BN) * BN;
        rc = ensure(ctx, R.xq, (size_t)(nq_pad / BN) * L.nbk * KBLOCK_B, "subset tiles");
        if (!rc) rc = ensure(ctx, R.pq, sizeof(float) * nq_pad, "subset norms");
        if (!rc) rc = ensure(ctx, R.mq, sizeof(float) * nq_pad, "subset norms");
        if (rc) return rc;
        CUSCAN_KERNEL(compact_positions_kernel, (unsigned)ceil_div(n, 256), 256, 0, s,
                      as<int32_t>(R.act_flag), as<int32_t>(R.act_idx), n, as<int32_t>(R.act_pos));
        CUSCAN_LAUNCH(ctx, "compact_positions_kernel");
        qpos = as<int32_t>(R.act_pos);
        if ((rc = tile_rows(ctx, R, xp, nq, d, L.d_pad, nq_pad, qpos, as<uint8_t>(R.xq),
                            as<float>(R.pq), as<float>(R.mq), s)))
            return rc;
        QuerySet Q;
        Q.xq = as<uint8_t>(R.xq);
        Q.pq = as<float>(R.pq);
        Q.mq = as<float>(R.mq);
        Q.nq = nq;
        Q.qpos = qpos;
        Q.rowlb = as<float>(R.lbtmp);
        rc = run_screen<M, MODE_BORUVKA>(ctx, R, L, n, d, corep, labp, clo, chi, s, nullptr, nullptr, Q);
    } else if (sym) {
        rc = run_screen<M, MODE_BORUVKA_SYM>(ctx, R, L, n, d, corep, labp, clo, chi, s);
    } else {
        QuerySet Q;
        Q.rowlb = as<float>(R.lbtmp);
        rc = run_screen<M, MODE_BORUVKA>(ctx, R, L, n, d, corep, labp, clo, chi, s, nullptr, nullptr, Q);
    }
    if (rc) return rc;
    if (!sym && nq > 0) {
        CUSCAN_KERNEL(update_row_lb_kernel, (unsigned)ceil_div(nq, 256), 256, 0, s,
                      as<float>(R.lbtmp), qpos, perm, nq, as<float>(R.rowlb));
        CUSCAN_LAUNCH(ctx, "update_row_lb_kernel");
    }
    R.screened_rows += nq;
    if (sym) ++R.symmetric_rounds;
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.count.ptr, 0, sizeof(int), s));
    const size_t rr_smem = sizeof(float) * RERANK_WARPS * (size_t)rerank_warp_floats(d);
    if ((rc = allow_dynamic_smem(ctx, rerank_boruvka_kernel, rr_smem))) return rc;
    if (nq > 0) {
        CUSCAN_KERNEL(rerank_boruvka_kernel, (unsigned)ceil_div(nq, (int64_t)RERANK_WARPS),
                      32 * RERANK_WARPS, rr_smem, s, xp, corep, labp, perm, nq, qpos, d,
                      as<int32_t>(R.cand_ids), as<int32_t>(R.rowcnt), BORUVKA_CAP,
                      sym ? as<int32_t>(R.colcnt) : nullptr, as<int32_t>(R.colbuf),
                      BORUVKA_COL_CAP, row_keys, as<int32_t>(R.fallback), as<int>(R.count));
        CUSCAN_LAUNCH(ctx, "rerank_boruvka_kernel");
    }
    int fallbacks = 0;
    if ((rc = read_screen_status(ctx, R, s, fallbacks))) return rc;
    if (fallback_rows) *fallback_rows += fallbacks;
    if (fallbacks > 0)
        return launch_candidates_fp32(ctx, xp, corep, labp, perm, n, d, row_keys, clo, chi, s,
                                      as<int32_t>(R.fallback), fallbacks);
    return CUSCAN_OK;
}

// The per-row terms of the bound for the debug entry point: (ps, pb, cm, m) with
// ps = (1 - C_B) p - abs_c, pb = (1 - C_B) p, cm = C_A m, so that the screen's bound of entry
// (r, c) is fmaf(-cm_r, m_c, fmaf(-2, acc_rc, pb_c) + ps_r) (screen units).
// An exact (plain f32) Borůvka round over the rows that can hold their component's cheapest
// edge. The rows are chosen as in the screened rounds: every component gets an upper bound of
// its cheapest cross edge from the kNN pairs (seed_bounds_kernel), and a row is skipped when its
// core distance or its lower bound from earlier rounds exceeds that bound. Every cross edge of a
// skipped row then weighs strictly more than the component's cheapest, so the round's winners
// (crates/hdbscan/src/kernels/boruvka.rs:68-140 over all rows) are unchanged. The rows scanned
// leave their exact cheapest cross edge as their lower bound for the next round.
int launch_candidates_exact_rows(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int d,
                                 const int32_t *knn_ids, const float *knn_sq, int k,
                                 const float *core, const int32_t *label, cudaStream_t s,
                                 int64_t *screened_rows) {
    const float *xp = as<float>(b.xp);
    const float *corep = as<float>(b.corep);
    const int32_t *labp = as<int32_t>(b.labp);
    const int32_t *perm = as<int32_t>(b.perm);
    unsigned long long *row_keys = as<unsigned long long>(b.row_keys);
    int32_t *clo = as<int32_t>(b.tile_lo), *chi = as<int32_t>(b.tile_hi);
    RefinedBuffers &R = b.refined;
    int rc = ensure(ctx, R.cbound, sizeof(uint32_t) * n, "component bounds");
    if (!rc) rc = ensure(ctx, R.urow, sizeof(uint32_t) * n, "row bounds");
    if (!rc) rc = ensure(ctx, R.count, 16, "row counts");
    if (!rc) rc = ensure(ctx, R.act_flag, sizeof(int32_t) * n, "active rows");
    if (!rc) rc = ensure(ctx, R.act_idx, sizeof(int32_t) * n, "active rows");
    if (!rc) rc = ensure(ctx, R.act_pos, sizeof(int32_t) * n, "active rows");
    if (!rc) rc = ensure(ctx, R.rowlb, sizeof(float) * n, "row lower bounds");
    if (rc) return rc;
    if (!R.lb_valid) {  // first round of the fit: no bounds yet
        CUSCAN_CUDA(ctx, cudaMemsetAsync(R.rowlb.ptr, 0, sizeof(float) * n, s));
        R.lb_valid = true;
    }
    CUSCAN_KERNEL(fill_u32_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, as<uint32_t>(R.cbound), n,
                  0x7f800000u);
    CUSCAN_KERNEL(seed_bounds_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, knn_ids, knn_sq, k,
                  core, label, n, as<uint32_t>(R.cbound));
    CUSCAN_CUDA(ctx, cudaMemsetAsync(R.count.ptr, 0, 2 * sizeof(int), s));
    CUSCAN_KERNEL(init_row_bounds_kernel, (unsigned)ceil_div(n, 256), 256, 0, s,
                  as<uint32_t>(R.cbound), labp, corep, as<float>(R.rowlb), perm, n,
                  as<uint32_t>(R.urow), as<int>(R.count), as<int32_t>(R.act_flag));
    CUSCAN_LAUNCH(ctx, "component bounds");
    if ((rc = scan_exclusive(ctx, as<int32_t>(R.act_flag), as<int32_t>(R.act_idx), n,
                             as<int32_t>(R.count) + 1, b.scan_tmp, s)))
        return rc;
    int counts[2] = {0, 0};  // rows without a component bound, rows that can hold an edge
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(counts, R.count.ptr, sizeof(counts), cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
    const int64_t active = counts[1];
    const int32_t *qpos = nullptr;
    if (active == n) {
        rc = launch_candidates_fp32(ctx, xp, corep, labp, perm, n, d, row_keys, clo, chi, s);
    } else if (active > 0) {
        CUSCAN_KERNEL(compact_positions_kernel, (unsigned)ceil_div(n, 256), 256, 0, s,
                      as<int32_t>(R.act_flag), as<int32_t>(R.act_idx), n, as<int32_t>(R.act_pos));
        CUSCAN_LAUNCH(ctx, "compact_positions_kernel");
        qpos = as<int32_t>(R.act_pos);
        rc = launch_candidates_fp32(ctx, xp, corep, labp, perm, n, d, row_keys, clo, chi, s, qpos,
                                    active);
    }
    if (rc) return rc;
    if (active > 0) {
        CUSCAN_KERNEL(row_lb_from_keys_kernel, (unsigned)ceil_div(active, 256), 256, 0, s, row_keys,
                      qpos, perm, active, as<float>(R.rowlb));
        CUSCAN_LAUNCH(ctx, "row_lb_from_keys_kernel");
    }
    if (screened_rows) *screened_rows += active;
    return CUSCAN_OK;
}

__global__ void debug_rows_kernel(const float *__restrict__ pnorm, const float *__restrict__ mnorm,
                                  int64_t n, float one_minus_cb, float abs_c, float c_a,
                                  float *__restrict__ rows) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float p = pnorm[r], m = mnorm[r];
    rows[4 * r + 0] = one_minus_cb * p - abs_c;
    rows[4 * r + 1] = one_minus_cb * p;
    rows[4 * r + 2] = c_a * m;
    rows[4 * r + 3] = m;
}

int debug_screen_tile(cuscan_ctx *ctx, ForestBuffers &b, const float *x, int64_t n, int d,
                      int operands, float *out, float *rows_out, float *chunk_out,
                      float *scale_out, cudaStream_t s) {
    RefinedBuffers &R = b.refined;
    R.have_scale = false;
    R.want_fp16 = operands == FMT_FP16;
    int rc = choose_operands(ctx, R, x, n, d, s);
    if (rc) return rc;
    if (operands == FMT_FP16 && !R.fp16)
        return fail(ctx, CUSCAN_INVALID_INPUT, "no fp16 scale for this data");
    R.split = operands == FMT_SPLIT;
    Layout L;
    if (!refined_layout(n, d, L, R.split))
        return fail(ctx, CUSCAN_CAPACITY, "shape outside the tensor-core tiling%s",
                    R.split ? " (split copies need d <= 64)" : "");
    if (scale_out) *scale_out = R.fp16 ? R.scale : 1.0f;
    rc = prep(ctx, R, L, x, n, d, nullptr, nullptr, s);
    if (!rc)
        rc = run_screen<32, MODE_KNN_LIST>(ctx, R, L, n, d, nullptr, nullptr, nullptr, nullptr, s,
                                           out, chunk_out);
    if (!rc && rows_out) {
        float ca, cb, abs_c;
        error_coefficients(d, L.d_pad, operand_format(R), R.fp16 ? R.amax_value * R.scale : R.amax_value, ca, cb, abs_c);
        CUSCAN_KERNEL(debug_rows_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, as<float>(R.pnorm),
                      as<float>(R.mnorm), n, 1.0f - cb, abs_c, ca, rows_out);
        CUSCAN_LAUNCH(ctx, "debug_rows_kernel");
    }
    if (!rc) {
        int fallbacks = 0;
        CUSCAN_CUDA(ctx, cudaMemsetAsync(R.count.ptr, 0, sizeof(int), s));
        rc = read_screen_status(ctx, R, s, fallbacks);
    }
    R.have_scale = false;
    R.split = false;
    R.fp16 = false;
    return rc;
}

}  // namespace cuscan
