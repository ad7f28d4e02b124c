// Borůvka round kernels with f32 direct differences (the "plain" arithmetic), and the CSR
// component reduction of the reference's HdbscanOps::component_reduce.
//
// Candidate rule (crates/hdbscan/src/kernels/boruvka.rs:68-140): for row i, the
// lexicographically smallest (w_ij, j) with w_ij = max(max(d2_ij, core_i), core_j) over rows j
// of another component. Here a (w, j) pair is packed into one 64-bit key
// (canonical weight bits << 32 | j): for non-negative weights the unsigned key order is exactly
// that lexicographic order, so partial results from any split of the reference range combine
// with a single atomicMin.
//
// The fused fit path calls the kernel on component-sorted rows. A (query block, reference
// tile) pair whose rows all carry one label holds only same-component pairs and is skipped
// before any distance is computed; tile label ranges are precomputed per 32-row tile.
#include <mutex>

#include "forest.cuh"

namespace cuscan {
namespace {

constexpr int QB = 128;
constexpr int RT = 32;
constexpr int RTP = 36;

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem, bool valid) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    int src_size = valid ? 4 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem),
                 "r"(src_size));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// Label range of each RT-row tile.
__global__ void tile_range_kernel(const int32_t *__restrict__ labels, int64_t n,
                                  int32_t *__restrict__ lo, int32_t *__restrict__ hi) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t tiles = ceil_div(n, RT);
    if (t >= tiles) return;
    int64_t a = t * RT, b = a + RT < n ? a + RT : n;
    int32_t mn = labels[a], mx = labels[a];
    for (int64_t i = a + 1; i < b; ++i) {
        int32_t l = labels[i];
        mn = l < mn ? l : mn;
        mx = l > mx ? l : mx;
    }
    lo[t] = mn;
    hi[t] = mx;
}

__device__ __forceinline__ void load_tile(float *tile, float *core_t, int32_t *lab_t,
                                          int32_t *id_t, const float *data, const float *core,
                                          const int32_t *labels, const int32_t *ids, int64_t n,
                                          int d, int64_t r0) {
    const int total = RT * d;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int r = e / d;
        int f = e - r * d;
        int64_t row = r0 + r;
        bool valid = row < n;
        cp_async4(&tile[f * RTP + r], valid ? data + row * (int64_t)d + f : data, valid);
    }
    if (threadIdx.x < RT) {
        int64_t row = r0 + threadIdx.x;
        bool valid = row < n;
        core_t[threadIdx.x] = valid ? core[row] : 0.0f;
        lab_t[threadIdx.x] = valid ? labels[row] : -1;
        id_t[threadIdx.x] = valid ? (ids ? ids[row] : (int32_t)row) : -1;
    }
}

// Per-tile row data of the candidate sweep, double-buffered in shared memory.
struct CandShared {
    float core_t[2][RT];
    int32_t lab_t[2][RT];
    int32_t id_t[2][RT];
    int32_t q_range[2];
};

// One block: QB query rows [q0, q0 + QB) against rows [r_begin, r_end); each query's cheapest
// cross-component key is folded into row_keys with atomicMin.
__device__ __forceinline__ void candidates_block(
    const float *__restrict__ data, const float *__restrict__ core,
    const int32_t *__restrict__ labels, const int32_t *__restrict__ ids, int64_t n, int d,
    const int32_t *__restrict__ tile_lo, const int32_t *__restrict__ tile_hi, int64_t q0,
    int64_t r_begin, int64_t r_end, unsigned long long *__restrict__ row_keys,
    const int32_t *__restrict__ qmap, int64_t nq, int64_t qoff, float *smem, CandShared &sh) {
    float *qs = smem;                       // [d][QB]
    float *tiles = smem + (size_t)d * QB;   // 2 x [d][RTP]
    float(&core_t)[2][RT] = sh.core_t;
    int32_t(&lab_t)[2][RT] = sh.lab_t;
    int32_t(&id_t)[2][RT] = sh.id_t;
    int32_t *q_range = sh.q_range;
    const int tid = threadIdx.x;
    const int64_t qi = q0 + tid;

    // query rows are positions qmap[qi] (or qoff + qi) of the same arrays
    const bool q_valid = qi < nq;
    const int64_t qpos = q_valid ? (qmap ? (int64_t)qmap[qi] : qoff + qi) : 0;
    const int32_t my_label = q_valid ? labels[qpos] : -1;
    const float my_core = q_valid ? core[qpos] : 0.0f;
    if (tid == 0) {
        q_range[0] = INT32_MAX;
        q_range[1] = INT32_MIN;
    }
    __syncthreads();
    if (q_valid) {
        atomicMin(&q_range[0], my_label);
        atomicMax(&q_range[1], my_label);
    }
    for (int e = tid; e < QB * d; e += QB) {
        int q = e / d;
        int f = e - q * d;
        int64_t row = q0 + q;
        int64_t src = row < nq ? (qmap ? (int64_t)qmap[row] : qoff + row) : 0;
        qs[f * QB + q] = row < nq ? data[src * (int64_t)d + f] : 0.0f;
    }
    __syncthreads();
    const int32_t qlo = q_range[0], qhi = q_range[1];
    const bool q_uniform = qlo == qhi;
    unsigned long long best = ~0ull;

    auto skip_tile = [&](int64_t r0) -> bool {
        int64_t t = r0 / RT;
        return q_uniform && tile_lo[t] == qlo && tile_hi[t] == qlo;
    };
    auto next_tile = [&](int64_t r0) -> int64_t {
        while (r0 < r_end && skip_tile(r0)) r0 += RT;
        return r0;
    };

    const int tile_floats = d * RTP;
    int buf = 0;
    int64_t r0 = next_tile(r_begin);
    if (r0 < r_end) {
        load_tile(tiles, core_t[0], lab_t[0], id_t[0], data, core, labels, ids, r_end, d, r0);
        cp_async_commit();
    }
    while (r0 < r_end) {
        const int64_t nxt = next_tile(r0 + RT);
        if (nxt < r_end) {
            load_tile(tiles + (buf ^ 1) * tile_floats, core_t[buf ^ 1], lab_t[buf ^ 1],
                      id_t[buf ^ 1], data, core, labels, ids, r_end, d, nxt);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const float *tile = tiles + buf * tile_floats;
        float acc[RT];
#pragma unroll
        for (int r = 0; r < RT; ++r) acc[r] = 0.0f;
        const float *qcol = qs + tid;
#pragma unroll 2
        for (int f = 0; f < d; ++f) {
            const float qv = qcol[f * QB];
            const float4 *row4 = reinterpret_cast<const float4 *>(tile + f * RTP);
#pragma unroll
            for (int r4 = 0; r4 < RT / 4; ++r4) {
                const float4 v = row4[r4];
                float t0 = qv - v.x, t1 = qv - v.y, t2 = qv - v.z, t3 = qv - v.w;
                acc[4 * r4 + 0] = __fmaf_rn(t0, t0, acc[4 * r4 + 0]);
                acc[4 * r4 + 1] = __fmaf_rn(t1, t1, acc[4 * r4 + 1]);
                acc[4 * r4 + 2] = __fmaf_rn(t2, t2, acc[4 * r4 + 2]);
                acc[4 * r4 + 3] = __fmaf_rn(t3, t3, acc[4 * r4 + 3]);
            }
        }
#pragma unroll
        for (int r = 0; r < RT; ++r) {
            const int32_t lj = lab_t[buf][r];
            if (lj >= 0 && lj != my_label) {
                float w = fmaxf(fmaxf(acc[r], my_core), core_t[buf][r]);
                if (!(w != w)) {
                    unsigned long long key =
                        ((unsigned long long)weight_key_bits(w) << 32) | (uint32_t)id_t[buf][r];
                    best = key < best ? key : best;
                }
            }
        }
        __syncthreads();
        buf ^= 1;
        r0 = nxt;
    }
    if (q_valid && best != ~0ull) {
        const int32_t out = ids ? ids[qpos] : (int32_t)qpos;
        atomicMin(&row_keys[out], best);
    }
}

__global__ void __launch_bounds__(QB) candidates_fp32_kernel(
    const float *__restrict__ data, const float *__restrict__ core,
    const int32_t *__restrict__ labels, const int32_t *__restrict__ ids, int64_t n, int d,
    const int32_t *__restrict__ tile_lo, const int32_t *__restrict__ tile_hi, int64_t ref_chunk,
    unsigned long long *__restrict__ row_keys, const int32_t *__restrict__ qmap, int64_t nq,
    int64_t qoff) {
    extern __shared__ __align__(16) float smem[];
    __shared__ CandShared sh;
    const int64_t r_begin = (int64_t)blockIdx.y * ref_chunk;
    int64_t r_end = r_begin + ref_chunk;
    if (r_end > n) r_end = n;
    candidates_block(data, core, labels, ids, n, d, tile_lo, tile_hi, (int64_t)blockIdx.x * QB,
                     r_begin, r_end, row_keys, qmap, nq, qoff, smem, sh);
}

// Packed fits: fit blockIdx.z (skipped unless its round runs), query block blockIdx.x,
// reference chunk blockIdx.y of `splits`, over the fit's component-sorted copies (the launch
// launch_candidates_fp32 makes for a fit alone).
__global__ void __launch_bounds__(QB) pack_candidates_kernel(const PackFit *__restrict__ fits,
                                                             int splits) {
    extern __shared__ __align__(16) float smem[];
    __shared__ CandShared sh;
    const PackFit &f = fits[blockIdx.z];
    const int64_t n = f.n, q0 = (int64_t)blockIdx.x * QB;
    if (q0 >= n || !*(volatile int32_t *)&f.kept_total[1]) return;
    const int64_t chunk = ceil_div(ceil_div(n, (int64_t)splits), (int64_t)RT) * RT;
    const int64_t r_begin = (int64_t)blockIdx.y * chunk;
    if (r_begin >= n) return;
    const int64_t r_end = r_begin + chunk < n ? r_begin + chunk : n;
    candidates_block(f.xp, f.corep, f.labp, f.perm, n, f.d, f.tile_lo, f.tile_hi, q0, r_begin,
                     r_end, f.row_keys, nullptr, n, 0, smem, sh);
}

__global__ void fill_u64_kernel(unsigned long long *p, int64_t n, unsigned long long v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void keys_to_candidates_kernel(const unsigned long long *__restrict__ keys, int64_t n,
                                          float *__restrict__ w, int32_t *__restrict__ dst) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long k = keys[i];
    if (k == ~0ull) {
        w[i] = CUSCAN_INF;
        dst[i] = (int32_t)n;
    } else {
        w[i] = __uint_as_float((uint32_t)(k >> 32));
        dst[i] = (int32_t)(uint32_t)k;
    }
}

// ---- CSR component reduction (component_reduce.rs semantics) ----

struct Fold {
    uint32_t key, bits, source, bad;
};

__device__ __forceinline__ void fold_take(Fold &a, const Fold &b) {
    if (b.key < a.key || (b.key == a.key && b.source < a.source)) {
        a.key = b.key;
        a.bits = b.bits;
        a.source = b.source;
    }
    a.bad = b.bad < a.bad ? b.bad : a.bad;
}

__device__ __forceinline__ Fold warp_fold(Fold v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Fold u;
        u.key = __shfl_xor_sync(0xffffffffu, v.key, o);
        u.bits = __shfl_xor_sync(0xffffffffu, v.bits, o);
        u.source = __shfl_xor_sync(0xffffffffu, v.source, o);
        u.bad = __shfl_xor_sync(0xffffffffu, v.bad, o);
        fold_take(v, u);
    }
    return v;
}

// One warp per tile of CSR positions [tile_starts[t], tile_ends[t]).
__global__ void reduce_tiles_kernel(const float *__restrict__ weights,
                                    const int32_t *__restrict__ indices,
                                    const int32_t *__restrict__ members,
                                    const int32_t *__restrict__ starts,
                                    const int32_t *__restrict__ ends, int64_t p, uint32_t n,
                                    Fold *__restrict__ partial) {
    int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    int lane = threadIdx.x & 31;
    if (t >= p) return;
    Fold acc{0xffffffffu, 0x7f800000u, n, n};
    // a malformed plan is clamped to the member array [0, n) and to member ids below n, so
    // it never reads outside the caller's buffers (a valid plan is unaffected)
    const int64_t lo = starts[t] > 0 ? starts[t] : 0;
    const int64_t hi = (int64_t)ends[t] < (int64_t)n ? (int64_t)ends[t] : (int64_t)n;
    for (int64_t pos = lo + lane; pos < hi; pos += 32) {
        uint32_t member = (uint32_t)members[pos];
        if (member >= n) continue;
        uint32_t original = __float_as_uint(weights[member]);
        int32_t destination = indices[member];
        Fold v{0xffffffffu, 0x7f800000u, n, n};
        if (numerical_bits(original) || destination >= (int32_t)n) {
            v.bad = member;
        } else if (destination >= 0) {
            v.key = (original & 0x7fffffffu) == 0 ? 0u : original;
            v.bits = original;
            v.source = member;
        }
        fold_take(acc, v);
    }
    acc = warp_fold(acc);
    if (lane == 0) partial[t] = acc;
}

// One warp per component over its tile partials; writes winner weight and 5-int metadata.
__global__ void reduce_components_kernel(const float *__restrict__ weights,
                                         const int32_t *__restrict__ indices,
                                         const int32_t *__restrict__ partial_offsets,
                                         const Fold *__restrict__ partial, int64_t c, int64_t p,
                                         uint32_t n, float *__restrict__ win_w,
                                         int32_t *__restrict__ win_meta) {
    int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    int lane = threadIdx.x & 31;
    if (s >= c) return;
    Fold acc{0xffffffffu, 0x7f800000u, n, n};
    // partials of a malformed plan outside [0, p) are not read (a valid plan is unaffected)
    const int64_t lo = partial_offsets[s] > 0 ? partial_offsets[s] : 0;
    const int64_t hi = partial_offsets[s + 1] < p ? partial_offsets[s + 1] : p;
    for (int64_t t = lo + lane; t < hi; t += 32)
        fold_take(acc, partial[t]);
    acc = warp_fold(acc);
    if (lane != 0) return;
    int32_t destination = acc.source < n ? indices[acc.source] : -1;
    int32_t kind = 0, bad_destination = -1;
    if (acc.bad < n) {
        if (numerical_bits(__float_as_uint(weights[acc.bad]))) {
            kind = 1;
        } else {
            kind = 2;
            bad_destination = indices[acc.bad];
        }
    }
    win_w[s] = __uint_as_float(acc.bits);
    int32_t *m = win_meta + s * 5;
    m[0] = acc.source < n ? (int32_t)acc.source : -1;
    m[1] = destination;
    m[2] = (int32_t)acc.bad;
    m[3] = kind;
    m[4] = bad_destination;
}

}  // namespace

int launch_tile_ranges(cuscan_ctx *ctx, const int32_t *labels, int64_t n, int32_t *tile_lo,
                       int32_t *tile_hi, cudaStream_t s) {
    const int64_t tiles = ceil_div(n, RT);
    CUSCAN_KERNEL(tile_range_kernel, (unsigned)ceil_div(tiles, 256), 256, 0, s, labels, n,
                  tile_lo, tile_hi);
    CUSCAN_LAUNCH(ctx, "tile_range_kernel");
    return CUSCAN_OK;
}

int launch_candidates_fp32(cuscan_ctx *ctx, const float *data, const float *core_sq,
                           const int32_t *labels, const int32_t *ids, int64_t n, int d,
                           unsigned long long *row_keys, int32_t *tile_lo, int32_t *tile_hi,
                           cudaStream_t s, const int32_t *qmap, int64_t nq, int64_t qoff) {
    if (!qmap && qoff == 0 && nq == 0) nq = n;
    if (nq == 0) return CUSCAN_OK;
    int rc = launch_tile_ranges(ctx, labels, n, tile_lo, tile_hi, s);
    if (rc) return rc;
    const int64_t qblocks = ceil_div(nq, QB);
    int64_t splits = 1;
    const int64_t target = 2 * (int64_t)ctx->sm_count;
    if (qblocks < target) splits = ceil_div(target, qblocks);
    const int64_t max_splits = ceil_div(n, (int64_t)RT * 8);
    if (splits > max_splits) splits = max_splits;
    if (splits > 64) splits = 64;
    if (splits < 1) splits = 1;
    int64_t chunk = ceil_div(ceil_div(n, splits), RT) * RT;
    splits = ceil_div(n, chunk);
    const size_t smem = ((size_t)d * QB + 2 * (size_t)d * RTP) * sizeof(float);
    if (smem > 200 * 1024)
        return fail(ctx, CUSCAN_CAPACITY,
                    "feature count %d exceeds the shared-memory staging limit of the Boruvka "
                    "kernel (at most 256 features)", d);
    if (int rc = allow_dynamic_smem(ctx, candidates_fp32_kernel, smem)) return rc;
    dim3 grid((unsigned)qblocks, (unsigned)splits);
    CUSCAN_KERNEL(candidates_fp32_kernel, grid, QB, smem, s, data, core_sq, labels, ids, n, d,
                  tile_lo, tile_hi, chunk, row_keys, qmap, nq, qoff);
    CUSCAN_LAUNCH(ctx, "candidates_fp32_kernel");
    return CUSCAN_OK;
}

int launch_pack_candidates(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max,
                           int d_max, int splits, cudaStream_t s) {
    const size_t smem = ((size_t)d_max * QB + 2 * (size_t)d_max * RTP) * sizeof(float);
    if (smem > 200 * 1024)
        return fail(ctx, CUSCAN_CAPACITY, "feature count %d exceeds the Boruvka staging limit",
                    d_max);
    if (int rc = allow_dynamic_smem(ctx, pack_candidates_kernel, smem)) return rc;
    dim3 grid((unsigned)ceil_div(n_max, QB), (unsigned)splits, (unsigned)count);
    CUSCAN_KERNEL(pack_candidates_kernel, grid, QB, smem, s, fits, splits);
    CUSCAN_LAUNCH(ctx, "pack_candidates_kernel");
    return CUSCAN_OK;
}

int launch_fill_u64(cuscan_ctx *ctx, unsigned long long *p, int64_t n, unsigned long long v,
                    cudaStream_t s) {
    if (n <= 0) return CUSCAN_OK;
    CUSCAN_KERNEL(fill_u64_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, p, n, v);
    CUSCAN_LAUNCH(ctx, "fill_u64_kernel");
    return CUSCAN_OK;
}

int launch_keys_to_candidates(cuscan_ctx *ctx, const unsigned long long *keys, int64_t n,
                              float *w, int32_t *dst, cudaStream_t s) {
    CUSCAN_KERNEL(keys_to_candidates_kernel, (unsigned)ceil_div(n, 256), 256, 0, s, keys, n, w, dst);
    CUSCAN_LAUNCH(ctx, "keys_to_candidates_kernel");
    return CUSCAN_OK;
}

int launch_component_reduce(cuscan_ctx *ctx, const float *weights, const int32_t *indices,
                            const int32_t *members, const int32_t *starts, const int32_t *ends,
                            const int32_t *partial_offsets, int64_t n, int64_t p, int64_t c,
                            float *win_w, int32_t *win_meta, Buffer &scratch, cudaStream_t s) {
    if (c == 0) return CUSCAN_OK;
    int rc = ensure(ctx, scratch, (size_t)(p > 0 ? p : 1) * sizeof(Fold), "component partials");
    if (rc) return rc;
    if (p > 0) {
        CUSCAN_KERNEL(reduce_tiles_kernel, (unsigned)ceil_div(p * 32, 256), 256, 0, s, 
            weights, indices, members, starts, ends, p, (uint32_t)n, as<Fold>(scratch));
        CUSCAN_LAUNCH(ctx, "reduce_tiles_kernel");
    }
    CUSCAN_KERNEL(reduce_components_kernel, (unsigned)ceil_div(c * 32, 256), 256, 0, s, 
        weights, indices, partial_offsets, as<Fold>(scratch), c, p, (uint32_t)n, win_w, win_meta);
    CUSCAN_LAUNCH(ctx, "reduce_components_kernel");
    return CUSCAN_OK;
}

// ---------------------------------------------------------------------------------------------
// Component reduction without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need this reduction: a host
// whose device memory is owned by another framework's caching pool, a real-time loop that must
// not take the implicit synchronisation of cudaMalloc/cudaFree, or a plugin that is handed
// device buffers and nothing else. For them the per-tile partial results live in a fixed
// array of static device memory that the CUDA module owns: every GPU that loads this library
// keeps NOALLOC_MAX_TILES * 16 bytes (1 MiB) for it until the process exits.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int64_t NOALLOC_MAX_TILES = 65536;  // == CUSCAN_NOALLOC_MAX_TILES in the header

static __device__ __align__(256) Fold g_noalloc_partials[NOALLOC_MAX_TILES];

// The array's address on each device. In host code the symbol is only a host-side stand-in;
// the device address is fetched once per device with that device current.
std::mutex g_noalloc_mutex;
Fold *g_noalloc_ptr[64] = {};

void set_err(char *err, size_t len, const char *msg) {
    if (err && len) {
        snprintf(err, len, "%s", msg);
    }
}

}  // namespace

}  // namespace cuscan

extern "C" int cuscan_component_reduce_noalloc(
    const float *weights, const int32_t *indices, const int32_t *members,
    const int32_t *tile_starts, const int32_t *tile_ends, const int32_t *partial_offsets,
    int64_t n, int64_t p, int64_t c, float *win_weights, int32_t *win_meta, void *stream,
    char *err, size_t err_len) {
    using namespace cuscan;
    if (n < 0 || p < 0 || c < 0 || c > n || p > n) {
        set_err(err, err_len, "component_reduce_noalloc received inconsistent sizes");
        return CUSCAN_INVALID_INPUT;
    }
    if (n > INT32_MAX) {
        set_err(err, err_len, "component member index exceeds the supported integer range");
        return CUSCAN_OVERFLOW;
    }
    if (p > NOALLOC_MAX_TILES) {
        char msg[160];
        snprintf(msg, sizeof(msg),
                 "component_reduce_noalloc supports at most %lld tiles (got %lld); use "
                 "cuscan_component_reduce for larger plans",
                 (long long)NOALLOC_MAX_TILES, (long long)p);
        set_err(err, err_len, msg);
        return CUSCAN_CAPACITY;
    }
    if (c == 0) return CUSCAN_OK;
    int device = -1;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess || device < 0 || device >= 64) {
        cudaGetLastError();
        set_err(err, err_len, "no usable current CUDA device");
        return CUSCAN_BACKEND_UNAVAILABLE;
    }
    Fold *scratch = nullptr;
    {
        // first call on a device: resolve the static array's device address (done once)
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[device]) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_partials);
            if (e != cudaSuccess || !ptr) {
                cudaGetLastError();
                set_err(err, err_len, "cudaGetSymbolAddress of the static partials failed");
                return CUSCAN_BACKEND_UNAVAILABLE;
            }
            g_noalloc_ptr[device] = static_cast<Fold *>(ptr);
        }
        scratch = g_noalloc_ptr[device];
    }
    // every tile writes its own partial, so no clearing of the shared array is needed
    cudaStream_t s = (cudaStream_t)stream;
    if (p > 0) {
        CUSCAN_KERNEL(reduce_tiles_kernel, (unsigned)ceil_div(p * 32, 256), 256, 0, s, weights,
                      indices, members, tile_starts, tile_ends, p, (uint32_t)n, scratch);
    }
    CUSCAN_KERNEL(reduce_components_kernel, (unsigned)ceil_div(c * 32, 256), 256, 0, s, weights,
                  indices, partial_offsets, scratch, c, p, (uint32_t)n, win_weights, win_meta);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_err(err, err_len, cudaGetErrorString(e));
        return CUSCAN_BACKEND_UNAVAILABLE;
    }
    return CUSCAN_OK;
}
