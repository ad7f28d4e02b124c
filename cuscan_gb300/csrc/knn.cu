// Exact k-nearest-neighbour sweep with f32 direct differences (the "plain" arithmetic).
//
// Semantics follow exact_kernel (crates/cuscan-common/src/kernels/neighbors.rs:17-76): every
// squared distance is acc = fmaf(q_f - r_f, q_f - r_f, acc) over features in order, rows are
// ordered by (distance, id), self is excluded by global id, empty slots hold (pad, nr).
//
// Layout: one thread owns one query row (its features staged once in shared memory as
// [feature][query] so the per-feature reads are conflict free); reference rows stream through
// a double-buffered shared tile [feature][RT] filled with 4-byte cp.async copies, and each
// thread keeps RT running distances in registers. Per feature and per 4 references that is one
// broadcast 16-byte shared load, four FADD and four FFMA. The running top-K list lives in
// registers and is updated with a fully unrolled predicated insertion; after the first few
// tiles almost every candidate fails the threshold test, so the list costs one compare per
// pair. When there are too few query blocks to fill the 152 SMs the reference range is split
// across blocks and the partial lists are merged by a second kernel.
#include <limits>

#include "forest.cuh"

namespace cuscan {
namespace {

constexpr int QB = 128;  // queries (threads) per block
constexpr int RT = 32;   // references per shared tile
constexpr int RTP = 36;  // padded tile row (keeps 16-byte alignment, spreads store banks)

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

// Copy reference rows [r0, r0+RT) into tile[f*RTP + r] (zero fill past nr).
__device__ __forceinline__ void load_ref_tile(float *tile, const float *ref, int64_t nr, int d,
                                              int64_t r0) {
    const int total = RT * d;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int r = e / d;
        int f = e - r * d;
        int64_t row = r0 + r;
        bool valid = row < nr;
        const float *src = valid ? ref + row * (int64_t)d + f : ref;
        cp_async4(&tile[f * RTP + r], src, valid);
    }
}

// Sorted register list insertion: (x, j) is known to beat slot K-1.
template <int K>
__device__ __forceinline__ void list_insert(float (&ld)[K], int (&li)[K], float x, int j) {
#pragma unroll
    for (int s = K - 1; s >= 0; --s) {
        bool here = knn_better(x, j, ld[s], li[s]);
        bool prev = (s > 0) ? knn_better(x, j, ld[s > 0 ? s - 1 : 0], li[s > 0 ? s - 1 : 0]) : false;
        if (here) {
            if (prev) {
                ld[s] = ld[s - 1 < 0 ? 0 : s - 1];
                li[s] = li[s - 1 < 0 ? 0 : s - 1];
            } else {
                ld[s] = x;
                li[s] = j;
            }
        }
    }
}

// One block: QB query rows [q0, q0 + QB) x reference rows [r_begin, r_end). Writes the K-best
// list of each query (first k entries) to out_ids/out_dist rows of width k, at split * stride
// (partial lists when split); with stride 0 a query qi goes to row qmap[qi] when qmap is set.
template <int K>
__device__ __forceinline__ void knn_block(
    const float *__restrict__ query, int64_t nq, const float *__restrict__ ref, int64_t nr, int d,
    int k, int exclude_self, int64_t query_offset, float pad, int64_t q0, int64_t r_begin,
    int64_t r_end, int32_t *__restrict__ out_ids, float *__restrict__ out_dist,
    int64_t out_split_stride, int64_t split, const int32_t *__restrict__ qmap, float *smem) {
    float *qs = smem;                         // [d][QB]
    float *tiles = smem + (size_t)d * QB;     // 2 x [d][RTP]
    const int tid = threadIdx.x;
    const int64_t qi = q0 + tid;

    // stage this block's queries transposed (qmap selects a subset of query rows)
    for (int e = tid; e < QB * d; e += QB) {
        int q = e / d;
        int f = e - q * d;
        int64_t row = q0 + q;
        int64_t src = row < nq ? (qmap ? (int64_t)qmap[row] : row) : 0;
        qs[f * QB + q] = row < nq ? query[src * (int64_t)d + f] : 0.0f;
    }

    float ld[K];
    int li[K];
#pragma unroll
    for (int s = 0; s < K; ++s) {
        ld[s] = pad;
        li[s] = (int)nr;
    }
    const int64_t self =
        exclude_self ? (qmap ? (qi < nq ? (int64_t)qmap[qi] : -1) : query_offset + qi) : -1;

    const int tile_floats = d * RTP;
    int buf = 0;
    if (r_begin < r_end) {
        load_ref_tile(tiles, ref, r_end, d, r_begin);
        cp_async_commit();
    }
    for (int64_t r0 = r_begin; r0 < r_end; r0 += RT) {
        const int64_t next = r0 + RT;
        if (next < r_end) {
            load_ref_tile(tiles + (buf ^ 1) * tile_floats, ref, r_end, d, next);
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
            const int64_t j = r0 + r;
            const float x = acc[r];
            if (j < r_end && j != self && knn_better(x, (int)j, ld[K - 1], li[K - 1]))
                list_insert<K>(ld, li, x, (int)j);
        }
        __syncthreads();
        buf ^= 1;
    }
    if (qi < nq) {
        // partial lists (split > 1) stay compact; final rows go to their mapped row
        const int64_t orow = (qmap && out_split_stride == 0) ? (int64_t)qmap[qi] : qi;
        int32_t *oi = out_ids + split * out_split_stride + orow * k;
        float *od = out_dist + split * out_split_stride + orow * k;
#pragma unroll
        for (int s = 0; s < K; ++s) {
            if (s < k) {
                oi[s] = li[s];
                od[s] = ld[s];
            }
        }
    }
}

template <int K>
__global__ void __launch_bounds__(QB) knn_fp32_kernel(
    const float *__restrict__ query, int64_t nq, const float *__restrict__ ref, int64_t nr, int d,
    int k, int exclude_self, int64_t query_offset, float pad, int64_t ref_chunk,
    int32_t *__restrict__ out_ids, float *__restrict__ out_dist, int64_t out_split_stride,
    const int32_t *__restrict__ qmap) {
    extern __shared__ __align__(16) float smem[];
    const int64_t r_begin = (int64_t)blockIdx.y * ref_chunk;
    int64_t r_end = r_begin + ref_chunk;
    if (r_end > nr) r_end = nr;
    knn_block<K>(query, nq, ref, nr, d, k, exclude_self, query_offset, pad,
                 (int64_t)blockIdx.x * QB, r_begin, r_end, out_ids, out_dist, out_split_stride,
                 (int64_t)blockIdx.y, qmap, smem);
}

// Packed fits: fit blockIdx.z, query block blockIdx.x, reference chunk blockIdx.y of `splits`
// (the self-kNN of launch_exact_knn_fp32: squared distances, self excluded, +inf padding).
// Fits with k > K take the per-fit launch instead.
template <int K>
__global__ void __launch_bounds__(QB) pack_knn_kernel(const PackFit *__restrict__ fits,
                                                      int splits) {
    extern __shared__ __align__(16) float smem[];
    const PackFit &f = fits[blockIdx.z];
    const int64_t n = f.n, q0 = (int64_t)blockIdx.x * QB;
    const int k = f.k;
    if (k > K || q0 >= n) return;
    const int64_t chunk = ceil_div(ceil_div(n, (int64_t)splits), (int64_t)RT) * RT;
    const int64_t r_begin = (int64_t)blockIdx.y * chunk;
    const int64_t r_end = r_begin + chunk < n ? r_begin + chunk : n;
    if (splits > 1)
        knn_block<K>(f.x, n, f.x, n, f.d, k, 1, 0, CUSCAN_INF, q0, r_begin, r_end, f.part_ids,
                     f.part_dist, n * k, (int64_t)blockIdx.y, nullptr, smem);
    else
        knn_block<K>(f.x, n, f.x, n, f.d, k, 1, 0, CUSCAN_INF, q0, r_begin, r_end, f.ids, f.dsq,
                     0, 0, nullptr, smem);
}

// Merge `splits` sorted partial lists of query q into the final top-k (row orow).
template <int K>
__device__ __forceinline__ void knn_merge_row(const int32_t *__restrict__ part_ids,
                                              const float *__restrict__ part_dist, int64_t q,
                                              int64_t orow, int k, int splits,
                                              int64_t split_stride, float pad, int64_t nr,
                                              int squared, int32_t *__restrict__ ids,
                                              float *__restrict__ dist) {
    float ld[K];
    int li[K];
#pragma unroll
    for (int s = 0; s < K; ++s) {
        ld[s] = pad;
        li[s] = (int)nr;
    }
    for (int sp = 0; sp < splits; ++sp) {
        const int32_t *pi = part_ids + sp * split_stride + q * k;
        const float *pd = part_dist + sp * split_stride + q * k;
        for (int s = 0; s < k; ++s) {
            float x = pd[s];
            int j = pi[s];
            if (knn_better(x, j, ld[K - 1], li[K - 1])) list_insert<K>(ld, li, x, j);
        }
    }
#pragma unroll
    for (int s = 0; s < K; ++s) {
        if (s < k) {
            ids[orow * k + s] = li[s];
            float x = ld[s];
            dist[orow * k + s] = squared ? x : sqrtf(x);
        }
    }
}

template <int K>
__global__ void knn_merge_kernel(const int32_t *__restrict__ part_ids,
                                 const float *__restrict__ part_dist, int64_t nq, int k,
                                 int splits, int64_t split_stride, float pad, int64_t nr,
                                 int squared, int32_t *__restrict__ ids, float *__restrict__ dist,
                                 const int32_t *__restrict__ qmap) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    knn_merge_row<K>(part_ids, part_dist, q, qmap ? (int64_t)qmap[q] : q, k, splits, split_stride,
                     pad, nr, squared, ids, dist);
}

// Packed fits: the partial lists of fit blockIdx.y merged into its kNN lists.
template <int K>
__global__ void pack_knn_merge_kernel(const PackFit *__restrict__ fits, int splits) {
    const PackFit &f = fits[blockIdx.y];
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f.k > K || q >= f.n) return;
    knn_merge_row<K>(f.part_ids, f.part_dist, q, q, f.k, splits, f.n * f.k, CUSCAN_INF, f.n, 1,
                     f.ids, f.dsq);
}

__global__ void sqrt_rows_kernel(float *dist, int64_t count) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) dist[i] = sqrtf(dist[i]);
}

// General k: one thread per query keeps its list in the output row in global memory,
// exactly like the reference's serial kernel (used for k > 32).
__global__ void __launch_bounds__(QB) knn_fp32_wide_kernel(
    const float *__restrict__ query, int64_t nq, const float *__restrict__ ref, int64_t nr, int d,
    int k, int exclude_self, int64_t query_offset, float pad, int32_t *__restrict__ ids,
    float *__restrict__ dist) {
    extern __shared__ __align__(16) float smem[];
    float *qs = smem;
    float *tile = smem + (size_t)d * QB;
    const int tid = threadIdx.x;
    const int64_t q0 = (int64_t)blockIdx.x * QB;
    const int64_t qi = q0 + tid;
    for (int e = tid; e < QB * d; e += QB) {
        int q = e / d;
        int f = e - q * d;
        int64_t row = q0 + q;
        qs[f * QB + q] = row < nq ? query[row * (int64_t)d + f] : 0.0f;
    }
    int32_t *li = ids + (qi < nq ? qi : 0) * (int64_t)k;
    float *ld = dist + (qi < nq ? qi : 0) * (int64_t)k;
    if (qi < nq)
        for (int s = 0; s < k; ++s) {
            li[s] = (int32_t)nr;
            ld[s] = pad;
        }
    float worst_d = pad;
    int worst_i = (int)nr;
    const int64_t self = exclude_self ? query_offset + qi : -1;
    for (int64_t r0 = 0; r0 < nr; r0 += RT) {
        __syncthreads();
        load_ref_tile(tile, ref, nr, d, r0);
        cp_async_commit();
        cp_async_wait<0>();
        __syncthreads();
        float acc[RT];
#pragma unroll
        for (int r = 0; r < RT; ++r) acc[r] = 0.0f;
        for (int f = 0; f < d; ++f) {
            const float qv = qs[f * QB + tid];
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
        if (qi < nq) {
            for (int r = 0; r < RT; ++r) {
                const int64_t j = r0 + r;
                const float x = acc[r];
                if (j >= nr || j == self || !knn_better(x, (int)j, worst_d, worst_i)) continue;
                int slot = k - 1;
                while (slot > 0 && knn_better(x, (int)j, ld[slot - 1], li[slot - 1])) {
                    li[slot] = li[slot - 1];
                    ld[slot] = ld[slot - 1];
                    --slot;
                }
                li[slot] = (int32_t)j;
                ld[slot] = x;
                worst_d = ld[k - 1];
                worst_i = li[k - 1];
            }
        }
    }
}

// Split the reference range when the query blocks alone cannot fill the GPU: `splits` CTAs per
// query block, each over `chunk` references.
void knn_split_plan(const cuscan_ctx *ctx, int64_t nq, int64_t nr, int64_t &splits,
                    int64_t &chunk) {
    const int64_t qblocks = ceil_div(nq, QB);
    splits = 1;
    const int64_t target = 2 * (int64_t)ctx->sm_count;
    if (qblocks < target) splits = ceil_div(target, qblocks);
    const int64_t max_splits = ceil_div(nr, (int64_t)RT * 8);
    if (splits > max_splits) splits = max_splits;
    if (splits > 1024) splits = 1024;
    if (splits < 1) splits = 1;
    chunk = ceil_div(ceil_div(nr, splits), RT) * RT;
    splits = ceil_div(nr, chunk);
}

template <int K>
int run_knn(cuscan_ctx *ctx, const float *query, int64_t nq, const float *ref, int64_t nr, int d,
            int k, int exclude_self, int64_t query_offset, int squared, int32_t *ids, float *dist,
            cudaStream_t s, Buffer &scratch_ids, Buffer &scratch_dist, const int32_t *qmap) {
    const float pad = squared ? std::numeric_limits<float>::infinity() : 3.40282346638528859812e+38f;
    const int64_t qblocks = ceil_div(nq, QB);
    int64_t splits = 1, chunk = 0;
    knn_split_plan(ctx, nq, nr, splits, chunk);
    const size_t smem = ((size_t)d * QB + 2 * (size_t)d * RTP) * sizeof(float);
    if (int rc = allow_dynamic_smem(ctx, knn_fp32_kernel<K>, smem)) return rc;
    dim3 grid((unsigned)qblocks, (unsigned)splits);
    if (splits == 1) {
        CUSCAN_KERNEL(knn_fp32_kernel<K>, grid, QB, smem, s, query, nq, ref, nr, d, k,
                      exclude_self, query_offset, pad, chunk, ids, dist, 0, qmap);
        CUSCAN_LAUNCH(ctx, "knn_fp32_kernel");
        if (!squared && nq * k > 0) {
            if (qmap) return fail(ctx, CUSCAN_INVALID_INPUT, "row-subset kNN is squared only");
            CUSCAN_KERNEL(sqrt_rows_kernel, (unsigned)ceil_div(nq * k, 256), 256, 0, s, dist, nq * k);
            CUSCAN_LAUNCH(ctx, "sqrt_rows_kernel");
        }
        return CUSCAN_OK;
    }
    const int64_t stride = nq * k;
    int rc = ensure(ctx, scratch_ids, (size_t)(stride * splits) * sizeof(int32_t), "kNN partial ids");
    if (rc) return rc;
    rc = ensure(ctx, scratch_dist, (size_t)(stride * splits) * sizeof(float), "kNN partial distances");
    if (rc) return rc;
    CUSCAN_KERNEL(knn_fp32_kernel<K>, grid, QB, smem, s, query, nq, ref, nr, d, k, exclude_self,
                  query_offset, pad, chunk, as<int32_t>(scratch_ids), as<float>(scratch_dist),
                  stride, qmap);
    CUSCAN_LAUNCH(ctx, "knn_fp32_kernel");
    CUSCAN_KERNEL(knn_merge_kernel<K>, (unsigned)ceil_div(nq, 128), 128, 0, s,
                  as<int32_t>(scratch_ids), as<float>(scratch_dist), nq, k, (int)splits, stride,
                  pad, nr, squared, ids, dist, qmap);
    CUSCAN_LAUNCH(ctx, "knn_merge_kernel");
    return CUSCAN_OK;
}

}  // namespace

size_t exact_knn_scratch_elems(const cuscan_ctx *ctx, int64_t nq, int64_t nr, int k) {
    int64_t splits = 1, chunk = 0;
    knn_split_plan(ctx, nq, nr, splits, chunk);
    return splits > 1 ? (size_t)(nq * k * splits) : 0;
}

int launch_exact_knn_fp32(cuscan_ctx *ctx, const float *query, int64_t nq, const float *ref,
                          int64_t nr, int d, int k, int exclude_self, int64_t query_offset,
                          int squared, int32_t *ids, float *dist, cudaStream_t s,
                          Buffer &scratch_ids, Buffer &scratch_dist, const int32_t *qmap) {
    if (nq == 0) return CUSCAN_OK;
    const size_t smem_needed = ((size_t)d * QB + 2 * (size_t)d * RTP) * sizeof(float);
    if (smem_needed > 200 * 1024)
        return fail(ctx, CUSCAN_CAPACITY,
                    "feature count %d exceeds the shared-memory staging limit of the kNN kernel "
                    "(at most 256 features)", d);
    if (k == 1)  // nearest row only (the cell assignment of the bf16-refined fits)
        return run_knn<1>(ctx, query, nq, ref, nr, d, k, exclude_self, query_offset, squared, ids,
                          dist, s, scratch_ids, scratch_dist, qmap);
    if (k <= 8)
        return run_knn<8>(ctx, query, nq, ref, nr, d, k, exclude_self, query_offset, squared, ids,
                          dist, s, scratch_ids, scratch_dist, qmap);
    if (k <= 16)
        return run_knn<16>(ctx, query, nq, ref, nr, d, k, exclude_self, query_offset, squared,
                           ids, dist, s, scratch_ids, scratch_dist, qmap);
    if (k <= 32)
        return run_knn<32>(ctx, query, nq, ref, nr, d, k, exclude_self, query_offset, squared,
                           ids, dist, s, scratch_ids, scratch_dist, qmap);
    if (qmap) return fail(ctx, CUSCAN_CAPACITY, "row-subset kNN supports k <= 32");
    const float pad = squared ? std::numeric_limits<float>::infinity() : 3.40282346638528859812e+38f;
    const size_t smem = ((size_t)d * QB + (size_t)d * RTP) * sizeof(float);
    if (int rc = allow_dynamic_smem(ctx, knn_fp32_wide_kernel, smem)) return rc;
    CUSCAN_KERNEL(knn_fp32_wide_kernel, (unsigned)ceil_div(nq, QB), QB, smem, s,
        query, nq, ref, nr, d, k, exclude_self, query_offset, pad, ids, dist);
    CUSCAN_LAUNCH(ctx, "knn_fp32_wide_kernel");
    if (!squared) {
        CUSCAN_KERNEL(sqrt_rows_kernel, (unsigned)ceil_div(nq * k, 256), 256, 0, s, dist, nq * k);
        CUSCAN_LAUNCH(ctx, "sqrt_rows_kernel");
    }
    return CUSCAN_OK;
}

template <int K>
static int run_pack_knn(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max,
                        int d_max, int splits, cudaStream_t s, int64_t &launches) {
    const size_t smem = ((size_t)d_max * QB + 2 * (size_t)d_max * RTP) * sizeof(float);
    if (int rc = allow_dynamic_smem(ctx, pack_knn_kernel<K>, smem)) return rc;
    dim3 grid((unsigned)ceil_div(n_max, QB), (unsigned)splits, (unsigned)count);
    CUSCAN_KERNEL(pack_knn_kernel<K>, grid, QB, smem, s, fits, splits);
    ++launches;
    if (splits > 1) {
        dim3 mg((unsigned)ceil_div(n_max, 128), (unsigned)count);
        CUSCAN_KERNEL(pack_knn_merge_kernel<K>, mg, 128, 0, s, fits, splits);
        ++launches;
    }
    CUSCAN_LAUNCH(ctx, "pack_knn_kernel");
    return CUSCAN_OK;
}

int launch_pack_knn(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max, int d_max,
                    int k_max, int splits, cudaStream_t s, int64_t &launches) {
    if (((size_t)d_max * QB + 2 * (size_t)d_max * RTP) * sizeof(float) > 200 * 1024)
        return fail(ctx, CUSCAN_CAPACITY, "feature count %d exceeds the kNN staging limit", d_max);
    if (k_max <= 8) return run_pack_knn<8>(ctx, fits, count, n_max, d_max, splits, s, launches);
    if (k_max <= 16) return run_pack_knn<16>(ctx, fits, count, n_max, d_max, splits, s, launches);
    return run_pack_knn<32>(ctx, fits, count, n_max, d_max, splits, s, launches);
}

}  // namespace cuscan
