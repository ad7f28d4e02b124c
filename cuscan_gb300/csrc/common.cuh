// Shared definitions for the cuscan_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <cstdarg>
#include <string>

#include "cuscan_gb300.h"

#define CUSCAN_INF __int_as_float(0x7f800000)

namespace cuscan {

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs; grids are sized in multiples of this.

// Device workspace owned by a context; grows on demand and is reused across calls.
struct Buffer {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct FitWorkspace;  // defined in workspace.cuh

}  // namespace cuscan

struct cuscan_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int kind = 0;
    char err[1024] = {0};
    int sm_count = cuscan::kSMs;
    cuscan::FitWorkspace *fit = nullptr;
};

namespace cuscan {

// Record an error on the context and return its status code.
inline int fail(cuscan_ctx *ctx, int kind, const char *fmt, ...) {
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
        va_end(ap);
        ctx->kind = kind;
    }
    return kind;
}

inline void clear_error(cuscan_ctx *ctx) {
    if (ctx) {
        ctx->err[0] = 0;
        ctx->kind = 0;
    }
}

inline int cuda_fail(cuscan_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(ctx, CUSCAN_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(ctx, CUSCAN_BACKEND_UNAVAILABLE, "%s: %s", what, cudaGetErrorString(e));
}

#define CUSCAN_CUDA(ctx, call)                                   \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return ::cuscan::cuda_fail((ctx), _e, #call); \
    } while (0)

#define CUSCAN_LAUNCH(ctx, what)                                  \
    do {                                                          \
        cudaError_t _e = cudaGetLastError();                      \
        if (_e != cudaSuccess) return ::cuscan::cuda_fail((ctx), _e, what); \
    } while (0)

// Raise a kernel's dynamic shared-memory cap to the device's opt-in limit. Every call sets the
// same value, so a fit running on another host thread cannot lower the cap between this call
// and a launch that needs more (the attribute belongs to the kernel, not to a stream).
template <class Kernel>
inline int allow_dynamic_smem(cuscan_ctx *ctx, Kernel kernel, size_t bytes) {
    int optin = 0;
    CUSCAN_CUDA(ctx, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                            ctx->device));
    cudaFuncAttributes attr;
    CUSCAN_CUDA(ctx, cudaFuncGetAttributes(&attr, (const void *)kernel));
    const size_t cap = (size_t)optin - attr.sharedSizeBytes;
    if (bytes > cap)
        return fail(ctx, CUSCAN_CAPACITY, "a kernel needs %zu bytes of shared memory, the device "
                    "allows %zu", bytes, cap);
    CUSCAN_CUDA(ctx, cudaFuncSetAttribute((const void *)kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
    return CUSCAN_OK;
}

// Number of kernels this library has launched in the process (reported by
// cuscan_launch_count so callers can account for every launch of a timed region).
inline std::atomic<long long> &launch_counter() {
    static std::atomic<long long> counter{0};
    return counter;
}

// Launch a kernel and count it.
#define CUSCAN_KERNEL(kernel, grid, block, smem, stream, ...)                  \
    do {                                                                        \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);             \
        ::cuscan::launch_counter().fetch_add(1, std::memory_order_relaxed);     \
    } while (0)

inline cudaStream_t pick_stream(cuscan_ctx *ctx, void *stream) {
    return stream ? (cudaStream_t)stream : ctx->stream;
}

// Ensure a buffer holds at least `bytes`; contents are not preserved.
inline int ensure(cuscan_ctx *ctx, Buffer &b, size_t bytes, const char *what) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return CUSCAN_OK;
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, CUSCAN_MEMORY, "device allocation of %zu bytes for %s failed: %s", bytes,
                    what, cudaGetErrorString(e));
    }
    b.bytes = bytes;
    return CUSCAN_OK;
}

inline void release(Buffer &b) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

template <class T>
inline T *as(Buffer &b) {
    return reinterpret_cast<T *>(b.ptr);
}

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------------------

// Lexicographic "candidate (d, j) beats slot (ds, js)" used by every top-k list: smaller
// squared distance first, lower id on ties (neighbors.rs:51,56).
__device__ __forceinline__ bool knn_better(float d, int j, float ds, int js) {
    return d < ds || (d == ds && (unsigned)j < (unsigned)js);
}

// Non-negative float bit patterns order like their values; -0 is folded onto +0 so that a
// key comparison matches the reference's canonical weight key (component_reduce.rs:69-74).
__device__ __forceinline__ uint32_t weight_key_bits(float w) {
    uint32_t b = __float_as_uint(w);
    return (b & 0x7fffffffu) == 0 ? 0u : b;
}

// NaN or negative non-zero weight (component_reduce.rs:21-25).
__device__ __forceinline__ bool numerical_bits(uint32_t bits) {
    uint32_t magnitude = bits & 0x7fffffffu;
    return ((bits & 0x80000000u) != 0 && magnitude != 0) || magnitude > 0x7f800000u;
}

}  // namespace cuscan

// Kernel launchers shared between translation units.
namespace cuscan {

// kNN (knn.cu). All pointers are device pointers. With qmap (squared, k <= 32 only), query row
// i is row qmap[i] of `query`, excludes reference qmap[i] as itself and is written to output
// row qmap[i].
int launch_exact_knn_fp32(cuscan_ctx *ctx, const float *query, int64_t nq, const float *ref,
                          int64_t nr, int d, int k, int exclude_self, int64_t query_offset,
                          int squared, int32_t *ids, float *dist, cudaStream_t s,
                          Buffer &scratch_ids, Buffer &scratch_dist,
                          const int32_t *qmap = nullptr);

// Elements of each split-kNN partial list buffer (ids and distances) that launch_exact_knn_fp32
// uses for nq queries against nr references (0 when the reference range is not split).
size_t exact_knn_scratch_elems(const cuscan_ctx *ctx, int64_t nq, int64_t nr, int k);

// Borůvka candidates (boruvka.cu): per-row 64-bit keys (weight bits << 32 | reference id),
// minimised atomically into row_keys[] (which the caller fills with ~0 first). Rows are
// positions in `data`; ids maps a position to the original id used for tie-breaking and
// output (NULL = identity). tile_lo/tile_hi are scratch of ceil(n/32) ints each.
// With qmap, only the nq query positions qmap[0..nq) are scanned (against all n positions);
// without it, the positions [qoff, qoff + nq) (all n positions when nq and qoff are 0).
int launch_candidates_fp32(cuscan_ctx *ctx, const float *data, const float *core_sq,
                           const int32_t *labels, const int32_t *ids, int64_t n, int d,
                           unsigned long long *row_keys, int32_t *tile_lo, int32_t *tile_hi,
                           cudaStream_t s, const int32_t *qmap = nullptr, int64_t nq = 0,
                           int64_t qoff = 0);
// Label range (min, max) of every 32-row tile of `labels`.
int launch_tile_ranges(cuscan_ctx *ctx, const int32_t *labels, int64_t n, int32_t *tile_lo,
                       int32_t *tile_hi, cudaStream_t s);
int launch_fill_u64(cuscan_ctx *ctx, unsigned long long *p, int64_t n, unsigned long long v,
                    cudaStream_t s);
int launch_keys_to_candidates(cuscan_ctx *ctx, const unsigned long long *keys, int64_t n,
                              float *w, int32_t *dst, cudaStream_t s);
int launch_component_reduce(cuscan_ctx *ctx, const float *weights, const int32_t *indices,
                            const int32_t *members, const int32_t *starts, const int32_t *ends,
                            const int32_t *partial_offsets, int64_t n, int64_t p, int64_t c,
                            float *win_w, int32_t *win_meta, Buffer &scratch, cudaStream_t s);

}  // namespace cuscan
