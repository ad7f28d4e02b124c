// C ABI of cuscan_gb300: context management, the three backend operations and the fused
// device-resident fit core.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "forest.cuh"
#include "workspace.cuh"

namespace cuscan {

// Refined (bf16 tensor-core) sweeps; defined in refined.cu.
int refined_available();
int launch_knn_refined(cuscan_ctx *ctx, ForestBuffers &b, const float *x, int64_t n, int d, int k,
                       int32_t *ids, float *dist, cudaStream_t s, int64_t *refined_rows,
                       int64_t *fallback_rows, int64_t *rescreened_rows);
int launch_candidates_refined(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int d,
                              const int32_t *knn_ids, const float *knn_sq, int k,
                              const float *core, const int32_t *label, cudaStream_t s,
                              int64_t *fallback_rows);
int launch_candidates_exact_rows(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int d,
                                 const int32_t *knn_ids, const float *knn_sq, int k,
                                 const float *core, const int32_t *label, cudaStream_t s,
                                 int64_t *screened_rows);
int debug_screen_tile(cuscan_ctx *ctx, ForestBuffers &b, const float *x, int64_t n, int d,
                      int operands, float *out, float *rows_out, float *chunk_out,
                      float *scale_out, cudaStream_t s);
int refined_operand_format(const ForestBuffers &b);
size_t refined_workspace_bytes(int64_t n, int d, int k);

// Every device buffer a context holds.
static int workspace_buffers(FitWorkspace *f, Buffer **out) {
    Buffer *own[] = {&f->x, &f->ids, &f->dsq, &f->core, &f->label, &f->src, &f->dst, &f->w,
                     &f->op_keys, &f->op_tiles_lo, &f->op_tiles_hi, &f->op_partials,
                     &f->op_knn_ids, &f->op_knn_dist, &f->pred_q, &f->pred_ids,
                     &f->pred_dist};
    const int n_own = (int)(sizeof(own) / sizeof(own[0]));
    static_assert(sizeof(own) / sizeof(own[0]) == kOwnBufferCount, "buffer list");
    for (int i = 0; i < n_own; ++i) out[i] = own[i];
    return n_own + forest_buffers(f->forest, out + n_own);
}
constexpr int kWorkspaceBufferCount = kOwnBufferCount + kForestBufferCount;

}  // namespace cuscan

using namespace cuscan;

extern "C" {

const char *cuscan_version(void) { return "cuscan_gb300 0.1.0 (sm_103a)"; }

int64_t cuscan_launch_count(void) { return (int64_t)launch_counter().load(); }

int cuscan_ctx_create(int device, cuscan_ctx **out) {
    if (!out) return CUSCAN_INVALID_INPUT;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return CUSCAN_BACKEND_UNAVAILABLE;
    }
    if (device < 0 || device >= count) return CUSCAN_BACKEND_UNAVAILABLE;
    cuscan_ctx *ctx = new cuscan_ctx();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return CUSCAN_BACKEND_UNAVAILABLE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) {
        ctx->sm_count = prop.multiProcessorCount;
        if (prop.major < 10) {
            cudaStreamDestroy(ctx->stream);
            delete ctx;
            return CUSCAN_BACKEND_UNAVAILABLE;
        }
    }
    ctx->fit = new FitWorkspace();
    if (cudaMallocHost(&ctx->fit->host_status, sizeof(DevStatus)) != cudaSuccess) {
        cudaGetLastError();
        cuscan_ctx_destroy(ctx);
        return CUSCAN_MEMORY;
    }
    for (auto &ev : ctx->fit->ev) cudaEventCreate(&ev);
    *out = ctx;
    return CUSCAN_OK;
}

void cuscan_ctx_destroy(cuscan_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->fit) {
        FitWorkspace *f = ctx->fit;
        Buffer *all[kWorkspaceBufferCount];
        const int count = workspace_buffers(f, all);
        for (int i = 0; i < count; ++i) release(*all[i]);
        f->forest.status = nullptr;
        for (cudaEvent_t e : f->forest.refined.screen_ev)
            if (e) cudaEventDestroy(e);
        pack_destroy(f->pack);
        if (f->host_status) cudaFreeHost(f->host_status);
        for (auto &ev : f->ev)
            if (ev) cudaEventDestroy(ev);
        delete f;
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int64_t cuscan_ctx_reserved_bytes(const cuscan_ctx *ctx) {
    if (!ctx || !ctx->fit) return 0;
    Buffer *all[kWorkspaceBufferCount];
    const int count = workspace_buffers(ctx->fit, all);
    int64_t total = 0;
    for (int i = 0; i < count; ++i) total += (int64_t)all[i]->bytes;
    return total + pack_reserved_bytes(ctx->fit->pack);
}

int cuscan_ctx_release_workspace(cuscan_ctx *ctx) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    Buffer *all[kWorkspaceBufferCount];
    const int count = workspace_buffers(ctx->fit, all);
    for (int i = 0; i < count; ++i) release(*all[i]);
    ctx->fit->forest.status = nullptr;
    pack_release(ctx->fit->pack);
    return CUSCAN_OK;
}

int64_t cuscan_fit_workspace_bytes(int64_t n, int32_t d, int32_t min_samples, int32_t precision) {
    if (n < 2 || d <= 0 || min_samples <= 0) return 0;
    const size_t N = (size_t)n, D = (size_t)d;
    const size_t k = (size_t)((int64_t)min_samples < n - 1 ? min_samples : n - 1);
    size_t b = 4 * N * D + 8 * N * k + 5 * 4 * N;  // input copy, kNN lists, core/label/MST arrays
    b += 18 * 4 * N + 4 * N * D + 16 * N;          // forest arrays, sorted copy, 64-bit keys
    b += 2 * 4 * (N / 32 + 2) + 64 + sizeof(DevStatus) + 4 * (N / 1024 + 2);  // tiles, scan
    // split-kNN partial lists: at most 2 * SMs + query blocks blocks of 128 rows
    b += 8 * k * 128 * (size_t)(2 * 2 * kSMs + ceil_div(n, 128));
    if (precision == CUSCAN_PRECISION_BF16_REFINED || precision == CUSCAN_PRECISION_FP16_REFINED)
        b += refined_workspace_bytes(n, d, (int)k);
    else if (n >= 2048)  // exact rounds over a row subset: bounds, flags, positions, counts
        b += 7 * 4 * N + 64;
    return (int64_t)b + (1 << 20);
}

const char *cuscan_last_error(const cuscan_ctx *ctx) { return ctx ? ctx->err : "null context"; }
int cuscan_error_kind(const cuscan_ctx *ctx) { return ctx ? ctx->kind : CUSCAN_INVALID_INPUT; }
void *cuscan_ctx_stream(cuscan_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int cuscan_exact_knn(cuscan_ctx *ctx, const float *query, int64_t nq, const float *reference,
                     int64_t nr, int32_t d, int32_t k, int32_t exclude_self,
                     int64_t query_offset, int32_t squared, int32_t *ids_out, float *dist_out,
                     void *stream) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (nq < 0 || nr <= 0 || d <= 0 || k <= 0)
        return fail(ctx, CUSCAN_INVALID_INPUT, "exact_knn needs nq >= 0, nr > 0, d > 0, k > 0");
    if (nr > INT32_MAX - 1 || nq > INT32_MAX)
        return fail(ctx, CUSCAN_OVERFLOW, "row count exceeds the supported integer range");
    if (nq > 0 && (!query || !reference || !ids_out || !dist_out))
        return fail(ctx, CUSCAN_INVALID_INPUT, "exact_knn received a null pointer");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    // The kNN of a point set against itself (the fit's core-distance sweep) takes the tensor-core
    // screen with exact re-rank, whose rows equal the exact sweep's bit for bit; it falls back to
    // the exact sweep itself for shapes outside the screen's tiling (fewer than 2048 rows,
    // k > 32, more than 128 features, values that overflow f32).
    if (query == reference && nq == nr && query_offset == 0 && exclude_self && squared &&
        nr >= 2048 && k <= 32 && refined_available()) {
        ForestBuffers &b = ctx->fit->forest;
        int rc = forest_reserve(ctx, b, nr, d);
        if (rc) return rc;
        b.refined.want_fp16 = false;
        b.refined.have_scale = false;
        b.refined.split = false;
        b.refined.screen_timed = false;
        int64_t refined_rows = 0, fallback_rows = 0, rescreened_rows = 0;
        return launch_knn_refined(ctx, b, reference, nr, d, k, ids_out, dist_out, s, &refined_rows,
                                  &fallback_rows, &rescreened_rows);
    }
    return launch_exact_knn_fp32(ctx, query, nq, reference, nr, d, k, exclude_self, query_offset,
                                 squared, ids_out, dist_out, s, ctx->fit->op_knn_ids,
                                 ctx->fit->op_knn_dist);
}

int cuscan_boruvka_candidates(cuscan_ctx *ctx, const float *data, const float *core_sq,
                              const int32_t *components, int64_t n, int32_t d, float *weights_out,
                              int32_t *destinations_out, void *stream) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (n <= 0 || d <= 0)
        return fail(ctx, CUSCAN_INVALID_INPUT, "Boruvka candidate input must contain at least one row");
    if (n > INT32_MAX - 1) return fail(ctx, CUSCAN_OVERFLOW, "Boruvka row indices");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    FitWorkspace *f = ctx->fit;
    int rc = ensure(ctx, f->op_keys, sizeof(unsigned long long) * n, "candidate keys");
    if (!rc) rc = ensure(ctx, f->op_tiles_lo, sizeof(int32_t) * (ceil_div(n, 32) + 1), "tiles");
    if (!rc) rc = ensure(ctx, f->op_tiles_hi, sizeof(int32_t) * (ceil_div(n, 32) + 1), "tiles");
    if (rc) return rc;
    unsigned long long *keys = as<unsigned long long>(f->op_keys);
    if ((rc = launch_fill_u64(ctx, keys, n, ~0ull, s))) return rc;
    if ((rc = launch_candidates_fp32(ctx, data, core_sq, components, nullptr, n, d, keys,
                                     as<int32_t>(f->op_tiles_lo), as<int32_t>(f->op_tiles_hi), s)))
        return rc;
    return launch_keys_to_candidates(ctx, keys, n, weights_out, destinations_out, s);
}

int cuscan_component_reduce(cuscan_ctx *ctx, const float *weights, const int32_t *indices,
                            const int32_t *members, const int32_t *tile_starts,
                            const int32_t *tile_ends, const int32_t *partial_offsets, int64_t n,
                            int64_t p, int64_t c, float *win_weights, int32_t *win_meta,
                            void *stream) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (n < 0 || p < 0 || c < 0 || c > n || p > n)
        return fail(ctx, CUSCAN_INVALID_INPUT, "component_reduce received inconsistent sizes");
    if (n > INT32_MAX) return fail(ctx, CUSCAN_OVERFLOW, "component member index");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    return launch_component_reduce(ctx, weights, indices, members, tile_starts, tile_ends,
                                   partial_offsets, n, p, c, win_weights, win_meta,
                                   ctx->fit->op_partials, pick_stream(ctx, stream));
}

static int read_status(cuscan_ctx *ctx, DevStatus *dev, DevStatus *host, cudaStream_t s) {
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(host, dev, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
    return CUSCAN_OK;
}

static int status_error(cuscan_ctx *ctx, int kind) {
    switch (kind) {
        case 1:
            return fail(ctx, CUSCAN_NUMERICAL,
                        "Boruvka candidate weight must be nonnegative and not NaN");
        case 2:
            return fail(ctx, CUSCAN_INVALID_INPUT, "candidate index is out of range");
        default:
            return fail(ctx, CUSCAN_NUMERICAL, "Boruvka round made no progress");
    }
}

static float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

int cuscan_fit_core_device(cuscan_ctx *ctx, const float *data, int64_t n, int32_t d,
                           int32_t min_samples, int32_t precision, int32_t *knn_ids,
                           float *knn_sq, float *core_sq, uint32_t *mst_src, uint32_t *mst_dst,
                           float *mst_wsq, int64_t *n_edges, cuscan_fit_stats *stats,
                           void *stream) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (n_edges) *n_edges = 0;
    if (stats) memset(stats, 0, sizeof(*stats));
    if (min_samples <= 0) return fail(ctx, CUSCAN_INVALID_CONFIG, "min_samples must be positive");
    if (n < 2 || d <= 0)
        return fail(ctx, CUSCAN_INVALID_INPUT, "the fit core needs at least two rows and one feature");
    if (n > INT32_MAX - 1)
        return fail(ctx, CUSCAN_INVALID_INPUT, "row count %lld exceeds the supported maximum",
                    (long long)n);
    if (precision != CUSCAN_PRECISION_PLAIN && precision != CUSCAN_PRECISION_BF16_REFINED &&
        precision != CUSCAN_PRECISION_FP16_REFINED)
        return fail(ctx, CUSCAN_INVALID_CONFIG, "unknown precision %d", precision);
    const bool refined = precision != CUSCAN_PRECISION_PLAIN;
    if (refined && !refined_available())
        return fail(ctx, CUSCAN_BACKEND_UNAVAILABLE,
                    "refined sweeps are not available for this shape");
    if (!data || !knn_ids || !knn_sq || !core_sq || !mst_src || !mst_dst || !mst_wsq)
        return fail(ctx, CUSCAN_INVALID_INPUT, "fit_core_device received a null pointer");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    FitWorkspace *f = ctx->fit;
    ForestBuffers &b = f->forest;
    int rc = forest_reserve(ctx, b, n, d);
    if (!rc) rc = ensure(ctx, f->label, sizeof(int32_t) * n, "point labels");
    if (rc) return rc;
    const int k = (int)((int64_t)min_samples < n - 1 ? min_samples : n - 1);
    int32_t *label = as<int32_t>(f->label);
    cudaEvent_t *ev = f->ev;
    int64_t refined_rows = 0, fallback_rows = 0, boruvka_fallback_rows = 0, rescreened_rows = 0;
    b.refined.want_fp16 = precision == CUSCAN_PRECISION_FP16_REFINED;
    b.refined.have_scale = false;
    b.refined.split = false;
    b.refined.tile_pairs = 0;
    b.refined.screened_rows = 0;
    b.refined.symmetric_rounds = 0;
    b.refined.lb_valid = false;
    b.refined.screen_timed = false;

    CUSCAN_CUDA(ctx, cudaMemsetAsync(b.status, 0, sizeof(DevStatus), s));
    CUSCAN_CUDA(ctx, cudaEventRecord(ev[0], s));
    // ---- core_distances: exact kNN sweep (estimator.rs:591-657) + core column ----
    if (refined)
        rc = launch_knn_refined(ctx, b, data, n, d, k, knn_ids, knn_sq, s, &refined_rows,
                                &fallback_rows, &rescreened_rows);
    else
        rc = launch_exact_knn_fp32(ctx, data, n, data, n, d, k, 1, 0, 1, knn_ids, knn_sq, s,
                                   b.knn_ids_tmp, b.knn_dist_tmp);
    if (rc) return rc;
    CUSCAN_CUDA(ctx, cudaEventRecord(ev[1], s));
    if ((rc = forest_core(ctx, knn_sq, n, k, min_samples, core_sq, s))) return rc;
    CUSCAN_CUDA(ctx, cudaEventRecord(ev[2], s));
    // ---- mst: kNN seed then Borůvka rounds (estimator.rs:689-874) ----
    if ((rc = forest_seed(ctx, b, core_sq, knn_ids, knn_sq, n, k, label, mst_src, mst_dst,
                          mst_wsq, s)))
        return rc;
    DevStatus *hs = f->host_status;
    if ((rc = read_status(ctx, b.status, hs, s))) return rc;
    if (hs->err_kind) return status_error(ctx, hs->err_kind);
    const int64_t seed_edges = (int64_t)hs->edges;
    const int64_t after_seed = (int64_t)hs->components;
    int64_t components = (int64_t)hs->components;
    int64_t rounds = 0;
    double cand_ms = 0.0, cross_pairs = 0.0;
    f->round_count = 0;
    // exact rounds of fits of at least 2048 rows scan only the rows that can hold their
    // component's cheapest edge (smaller fits scan every row: one host read per round fewer)
    const bool exact_rows = !refined && n >= 2048;
    while (components > 1) {
        const int64_t rows0 = b.refined.screened_rows, tiles0 = b.refined.tile_pairs;
        if (rounds > 64) return fail(ctx, CUSCAN_NUMERICAL, "Boruvka did not converge");
        if ((rc = forest_sort_by_component(ctx, b, data, core_sq, label, n, d, s))) return rc;
        unsigned long long *row_keys = as<unsigned long long>(b.row_keys);
        if ((rc = launch_fill_u64(ctx, row_keys, n, ~0ull, s))) return rc;
        CUSCAN_CUDA(ctx, cudaEventRecord(ev[4], s));
        if (refined)
            rc = launch_candidates_refined(ctx, b, n, d, knn_ids, knn_sq, k, core_sq, label, s,
                                           &boruvka_fallback_rows);
        else if (exact_rows)
            rc = launch_candidates_exact_rows(ctx, b, n, d, knn_ids, knn_sq, k, core_sq, label, s,
                                              &b.refined.screened_rows);
        else
            rc = launch_candidates_fp32(ctx, as<float>(b.xp), as<float>(b.corep),
                                        as<int32_t>(b.labp), as<int32_t>(b.perm), n, d, row_keys,
                                        as<int32_t>(b.tile_lo), as<int32_t>(b.tile_hi), s);
        if (rc) return rc;
        CUSCAN_CUDA(ctx, cudaEventRecord(ev[5], s));
        if ((rc = forest_round(ctx, b, n, components, label, mst_src, mst_dst, mst_wsq, s,
                               refined || exact_rows)))
            return rc;
        if ((rc = read_status(ctx, b.status, hs, s))) return rc;
        cand_ms += elapsed(ev[4], ev[5]);
        cross_pairs += (double)n * (double)n - hs->same_pairs;
        if (f->round_count < FitWorkspace::kMaxRoundLog) {
            const int r = f->round_count++;
            f->round_rows[r] = refined || exact_rows ? b.refined.screened_rows - rows0 : n;
            f->round_tiles[r] = b.refined.tile_pairs - tiles0;
            f->round_ms[r] = elapsed(ev[4], ev[5]);
            f->round_cross[r] = (double)n * (double)n - hs->same_pairs;
        }
        if (hs->err_kind) return status_error(ctx, hs->err_kind);
        ++rounds;
        components = (int64_t)hs->components;
    }
    // total weight of the tree in f64 on the device (finalize_mst's per-edge sqrt, summed)
    if ((rc = forest_mst_weight(ctx, b, mst_wsq, (int64_t)hs->edges, s))) return rc;
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(&hs->mst_weight, &b.status->mst_weight, sizeof(double),
                                     cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaEventRecord(ev[3], s));
    CUSCAN_CUDA(ctx, cudaEventSynchronize(ev[3]));
    if ((int64_t)hs->edges != n - 1)
        return fail(ctx, CUSCAN_NUMERICAL, "Boruvka produced an incomplete spanning tree");
    if (n_edges) *n_edges = (int64_t)hs->edges;
    if (stats) {
        stats->core_ms = elapsed(ev[0], ev[2]);
        stats->mst_ms = elapsed(ev[2], ev[3]);
        stats->knn_kernel_ms = elapsed(ev[0], ev[1]);
        stats->candidate_kernel_ms = cand_ms;
        stats->rounds = rounds;
        stats->seed_edges = seed_edges;
        stats->components_after_seed = after_seed;
        stats->refined_rows = refined_rows;
        stats->fallback_rows = fallback_rows;
        stats->boruvka_fallback_rows = boruvka_fallback_rows;
        stats->cross_pairs = cross_pairs;
        stats->rescreened_rows = rescreened_rows;
        stats->screen_tile_pairs = b.refined.tile_pairs;
        stats->boruvka_screened_rows = b.refined.screened_rows;
        stats->symmetric_rounds = b.refined.symmetric_rounds;
        stats->mst_weight = hs->mst_weight;
        stats->knn_screen_ms =
            b.refined.screen_timed ? elapsed(b.refined.screen_ev[0], b.refined.screen_ev[1]) : 0.0;
        stats->operand_format = refined ? refined_operand_format(b) : -1;
    }
    return CUSCAN_OK;
}

int cuscan_fit_core(cuscan_ctx *ctx, const float *data, int64_t n, int32_t d,
                    int32_t min_samples, int32_t precision, int32_t *knn_ids, float *knn_sq,
                    float *core_sq, uint32_t *mst_src, uint32_t *mst_dst, float *mst_wsq,
                    int64_t *n_edges, cuscan_fit_stats *stats) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (min_samples <= 0) return fail(ctx, CUSCAN_INVALID_CONFIG, "min_samples must be positive");
    if (n < 2 || d <= 0)
        return fail(ctx, CUSCAN_INVALID_INPUT, "the fit core needs at least two rows and one feature");
    if (!data || !core_sq || !mst_src || !mst_dst || !mst_wsq)
        return fail(ctx, CUSCAN_INVALID_INPUT, "fit_core received a null pointer");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    FitWorkspace *f = ctx->fit;
    cudaStream_t s = ctx->stream;
    const int64_t k = (int64_t)min_samples < n - 1 ? min_samples : n - 1;
    int rc = ensure(ctx, f->x, sizeof(float) * n * d, "input rows");
    if (!rc) rc = ensure(ctx, f->ids, sizeof(int32_t) * n * k, "kNN ids");
    if (!rc) rc = ensure(ctx, f->dsq, sizeof(float) * n * k, "kNN distances");
    if (!rc) rc = ensure(ctx, f->core, sizeof(float) * n, "core distances");
    if (!rc) rc = ensure(ctx, f->src, sizeof(uint32_t) * n, "MST sources");
    if (!rc) rc = ensure(ctx, f->dst, sizeof(uint32_t) * n, "MST destinations");
    if (!rc) rc = ensure(ctx, f->w, sizeof(float) * n, "MST weights");
    if (rc) return rc;
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(f->x.ptr, data, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
    int64_t m = 0;
    rc = cuscan_fit_core_device(ctx, as<float>(f->x), n, d, min_samples, precision,
                                as<int32_t>(f->ids), as<float>(f->dsq), as<float>(f->core),
                                as<uint32_t>(f->src), as<uint32_t>(f->dst), as<float>(f->w), &m,
                                stats, s);
    if (rc) return rc;
    if (knn_ids)
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(knn_ids, f->ids.ptr, sizeof(int32_t) * n * k,
                                         cudaMemcpyDeviceToHost, s));
    if (knn_sq)
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(knn_sq, f->dsq.ptr, sizeof(float) * n * k,
                                         cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(core_sq, f->core.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(mst_src, f->src.ptr, sizeof(uint32_t) * m, cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(mst_dst, f->dst.ptr, sizeof(uint32_t) * m, cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(mst_wsq, f->w.ptr, sizeof(float) * m, cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
    if (n_edges) *n_edges = m;
    return CUSCAN_OK;
}

int cuscan_fit_round_stats(const cuscan_ctx *ctx, int32_t max_rounds, int64_t *rows,
                           int64_t *tiles, double *ms, double *cross_pairs) {
    if (!ctx || !ctx->fit || max_rounds < 0) return -1;
    const FitWorkspace *f = ctx->fit;
    const int count = f->round_count < max_rounds ? f->round_count : max_rounds;
    for (int r = 0; r < count; ++r) {
        if (rows) rows[r] = f->round_rows[r];
        if (tiles) tiles[r] = f->round_tiles[r];
        if (ms) ms[r] = f->round_ms[r];
        if (cross_pairs) cross_pairs[r] = f->round_cross[r];
    }
    return f->round_count;
}

// ---- row shards: one fit split by query rows over ranks that exchange row keys ----
int cuscan_shard_seed(cuscan_ctx *ctx, int64_t n, int32_t d, int32_t min_samples,
                      const int32_t *knn_ids, const float *knn_sq, float *core_sq,
                      int32_t *labels, uint32_t *mst_src, uint32_t *mst_dst, float *mst_wsq,
                      int64_t *n_edges, int64_t *components, void *stream) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (n < 2 || d <= 0) return fail(ctx, CUSCAN_INVALID_INPUT, "a fit needs at least two rows");
    if (min_samples <= 0) return fail(ctx, CUSCAN_INVALID_CONFIG, "min_samples must be positive");
    if (n > INT32_MAX - 1) return fail(ctx, CUSCAN_OVERFLOW, "row indices");
    if (!knn_ids || !knn_sq || !core_sq || !labels || !mst_src || !mst_dst || !mst_wsq)
        return fail(ctx, CUSCAN_INVALID_INPUT, "null buffer");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    FitWorkspace *f = ctx->fit;
    ForestBuffers &b = f->forest;
    int rc = forest_reserve(ctx, b, n, d);
    if (rc) return rc;
    const int k = (int)((int64_t)min_samples < n - 1 ? min_samples : n - 1);
    CUSCAN_CUDA(ctx, cudaMemsetAsync(b.status, 0, sizeof(DevStatus), s));
    if ((rc = forest_core(ctx, knn_sq, n, k, min_samples, core_sq, s))) return rc;
    if ((rc = forest_seed(ctx, b, core_sq, knn_ids, knn_sq, n, k, labels, mst_src, mst_dst,
                          mst_wsq, s)))
        return rc;
    DevStatus *hs = f->host_status;
    if ((rc = read_status(ctx, b.status, hs, s))) return rc;
    if (hs->err_kind) return status_error(ctx, hs->err_kind);
    if (n_edges) *n_edges = (int64_t)hs->edges;
    if (components) *components = (int64_t)hs->components;
    return CUSCAN_OK;
}

int cuscan_shard_round_keys(cuscan_ctx *ctx, const float *data, const float *core_sq,
                            const int32_t *labels, int64_t n, int32_t d, int64_t row_begin,
                            int64_t row_end, uint64_t *row_keys, void *stream) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (n <= 0 || d <= 0 || row_begin < 0 || row_end > n || row_begin > row_end || !row_keys)
        return fail(ctx, CUSCAN_INVALID_INPUT, "row range [%lld, %lld) outside the %lld rows",
                    (long long)row_begin, (long long)row_end, (long long)n);
    if (n > INT32_MAX - 1) return fail(ctx, CUSCAN_OVERFLOW, "row indices");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    FitWorkspace *f = ctx->fit;
    int rc = ensure(ctx, f->op_tiles_lo, sizeof(int32_t) * (ceil_div(n, 32) + 1), "tiles");
    if (!rc) rc = ensure(ctx, f->op_tiles_hi, sizeof(int32_t) * (ceil_div(n, 32) + 1), "tiles");
    if (rc) return rc;
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(row_keys);
    if ((rc = launch_fill_u64(ctx, keys, n, ~0ull, s))) return rc;
    if (row_end == row_begin) return CUSCAN_OK;
    return launch_candidates_fp32(ctx, data, core_sq, labels, nullptr, n, d, keys,
                                  as<int32_t>(f->op_tiles_lo), as<int32_t>(f->op_tiles_hi), s,
                                  nullptr, row_end - row_begin, row_begin);
}

int cuscan_shard_round_merge(cuscan_ctx *ctx, const float *data, const float *core_sq,
                             int32_t *labels, int64_t n, int32_t d, const uint64_t *row_keys,
                             uint32_t *mst_src, uint32_t *mst_dst, float *mst_wsq,
                             int64_t *n_edges, int64_t *components, double *mst_weight,
                             void *stream) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (n < 2 || d <= 0 || !row_keys) return fail(ctx, CUSCAN_INVALID_INPUT, "bad round input");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    FitWorkspace *f = ctx->fit;
    ForestBuffers &b = f->forest;
    if (!b.status) return fail(ctx, CUSCAN_INVALID_INPUT, "no shard seed on this context");
    DevStatus *hs = f->host_status;
    int rc = read_status(ctx, b.status, hs, s);
    if (rc) return rc;
    const int64_t before = (int64_t)hs->components;
    if (before > 1) {
        if ((rc = forest_sort_by_component(ctx, b, data, core_sq, labels, n, d, s))) return rc;
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(b.row_keys.ptr, row_keys, sizeof(uint64_t) * n,
                                         cudaMemcpyDeviceToDevice, s));
        if ((rc = forest_round(ctx, b, n, before, labels, mst_src, mst_dst, mst_wsq, s, 0)))
            return rc;
        if ((rc = read_status(ctx, b.status, hs, s))) return rc;
        if (hs->err_kind) return status_error(ctx, hs->err_kind);
    }
    if (hs->components == 1 && mst_weight) {
        if ((rc = forest_mst_weight(ctx, b, mst_wsq, (int64_t)hs->edges, s))) return rc;
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(&hs->mst_weight, &b.status->mst_weight, sizeof(double),
                                         cudaMemcpyDeviceToHost, s));
        CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
        *mst_weight = hs->mst_weight;
    }
    if (n_edges) *n_edges = (int64_t)hs->edges;
    if (components) *components = (int64_t)hs->components;
    return CUSCAN_OK;
}

int cuscan_debug_screen_tile_operands(cuscan_ctx *ctx, const float *data, int64_t n, int32_t d,
                                      int32_t operands, float *tile_out, float *rows_out,
                                      float *chunk_out, float *scale_out, void *stream) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (n < 256 || d <= 0 || !data || !tile_out)
        return fail(ctx, CUSCAN_INVALID_INPUT, "debug tile needs n >= 256 rows");
    if (operands < 0 || operands > 2)
        return fail(ctx, CUSCAN_INVALID_INPUT, "unknown operand format");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    int rc = forest_reserve(ctx, ctx->fit->forest, n, d);
    if (rc) return rc;
    return debug_screen_tile(ctx, ctx->fit->forest, data, n, d, operands, tile_out, rows_out,
                             chunk_out, scale_out, s);
}

int cuscan_debug_screen_tile(cuscan_ctx *ctx, const float *data, int64_t n, int32_t d,
                             float *tile_out, void *stream) {
    return cuscan_debug_screen_tile_operands(ctx, data, n, d, 0, tile_out, nullptr, nullptr,
                                             nullptr, stream);
}

}  // extern "C"
