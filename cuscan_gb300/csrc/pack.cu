// Packed small fits: the fit cores of several small point sets, every step of every fit in one
// launch.
//
// A small fit (fewer than 2048 rows) is a handful of short kernels, and the host reads the
// component count after the seed and after every Borůvka round
// (crates/hdbscan/src/estimator.rs:689-874 does the same on its host). Its time goes to launch
// and synchronisation latency, not to the kernels. A pack runs the same steps for all of its fits
// at once, each step one launch over every fit: the fits' sizes and device buffers sit in an
// array of PackFit descriptors in device memory, and each block of a grouped kernel takes its
// fit from the grid (forest.cuh):
//   1. one copy in: the descriptors and every fit's rows;
//   2. exact kNN lists (pack_knn_kernel; a merge of partial lists when the reference range of
//      each fit is split to fill the GPU);
//   3. core column, kNN seed and its merge, one CTA per fit (pack_seed_kernel);
//   4. Borůvka rounds: per round the component sort (pack_sort_kernel, one CTA per fit), the
//      sorted copy of the rows (pack_gather_kernel), the exact candidate sweep
//      (pack_candidates_kernel) and the winners and merge (pack_merge_kernel, one CTA per
//      fit). A fit whose forest is complete skips the rest of the rounds on the device. The
//      host launches rounds in batches (three, then two at a time) and reads one counter after
//      each batch: the fits that need another round;
//   5. the f64 MST weight, one CTA per fit;
//   6. one copy out: every fit's status block and outputs.
// A pack of eight fits that finish in three rounds takes 16 launches and one host read between
// the copies, where the same fits alone take about 26 launches and 4 host reads each.
//
// Each step is the kernel body a fit alone runs for fewer than 2048 rows, in every precision
// (the exact f32 kNN and candidate sweeps, the single-CTA forest steps of forest.cu), with the
// same pointer-doubling step counts, so every output is bit identical to cuscan_fit_core's.
// Splitting the reference range differently does not change the lists: the kNN merge and the
// candidate keys are exact minima in a total order. Fits with k > 32 take the per-fit kNN
// launch (the wide kernel, as alone).
//
// The reference has no counterpart: its serving layer does not exist and its small fits run
// one host-driven round at a time.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "forest.cuh"
#include "workspace.cuh"

namespace cuscan {

struct PackWorkspace {
    Buffer arena;             // device: descriptors and rows | outputs | per-fit work arrays
    void *staging = nullptr;  // pinned mirror of the first two regions (same offsets)
    size_t staging_bytes = 0;
    cudaEvent_t ev[3] = {};   // pack start, kNN lists done, weights done
    int64_t launches = 0, host_reads = 0;  // of the latest pack
};

namespace {

constexpr int kKnnRows = 128;      // query rows per block of the kNN and candidate sweeps
constexpr int kGroupedMaxK = 32;   // larger k takes the per-fit kNN launch
constexpr int kFirstBatch = 3;     // rounds launched before the first host read
constexpr int kNextBatch = 2;

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

int item_k(const cuscan_fit_item &it) {
    return (int)((int64_t)it.min_samples < it.n - 1 ? it.min_samples : it.n - 1);
}

int status_to_error(cuscan_ctx *ctx, int kind, int item) {
    switch (kind) {
        case 1:
            return fail(ctx, CUSCAN_NUMERICAL,
                        "fit %d: Boruvka candidate weight must be nonnegative and not NaN", item);
        case 2:
            return fail(ctx, CUSCAN_INVALID_INPUT, "fit %d: candidate index is out of range", item);
        case kPackErrNoConvergence:
            return fail(ctx, CUSCAN_NUMERICAL, "fit %d: Boruvka did not converge", item);
        default:
            return fail(ctx, CUSCAN_NUMERICAL, "fit %d: Boruvka round made no progress", item);
    }
}

int validate(cuscan_ctx *ctx, const cuscan_fit_item &it, int i) {
    if (!it.data || !it.core_sq || !it.mst_src || !it.mst_dst || !it.mst_wsq)
        return fail(ctx, CUSCAN_INVALID_INPUT, "fit %d received a null pointer", i);
    if (it.min_samples <= 0)
        return fail(ctx, CUSCAN_INVALID_CONFIG, "fit %d: min_samples must be positive", i);
    if (it.n < 2 || it.n > CUSCAN_PACK_MAX_ROWS)
        return fail(ctx, CUSCAN_INVALID_INPUT,
                    "fit %d: a packed fit needs 2 to %d rows, got %lld", i, CUSCAN_PACK_MAX_ROWS,
                    (long long)it.n);
    if (it.d <= 0 || it.d > CUSCAN_PACK_MAX_FEATURES)
        return fail(ctx, CUSCAN_INVALID_INPUT, "fit %d: a packed fit needs 1 to %d features", i,
                    CUSCAN_PACK_MAX_FEATURES);
    if (it.precision != CUSCAN_PRECISION_PLAIN && it.precision != CUSCAN_PRECISION_BF16_REFINED &&
        it.precision != CUSCAN_PRECISION_FP16_REFINED)
        return fail(ctx, CUSCAN_INVALID_CONFIG, "fit %d: unknown precision %d", i, it.precision);
    return CUSCAN_OK;
}

float elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();
        ms = 0.0f;
    }
    return ms;
}

// Byte offsets of one fit's arrays in the arena. Region 1 (copied in): the descriptors, then
// every fit's rows. Region 2 (copied out): the round counters, then every fit's status block and
// outputs. Region 3: work arrays that stay on the device.
struct FitLayout {
    size_t x;
    size_t status, core, src, dst, w, ids, dsq;
    size_t label, next, ja, ma, jb, mb, keep, pos, parent, minlab, kept, esrc, edst, ew;
    size_t cnt, start, fill, perm, labp, xp, corep, row_keys, comp_keys, tile_lo, tile_hi;
    size_t part_ids, part_dist;
};

struct PackLayout {
    std::vector<FitLayout> fit;
    size_t in_bytes = 0;   // region 1 is [0, in_bytes)
    size_t more = 0;       // region 2 is [more, out_end)
    size_t out_end = 0;
    size_t total = 0;
};

// Reference-range chunks of the kNN and candidate sweeps: enough blocks to fill the GPU twice
// over (the plan of a fit alone), chunks of at least 256 rows.
int64_t pack_splits(const cuscan_ctx *ctx, int count, int64_t n_max) {
    const int64_t blocks = (int64_t)count * ceil_div(n_max, kKnnRows);
    const int64_t target = 2 * (int64_t)ctx->sm_count;
    int64_t splits = blocks < target ? ceil_div(target, blocks) : 1;
    const int64_t cap = ceil_div(n_max, 256);
    if (splits > cap) splits = cap;
    if (splits > 64) splits = 64;
    return splits < 1 ? 1 : splits;
}

PackLayout make_layout(const cuscan_fit_item *items, int count, int64_t splits) {
    PackLayout L;
    L.fit.resize((size_t)count);
    size_t off = align256(sizeof(PackFit) * (size_t)count);
    auto take = [&off](size_t bytes) {
        const size_t at = off;
        off = align256(off + bytes);
        return at;
    };
    for (int i = 0; i < count; ++i)
        L.fit[i].x = take(sizeof(float) * (size_t)items[i].n * items[i].d);
    L.in_bytes = off;
    L.more = take(sizeof(int) * (kPackMaxRounds + 2));
    for (int i = 0; i < count; ++i) {
        const cuscan_fit_item &it = items[i];
        const size_t n = (size_t)it.n, nk = n * (size_t)item_k(it);
        FitLayout &F = L.fit[i];
        F.status = take(sizeof(DevStatus));
        F.core = take(4 * n);
        F.src = take(4 * n);
        F.dst = take(4 * n);
        F.w = take(4 * n);
        F.ids = it.knn_ids ? take(4 * nk) : 0;
        F.dsq = it.knn_sq ? take(4 * nk) : 0;
    }
    L.out_end = off;
    for (int i = 0; i < count; ++i) {
        const cuscan_fit_item &it = items[i];
        const size_t n = (size_t)it.n, nk = n * (size_t)item_k(it), nd = n * (size_t)it.d;
        FitLayout &F = L.fit[i];
        if (!it.knn_ids) F.ids = take(4 * nk);
        if (!it.knn_sq) F.dsq = take(4 * nk);
        for (size_t *p : {&F.label, &F.next, &F.ja, &F.ma, &F.jb, &F.mb, &F.keep, &F.pos,
                          &F.parent, &F.minlab, &F.esrc, &F.edst, &F.ew, &F.cnt, &F.start,
                          &F.fill, &F.perm, &F.labp, &F.corep})
            *p = take(4 * n);
        F.kept = take(2 * sizeof(int32_t));
        F.xp = take(4 * nd);
        F.row_keys = take(8 * n);
        F.comp_keys = take(8 * n);
        F.tile_lo = take(4 * (n / 32 + 1));
        F.tile_hi = take(4 * (n / 32 + 1));
        const size_t parts = splits > 1 && item_k(it) <= kGroupedMaxK ? nk * (size_t)splits : 0;
        F.part_ids = take(4 * parts);
        F.part_dist = take(4 * parts);
    }
    L.total = off;
    return L;
}

PackFit describe(const cuscan_fit_item &it, const FitLayout &F, char *base) {
    PackFit f;
    std::memset(&f, 0, sizeof(f));
    f.x = reinterpret_cast<const float *>(base + F.x);
    f.n = it.n;
    f.d = it.d;
    f.k = item_k(it);
    f.min_samples = it.min_samples;
    // a fit alone lets rows lack a candidate on the refined paths only (api.cu)
    f.allow_empty = it.precision != CUSCAN_PRECISION_PLAIN;
    f.ids = reinterpret_cast<int32_t *>(base + F.ids);
    f.dsq = reinterpret_cast<float *>(base + F.dsq);
    f.core = reinterpret_cast<float *>(base + F.core);
    f.label = reinterpret_cast<int32_t *>(base + F.label);
    f.src = reinterpret_cast<uint32_t *>(base + F.src);
    f.dst = reinterpret_cast<uint32_t *>(base + F.dst);
    f.w = reinterpret_cast<float *>(base + F.w);
    f.next = reinterpret_cast<int32_t *>(base + F.next);
    f.ja = reinterpret_cast<int32_t *>(base + F.ja);
    f.ma = reinterpret_cast<int32_t *>(base + F.ma);
    f.jb = reinterpret_cast<int32_t *>(base + F.jb);
    f.mb = reinterpret_cast<int32_t *>(base + F.mb);
    f.keep = reinterpret_cast<int32_t *>(base + F.keep);
    f.pos = reinterpret_cast<int32_t *>(base + F.pos);
    f.parent = reinterpret_cast<int32_t *>(base + F.parent);
    f.minlab = reinterpret_cast<int32_t *>(base + F.minlab);
    f.kept_total = reinterpret_cast<int32_t *>(base + F.kept);
    f.esrc = reinterpret_cast<uint32_t *>(base + F.esrc);
    f.edst = reinterpret_cast<uint32_t *>(base + F.edst);
    f.ew = reinterpret_cast<float *>(base + F.ew);
    f.cnt = reinterpret_cast<int32_t *>(base + F.cnt);
    f.start = reinterpret_cast<int32_t *>(base + F.start);
    f.fill = reinterpret_cast<int32_t *>(base + F.fill);
    f.perm = reinterpret_cast<int32_t *>(base + F.perm);
    f.labp = reinterpret_cast<int32_t *>(base + F.labp);
    f.xp = reinterpret_cast<float *>(base + F.xp);
    f.corep = reinterpret_cast<float *>(base + F.corep);
    f.row_keys = reinterpret_cast<unsigned long long *>(base + F.row_keys);
    f.comp_keys = reinterpret_cast<unsigned long long *>(base + F.comp_keys);
    f.tile_lo = reinterpret_cast<int32_t *>(base + F.tile_lo);
    f.tile_hi = reinterpret_cast<int32_t *>(base + F.tile_hi);
    f.part_ids = reinterpret_cast<int32_t *>(base + F.part_ids);
    f.part_dist = reinterpret_cast<float *>(base + F.part_dist);
    f.status = reinterpret_cast<DevStatus *>(base + F.status);
    return f;
}

int make_workspace(cuscan_ctx *ctx) {
    FitWorkspace *f = ctx->fit;
    if (f->pack) return CUSCAN_OK;
    PackWorkspace *p = new PackWorkspace();
    cudaError_t e = cudaSuccess;
    for (auto &ev : p->ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e != cudaSuccess) {
        pack_destroy(p);
        return cuda_fail(ctx, e, "pack events");
    }
    f->pack = p;
    return CUSCAN_OK;
}

}  // namespace

int64_t pack_reserved_bytes(const PackWorkspace *p) { return p ? (int64_t)p->arena.bytes : 0; }

void pack_release(PackWorkspace *p) {
    if (!p) return;
    release(p->arena);
    if (p->staging) cudaFreeHost(p->staging);
    p->staging = nullptr;
    p->staging_bytes = 0;
}

void pack_destroy(PackWorkspace *p) {
    if (!p) return;
    pack_release(p);
    for (auto &e : p->ev)
        if (e) cudaEventDestroy(e);
    delete p;
}

}  // namespace cuscan

using namespace cuscan;

extern "C" int cuscan_fit_core_packed_launch_stats(cuscan_ctx *ctx, int64_t *launches,
                                                   int64_t *host_reads) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    const PackWorkspace *p = ctx->fit ? ctx->fit->pack : nullptr;
    if (launches) *launches = p ? p->launches : 0;
    if (host_reads) *host_reads = p ? p->host_reads : 0;
    return CUSCAN_OK;
}

extern "C" int cuscan_fit_core_packed(cuscan_ctx *ctx, cuscan_fit_item *items, int32_t count) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    if (!items || count < 1 || count > CUSCAN_PACK_MAX_FITS)
        return fail(ctx, CUSCAN_INVALID_INPUT, "a pack holds 1 to %d fits", CUSCAN_PACK_MAX_FITS);
    for (int i = 0; i < count; ++i) {
        items[i].status = CUSCAN_OK;
        items[i].n_edges = 0;
        std::memset(&items[i].stats, 0, sizeof(items[i].stats));
    }
    for (int i = 0; i < count; ++i)
        if (int rc = validate(ctx, items[i], i)) {
            items[i].status = rc;
            return rc;
        }
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    int rc = make_workspace(ctx);
    if (rc) return rc;
    PackWorkspace &P = *ctx->fit->pack;
    P.launches = 0;
    P.host_reads = 0;

    int64_t n_max = 0;
    int d_max = 0, k_max = 0;
    for (int i = 0; i < count; ++i) {
        n_max = std::max(n_max, items[i].n);
        d_max = std::max(d_max, items[i].d);
        if (item_k(items[i]) <= kGroupedMaxK) k_max = std::max(k_max, item_k(items[i]));
    }
    const int64_t splits = pack_splits(ctx, count, n_max);
    const PackLayout L = make_layout(items, count, splits);
    cudaStream_t s = ctx->stream;
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
    if ((rc = ensure(ctx, P.arena, L.total, "packed fits"))) return rc;
    if (P.staging_bytes < L.out_end) {
        if (P.staging) cudaFreeHost(P.staging);
        P.staging = nullptr;
        P.staging_bytes = 0;
        CUSCAN_CUDA(ctx, cudaMallocHost(&P.staging, L.out_end));
        P.staging_bytes = L.out_end;
    }
    char *base = static_cast<char *>(P.arena.ptr);
    char *stg = static_cast<char *>(P.staging);
    PackFit *host_fits = reinterpret_cast<PackFit *>(stg);
    for (int i = 0; i < count; ++i) {
        host_fits[i] = describe(items[i], L.fit[i], base);
        std::memcpy(stg + L.fit[i].x, items[i].data,
                    sizeof(float) * (size_t)items[i].n * items[i].d);
    }
    const PackFit *fits = reinterpret_cast<const PackFit *>(base);
    int *more = reinterpret_cast<int *>(base + L.more);

    CUSCAN_CUDA(ctx, cudaEventRecord(P.ev[0], s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(base, stg, L.in_bytes, cudaMemcpyHostToDevice, s));
    if (k_max > 0 &&
        (rc = pack_knn(ctx, fits, count, n_max, d_max, k_max, (int)splits, s, P.launches)))
        return rc;
    for (int i = 0; i < count; ++i) {
        if (item_k(items[i]) <= kGroupedMaxK) continue;
        Buffer unused_ids, unused_dist;  // the wide kernel keeps no partial lists
        const PackFit &f = host_fits[i];
        if ((rc = launch_exact_knn_fp32(ctx, f.x, f.n, f.x, f.n, f.d, f.k, 1, 0, 1, f.ids, f.dsq,
                                        s, unused_ids, unused_dist)))
            return rc;
        ++P.launches;
    }
    CUSCAN_CUDA(ctx, cudaEventRecord(P.ev[1], s));
    if ((rc = pack_seed(ctx, fits, count, more, s))) return rc;
    ++P.launches;
    int r = 0;
    for (int batch = kFirstBatch; r < kPackMaxRounds + 2; batch = kNextBatch) {
        for (int b = 0; b < batch && r < kPackMaxRounds + 2; ++b, ++r) {
            if ((rc = pack_round(ctx, fits, count, n_max, d_max, (int)splits, r, more, s)))
                return rc;
            P.launches += 4;
        }
        int *due = reinterpret_cast<int *>(stg + L.more) + (r - 1);
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(due, more + (r - 1), sizeof(int),
                                         cudaMemcpyDeviceToHost, s));
        CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
        ++P.host_reads;
        if (*due == 0) break;
    }
    if ((rc = pack_weight(ctx, fits, count, s))) return rc;
    ++P.launches;
    CUSCAN_CUDA(ctx, cudaEventRecord(P.ev[2], s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(stg + L.more, base + L.more, L.out_end - L.more,
                                     cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));

    // results
    const float knn_ms = elapsed_ms(P.ev[0], P.ev[1]);
    const float mst_ms = elapsed_ms(P.ev[1], P.ev[2]);
    int first = CUSCAN_OK;
    char first_err[sizeof(ctx->err)] = {0};
    for (int i = 0; i < count; ++i) {
        cuscan_fit_item &it = items[i];
        const FitLayout &F = L.fit[i];
        DevStatus hs;
        std::memcpy(&hs, stg + F.status, sizeof(hs));
        const int64_t n = it.n, k = item_k(it);
        int item_rc = CUSCAN_OK;
        if (hs.err_kind)
            item_rc = status_to_error(ctx, hs.err_kind, i);
        else if ((int64_t)hs.edges != n - 1)
            item_rc = fail(ctx, CUSCAN_NUMERICAL,
                           "fit %d: Boruvka produced an incomplete spanning tree", i);
        it.status = item_rc;
        if (item_rc) {
            if (!first) {
                first = item_rc;
                std::memcpy(first_err, ctx->err, sizeof(first_err));
            }
            continue;
        }
        it.n_edges = (int64_t)hs.edges;
        std::memcpy(it.core_sq, stg + F.core, sizeof(float) * n);
        std::memcpy(it.mst_src, stg + F.src, sizeof(uint32_t) * (n - 1));
        std::memcpy(it.mst_dst, stg + F.dst, sizeof(uint32_t) * (n - 1));
        std::memcpy(it.mst_wsq, stg + F.w, sizeof(float) * (n - 1));
        if (it.knn_ids) std::memcpy(it.knn_ids, stg + F.ids, sizeof(int32_t) * n * k);
        if (it.knn_sq) std::memcpy(it.knn_sq, stg + F.dsq, sizeof(float) * n * k);
        cuscan_fit_stats &S = it.stats;
        S.core_ms = knn_ms;
        S.knn_kernel_ms = knn_ms;
        S.mst_ms = mst_ms;
        S.rounds = (int64_t)hs.rounds;
        S.seed_edges = (int64_t)hs.seed_edges;
        S.components_after_seed = (int64_t)hs.components_after_seed;
        S.cross_pairs = hs.cross_pairs;
        S.mst_weight = hs.mst_weight;
        S.operand_format = -1;  // packed fits run the exact kernels
    }
    clear_error(ctx);
    if (first) {
        std::memcpy(ctx->err, first_err, sizeof(first_err));
        ctx->kind = first;
    }
    return first;
}
