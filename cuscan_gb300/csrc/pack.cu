// Packed small fits: several fit cores of small point sets in ONE CUDA graph launch.
//
// A small fit (fewer than 2048 rows) is made of about a hundred short kernels, and the host
// reads the component count after the seed and after every Borůvka round
// (crates/hdbscan/src/estimator.rs:689-874 does the same on its host). Its time goes to launch
// and synchronisation latency, not to the kernels. Here the fit of each point set is captured
// as one branch of a CUDA graph: copy in, exact kNN sweep and core column, kNN seed, the
// Borůvka rounds, the f64 MST weight, copy out. The branches of a pack run side by side. The
// round loop is a conditional WHILE node; a one-thread kernel at the end of each round sets its
// condition on the device (more than one component, no error, at most the host driver's round
// limit), so no host round trip happens inside a fit. The host launches the graph once and
// synchronises once per pack.
//
// Every pack of a given size has the same graph topology, so the graph is instantiated once
// per pack size and context and then updated in place (cudaGraphExecUpdate with the newly
// captured graph: new pointers, row counts and copy sizes). Measured on a pack of 8 fits (440
// top-level nodes): capture 4.0 ms, instantiation 7.1 ms, update 0.7 ms of host time.
// Each capture creates its round loops' conditional handles anew. An updated graph is launched
// only when every new handle has the same value as the handle of the same branch when the graph
// was instantiated: its kernels then set exactly the conditions the instantiated graph's
// kernels set. Otherwise the graph is instantiated again. The handles also take their default
// (0, no round) at every launch, so no condition value outlives a launch.
//
// Each branch runs the kernels cuscan_fit_core_device runs for the same input: below 2048 rows
// every precision takes the exact f32 kernels, so the outputs are bit identical. One launch
// parameter differs: the cycle breaking of the seed and of every round takes its
// pointer-doubling step count from the largest packed row count (CUSCAN_PACK_MAX_ROWS) instead
// of from the current component count, which the host no longer reads; every pack of a given
// size then has the same graph topology. Any count of at least log2(active nodes) + 1 steps
// reaches the same fixed point (forest.cu), so the edges do not change.
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

struct PackBranch {
    ForestBuffers forest;
    cudaGraphConditionalHandle loop = 0;  // round loop handle of the latest capture
    Buffer x, ids, dsq, core, label, src, dst, w;
    cudaStream_t stream = nullptr;   // capture stream of this branch
    cudaEvent_t join = nullptr;      // joins the branch back into the pack's stream
    cudaEvent_t ev[3] = {};          // start, core distances done, weight done (timing)
};

struct PackWorkspace {
    std::vector<PackBranch *> branches;
    cudaGraphExec_t exec[CUSCAN_PACK_MAX_FITS + 1] = {};  // per pack size, updated in place
    // the branches' round loop handles when exec[count] was instantiated
    cudaGraphConditionalHandle exec_loop[CUSCAN_PACK_MAX_FITS + 1][CUSCAN_PACK_MAX_FITS] = {};
    int64_t instantiations = 0, updates = 0;
    cudaStream_t body = nullptr;     // captures the round-loop bodies
    cudaEvent_t fork = nullptr;
    void *staging = nullptr;         // pinned: every fit's input rows, then every fit's outputs
    size_t staging_bytes = 0;
};

namespace {

constexpr int kBranchOwnBuffers = 8;
constexpr int kBranchBufferCount = kBranchOwnBuffers + kForestBufferCount;
constexpr unsigned long long kMaxRounds = 64;  // the host driver's limit (api.cu)
constexpr int kErrNoConvergence = 8;

int branch_buffers(PackBranch *b, Buffer **out) {
    Buffer *own[] = {&b->x, &b->ids, &b->dsq, &b->core, &b->label, &b->src, &b->dst, &b->w};
    static_assert(sizeof(own) / sizeof(own[0]) == kBranchOwnBuffers, "buffer list");
    for (int i = 0; i < kBranchOwnBuffers; ++i) out[i] = own[i];
    return kBranchOwnBuffers + forest_buffers(b->forest, out + kBranchOwnBuffers);
}

// Condition of the round loop after the seed; records the seed's results.
__global__ void loop_enter_kernel(DevStatus *st, cudaGraphConditionalHandle loop) {
    st->seed_edges = st->edges;
    st->components_after_seed = st->components;
    st->rounds = 0;
    st->cross_pairs = 0.0;
    cudaGraphSetConditional(loop, st->components > 1 && st->err_kind == 0 ? 1u : 0u);
}

// End of a round: count it and its ordered cross-component pairs, then decide whether another
// round runs. A round limit keeps the loop finite whatever the data.
__global__ void loop_next_kernel(DevStatus *st, double n_squared, cudaGraphConditionalHandle loop) {
    st->rounds += 1;
    st->cross_pairs += n_squared - st->same_pairs;
    bool more = st->components > 1 && st->err_kind == 0;
    if (more && st->rounds > kMaxRounds) {
        st->err_kind = kErrNoConvergence;
        more = false;
    }
    cudaGraphSetConditional(loop, more ? 1u : 0u);
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Offsets of one fit's regions in the pinned staging buffer.
struct Staging {
    size_t in, status, core, src, dst, w, ids, dsq;
};

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
        case kErrNoConvergence:
            return fail(ctx, CUSCAN_NUMERICAL, "fit %d: Boruvka did not converge", item);
        default:
            return fail(ctx, CUSCAN_NUMERICAL, "fit %d: Boruvka round made no progress", item);
    }
}

void destroy_branch(PackBranch *b) {
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->join) cudaEventDestroy(b->join);
    for (auto &e : b->ev)
        if (e) cudaEventDestroy(e);
    delete b;
}

// Streams and events are created whole or not at all: a workspace or branch is kept only once
// every handle it needs exists.
int make_workspace(cuscan_ctx *ctx, int count) {
    FitWorkspace *f = ctx->fit;
    if (!f->pack) {
        PackWorkspace *p = new PackWorkspace();
        cudaError_t e = cudaStreamCreateWithFlags(&p->body, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            pack_destroy(p);
            return cuda_fail(ctx, e, "pack streams");
        }
        f->pack = p;
    }
    PackWorkspace &P = *f->pack;
    while ((int)P.branches.size() < count) {
        PackBranch *b = new PackBranch();
        cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
        for (auto &ev : b->ev)
            if (e == cudaSuccess) e = cudaEventCreate(&ev);
        if (e != cudaSuccess) {
            destroy_branch(b);
            return cuda_fail(ctx, e, "pack branch streams");
        }
        P.branches.push_back(b);
    }
    return CUSCAN_OK;
}

// Every buffer a branch touches, sized before capture: nothing allocates while capturing.
int reserve_branch(cuscan_ctx *ctx, PackBranch &br, const cuscan_fit_item &it) {
    const int64_t n = it.n;
    const int d = it.d, k = item_k(it);
    int rc = forest_reserve(ctx, br.forest, n, d);
    if (!rc) rc = ensure(ctx, br.x, sizeof(float) * n * d, "packed input rows");
    if (!rc) rc = ensure(ctx, br.ids, sizeof(int32_t) * n * k, "packed kNN ids");
    if (!rc) rc = ensure(ctx, br.dsq, sizeof(float) * n * k, "packed kNN distances");
    if (!rc) rc = ensure(ctx, br.core, sizeof(float) * n, "packed core distances");
    if (!rc) rc = ensure(ctx, br.label, sizeof(int32_t) * n, "packed labels");
    if (!rc) rc = ensure(ctx, br.src, sizeof(uint32_t) * n, "packed MST sources");
    if (!rc) rc = ensure(ctx, br.dst, sizeof(uint32_t) * n, "packed MST destinations");
    if (!rc) rc = ensure(ctx, br.w, sizeof(float) * n, "packed MST weights");
    const size_t split = exact_knn_scratch_elems(ctx, n, n, k);
    if (!rc) rc = ensure(ctx, br.forest.knn_ids_tmp, sizeof(int32_t) * split, "packed kNN partials");
    if (!rc) rc = ensure(ctx, br.forest.knn_dist_tmp, sizeof(float) * split, "packed kNN partials");
    // exclusive scans over n entries keep one int per 1024-entry tile
    if (!rc) rc = ensure(ctx, br.forest.scan_tmp, sizeof(int32_t) * ceil_div(n, 1024), "scan tile sums");
    return rc;
}

// One Borůvka round of a branch (the body of the while loop), captured on stream s.
int capture_round(cuscan_ctx *ctx, PackBranch &br, const cuscan_fit_item &it,
                  cudaGraphConditionalHandle loop, cudaStream_t s) {
    ForestBuffers &b = br.forest;
    const int64_t n = it.n;
    const int d = it.d;
    int32_t *label = as<int32_t>(br.label);
    int rc = forest_sort_by_component(ctx, b, as<float>(br.x), as<float>(br.core), label, n, d, s);
    if (!rc) rc = launch_fill_u64(ctx, as<unsigned long long>(b.row_keys), n, ~0ull, s);
    if (!rc)
        rc = launch_candidates_fp32(ctx, as<float>(b.xp), as<float>(b.corep), as<int32_t>(b.labp),
                                    as<int32_t>(b.perm), n, d, as<unsigned long long>(b.row_keys),
                                    as<int32_t>(b.tile_lo), as<int32_t>(b.tile_hi), s);
    // the component count is known only on the device: the pointer doubling takes the step
    // count of the largest packed fit, so that every pack of a given size has the same graph
    // topology (any count >= log2(active nodes) + 1 reaches the same fixed point)
    if (!rc)
        rc = forest_round(ctx, b, n, CUSCAN_PACK_MAX_ROWS, label, as<uint32_t>(br.src), as<uint32_t>(br.dst),
                          as<float>(br.w), s, it.precision != CUSCAN_PRECISION_PLAIN);
    if (rc) return rc;
    CUSCAN_KERNEL(loop_next_kernel, 1, 1, 0, s, b.status, (double)n * (double)n, loop);
    CUSCAN_LAUNCH(ctx, "loop_next_kernel");
    return CUSCAN_OK;
}

// The whole fit of one item as a branch, captured on the branch stream.
int capture_branch(cuscan_ctx *ctx, PackWorkspace &P, PackBranch &br, const cuscan_fit_item &it,
                   const Staging &st) {
    cudaStream_t s = br.stream;
    ForestBuffers &b = br.forest;
    char *stg = static_cast<char *>(P.staging);
    const int64_t n = it.n;
    const int d = it.d, k = item_k(it);
    float *x = as<float>(br.x), *dsq = as<float>(br.dsq), *core = as<float>(br.core);
    int32_t *ids = as<int32_t>(br.ids), *label = as<int32_t>(br.label);
    uint32_t *src = as<uint32_t>(br.src), *dst = as<uint32_t>(br.dst);
    float *w = as<float>(br.w);
    CUSCAN_CUDA(ctx, cudaEventRecordWithFlags(br.ev[0], s, cudaEventRecordExternal));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(x, stg + st.in, sizeof(float) * n * d,
                                     cudaMemcpyHostToDevice, s));
    CUSCAN_CUDA(ctx, cudaMemsetAsync(b.status, 0, sizeof(DevStatus), s));
    int rc = launch_exact_knn_fp32(ctx, x, n, x, n, d, k, 1, 0, 1, ids, dsq, s, b.knn_ids_tmp,
                                   b.knn_dist_tmp);
    if (!rc) rc = forest_core(ctx, dsq, n, k, it.min_samples, core, s);
    if (rc) return rc;
    CUSCAN_CUDA(ctx, cudaEventRecordWithFlags(br.ev[1], s, cudaEventRecordExternal));
    if ((rc = forest_seed(ctx, b, core, ids, dsq, n, k, label, src, dst, w, s,
                          CUSCAN_PACK_MAX_ROWS)))
        return rc;

    // the round loop: a while node after the kernel that sets its first condition
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    CUSCAN_CUDA(ctx, cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, nullptr, nullptr, nullptr));
    cudaGraphConditionalHandle loop;
    CUSCAN_CUDA(ctx, cudaGraphConditionalHandleCreate(&loop, graph, 0, cudaGraphCondAssignDefault));
    br.loop = loop;
    CUSCAN_KERNEL(loop_enter_kernel, 1, 1, 0, s, b.status, loop);
    CUSCAN_LAUNCH(ctx, "loop_enter_kernel");
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    CUSCAN_CUDA(ctx, cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    CUSCAN_CUDA(ctx, cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CUSCAN_CUDA(ctx, cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                                         cudaStreamSetCaptureDependencies));
    CUSCAN_CUDA(ctx, cudaStreamBeginCaptureToGraph(P.body, body, nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeRelaxed));
    rc = capture_round(ctx, br, it, loop, P.body);
    cudaGraph_t captured = nullptr;
    const cudaError_t e = cudaStreamEndCapture(P.body, &captured);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "capture of the round loop");

    if ((rc = forest_mst_weight(ctx, b, w, n - 1, s))) return rc;
    CUSCAN_CUDA(ctx, cudaEventRecordWithFlags(br.ev[2], s, cudaEventRecordExternal));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(stg + st.status, b.status, sizeof(DevStatus),
                                     cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(stg + st.core, core, sizeof(float) * n,
                                     cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(stg + st.src, src, sizeof(uint32_t) * (n - 1),
                                     cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(stg + st.dst, dst, sizeof(uint32_t) * (n - 1),
                                     cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(stg + st.w, w, sizeof(float) * (n - 1),
                                     cudaMemcpyDeviceToHost, s));
    if (it.knn_ids)
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(stg + st.ids, ids, sizeof(int32_t) * n * k,
                                         cudaMemcpyDeviceToHost, s));
    if (it.knn_sq)
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(stg + st.dsq, dsq, sizeof(float) * n * k,
                                         cudaMemcpyDeviceToHost, s));
    return CUSCAN_OK;
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

}  // namespace

int64_t pack_reserved_bytes(const PackWorkspace *p) {
    if (!p) return 0;
    int64_t total = 0;
    Buffer *all[kBranchBufferCount];
    for (PackBranch *b : p->branches) {
        const int c = branch_buffers(b, all);
        for (int i = 0; i < c; ++i) total += (int64_t)all[i]->bytes;
    }
    return total;
}

static void drop_execs(PackWorkspace *p) {
    for (cudaGraphExec_t &e : p->exec) {
        if (e) cudaGraphExecDestroy(e);
        e = nullptr;
    }
}

void pack_release(PackWorkspace *p) {
    if (!p) return;
    drop_execs(p);  // they point at the buffers released here
    Buffer *all[kBranchBufferCount];
    for (PackBranch *b : p->branches) {
        const int c = branch_buffers(b, all);
        for (int i = 0; i < c; ++i) release(*all[i]);
        b->forest.status = nullptr;
    }
    if (p->staging) cudaFreeHost(p->staging);
    p->staging = nullptr;
    p->staging_bytes = 0;
}

void pack_destroy(PackWorkspace *p) {
    if (!p) return;
    pack_release(p);  // also drops the instantiated graphs
    for (PackBranch *b : p->branches) destroy_branch(b);
    if (p->body) cudaStreamDestroy(p->body);
    if (p->fork) cudaEventDestroy(p->fork);
    delete p;
}

}  // namespace cuscan

using namespace cuscan;

extern "C" int cuscan_fit_core_packed_graph_stats(cuscan_ctx *ctx, int64_t *instantiations,
                                                  int64_t *updates) {
    if (!ctx) return CUSCAN_INVALID_INPUT;
    const PackWorkspace *p = ctx->fit ? ctx->fit->pack : nullptr;
    if (instantiations) *instantiations = p ? p->instantiations : 0;
    if (updates) *updates = p ? p->updates : 0;
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
    int rc = make_workspace(ctx, count);
    if (rc) return rc;
    PackWorkspace &P = *ctx->fit->pack;

    // pinned staging: inputs, then outputs, each region 256-byte aligned
    std::vector<Staging> st((size_t)count);
    size_t off = 0;
    for (int i = 0; i < count; ++i) {
        st[i].in = off;
        off = align256(off + sizeof(float) * (size_t)items[i].n * items[i].d);
    }
    for (int i = 0; i < count; ++i) {
        const size_t n = (size_t)items[i].n, nk = n * (size_t)item_k(items[i]);
        st[i].status = off;
        off = align256(off + sizeof(DevStatus));
        st[i].core = off;
        off = align256(off + 4 * n);
        st[i].src = off;
        off = align256(off + 4 * (n - 1));
        st[i].dst = off;
        off = align256(off + 4 * (n - 1));
        st[i].w = off;
        off = align256(off + 4 * (n - 1));
        st[i].ids = off;
        off = align256(off + (items[i].knn_ids ? 4 * nk : 0));
        st[i].dsq = off;
        off = align256(off + (items[i].knn_sq ? 4 * nk : 0));
    }
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (P.staging_bytes < off) {
        if (P.staging) cudaFreeHost(P.staging);
        P.staging = nullptr;
        P.staging_bytes = 0;
        CUSCAN_CUDA(ctx, cudaMallocHost(&P.staging, off));
        P.staging_bytes = off;
    }
    for (int i = 0; i < count; ++i) {
        if ((rc = reserve_branch(ctx, *P.branches[i], items[i]))) {
            items[i].status = rc;
            return rc;
        }
        std::memcpy(static_cast<char *>(P.staging) + st[i].in, items[i].data,
                    sizeof(float) * (size_t)items[i].n * items[i].d);
    }

    // capture: fork one branch per fit from the pack stream, join them all back
    cudaStream_t s0 = ctx->stream;
    CUSCAN_CUDA(ctx, cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed));
    int captured = 0;
    cudaError_t e = cudaEventRecord(P.fork, s0);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "fork of the pack graph");
    for (int i = 0; i < count && !rc; ++i) {
        PackBranch &br = *P.branches[i];
        e = cudaStreamWaitEvent(br.stream, P.fork, 0);
        if (e != cudaSuccess) {
            rc = cuda_fail(ctx, e, "fork of a pack branch");
            break;
        }
        ++captured;
        rc = capture_branch(ctx, P, br, items[i], st[i]);
        if (rc) items[i].status = rc;
    }
    // every forked branch joins the pack stream, also after a failure, so the capture ends
    for (int i = 0; i < captured; ++i) {
        PackBranch &br = *P.branches[i];
        cudaEventRecord(br.join, br.stream);
        cudaStreamWaitEvent(s0, br.join, 0);
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s0, &graph);
    if (!rc && e != cudaSuccess) rc = cuda_fail(ctx, e, "capture of the pack graph");
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return rc;
    }
    // the instantiated graph of this pack size takes the new graph's parameters; a graph that
    // does not match (or the first pack of this size) is instantiated
    cudaGraphExec_t &exec = P.exec[count];
    bool updated = false;
    bool same_handles = true;
    for (int i = 0; i < count; ++i) same_handles &= P.branches[i]->loop == P.exec_loop[count][i];
    if (exec && !same_handles) {
        cudaGraphExecDestroy(exec);
        exec = nullptr;
    }
    if (exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(exec, graph, &info) == cudaSuccess) {
            updated = true;
            ++P.updates;
        } else {
            cudaGetLastError();
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
    }
    if (!updated) {
        e = cudaGraphInstantiate(&exec, graph, 0);
        if (e != cudaSuccess) {
            exec = nullptr;
            cudaGraphDestroy(graph);
            return cuda_fail(ctx, e, "instantiation of the pack graph");
        }
        ++P.instantiations;
        for (int i = 0; i < count; ++i) P.exec_loop[count][i] = P.branches[i]->loop;
    }
    cudaGraphDestroy(graph);
    e = cudaGraphLaunch(exec, s0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s0);
    if (e != cudaSuccess) {
        cudaGraphExecDestroy(exec);
        exec = nullptr;
        return cuda_fail(ctx, e, "pack graph");
    }

    // results
    const char *stg = static_cast<const char *>(P.staging);
    int first = CUSCAN_OK;
    char first_err[sizeof(ctx->err)] = {0};
    for (int i = 0; i < count; ++i) {
        cuscan_fit_item &it = items[i];
        PackBranch &br = *P.branches[i];
        DevStatus hs;
        std::memcpy(&hs, stg + st[i].status, sizeof(hs));
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
        std::memcpy(it.core_sq, stg + st[i].core, sizeof(float) * n);
        std::memcpy(it.mst_src, stg + st[i].src, sizeof(uint32_t) * (n - 1));
        std::memcpy(it.mst_dst, stg + st[i].dst, sizeof(uint32_t) * (n - 1));
        std::memcpy(it.mst_wsq, stg + st[i].w, sizeof(float) * (n - 1));
        if (it.knn_ids) std::memcpy(it.knn_ids, stg + st[i].ids, sizeof(int32_t) * n * k);
        if (it.knn_sq) std::memcpy(it.knn_sq, stg + st[i].dsq, sizeof(float) * n * k);
        cuscan_fit_stats &S = it.stats;
        S.core_ms = elapsed_ms(br.ev[0], br.ev[1]);
        S.knn_kernel_ms = S.core_ms;
        S.mst_ms = elapsed_ms(br.ev[1], br.ev[2]);
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
