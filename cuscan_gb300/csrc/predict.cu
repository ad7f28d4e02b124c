// approximate_predict: the prediction hierarchy of a fitted model and exact candidate searches
// on the device.
//
// The hierarchy is the reference's PredictionHierarchy (crates/hdbscan-core/src/prediction.rs):
// cluster nodes of the final condensed tree with the selected label and the selected anchor's
// maximum lambda propagated top down (new, prediction.rs:433-700), every finite training point
// attached to its condensed-tree parent with its departure lambda, and the per-query candidate
// math (predict_row, prediction.rs:855-925). All of that is f64 host arithmetic, as in the
// reference.
//
// The device does the two searches of crates/hdbscan/src/prediction.rs:1658-1978:
//  - prediction cores: each finite training row against all of them, self included, width s;
//    the core is the Euclidean distance at rank s - 1 (computed once per predictor);
//  - queries: each query row against the finite training rows, width 2 s, ordered by
//    (squared distance, compact id).
// Both use the exact f32 kNN kernel, so the distances are the reference's f32 values.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "forest.cuh"
#include "workspace.cuh"

struct cuscan_predictor {
    int device = -1;            // -1: host-only (candidate math without device searches)
    int64_t n_finite = 0;
    int32_t d = 0;
    int32_t s = 0;               // min_samples
    std::vector<uint32_t> finite_index;
    // cluster nodes (index 0 is the root); empty for the no-cluster-tree state
    std::vector<int64_t> node_id, node_parent;
    std::vector<double> node_birth, node_max;
    std::vector<int32_t> node_label;
    // attachment of each compact finite row
    std::vector<int64_t> point_node;
    std::vector<double> point_departure;
    std::vector<double> cores;   // prediction core distances (Euclidean, f64)
    float *train = nullptr;      // device copy of the finite training rows [n_finite, d]
};

namespace cuscan {
namespace {

int invalid(cuscan_ctx *ctx, const std::string &msg) {
    return fail(ctx, CUSCAN_INVALID_INPUT, "%s", msg.c_str());
}

bool is_finite_row(const std::vector<uint32_t> &fi, int64_t raw, int64_t *pos = nullptr) {
    auto it = std::lower_bound(fi.begin(), fi.end(), (uint32_t)raw);
    if (raw < 0 || raw > (int64_t)UINT32_MAX || it == fi.end() || (int64_t)*it != raw) return false;
    if (pos) *pos = it - fi.begin();
    return true;
}

// PredictionHierarchy::new (prediction.rs:433-700) on the raw-id condensed tree.
int build_hierarchy(cuscan_ctx *ctx, cuscan_predictor &P, const int64_t *parent,
                    const int64_t *child, const float *lambda, const float *size, int64_t rows,
                    const int32_t *labels, int64_t raw_n) {
    const std::vector<uint32_t> &fi = P.finite_index;
    if (raw_n > INT32_MAX) return fail(ctx, CUSCAN_OVERFLOW, "raw point index");
    if (fi.empty()) return invalid(ctx, "prediction requires at least one finite training point");
    for (size_t i = 1; i < fi.size(); ++i)
        if (fi[i - 1] >= fi[i]) return invalid(ctx, "finite index must be strictly ascending");
    if ((int64_t)fi.back() >= raw_n) return invalid(ctx, "finite index refers past the raw row count");
    {
        size_t next = 0;
        for (int64_t raw = 0; raw < raw_n; ++raw) {
            const bool finite = next < fi.size() && (int64_t)fi[next] == raw;
            if (finite) ++next;
            if (labels[raw] < -1 || (!finite && labels[raw] != -1))
                return invalid(ctx, "invalid fitted label " + std::to_string(labels[raw]) +
                                        " for row " + std::to_string(raw));
        }
    }
    for (int64_t r = 0; r < rows; ++r) {
        const int64_t p = parent[r], c = child[r];
        const float l = lambda[r], z = size[r];
        if (p < raw_n)
            return invalid(ctx, "condensed tree row " + std::to_string(r) + " has point id " +
                                    std::to_string(p) + " as a parent");
        if (std::isnan(l) || l < 0.0f)
            return invalid(ctx, "condensed tree row " + std::to_string(r) + " has invalid lambda");
        if (!std::isfinite(z) || z < 1.0f)
            return invalid(ctx, "condensed tree row " + std::to_string(r) +
                                    " has invalid child size");
        const bool is_point = c >= 0 && c < raw_n;
        const bool is_cluster = z > 1.0f;
        if (is_point == is_cluster)
            return invalid(ctx, "condensed tree row " + std::to_string(r) +
                                    " mixes point/cluster child");
        if (is_cluster && c <= p)
            return invalid(ctx, "cluster edge " + std::to_string(p) + " -> " + std::to_string(c) +
                                    " does not increase the cluster id");
    }
    std::vector<int64_t> cluster_rows;
    for (int64_t r = 0; r < rows; ++r)
        if (size[r] > 1.0f) cluster_rows.push_back(r);

    if (cluster_rows.empty()) {
        // root-only trees: one parent, each finite point exactly once
        if (rows == 0 && fi.size() >= 2)
            return invalid(ctx, "condensed tree has no rows for several finite training points");
        if (rows > 0) {
            for (int64_t r = 0; r < rows; ++r)
                if (parent[r] != parent[0])
                    return invalid(ctx, "root-only condensed tree has several parents");
            std::vector<char> seen(fi.size(), 0);
            for (int64_t r = 0; r < rows; ++r) {
                int64_t pos;
                if (!is_finite_row(fi, child[r], &pos)) continue;
                if (seen[pos]) return invalid(ctx, "training point has more than one condensed tree row");
                seen[pos] = 1;
            }
            for (size_t i = 0; i < fi.size(); ++i)
                if (!seen[i]) return invalid(ctx, "finite training point has no condensed tree row");
        }
        return CUSCAN_OK;  // no-cluster-tree state: nodes stay empty
    }

    int64_t root_id = parent[cluster_rows[0]];
    for (int64_t r : cluster_rows) root_id = std::min(root_id, parent[r]);
    std::unordered_map<int64_t, int64_t> node_of;
    node_of.reserve(cluster_rows.size() * 2 + 2);
    node_of[root_id] = 0;
    P.node_id.assign(1, root_id);
    for (int64_t r : cluster_rows) {
        if (!node_of.emplace(child[r], (int64_t)P.node_id.size()).second)
            return invalid(ctx, "cluster " + std::to_string(child[r]) +
                                    " has more than one parent edge or is the root");
        P.node_id.push_back(child[r]);
    }
    const size_t nn = P.node_id.size();
    P.node_parent.assign(nn, -1);
    P.node_birth.assign(nn, 0.0);
    P.node_label.assign(nn, -1);
    P.node_max.assign(nn, 0.0);
    for (size_t o = 0; o < cluster_rows.size(); ++o) {
        auto it = node_of.find(parent[cluster_rows[o]]);
        if (it == node_of.end())
            return invalid(ctx, "cluster parent is neither the root nor a child cluster");
        P.node_parent[o + 1] = it->second;
        P.node_birth[o + 1] = (double)lambda[cluster_rows[o]];
    }
    // maximum lambda of every node over its rows; point attachments; label anchors
    std::vector<double> max_lambda(nn, 0.0);
    std::vector<char> seen(nn, 0);
    P.point_node.assign(fi.size(), -1);
    P.point_departure.assign(fi.size(), 0.0);
    std::unordered_map<int32_t, int64_t> anchors;
    for (int64_t r = 0; r < rows; ++r) {
        auto it = node_of.find(parent[r]);
        if (it == node_of.end())
            return invalid(ctx, "condensed tree parent " + std::to_string(parent[r]) +
                                    " is not part of the cluster tree");
        const int64_t node = it->second;
        const double l = (double)lambda[r];
        if (!seen[node] || l > max_lambda[node]) {
            max_lambda[node] = l;
            seen[node] = 1;
        }
        int64_t pos;
        if (!is_finite_row(fi, child[r], &pos)) continue;
        if (P.point_node[pos] >= 0)
            return invalid(ctx, "training point " + std::to_string(child[r]) +
                                    " has more than one condensed tree row");
        P.point_node[pos] = node;
        P.point_departure[pos] = l;
        const int32_t label = labels[child[r]];
        if (label >= 0) {
            auto a = anchors.emplace(label, parent[r]).first;
            if (parent[r] < a->second) a->second = parent[r];
        }
    }
    for (size_t i = 0; i < fi.size(); ++i)
        if (P.point_node[i] < 0)
            return invalid(ctx, "finite training point " + std::to_string(fi[i]) +
                                    " has no condensed tree row");
    std::vector<int32_t> anchor_label(nn, -1);
    std::vector<char> anchored(nn, 0);
    for (const auto &a : anchors) {
        const int64_t node = node_of[a.second];
        if (anchored[node])
            return invalid(ctx, "two fitted labels share one selected cluster");
        anchored[node] = 1;
        anchor_label[node] = a.first;
    }
    // top down: a node's own anchor wins over the inherited values
    std::vector<int64_t> child_start(nn + 1, 0), fill, children(nn > 0 ? nn - 1 : 0);
    for (size_t i = 1; i < nn; ++i) child_start[P.node_parent[i] + 1] += 1;
    for (size_t i = 0; i < nn; ++i) child_start[i + 1] += child_start[i];
    fill = child_start;
    for (size_t i = 1; i < nn; ++i) children[fill[P.node_parent[i]]++] = (int64_t)i;
    std::vector<int64_t> stack{0};
    size_t visited = 0;
    while (!stack.empty()) {
        const int64_t node = stack.back();
        stack.pop_back();
        ++visited;
        for (int64_t c = child_start[node]; c < child_start[node + 1]; ++c)
            stack.push_back(children[c]);
        if (anchored[node]) {
            P.node_label[node] = anchor_label[node];
            P.node_max[node] = max_lambda[node];
        } else if (P.node_parent[node] >= 0) {
            P.node_label[node] = P.node_label[P.node_parent[node]];
            P.node_max[node] = P.node_max[P.node_parent[node]];
        }
    }
    if (visited != nn) return invalid(ctx, "cluster tree is not connected to its root");
    return CUSCAN_OK;
}

// predict_row (prediction.rs:855-925): first minimum mutual-reachability candidate, then the
// ascent from its attachment while the parent edge was born at or after the query's lambda.
int predict_row(cuscan_ctx *ctx, const cuscan_predictor &P, const int32_t *ids,
                const double *dist, int32_t *label, double *strength, int32_t *connector) {
    const int width = 2 * P.s;
    for (int c = 0; c < width; ++c)
        if (!std::isfinite(dist[c]) || dist[c] < 0.0)
            return fail(ctx, CUSCAN_NUMERICAL, "invalid candidate distance %g", dist[c]);
    const double query_core = dist[P.s];
    int best = -1;
    double best_mrd = 0.0;
    for (int c = 0; c < width; ++c) {
        const int32_t id = ids[c];
        if (id < 0 || (int64_t)id >= P.n_finite)
            return fail(ctx, CUSCAN_NUMERICAL, "invalid candidate id %d", id);
        const double core = P.cores[id];
        if (!std::isfinite(core) || core < 0.0)
            return fail(ctx, CUSCAN_NUMERICAL, "invalid prediction core distance %g", core);
        const double mrd = std::max(std::max(core, query_core), dist[c]);
        if (best < 0 || mrd < best_mrd) {
            best = c;
            best_mrd = mrd;
        }
    }
    const int32_t conn = ids[best];
    const double lam = best_mrd > 0.0 ? 1.0 / best_mrd : DBL_MAX;
    int64_t cluster = P.point_node[conn];
    if (P.point_departure[conn] > lam) {
        const int64_t root_id = P.node_id[0];
        while (P.node_id[cluster] > root_id) {
            const int64_t parent = P.node_parent[cluster];
            if (parent >= 0 && P.node_birth[cluster] >= lam) cluster = parent;
            else break;
        }
    }
    const int32_t lab = P.node_label[cluster];
    const double mx = P.node_max[cluster];
    if (lab < 0) {
        *label = -1;
        *strength = 0.0;
    } else if (mx > 0.0) {
        *label = lab;
        *strength = std::min(mx, lam) / mx;
    } else {
        *label = lab;
        *strength = 1.0;
    }
    *connector = (int32_t)P.finite_index[conn];
    return CUSCAN_OK;
}

int euclidean(cuscan_ctx *ctx, float sq, double *out) {
    if (!std::isfinite(sq) || sq < 0.0f)
        return fail(ctx, CUSCAN_NUMERICAL, "neighbor search returned invalid squared distance %g",
                    (double)sq);
    *out = std::sqrt((double)sq);
    return CUSCAN_OK;
}

}  // namespace
}  // namespace cuscan

using namespace cuscan;

namespace {
int predict_candidates(cuscan_ctx *ctx, const cuscan_predictor *p, const int32_t *ids,
                       const double *distances, int64_t m, int32_t *labels, double *strengths,
                       int32_t *connecting_points);
int predict_queries(cuscan_ctx *ctx, const cuscan_predictor *p, const float *queries, int64_t m,
                    int32_t *labels, double *strengths, int32_t *connecting_points);
}  // namespace

extern "C" {

static int create_predictor(cuscan_ctx *ctx, const float *train, int64_t n_finite, int32_t d,
                            int32_t min_samples, const int64_t *tree_parent,
                            const int64_t *tree_child, const float *tree_lambda,
                            const float *tree_child_size, int64_t tree_rows,
                            const int32_t *labels, int64_t raw_n, const uint32_t *finite_index,
                            const double *prediction_core, cuscan_predictor **out) {
    *out = nullptr;
    if (min_samples <= 0) return fail(ctx, CUSCAN_INVALID_INPUT, "min_samples must be positive");
    if (n_finite <= 0 || d <= 0 || raw_n < n_finite || tree_rows < 0 || !labels || !finite_index ||
        (tree_rows > 0 && (!tree_parent || !tree_child || !tree_lambda || !tree_child_size)))
        return fail(ctx, CUSCAN_INVALID_INPUT, "invalid predictor arguments");
    if (n_finite > INT32_MAX - 1) return fail(ctx, CUSCAN_OVERFLOW, "training row count");
    if (!train && !prediction_core)
        return fail(ctx, CUSCAN_INVALID_INPUT,
                    "a predictor without training rows needs its prediction core distances");
    if (train && !ctx->fit)
        return fail(ctx, CUSCAN_INVALID_INPUT, "a predictor with training rows needs a context");
    auto P = std::make_unique<cuscan_predictor>();
    P->n_finite = n_finite;
    P->d = d;
    P->s = min_samples;
    P->finite_index.assign(finite_index, finite_index + n_finite);
    int rc = build_hierarchy(ctx, *P, tree_parent, tree_child, tree_lambda, tree_child_size,
                             tree_rows, labels, raw_n);
    if (rc) return rc;
    const bool clustered = !P->node_id.empty();
    if (clustered && 2 * (int64_t)min_samples > n_finite)
        return fail(ctx, CUSCAN_INVALID_INPUT,
                    "approximate_predict needs 2*min_samples = %lld neighbors but the model has "
                    "only %lld finite training points",
                    2 * (long long)min_samples, (long long)n_finite);
    if (prediction_core) {
        P->cores.assign(prediction_core, prediction_core + n_finite);
        for (double c : P->cores)
            if (!std::isfinite(c) || c < 0.0)
                return fail(ctx, CUSCAN_NUMERICAL, "invalid prediction core distance %g", c);
    }
    if (train && clustered) {
        CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
        cudaStream_t s = ctx->stream;
        const size_t bytes = sizeof(float) * (size_t)n_finite * d;
        cudaError_t e = cudaMalloc(&P->train, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, CUSCAN_MEMORY, "device allocation of %zu bytes for the training rows "
                        "failed", bytes);
        }
        P->device = ctx->device;
        std::unique_ptr<cuscan_predictor, void (*)(cuscan_predictor *)> guard(
            P.get(), [](cuscan_predictor *q) {
                if (q->train) cudaFree(q->train);
                q->train = nullptr;
            });
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(P->train, train, bytes, cudaMemcpyHostToDevice, s));
        if (!prediction_core) {
            // training cores: self-inclusive rows of width s, Euclidean value at rank s - 1
            P->cores.assign(n_finite, 0.0);
            if (min_samples > 1) {
                FitWorkspace *f = ctx->fit;
                const int k = min_samples;
                rc = ensure(ctx, f->pred_ids, sizeof(int32_t) * n_finite * k, "core ids");
                if (!rc) rc = ensure(ctx, f->pred_dist, sizeof(float) * n_finite * k, "core distances");
                if (!rc) rc = launch_exact_knn_fp32(ctx, P->train, n_finite, P->train, n_finite, d, k,
                                                    0, 0, 1, as<int32_t>(f->pred_ids),
                                                    as<float>(f->pred_dist), s, f->op_knn_ids,
                                                    f->op_knn_dist);
                if (rc) return rc;
                std::vector<float> sq((size_t)n_finite * k);
                CUSCAN_CUDA(ctx, cudaMemcpyAsync(sq.data(), f->pred_dist.ptr, sizeof(float) * sq.size(),
                                                 cudaMemcpyDeviceToHost, s));
                CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
                for (int64_t i = 0; i < n_finite; ++i)
                    if ((rc = euclidean(ctx, sq[(size_t)i * k + k - 1], &P->cores[i]))) return rc;
            }
        }
        CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
        guard.release();
    } else if (!prediction_core) {
        P->cores.assign(n_finite, 0.0);  // no cluster tree: cores are never read
    }
    *out = P.release();
    return CUSCAN_OK;
}

int cuscan_predictor_create(cuscan_ctx *ctx, const float *train, int64_t n_finite, int32_t d,
                            int32_t min_samples, const int64_t *tree_parent,
                            const int64_t *tree_child, const float *tree_lambda,
                            const float *tree_child_size, int64_t tree_rows,
                            const int32_t *labels, int64_t raw_n, const uint32_t *finite_index,
                            const double *prediction_core, cuscan_predictor **out, char *err,
                            size_t err_len) {
    if (!out) return CUSCAN_INVALID_INPUT;
    cuscan_ctx local;  // collects the message when no context is given
    cuscan_ctx *ectx = ctx ? ctx : &local;
    clear_error(ectx);
    if (train && !ctx) {
        *out = nullptr;
        if (err && err_len) std::snprintf(err, err_len, "training rows need a device context");
        return CUSCAN_INVALID_INPUT;
    }
    const int rc = create_predictor(ectx, train, n_finite, d, min_samples, tree_parent, tree_child,
                                    tree_lambda, tree_child_size, tree_rows, labels, raw_n,
                                    finite_index, prediction_core, out);
    if (rc && err && err_len) std::snprintf(err, err_len, "%s", ectx->err);
    return rc;
}

void cuscan_predictor_destroy(cuscan_predictor *p) {
    if (!p) return;
    if (p->train) {
        cudaSetDevice(p->device);
        cudaFree(p->train);
    }
    delete p;
}

// ---- portable state (crates/hdbscan-core/src/prediction.rs:161-433) ----

int cuscan_predictor_state_shape(const cuscan_predictor *p, int64_t *n_finite,
                                 int64_t *cluster_nodes) {
    if (!p) return CUSCAN_INVALID_INPUT;
    const bool tree = !p->node_id.empty();
    if (n_finite) *n_finite = tree ? p->n_finite : 0;
    if (cluster_nodes) *cluster_nodes = (int64_t)p->node_id.size();
    return CUSCAN_OK;
}

int cuscan_predictor_export(cuscan_ctx *ctx, const cuscan_predictor *p, float *geometry,
                            uint32_t *finite_index, uint64_t *node_ids,
                            uint64_t *node_parent_indices, double *node_birth_lambdas,
                            int32_t *node_labels, double *node_max_lambdas,
                            uint64_t *point_node_indices, double *point_departure_lambdas,
                            double *prediction_cores) {
    if (!p) return CUSCAN_INVALID_INPUT;
    if (p->node_id.empty()) return CUSCAN_OK;  // no-cluster-tree state: nothing to export
    cuscan_ctx local;
    cuscan_ctx *ectx = ctx ? ctx : &local;
    if (!finite_index || !node_ids || !node_parent_indices || !node_birth_lambdas ||
        !node_labels || !node_max_lambdas || !point_node_indices || !point_departure_lambdas ||
        !prediction_cores)
        return fail(ectx, CUSCAN_INVALID_INPUT, "predictor export received a null pointer");
    clear_error(ectx);
    // A host-only predictor (no device rows) exports its columns without geometry.
    if (p->train) {
        if (!ctx || !geometry)
            return fail(ectx, CUSCAN_INVALID_INPUT, "predictor geometry export needs a context "
                        "and a buffer");
        if (p->device != ctx->device)
            return fail(ctx, CUSCAN_INVALID_INPUT, "the predictor's training rows are not on this "
                        "device");
        CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
        CUSCAN_CUDA(ctx, cudaMemcpyAsync(geometry, p->train, sizeof(float) * p->n_finite * p->d,
                                         cudaMemcpyDeviceToHost, ctx->stream));
    } else if (geometry) {
        return fail(ectx, CUSCAN_INVALID_INPUT, "this predictor holds no training rows");
    }
    const size_t nn = p->node_id.size();
    for (size_t i = 0; i < nn; ++i) {
        node_ids[i] = (uint64_t)p->node_id[i];
        node_parent_indices[i] = p->node_parent[i] < 0 ? UINT64_MAX : (uint64_t)p->node_parent[i];
        node_birth_lambdas[i] = p->node_birth[i];
        node_labels[i] = p->node_label[i];
        node_max_lambdas[i] = p->node_max[i];
    }
    for (int64_t i = 0; i < p->n_finite; ++i) {
        finite_index[i] = p->finite_index[i];
        point_node_indices[i] = (uint64_t)p->point_node[i];
        point_departure_lambdas[i] = p->point_departure[i];
        prediction_cores[i] = p->cores[i];
    }
    if (p->train) CUSCAN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CUSCAN_OK;
}

namespace {
// PredictionHierarchy::from_state (prediction.rs:279-433): every column is untrusted.
int import_state(cuscan_ctx *ctx, cuscan_predictor &P, int64_t nn, const uint64_t *node_ids,
                 const uint64_t *parents, const double *births, const int32_t *labels,
                 const double *maxes, const uint64_t *point_nodes, const double *departures) {
    const int64_t nf = P.n_finite;
    if (nf > INT32_MAX || nn > INT32_MAX)
        return fail(ctx, CUSCAN_OVERFLOW, "portable prediction hierarchy count");
    for (int64_t i = 0; i < nf; ++i)
        if (P.finite_index[i] > (uint32_t)INT32_MAX ||
            (i > 0 && P.finite_index[i - 1] >= P.finite_index[i]))
            return invalid(ctx, "portable finite index must be strictly ascending and fit i32");
    std::unordered_map<uint64_t, int64_t> seen;
    seen.reserve((size_t)nn * 2);
    uint64_t min_id = UINT64_MAX;
    for (int64_t i = 0; i < nn; ++i) {
        if (!seen.emplace(node_ids[i], i).second)
            return invalid(ctx, "portable hierarchy node ids are not unique");
        min_id = node_ids[i] < min_id ? node_ids[i] : min_id;
    }
    if (node_ids[0] != min_id)
        return invalid(ctx, "portable hierarchy root is not the minimum node id");
    uint64_t zero_bits = 0, b0 = 0;
    std::memcpy(&b0, &births[0], sizeof(b0));
    if (parents[0] != UINT64_MAX || b0 != zero_bits)
        return invalid(ctx, "portable hierarchy root sentinel or birth lambda is not canonical");
    for (int64_t i = 1; i < nn; ++i) {
        const uint64_t par = parents[i];
        if (par >= (uint64_t)nn || par == (uint64_t)i || node_ids[par] >= node_ids[i] ||
            node_ids[i] <= node_ids[0])
            return invalid(ctx, "portable hierarchy parent graph is invalid");
    }
    std::unordered_map<int32_t, int> used;
    if (labels[0] >= 0) used.emplace(labels[0], 1);
    for (int64_t i = 0; i < nn; ++i) {
        if (std::isnan(births[i]) || births[i] < 0.0 || std::isnan(maxes[i]) || maxes[i] < 0.0 ||
            labels[i] < -1)
            return invalid(ctx, "portable hierarchy contains an invalid lambda or label");
        if (i == 0) {
            uint64_t mb = 0;
            std::memcpy(&mb, &maxes[0], sizeof(mb));
            if (labels[0] == -1 && mb != zero_bits)
                return invalid(ctx, "unmapped portable hierarchy root must have canonical zero "
                                    "maximum");
        } else {
            const int64_t par = (int64_t)parents[i];
            if (labels[i] == labels[par]) {
                uint64_t a = 0, b = 0;
                std::memcpy(&a, &maxes[i], sizeof(a));
                std::memcpy(&b, &maxes[par], sizeof(b));
                if (a != b)
                    return invalid(ctx, "inherited portable hierarchy maximum differs from its "
                                        "parent");
            } else if (labels[i] < 0 || !used.emplace(labels[i], 1).second) {
                return invalid(ctx, "portable hierarchy anchor labels are invalid or duplicated");
            }
        }
    }
    for (int64_t i = 0; i < nf; ++i)
        if (point_nodes[i] >= (uint64_t)nn || std::isnan(departures[i]) || departures[i] < 0.0)
            return invalid(ctx, "portable point attachment is invalid");
    P.node_id.resize((size_t)nn);
    P.node_parent.resize((size_t)nn);
    P.node_birth.assign(births, births + nn);
    P.node_label.assign(labels, labels + nn);
    P.node_max.assign(maxes, maxes + nn);
    for (int64_t i = 0; i < nn; ++i) {
        P.node_id[i] = (int64_t)node_ids[i];
        P.node_parent[i] = i == 0 ? -1 : (int64_t)parents[i];
    }
    P.point_node.resize((size_t)nf);
    for (int64_t i = 0; i < nf; ++i) P.point_node[i] = (int64_t)point_nodes[i];
    P.point_departure.assign(departures, departures + nf);
    return CUSCAN_OK;
}
}  // namespace

int cuscan_predictor_from_state(cuscan_ctx *ctx, const float *geometry, int64_t n_finite,
                                int32_t d, int32_t min_samples, const uint32_t *finite_index,
                                int64_t cluster_nodes, const uint64_t *node_ids,
                                const uint64_t *node_parent_indices,
                                const double *node_birth_lambdas, const int32_t *node_labels,
                                const double *node_max_lambdas,
                                const uint64_t *point_node_indices,
                                const double *point_departure_lambdas,
                                const double *prediction_cores, cuscan_predictor **out,
                                char *err, size_t err_len) {
    if (!out) return CUSCAN_INVALID_INPUT;
    *out = nullptr;
    cuscan_ctx local;
    cuscan_ctx *ectx = ctx ? ctx : &local;
    clear_error(ectx);
    auto finish = [&](int rc) {
        if (rc && err && err_len) std::snprintf(err, err_len, "%s", ectx->err);
        return rc;
    };
    if (d <= 0 || min_samples <= 0)
        return finish(fail(ectx, CUSCAN_INVALID_INPUT,
                           "predictor feature count and min_samples must be positive"));
    auto P = std::make_unique<cuscan_predictor>();
    P->d = d;
    P->s = min_samples;
    if (n_finite == 0 && cluster_nodes == 0) {  // the no-cluster-tree state
        *out = P.release();
        return CUSCAN_OK;
    }
    if (n_finite <= 0 || cluster_nodes <= 0)
        return finish(invalid(ectx, "portable prediction hierarchy has a partially empty column set"));
    if (!finite_index || !node_ids || !node_parent_indices || !node_birth_lambdas ||
        !node_labels || !node_max_lambdas || !point_node_indices || !point_departure_lambdas ||
        !prediction_cores)
        return finish(fail(ectx, CUSCAN_INVALID_INPUT, "predictor state received a null pointer"));
    if (2 * (int64_t)min_samples > n_finite)
        return finish(invalid(ectx, "predictor min_samples exceeds candidate-width limit"));
    if (geometry && !ctx)
        return finish(fail(ectx, CUSCAN_INVALID_INPUT, "predictor geometry needs a device context"));
    P->n_finite = n_finite;
    P->finite_index.assign(finite_index, finite_index + n_finite);
    int rc = import_state(ectx, *P, cluster_nodes, node_ids, node_parent_indices,
                          node_birth_lambdas, node_labels, node_max_lambdas, point_node_indices,
                          point_departure_lambdas);
    if (rc) return finish(rc);
    P->cores.assign(prediction_cores, prediction_cores + n_finite);
    // import_predictor_state (crates/hdbscan/src/prediction.rs:1411-1424).
    for (double c : P->cores) {
        if (!std::isfinite(c) || c < 0.0)
            return finish(invalid(ectx, "prediction cores must be finite, nonnegative, and match "
                                        "finite rows"));
        uint64_t bits = 0;
        std::memcpy(&bits, &c, sizeof(bits));
        if (min_samples == 1 && bits != 0)
            return finish(invalid(ectx, "rank-one prediction cores must be canonical positive zero"));
    }
    if (!geometry) {  // host-only: the candidate math without device searches
        *out = P.release();
        return CUSCAN_OK;
    }
    for (int64_t i = 0; i < n_finite * (int64_t)d; ++i)
        if (!std::isfinite(geometry[i]))
            return finish(invalid(ectx, "predictor geometry must be finite"));
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = sizeof(float) * (size_t)n_finite * d;
    cudaError_t e = cudaMalloc(&P->train, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return finish(fail(ctx, CUSCAN_MEMORY, "device allocation of %zu bytes for the training "
                           "rows failed", bytes));
    }
    P->device = ctx->device;
    e = cudaMemcpyAsync(P->train, geometry, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(P->train);
        P->train = nullptr;
        return finish(cuda_fail(ctx, e, "predictor geometry upload"));
    }
    *out = P.release();
    return CUSCAN_OK;
}

int cuscan_predictor_shape(const cuscan_predictor *p, int64_t *n_finite, int32_t *d,
                           int32_t *min_samples) {
    if (!p) return CUSCAN_INVALID_INPUT;
    if (n_finite) *n_finite = p->n_finite;
    if (d) *d = p->d;
    if (min_samples) *min_samples = p->s;
    return CUSCAN_OK;
}

int64_t cuscan_predict_workspace_bytes(const cuscan_predictor *p, int64_t m) {
    if (!p || m <= 0) return 0;
    const int64_t k = 2 * (int64_t)p->s;
    // query rows, candidate ids and distances, split-search partial lists
    const int64_t split = 8 * k * 128 * (4 * (int64_t)kSMs + ceil_div(m, (int64_t)128));
    return (int64_t)sizeof(float) * m * p->d + 8 * m * k + split + (1 << 20);
}

int cuscan_predictor_no_cluster_tree(const cuscan_predictor *p) {
    return p && p->node_id.empty() ? 1 : 0;
}

int cuscan_predictor_read_cores(const cuscan_predictor *p, double *out) {
    if (!p || !out) return CUSCAN_INVALID_INPUT;
    std::memcpy(out, p->cores.data(), sizeof(double) * p->cores.size());
    return CUSCAN_OK;
}

int cuscan_predictor_predict_candidates(const cuscan_predictor *p, const int32_t *ids,
                                        const double *distances, int64_t m, int32_t *labels,
                                        double *strengths, int32_t *connecting_points, char *err,
                                        size_t err_len) {
    if (!p) return CUSCAN_INVALID_INPUT;
    cuscan_ctx local;  // collects the message
    cuscan_ctx *ctx = &local;
    const int rc = predict_candidates(ctx, p, ids, distances, m, labels, strengths,
                                      connecting_points);
    if (rc && err && err_len) std::snprintf(err, err_len, "%s", ctx->err);
    return rc;
}

int cuscan_predictor_predict(cuscan_ctx *ctx, const cuscan_predictor *p, const float *queries,
                             int64_t m, int32_t *labels, double *strengths,
                             int32_t *connecting_points) {
    if (!ctx || !p) return CUSCAN_INVALID_INPUT;
    clear_error(ctx);
    return predict_queries(ctx, p, queries, m, labels, strengths, connecting_points);
}

}  // extern "C"

namespace {

int predict_candidates(cuscan_ctx *ctx, const cuscan_predictor *p, const int32_t *ids,
                       const double *distances, int64_t m, int32_t *labels, double *strengths,
                       int32_t *connecting_points) {
    if (m < 0 || (m > 0 && (!ids || !distances || !labels || !strengths || !connecting_points)))
        return fail(ctx, CUSCAN_INVALID_INPUT, "invalid candidate batch");
    if (p->node_id.empty())
        return fail(ctx, CUSCAN_INVALID_INPUT,
                    "model has no cluster tree; use the no-cluster-tree shortcut");
    const int width = 2 * p->s;
    for (int64_t q = 0; q < m; ++q) {
        int rc = predict_row(ctx, *p, ids + q * width, distances + q * width, labels + q,
                             strengths + q, connecting_points + q);
        if (rc) return rc;
    }
    return CUSCAN_OK;
}

int predict_queries(cuscan_ctx *ctx, const cuscan_predictor *p, const float *queries, int64_t m,
                    int32_t *labels, double *strengths, int32_t *connecting_points) {
    if (m <= 0 || !queries || !labels || !strengths || !connecting_points)
        return fail(ctx, CUSCAN_INVALID_INPUT, "X must contain at least one row and one feature");
    if (p->node_id.empty()) {  // no-cluster-tree shortcut: all noise, zero strength, -1
        for (int64_t q = 0; q < m; ++q) {
            labels[q] = -1;
            strengths[q] = 0.0;
            connecting_points[q] = -1;
        }
        return CUSCAN_OK;
    }
    if (!p->train || p->device != ctx->device)
        return fail(ctx, CUSCAN_INVALID_INPUT, "the predictor's training rows are not on this device");
    for (int64_t i = 0; i < m * (int64_t)p->d; ++i)
        if (!std::isfinite(queries[i]))
            return fail(ctx, CUSCAN_INVALID_INPUT, "X must contain only finite values");
    CUSCAN_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    FitWorkspace *f = ctx->fit;
    const int k = 2 * p->s;
    int rc = ensure(ctx, f->pred_q, sizeof(float) * m * p->d, "query rows");
    if (!rc) rc = ensure(ctx, f->pred_ids, sizeof(int32_t) * m * k, "query candidates");
    if (!rc) rc = ensure(ctx, f->pred_dist, sizeof(float) * m * k, "query candidate distances");
    if (rc) return rc;
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(f->pred_q.ptr, queries, sizeof(float) * m * p->d,
                                     cudaMemcpyHostToDevice, s));
    if ((rc = launch_exact_knn_fp32(ctx, as<float>(f->pred_q), m, p->train, p->n_finite, p->d, k,
                                    0, 0, 1, as<int32_t>(f->pred_ids), as<float>(f->pred_dist), s,
                                    f->op_knn_ids, f->op_knn_dist)))
        return rc;
    std::vector<int32_t> ids((size_t)m * k);
    std::vector<float> sq((size_t)m * k);
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(ids.data(), f->pred_ids.ptr, sizeof(int32_t) * ids.size(),
                                     cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaMemcpyAsync(sq.data(), f->pred_dist.ptr, sizeof(float) * sq.size(),
                                     cudaMemcpyDeviceToHost, s));
    CUSCAN_CUDA(ctx, cudaStreamSynchronize(s));
    std::vector<double> dist((size_t)k);
    for (int64_t q = 0; q < m; ++q) {
        for (int c = 0; c < k; ++c)
            if ((rc = euclidean(ctx, sq[(size_t)q * k + c], &dist[c]))) return rc;
        if ((rc = predict_row(ctx, *p, ids.data() + q * k, dist.data(), labels + q, strengths + q,
                              connecting_points + q)))
            return rc;
    }
    return CUSCAN_OK;
}

}  // namespace

