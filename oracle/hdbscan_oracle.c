/*
 * CPU restatement of cuscan's exact HDBSCAN fit core (core distances + Boruvka MST).
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle that the CUDA path is checked against
 * and the timed CPU baseline. Nothing in the shipped library links, loads or calls it.
 *
 * Every function restates one piece of the reference (lega0208/cuscan v0.1.3); the cited
 * file:line is the reference source it follows, relative to the reference project root.
 *
 * Arithmetic contract (parity-critical):
 *  - squared distances are f32, accumulated sequentially in feature order as
 *    acc = fmaf(x_f - y_f, x_f - y_f, acc): the reference writes `distance += delta * delta`
 *    (crates/cuscan-common/src/kernels/neighbors.rs:44-48,
 *     crates/hdbscan/src/kernels/boruvka.rs:97-101) and both of its JIT back ends (NVRTC and
 *    LLVM `llvm.fmuladd`) contract that statement into a fused multiply-add.
 *    Build with -ffp-contract=off so that only the explicit fmaf calls fuse.
 *  - Boruvka weights are max(max(d2, core_i), core_j) in f32 (boruvka.rs:102).
 *  - MST weights are finalised as sqrt((double) w_sq) (crates/hdbscan-core/src/mst.rs:501-512).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Status codes shared with the product C ABI; they mirror HdbscanError
 * (crates/hdbscan-core/src/error.rs:8-19). */
enum {
    ORC_OK = 0,
    ORC_INVALID_CONFIG = 1,
    ORC_INVALID_INPUT = 2,
    ORC_BACKEND_UNAVAILABLE = 3,
    ORC_NUMERICAL = 4,
    ORC_OVERFLOW = 5,
    ORC_CAPACITY = 6,
    ORC_MEMORY = 7,
};

#define ORC_INF (__builtin_inff())
#define ORC_FLT_MAX 3.40282346638528859812e+38f

static inline uint32_t f2u(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
}
static inline float u2f(uint32_t u) {
    float x;
    memcpy(&x, &u, 4);
    return x;
}

static int g_threads = 0;

/* Number of host threads the parallel loops use (0 = OpenMP default). */
void orc_set_threads(int threads) { g_threads = threads; }

int orc_max_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* Sequential-FMA squared distance (neighbors.rs:44-48 under contraction). */
static inline float sq_dist(const float *a, const float *b, int d) {
    float acc = 0.0f;
    for (int f = 0; f < d; ++f) {
        float delta = a[f] - b[f];
        acc = fmaf(delta, delta, acc);
    }
    return acc;
}

/* Squared distance with unfused `sum += delta * delta`, as the reference's host oracle
 * writes it (crates/hdbscan-core/src/oracle.rs:188-195). Kept as a cross-check only. */
static inline float sq_dist_unfused(const float *a, const float *b, int d) {
    float acc = 0.0f;
    for (int f = 0; f < d; ++f) {
        float delta = a[f] - b[f];
        float prod = delta * delta;
        acc = acc + prod;
    }
    return acc;
}

void orc_pair_distances(const float *x, const float *y, int64_t m, int d, int fused, float *out) {
    for (int64_t i = 0; i < m; ++i)
        out[i] = fused ? sq_dist(x + i * d, y + i * d, d) : sq_dist_unfused(x + i * d, y + i * d, d);
}

/*
 * Exact kNN of `query` rows against `reference` rows, ordered by (d2, id), with optional
 * self exclusion by global id (query_offset + row). Follows exact_kernel
 * (crates/cuscan-common/src/kernels/neighbors.rs:17-76): slots start as (pad, nr) with
 * pad = +inf for squared output and FLT_MAX otherwise; a candidate enters when it beats the
 * worst slot by distance, or ties it with a lower id; unsquared output takes sqrtf at the end.
 */
int orc_exact_neighbors(const float *query, int64_t nq, const float *reference, int64_t nr,
                        int d, int k, int exclude_self, int64_t query_offset, int squared,
                        int32_t *ids, float *dist) {
    if (nq < 0 || nr <= 0 || d <= 0 || k <= 0) return ORC_INVALID_INPUT;
    if (nr > INT32_MAX) return ORC_OVERFLOW;
    const float pad = squared ? ORC_INF : ORC_FLT_MAX;
#pragma omp parallel for schedule(dynamic, 16) num_threads(orc_max_threads())
    for (int64_t row = 0; row < nq; ++row) {
        int32_t *id = ids + row * k;
        float *ds = dist + row * k;
        for (int s = 0; s < k; ++s) {
            id[s] = (int32_t)nr;
            ds[s] = pad;
        }
        const float *q = query + row * d;
        const int64_t self = query_offset + row;
        for (int64_t r = 0; r < nr; ++r) {
            if (exclude_self && r == self) continue;
            float distance = sq_dist(q, reference + r * d, d);
            int w = k - 1;
            if (distance < ds[w] || (distance == ds[w] && r < (int64_t)(uint32_t)id[w])) {
                int slot = k - 1;
                while (slot > 0) {
                    int p = slot - 1;
                    if (distance < ds[p] || (distance == ds[p] && r < (int64_t)(uint32_t)id[p])) {
                        id[slot] = id[p];
                        ds[slot] = ds[p];
                        --slot;
                    } else {
                        break;
                    }
                }
                id[slot] = (int32_t)r;
                ds[slot] = distance;
            }
        }
        if (!squared)
            for (int s = 0; s < k; ++s) ds[s] = sqrtf(ds[s]);
    }
    return ORC_OK;
}

/*
 * Blocked forms of the two all-pairs loops, for checking large fits in reasonable time.
 * ORC_RB reference rows are copied feature-major into a per-thread block, so that the
 * sequential fmaf chains of ORC_RB pairs advance together (one vector FMA per feature where
 * the compiler vectorises). Each pair still evaluates acc = fmaf(q_f - r_f, q_f - r_f, acc) in
 * feature order from 0, exactly sq_dist, and the candidates of a row are offered in ascending
 * reference order, so outputs are bit-identical to the row-at-a-time loops
 * (tests/test_oracle_consistency.py checks this). The row-at-a-time loops remain the timed
 * CPU baseline: they are the reference's own per-row loop structure.
 */
#define ORC_RB 16
#define ORC_QB 64
static int g_blocked = 1;

/* 1: orc_fit_core uses the blocked loops (default); 0: the row-at-a-time loops. */
void orc_set_blocked(int on) { g_blocked = on ? 1 : 0; }

/* Copy reference rows [r0, r0 + nb) feature-major into tb[d][ORC_RB] (zero padded). */
static void transpose_block(const float *reference, int64_t r0, int nb, int d, float *tb) {
    for (int j = 0; j < ORC_RB; ++j) {
        if (j < nb) {
            const float *src = reference + (r0 + j) * d;
            for (int f = 0; f < d; ++f) tb[f * ORC_RB + j] = src[f];
        } else {
            for (int f = 0; f < d; ++f) tb[f * ORC_RB + j] = 0.0f;
        }
    }
}

/* Sequential-FMA squared distances of one query row to the ORC_RB rows of a block. */
static inline void block_dists(const float *q, const float *tb, int d, float *acc) {
    for (int j = 0; j < ORC_RB; ++j) acc[j] = 0.0f;
    for (int f = 0; f < d; ++f) {
        const float qf = q[f];
        const float *t = tb + f * ORC_RB;
        for (int j = 0; j < ORC_RB; ++j) {
            const float delta = qf - t[j];
            acc[j] = fmaf(delta, delta, acc[j]);
        }
    }
}

/* Blocked orc_exact_neighbors: the same slots, ties and padding. */
int orc_exact_neighbors_blocked(const float *query, int64_t nq, const float *reference,
                                int64_t nr, int d, int k, int exclude_self, int64_t query_offset,
                                int squared, int32_t *ids, float *dist) {
    if (nq < 0 || nr <= 0 || d <= 0 || k <= 0) return ORC_INVALID_INPUT;
    if (nr > INT32_MAX) return ORC_OVERFLOW;
    const float pad = squared ? ORC_INF : ORC_FLT_MAX;
    const int64_t chunks = (nq + ORC_QB - 1) / ORC_QB;
    int failed = 0;
#pragma omp parallel num_threads(orc_max_threads())
    {
        float *tb = (float *)malloc(sizeof(float) * (size_t)d * ORC_RB);
        if (!tb) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(dynamic, 1)
        for (int64_t ch = 0; ch < chunks; ++ch) {
            if (!tb) continue;
            const int64_t q0 = ch * ORC_QB, q1 = q0 + ORC_QB < nq ? q0 + ORC_QB : nq;
            for (int64_t row = q0; row < q1; ++row)
                for (int s = 0; s < k; ++s) {
                    ids[row * k + s] = (int32_t)nr;
                    dist[row * k + s] = pad;
                }
            float acc[ORC_RB];
            for (int64_t r0 = 0; r0 < nr; r0 += ORC_RB) {
                const int nb = (int)(nr - r0 < ORC_RB ? nr - r0 : ORC_RB);
                transpose_block(reference, r0, nb, d, tb);
                for (int64_t row = q0; row < q1; ++row) {
                    block_dists(query + row * d, tb, d, acc);
                    int32_t *id = ids + row * k;
                    float *ds = dist + row * k;
                    const int64_t self = query_offset + row;
                    for (int j = 0; j < nb; ++j) {
                        const int64_t r = r0 + j;
                        if (exclude_self && r == self) continue;
                        const float distance = acc[j];
                        const int w = k - 1;
                        if (distance < ds[w] ||
                            (distance == ds[w] && r < (int64_t)(uint32_t)id[w])) {
                            int slot = k - 1;
                            while (slot > 0) {
                                const int p = slot - 1;
                                if (distance < ds[p] ||
                                    (distance == ds[p] && r < (int64_t)(uint32_t)id[p])) {
                                    id[slot] = id[p];
                                    ds[slot] = ds[p];
                                    --slot;
                                } else {
                                    break;
                                }
                            }
                            id[slot] = (int32_t)r;
                            ds[slot] = distance;
                        }
                    }
                }
            }
            if (!squared)
                for (int64_t row = q0; row < q1; ++row)
                    for (int s = 0; s < k; ++s) dist[row * k + s] = sqrtf(dist[row * k + s]);
        }
        free(tb);
    }
    return failed ? ORC_MEMORY : ORC_OK;
}

/* Blocked orc_boruvka_candidates: the same (weight, j) minimum per row. */
int orc_boruvka_candidates_blocked(const float *x, const float *core_sq,
                                   const int32_t *components, int64_t n, int d, float *w_out,
                                   int32_t *dst_out) {
    if (n <= 0 || d <= 0) return ORC_INVALID_INPUT;
    const int64_t chunks = (n + ORC_QB - 1) / ORC_QB;
    int failed = 0;
#pragma omp parallel num_threads(orc_max_threads())
    {
        float *tb = (float *)malloc(sizeof(float) * (size_t)d * ORC_RB);
        if (!tb) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(dynamic, 1)
        for (int64_t ch = 0; ch < chunks; ++ch) {
            if (!tb) continue;
            const int64_t q0 = ch * ORC_QB, q1 = q0 + ORC_QB < n ? q0 + ORC_QB : n;
            for (int64_t i = q0; i < q1; ++i) {
                w_out[i] = ORC_INF;
                dst_out[i] = (int32_t)n;
            }
            float acc[ORC_RB];
            for (int64_t r0 = 0; r0 < n; r0 += ORC_RB) {
                const int nb = (int)(n - r0 < ORC_RB ? n - r0 : ORC_RB);
                transpose_block(x, r0, nb, d, tb);
                for (int64_t i = q0; i < q1; ++i) {
                    const int32_t ci = components[i];
                    int any = 0;
                    for (int j = 0; j < nb; ++j) any |= components[r0 + j] != ci;
                    if (!any) continue;
                    block_dists(x + i * d, tb, d, acc);
                    const float core = core_sq[i];
                    float best = w_out[i];
                    int64_t best_index = dst_out[i];
                    for (int j = 0; j < nb; ++j) {
                        const int64_t r = r0 + j;
                        if (components[r] == ci) continue;
                        const float weight = fmaxf(fmaxf(acc[j], core), core_sq[r]);
                        if (weight < best || (weight == best && r < best_index)) {
                            best = weight;
                            best_index = r;
                        }
                    }
                    w_out[i] = best;
                    dst_out[i] = (int32_t)best_index;
                }
            }
        }
        free(tb);
    }
    return failed ? ORC_MEMORY : ORC_OK;
}

/*
 * Core distances from a kNN row block (crates/hdbscan/src/estimator.rs:668-676):
 * +inf when min_samples >= n, 0 when min_samples == 1, else column min_samples-1.
 */
void orc_core_from_knn(const float *knn_sq, int64_t n, int k, int min_samples, float *core_sq) {
    for (int64_t i = 0; i < n; ++i) {
        if ((int64_t)min_samples >= n)
            core_sq[i] = ORC_INF;
        else if (min_samples == 1)
            core_sq[i] = 0.0f;
        else
            core_sq[i] = knn_sq[i * k + min_samples - 1];
    }
}

/* ---- Union-by-rank DSU (crates/hdbscan-core/src/dsu.rs:7-59) ---- */
typedef struct {
    int64_t *parent;
    uint32_t *rank;
    int64_t n;
} dsu_t;

static int dsu_init(dsu_t *s, int64_t n) {
    s->n = n;
    s->parent = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    s->rank = (uint32_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(uint32_t));
    if (!s->parent || !s->rank) return ORC_MEMORY;
    for (int64_t i = 0; i < n; ++i) s->parent[i] = i;
    return ORC_OK;
}
static void dsu_free(dsu_t *s) {
    free(s->parent);
    free(s->rank);
}
/* find with path halving (dsu.rs:31-38) */
static inline int64_t dsu_find(dsu_t *s, int64_t x) {
    while (s->parent[x] != x) {
        int64_t p = s->parent[x];
        s->parent[x] = s->parent[p];
        x = p;
    }
    return x;
}
/* union of two roots; the first argument wins rank ties (dsu.rs:41-52) */
static inline void dsu_union_roots(dsu_t *s, int64_t x, int64_t y) {
    if (x == y) return;
    if (s->rank[x] < s->rank[y]) {
        int64_t t = x;
        x = y;
        y = t;
    }
    s->parent[y] = x;
    if (s->rank[x] == s->rank[y]) s->rank[x] += 1;
}

/*
 * Seed forest from kNN rows (crates/hdbscan-core/src/mst.rs:368-420): for each point in
 * order, the first non-padding neighbour j with core_i >= core_j is the only one
 * considered; it becomes edge (i, j, max(core_i, d2_ij)) when i and j are in different
 * trees. Returns the edge count through *n_edges.
 */
static int init_from_knn(const float *core_sq, const int32_t *neighbors, const float *knn_sq,
                         int64_t n, int k, dsu_t *dsu, uint32_t *src, uint32_t *dst, float *wsq,
                         int64_t *n_edges) {
    int64_t e = 0;
    for (int64_t i = 0; i < n; ++i) {
        float core_i = core_sq[i];
        for (int j = 0; j < k; ++j) {
            int32_t t = neighbors[i * k + j];
            if (t < 0) continue;
            if ((int64_t)t >= n) return ORC_INVALID_INPUT;
            if (core_i >= core_sq[t]) {
                int64_t a = dsu_find(dsu, i), b = dsu_find(dsu, t);
                if (a != b) {
                    float d2 = knn_sq[i * k + j];
                    src[e] = (uint32_t)i;
                    dst[e] = (uint32_t)t;
                    wsq[e] = fmaxf(core_i, d2); /* Rust f32::max */
                    ++e;
                    dsu_union_roots(dsu, a, b);
                }
                break;
            }
        }
    }
    *n_edges = e;
    return ORC_OK;
}

int orc_init_from_knn(const float *core_sq, const int32_t *neighbors, const float *knn_sq,
                      int64_t n, int k, uint32_t *src, uint32_t *dst, float *wsq,
                      int64_t *n_edges, int32_t *labels_out) {
    dsu_t s;
    int rc = dsu_init(&s, n);
    if (rc) return rc;
    rc = init_from_knn(core_sq, neighbors, knn_sq, n, k, &s, src, dst, wsq, n_edges);
    if (!rc && labels_out)
        for (int64_t i = 0; i < n; ++i) labels_out[i] = (int32_t)dsu_find(&s, i);
    dsu_free(&s);
    return rc;
}

/*
 * Per-row Boruvka candidates (crates/hdbscan/src/kernels/boruvka.rs:68-140): for row i the
 * lexicographically smallest (max(max(d2, core_i), core_j), j) over j with
 * components[j] != components[i]; rows with no candidate keep (+inf, n).
 */
int orc_boruvka_candidates(const float *x, const float *core_sq, const int32_t *components,
                           int64_t n, int d, float *w_out, int32_t *dst_out) {
    if (n <= 0 || d <= 0) return ORC_INVALID_INPUT;
#pragma omp parallel for schedule(dynamic, 16) num_threads(orc_max_threads())
    for (int64_t i = 0; i < n; ++i) {
        int32_t ci = components[i];
        float core = core_sq[i];
        float best = ORC_INF;
        int64_t best_index = n;
        const float *xi = x + i * d;
        for (int64_t j = 0; j < n; ++j) {
            if (components[j] == ci) continue;
            float distance = sq_dist(xi, x + j * d, d);
            float weight = fmaxf(fmaxf(distance, core), core_sq[j]);
            if (weight < best || (weight == best && j < best_index)) {
                best = weight;
                best_index = j;
            }
        }
        w_out[i] = best;
        dst_out[i] = (int32_t)best_index;
    }
    return ORC_OK;
}

/* Same rule for the rows [row_begin, row_end) only (used to time a bounded sample). */
int orc_boruvka_candidates_rows(const float *x, const float *core_sq, const int32_t *components,
                                int64_t n, int d, int64_t row_begin, int64_t row_end,
                                float *w_out, int32_t *dst_out) {
    if (n <= 0 || d <= 0 || row_begin < 0 || row_end > n || row_begin > row_end)
        return ORC_INVALID_INPUT;
#pragma omp parallel for schedule(dynamic, 4) num_threads(orc_max_threads())
    for (int64_t i = row_begin; i < row_end; ++i) {
        int32_t ci = components[i];
        float core = core_sq[i];
        float best = ORC_INF;
        int64_t best_index = n;
        const float *xi = x + i * d;
        for (int64_t j = 0; j < n; ++j) {
            if (components[j] == ci) continue;
            float distance = sq_dist(xi, x + j * d, d);
            float weight = fmaxf(fmaxf(distance, core), core_sq[j]);
            if (weight < best || (weight == best && j < best_index)) {
                best = weight;
                best_index = j;
            }
        }
        w_out[i - row_begin] = best;
        dst_out[i - row_begin] = (int32_t)best_index;
    }
    return ORC_OK;
}

/*
 * Stable first-appearance CSR plan (crates/hdbscan-core/src/mst.rs:30-147).
 * Outputs: members[n], offsets[c+1], tile_starts/ends[p], partial_offsets[c+1].
 * Arrays must be sized for the worst case (c <= n, p <= n). Returns c and p.
 */
int orc_component_plan(const int32_t *labels, int64_t n, int tile_width, int32_t *members,
                       int32_t *offsets, int32_t *tile_starts, int32_t *tile_ends,
                       int32_t *partial_offsets, int64_t *c_out, int64_t *p_out) {
    if (n > INT32_MAX) return ORC_OVERFLOW;
    if (tile_width <= 0) return ORC_INVALID_INPUT;
    int32_t *slots = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int64_t *counts = (int64_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(int64_t));
    int64_t *cursor = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (!slots || !counts || !cursor) {
        free(slots);
        free(counts);
        free(cursor);
        return ORC_MEMORY;
    }
    for (int64_t i = 0; i < n; ++i) slots[i] = -1;
    int64_t c = 0;
    for (int64_t i = 0; i < n; ++i) {
        int32_t l = labels[i];
        if (l < 0 || (int64_t)l >= n) {
            free(slots);
            free(counts);
            free(cursor);
            return ORC_INVALID_INPUT;
        }
        if (slots[l] == -1) slots[l] = (int32_t)c++;
        counts[slots[l]] += 1;
    }
    offsets[0] = 0;
    partial_offsets[0] = 0;
    int64_t partial = 0;
    for (int64_t s = 0; s < c; ++s) {
        offsets[s + 1] = (int32_t)(offsets[s] + counts[s]);
        partial += (counts[s] + tile_width - 1) / tile_width;
        partial_offsets[s + 1] = (int32_t)partial;
    }
    for (int64_t s = 0; s < c; ++s) cursor[s] = offsets[s];
    for (int64_t i = 0; i < n; ++i) {
        int32_t s = slots[labels[i]];
        members[cursor[s]++] = (int32_t)i;
    }
    int64_t t = 0;
    for (int64_t s = 0; s < c; ++s) {
        int64_t start = offsets[s], end = offsets[s + 1];
        while (start < end) {
            int64_t te = start + tile_width < end ? start + tile_width : end;
            tile_starts[t] = (int32_t)start;
            tile_ends[t] = (int32_t)te;
            ++t;
            start = te;
        }
    }
    *c_out = c;
    *p_out = t;
    free(slots);
    free(counts);
    free(cursor);
    return ORC_OK;
}

/* NaN or negative nonzero weight bits (crates/hdbscan/src/kernels/component_reduce.rs:21-25). */
static inline int numerical_bits(uint32_t bits) {
    uint32_t magnitude = bits & 0x7fffffffu;
    return ((bits & 0x80000000u) != 0 && magnitude != 0) || magnitude > 0x7f800000u;
}

/*
 * Per-component winner over CSR-ordered members (component_reduce.rs:61-76, 129-153,
 * 317-353). The key is the weight's bit pattern with -0 canonicalised to 0; ties go to the
 * smaller source; the winner keeps its original weight bits. The earliest (smallest) member
 * whose weight is numerical or whose destination is >= n is reported as the bad row, with
 * kind 1 (numerical) or 2 (destination out of range, carrying that destination).
 * meta is row-major [c, 5] = (source, destination, bad_row, kind, bad_destination).
 * Tiles only partition the work in the reference; the winner does not depend on them.
 */
int orc_component_reduce(const float *weights, const int32_t *indices, const int32_t *members,
                         const int32_t *offsets, int64_t n, int64_t c, float *win_w,
                         int32_t *win_meta) {
    for (int64_t s = 0; s < c; ++s) {
        uint32_t key = 0xffffffffu, value = 0x7f800000u;
        int64_t source = n, bad = n;
        for (int64_t pos = offsets[s]; pos < offsets[s + 1]; ++pos) {
            int32_t member = members[pos];
            uint32_t original = f2u(weights[member]);
            int32_t destination = indices[member];
            if (numerical_bits(original) || (int64_t)destination >= n) {
                if (member < bad) bad = member;
            } else if (destination >= 0) {
                uint32_t k = (original & 0x7fffffffu) == 0 ? 0u : original;
                if (k < key || (k == key && member < source)) {
                    key = k;
                    value = original;
                    source = member;
                }
            }
        }
        int32_t destination = source < n ? indices[source] : -1;
        int32_t kind = 0, bad_destination = -1;
        if (bad < n) {
            if (numerical_bits(f2u(weights[bad]))) {
                kind = 1;
            } else {
                kind = 2;
                bad_destination = indices[bad];
            }
        }
        win_w[s] = u2f(value);
        int32_t *m = win_meta + s * 5;
        m[0] = source < n ? (int32_t)source : -1;
        m[1] = destination;
        m[2] = (int32_t)bad;
        m[3] = kind;
        m[4] = bad_destination;
    }
    return ORC_OK;
}

/*
 * Merge component winners in slot order (crates/hdbscan-core/src/mst.rs:152-285): validate,
 * raise the earliest error row (a numerical error beats an index error on the same row),
 * reject negative/NaN weights, then union winners whose endpoints are still apart.
 * "No progress" is a numerical error.
 */
static int merge_component_winners(dsu_t *dsu, const int32_t *members, const int32_t *offsets,
                                   int64_t n, int64_t c, const float *weights,
                                   const int32_t *meta, uint32_t *src, uint32_t *dst,
                                   float *wsq, int64_t *n_edges) {
    int have_err = 0;
    int32_t err_row = 0, err_kind = 0;
    for (int64_t s = 0; s < c; ++s) {
        const int32_t *m = meta + s * 5;
        int32_t source = m[0], destination = m[1], bad_row = m[2], kind = m[3], bad_dst = m[4];
        if ((source == -1) != (destination == -1)) return ORC_INVALID_INPUT;
        int in_seg_src = 0, in_seg_bad = 0;
        for (int64_t p = offsets[s]; p < offsets[s + 1]; ++p) {
            if (members[p] == source) in_seg_src = 1;
            if (members[p] == bad_row) in_seg_bad = 1;
        }
        if (source == -1) {
            if (f2u(weights[s]) != 0x7f800000u) return ORC_INVALID_INPUT;
        } else {
            if (source < 0 || source >= n || destination < 0 || destination >= n)
                return ORC_INVALID_INPUT;
            if (!in_seg_src) return ORC_INVALID_INPUT;
        }
        if (kind != 0) {
            if (!(kind == 1 || kind == 2) || bad_row < 0 || bad_row >= n) return ORC_INVALID_INPUT;
            if (!in_seg_bad) return ORC_INVALID_INPUT;
            if (kind == 2 && (bad_dst < 0 || bad_dst < n)) return ORC_INVALID_INPUT;
            if (kind == 1 && bad_dst != -1) return ORC_INVALID_INPUT;
            if (!have_err || bad_row < err_row || (bad_row == err_row && kind == 1)) {
                have_err = 1;
                err_row = bad_row;
                err_kind = kind;
            }
            continue;
        }
        if (bad_row != (int32_t)n || bad_dst != -1) return ORC_INVALID_INPUT;
    }
    if (have_err) return err_kind == 1 ? ORC_NUMERICAL : ORC_INVALID_INPUT;
    for (int64_t s = 0; s < c; ++s)
        if (meta[s * 5] >= 0 && (isnan(weights[s]) || weights[s] < 0.0f)) return ORC_NUMERICAL;
    int64_t before = *n_edges, e = before;
    for (int64_t s = 0; s < c; ++s) {
        const int32_t *m = meta + s * 5;
        if (m[0] < 0) continue;
        int64_t a = dsu_find(dsu, m[0]), b = dsu_find(dsu, m[1]);
        if (a != b) {
            src[e] = (uint32_t)m[0];
            dst[e] = (uint32_t)m[1];
            wsq[e] = weights[s];
            ++e;
            dsu_union_roots(dsu, a, b);
        }
    }
    *n_edges = e;
    if (e == before) return ORC_NUMERICAL;
    return ORC_OK;
}

typedef struct {
    int64_t rounds;
    int64_t seed_edges;
    int64_t components_after_seed;
    /* component sizes entering each round are appended here when non-NULL */
    int64_t *round_components; /* [max_rounds] */
    double *round_cross_pairs; /* [max_rounds] sum over ordered cross-component pairs */
    int64_t max_rounds;
} orc_fit_stats;

/*
 * Exact complete-graph fit core, brute-force route: core distances (estimator.rs:524-687,
 * BruteForce arm 591-657) then kNN-seeded Boruvka rounds (estimator.rs:689-874) until one
 * component remains. Outputs are the kNN rows (k = min(min_samples, n-1)), core_sq[n] and
 * the unsorted MST edges in reference merge order (seed edges, then each round's winners in
 * component slot order). knn_ids/knn_sq may be NULL only when the caller does not need them.
 */
int orc_fit_core(const float *x, int64_t n, int d, int min_samples, int32_t *knn_ids,
                 float *knn_sq, float *core_sq, uint32_t *src, uint32_t *dst, float *wsq,
                 int64_t *n_edges, orc_fit_stats *stats) {
    if (n <= 1 || d <= 0 || min_samples <= 0) return ORC_INVALID_INPUT;
    if (n > INT32_MAX) return ORC_OVERFLOW;
    int k = (int64_t)min_samples < n - 1 ? min_samples : (int)(n - 1);
    int rc = g_blocked ? orc_exact_neighbors_blocked(x, n, x, n, d, k, 1, 0, 1, knn_ids, knn_sq)
                       : orc_exact_neighbors(x, n, x, n, d, k, 1, 0, 1, knn_ids, knn_sq);
    if (rc) return rc;
    orc_core_from_knn(knn_sq, n, k, min_samples, core_sq);

    dsu_t dsu;
    rc = dsu_init(&dsu, n);
    if (rc) return rc;
    int64_t e = 0;
    rc = init_from_knn(core_sq, knn_ids, knn_sq, n, k, &dsu, src, dst, wsq, &e);
    if (rc) {
        dsu_free(&dsu);
        return rc;
    }
    if (stats) stats->seed_edges = e;

    size_t nn = (size_t)n;
    int32_t *labels = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *members = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *offsets = (int32_t *)malloc(sizeof(int32_t) * (nn + 1));
    int32_t *tstart = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *tend = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *poff = (int32_t *)malloc(sizeof(int32_t) * (nn + 1));
    float *cw = (float *)malloc(sizeof(float) * nn);
    int32_t *cd = (int32_t *)malloc(sizeof(int32_t) * nn);
    float *ww = (float *)malloc(sizeof(float) * nn);
    int32_t *wm = (int32_t *)malloc(sizeof(int32_t) * nn * 5);
    if (!labels || !members || !offsets || !tstart || !tend || !poff || !cw || !cd || !ww || !wm) {
        rc = ORC_MEMORY;
        goto done;
    }
    int64_t rounds = 0;
    for (;;) {
        for (int64_t i = 0; i < n; ++i) labels[i] = (int32_t)dsu_find(&dsu, i);
        int64_t c = 0, p = 0;
        rc = orc_component_plan(labels, n, 512, members, offsets, tstart, tend, poff, &c, &p);
        if (rc) goto done;
        if (rounds == 0 && stats) stats->components_after_seed = c;
        if (c <= 1) break;
        if (stats && stats->round_components && rounds < stats->max_rounds) {
            double same = 0.0;
            for (int64_t s = 0; s < c; ++s) {
                double sz = (double)(offsets[s + 1] - offsets[s]);
                same += sz * sz;
            }
            stats->round_components[rounds] = c;
            stats->round_cross_pairs[rounds] = (double)n * (double)n - same;
        }
        rc = g_blocked ? orc_boruvka_candidates_blocked(x, core_sq, labels, n, d, cw, cd)
                       : orc_boruvka_candidates(x, core_sq, labels, n, d, cw, cd);
        if (rc) goto done;
        rc = orc_component_reduce(cw, cd, members, offsets, n, c, ww, wm);
        if (rc) goto done;
        rc = merge_component_winners(&dsu, members, offsets, n, c, ww, wm, src, dst, wsq, &e);
        if (rc) goto done;
        ++rounds;
    }
    if (e != n - 1) rc = ORC_NUMERICAL;
    if (stats) stats->rounds = rounds;
    *n_edges = e;
done:
    free(labels);
    free(members);
    free(offsets);
    free(tstart);
    free(tend);
    free(poff);
    free(cw);
    free(cd);
    free(ww);
    free(wm);
    dsu_free(&dsu);
    return rc;
}

/*
 * Independent all-pairs Boruvka from singletons (crates/hdbscan-core/src/oracle.rs:70-168):
 * per point the (weight, j) minimum by total order, per root the strictly smaller weight
 * (earliest point wins ties), roots visited in ascending point order. Used as the
 * tie-robust weight check; production semantics are the kNN-seeded orc_fit_core.
 * Uses the unfused sum like that oracle when fused == 0.
 */
int orc_brute_force_mst(const float *x, int64_t n, int d, int min_samples, int fused,
                        uint32_t *src, uint32_t *dst, float *wsq, int64_t *n_edges) {
    if (n < 2) {
        *n_edges = 0;
        return ORC_OK;
    }
    int k = (int64_t)min_samples < n - 1 ? min_samples : (int)(n - 1);
    size_t nn = (size_t)n;
    int32_t *ids = (int32_t *)malloc(sizeof(int32_t) * nn * (size_t)k);
    float *kd = (float *)malloc(sizeof(float) * nn * (size_t)k);
    float *core = (float *)malloc(sizeof(float) * nn);
    int64_t *bi = (int64_t *)malloc(sizeof(int64_t) * nn);
    int64_t *bj = (int64_t *)malloc(sizeof(int64_t) * nn);
    float *bw = (float *)malloc(sizeof(float) * nn);
    unsigned char *has = (unsigned char *)malloc(nn);
    int64_t *root_of = (int64_t *)malloc(sizeof(int64_t) * nn);
    dsu_t dsu;
    int rc = dsu_init(&dsu, n);
    if (rc || !ids || !kd || !core || !bi || !bj || !bw || !has || !root_of) {
        rc = ORC_MEMORY;
        goto out;
    }
    {
        /* exact (d2, j)-ordered rows and the core rule of oracle.rs:21-67 */
        for (int64_t i = 0; i < n; ++i) {
            for (int s = 0; s < k; ++s) {
                ids[i * k + s] = (int32_t)n;
                kd[i * k + s] = ORC_INF;
            }
            for (int64_t j = 0; j < n; ++j) {
                if (j == i) continue;
                float dd = fused ? sq_dist(x + i * d, x + j * d, d)
                                 : sq_dist_unfused(x + i * d, x + j * d, d);
                int w = k - 1;
                if (dd < kd[i * k + w] || (dd == kd[i * k + w] && j < ids[i * k + w])) {
                    int slot = k - 1;
                    while (slot > 0 && (dd < kd[i * k + slot - 1] ||
                                        (dd == kd[i * k + slot - 1] && j < ids[i * k + slot - 1]))) {
                        ids[i * k + slot] = ids[i * k + slot - 1];
                        kd[i * k + slot] = kd[i * k + slot - 1];
                        --slot;
                    }
                    ids[i * k + slot] = (int32_t)j;
                    kd[i * k + slot] = dd;
                }
            }
            if (min_samples == 1)
                core[i] = 0.0f;
            else if (n <= min_samples)
                core[i] = ORC_INF;
            else
                core[i] = kd[i * k + min_samples - 1];
        }
    }
    int64_t e = 0, components = n;
    while (components > 1) {
        for (int64_t r = 0; r < n; ++r) has[r] = 0;
        for (int64_t i = 0; i < n; ++i) root_of[i] = dsu_find(&dsu, i);
        for (int64_t i = 0; i < n; ++i) {
            int64_t ri = root_of[i];
            int found = 0;
            int64_t pj = 0;
            float pw = 0.0f;
            for (int64_t j = 0; j < n; ++j) {
                if (root_of[j] == ri) continue;
                float dd = fused ? sq_dist(x + i * d, x + j * d, d)
                                 : sq_dist_unfused(x + i * d, x + j * d, d);
                float w = fmaxf(fmaxf(core[i], core[j]), dd);
                /* total_cmp on non-negative non-NaN floats is the numeric order */
                if (!found || w < pw || (w == pw && j < pj)) {
                    found = 1;
                    pw = w;
                    pj = j;
                }
            }
            if (found && (!has[ri] || pw < bw[ri])) {
                has[ri] = 1;
                bi[ri] = i;
                bj[ri] = pj;
                bw[ri] = pw;
            }
        }
        int64_t added = 0;
        for (int64_t r = 0; r < n; ++r) {
            if (dsu_find(&dsu, r) != r || !has[r]) continue;
            int64_t a = dsu_find(&dsu, bi[r]), b = dsu_find(&dsu, bj[r]);
            if (a != b) {
                src[e] = (uint32_t)bi[r];
                dst[e] = (uint32_t)bj[r];
                wsq[e] = bw[r];
                ++e;
                dsu_union_roots(&dsu, a, b);
                ++added;
            }
        }
        if (added == 0) {
            rc = ORC_NUMERICAL;
            goto out;
        }
        components -= added;
    }
    *n_edges = e;
out:
    free(ids);
    free(kd);
    free(core);
    free(bi);
    free(bj);
    free(bw);
    free(has);
    free(root_of);
    dsu_free(&dsu);
    return rc;
}

/* ---- finalize_mst + sort_mst (mst.rs:501-512; crates/hdbscan-core/src/linkage.rs:25-37) ---- */
typedef struct {
    uint32_t src, dst;
    double w;
} sorted_edge;

static int cmp_sorted_edge(const void *pa, const void *pb) {
    const sorted_edge *a = (const sorted_edge *)pa, *b = (const sorted_edge *)pb;
    /* total_cmp on values that are never NaN and never -0 after canonicalisation */
    if (a->w < b->w) return -1;
    if (a->w > b->w) return 1;
    if (a->src != b->src) return a->src < b->src ? -1 : 1;
    if (a->dst != b->dst) return a->dst < b->dst ? -1 : 1;
    return 0;
}

/* out is row-major [m, 3] doubles (src, dst, weight), the layout of minimum_spanning_tree_. */
int orc_finalize_mst(const uint32_t *src, const uint32_t *dst, const float *wsq, int64_t m,
                     double *out) {
    sorted_edge *e = (sorted_edge *)malloc(sizeof(sorted_edge) * (size_t)(m > 0 ? m : 1));
    if (!e) return ORC_MEMORY;
    for (int64_t i = 0; i < m; ++i) {
        e[i].src = src[i];
        e[i].dst = dst[i];
        double w = sqrt((double)wsq[i]);
        if (w == 0.0) w = 0.0;
        e[i].w = w;
    }
    qsort(e, (size_t)m, sizeof(sorted_edge), cmp_sorted_edge);
    for (int64_t i = 0; i < m; ++i) {
        out[i * 3 + 0] = (double)e[i].src;
        out[i * 3 + 1] = (double)e[i].dst;
        out[i * 3 + 2] = e[i].w;
    }
    free(e);
    return ORC_OK;
}

/* ------------------------------------------------------------------------------------------
 * approximate_predict (crates/hdbscan-core/src/prediction.rs). The hierarchy follows
 * PredictionHierarchy::new (prediction.rs:433-700) on a raw-id condensed tree; dense arrays
 * indexed by raw id stand in for the reference's hash maps. Prediction follows predict_row
 * (prediction.rs:855-925). Query candidates come from orc_exact_neighbors with self included
 * (crates/hdbscan/src/prediction.rs:1806-1978), cores from prediction.rs:94-120.
 * ---------------------------------------------------------------------------------------- */

/* Training prediction cores: self-inclusive exact rows of width s, Euclidean value at rank
 * s - 1 (0 for s == 1). */
int orc_prediction_cores(const float *train, int64_t n, int d, int s, double *out) {
    if (s <= 0 || n <= 0) return ORC_INVALID_INPUT;
    if (s == 1) {
        for (int64_t i = 0; i < n; ++i) out[i] = 0.0;
        return ORC_OK;
    }
    int32_t *ids = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * s);
    float *sq = (float *)malloc(sizeof(float) * (size_t)n * s);
    if (!ids || !sq) {
        free(ids);
        free(sq);
        return ORC_MEMORY;
    }
    int rc = orc_exact_neighbors(train, n, train, n, d, s, 0, 0, 1, ids, sq);
    for (int64_t i = 0; rc == ORC_OK && i < n; ++i) {
        const float v = sq[i * s + s - 1];
        if (!(v >= 0.0f) || v == ORC_INF) rc = ORC_NUMERICAL;
        else out[i] = sqrt((double)v);
    }
    free(ids);
    free(sq);
    return rc;
}

static int finite_pos(const uint32_t *fi, int64_t nf, int64_t raw) {
    int64_t lo = 0, hi = nf;
    while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if ((int64_t)fi[mid] < raw) lo = mid + 1;
        else hi = mid;
    }
    return (lo < nf && (int64_t)fi[lo] == raw) ? (int)lo : -1;
}

/* Predict m rows from candidate rows of width 2 s (compact ids, Euclidean f64 distances).
 * Returns ORC_OK, or the error class; *no_cluster is set when the tree has no clusters (the
 * outputs are then noise, 0, -1). */
int orc_predict_candidates(const int64_t *parent, const int64_t *child, const float *lambda,
                           const float *child_size, int64_t rows, const int32_t *labels,
                           int64_t raw_n, const uint32_t *finite_index, int64_t nf, int s,
                           const double *cores, const int32_t *cand_ids, const double *cand_dist,
                           int64_t m, int32_t *out_label, double *out_strength,
                           int32_t *out_conn, int *no_cluster) {
    int rc = ORC_OK;
    int64_t max_id = raw_n;
    for (int64_t r = 0; r < rows; ++r) {
        if (parent[r] < raw_n || child[r] < 0) return ORC_INVALID_INPUT;
        if (parent[r] > max_id) max_id = parent[r];
        if (child[r] > max_id) max_id = child[r];
        if (isnan(lambda[r]) || lambda[r] < 0.0f) return ORC_INVALID_INPUT;
        if (!(child_size[r] >= 1.0f) || child_size[r] == ORC_INF) return ORC_INVALID_INPUT;
        const int is_point = child[r] < raw_n, is_cluster = child_size[r] > 1.0f;
        if (is_point == is_cluster) return ORC_INVALID_INPUT;
        if (is_cluster && child[r] <= parent[r]) return ORC_INVALID_INPUT;
    }
    int64_t clusters = 0;
    for (int64_t r = 0; r < rows; ++r) clusters += child_size[r] > 1.0f;
    *no_cluster = clusters == 0;
    if (clusters == 0) {
        for (int64_t q = 0; q < m; ++q) {
            out_label[q] = -1;
            out_strength[q] = 0.0;
            out_conn[q] = -1;
        }
        return ORC_OK;
    }
    if (2 * (int64_t)s > nf) return ORC_INVALID_INPUT;
    const int64_t nn = clusters + 1;
    int64_t *node_of = (int64_t *)malloc(sizeof(int64_t) * (size_t)(max_id + 1));
    int64_t *nid = (int64_t *)malloc(sizeof(int64_t) * nn);
    int64_t *npar = (int64_t *)malloc(sizeof(int64_t) * nn);
    double *nbirth = (double *)malloc(sizeof(double) * nn);
    double *nmax = (double *)malloc(sizeof(double) * nn);
    double *maxl = (double *)malloc(sizeof(double) * nn);
    int32_t *nlab = (int32_t *)malloc(sizeof(int32_t) * nn);
    int64_t *anchor_of_label = NULL;  /* smallest parent id per label */
    int32_t *anchor_label = (int32_t *)malloc(sizeof(int32_t) * nn);
    int64_t *pnode = (int64_t *)malloc(sizeof(int64_t) * (size_t)nf);
    double *pdep = (double *)malloc(sizeof(double) * (size_t)nf);
    int32_t max_label = -1;
    for (int64_t r = 0; r < raw_n; ++r)
        if (labels[r] > max_label) max_label = labels[r];
    anchor_of_label = (int64_t *)malloc(sizeof(int64_t) * (size_t)(max_label + 2));
    if (!node_of || !nid || !npar || !nbirth || !nmax || !maxl || !nlab || !anchor_label ||
        !pnode || !pdep || !anchor_of_label) {
        rc = ORC_MEMORY;
        goto done;
    }
    for (int64_t i = 0; i <= max_id; ++i) node_of[i] = -1;
    {
        int64_t root = INT64_MAX;
        for (int64_t r = 0; r < rows; ++r)
            if (child_size[r] > 1.0f && parent[r] < root) root = parent[r];
        node_of[root] = 0;
        nid[0] = root;
        npar[0] = -1;
        nbirth[0] = 0.0;
        int64_t k = 1;
        for (int64_t r = 0; r < rows; ++r) {
            if (!(child_size[r] > 1.0f)) continue;
            if (node_of[child[r]] >= 0) { rc = ORC_INVALID_INPUT; goto done; }
            node_of[child[r]] = k;
            nid[k++] = child[r];
        }
        k = 1;
        for (int64_t r = 0; r < rows; ++r) {
            if (!(child_size[r] > 1.0f)) continue;
            if (node_of[parent[r]] < 0) { rc = ORC_INVALID_INPUT; goto done; }
            npar[k] = node_of[parent[r]];
            nbirth[k] = (double)lambda[r];
            ++k;
        }
    }
    for (int64_t i = 0; i < nn; ++i) {
        maxl[i] = -1.0; /* unseen */
        anchor_label[i] = -1;
    }
    for (int64_t i = 0; i < nf; ++i) pnode[i] = -1;
    for (int32_t l = 0; l <= max_label; ++l) anchor_of_label[l] = -1;
    for (int64_t r = 0; r < rows; ++r) {
        const int64_t node = node_of[parent[r]];
        if (node < 0) { rc = ORC_INVALID_INPUT; goto done; }
        const double l = (double)lambda[r];
        if (maxl[node] < 0.0 || l > maxl[node]) maxl[node] = l;
        const int pos = child[r] < raw_n ? finite_pos(finite_index, nf, child[r]) : -1;
        if (pos < 0) continue;
        if (pnode[pos] >= 0) { rc = ORC_INVALID_INPUT; goto done; }
        pnode[pos] = node;
        pdep[pos] = l;
        const int32_t lab = labels[child[r]];
        if (lab >= 0 && (anchor_of_label[lab] < 0 || parent[r] < anchor_of_label[lab]))
            anchor_of_label[lab] = parent[r];
    }
    for (int64_t i = 0; i < nf; ++i)
        if (pnode[i] < 0) { rc = ORC_INVALID_INPUT; goto done; }
    for (int32_t l = 0; l <= max_label; ++l) {
        if (anchor_of_label[l] < 0) continue;
        const int64_t node = node_of[anchor_of_label[l]];
        if (anchor_label[node] >= 0) { rc = ORC_INVALID_INPUT; goto done; }
        anchor_label[node] = l;
    }
    /* parents precede children in node order? Not in general: resolve by walking up with
     * memoisation, a node's value being its own anchor's or its parent's. */
    {
        int8_t *done_flag = (int8_t *)calloc((size_t)nn, 1);
        int64_t *path = (int64_t *)malloc(sizeof(int64_t) * nn);
        if (!done_flag || !path) {
            free(done_flag);
            free(path);
            rc = ORC_MEMORY;
            goto done;
        }
        for (int64_t i = 0; i < nn; ++i) {
            int64_t len = 0, v = i;
            while (v >= 0 && !done_flag[v]) {
                if (len >= nn) { rc = ORC_INVALID_INPUT; break; }  /* a cycle */
                path[len++] = v;
                v = npar[v];
            }
            if (rc) break;
            for (int64_t j = len - 1; j >= 0; --j) {
                const int64_t u = path[j];
                if (anchor_label[u] >= 0) {
                    nlab[u] = anchor_label[u];
                    nmax[u] = maxl[u] < 0.0 ? 0.0 : maxl[u];
                } else if (npar[u] >= 0) {
                    nlab[u] = nlab[npar[u]];
                    nmax[u] = nmax[npar[u]];
                } else {
                    nlab[u] = -1;
                    nmax[u] = 0.0;
                }
                done_flag[u] = 1;
            }
        }
        free(done_flag);
        free(path);
        if (rc) goto done;
    }
    for (int64_t q = 0; q < m && rc == ORC_OK; ++q) {
        const int32_t *ids = cand_ids + q * 2 * s;
        const double *dist = cand_dist + q * 2 * s;
        const double qcore = dist[s];
        int best = -1;
        double bmrd = 0.0;
        for (int c = 0; c < 2 * s; ++c) {
            if (!(dist[c] >= 0.0) || dist[c] == INFINITY) { rc = ORC_NUMERICAL; break; }
            if (ids[c] < 0 || ids[c] >= nf) { rc = ORC_NUMERICAL; break; }
            const double core = cores[ids[c]];
            double mrd = core > qcore ? core : qcore;
            if (dist[c] > mrd) mrd = dist[c];
            if (best < 0 || mrd < bmrd) {
                best = c;
                bmrd = mrd;
            }
        }
        if (rc) break;
        const int32_t conn = ids[best];
        const double lam = bmrd > 0.0 ? 1.0 / bmrd : 1.7976931348623157e308;
        int64_t cl = pnode[conn];
        if (pdep[conn] > lam) {
            while (nid[cl] > nid[0] && npar[cl] >= 0 && nbirth[cl] >= lam) cl = npar[cl];
        }
        if (nlab[cl] < 0) {
            out_label[q] = -1;
            out_strength[q] = 0.0;
        } else if (nmax[cl] > 0.0) {
            out_label[q] = nlab[cl];
            out_strength[q] = (nmax[cl] < lam ? nmax[cl] : lam) / nmax[cl];
        } else {
            out_label[q] = nlab[cl];
            out_strength[q] = 1.0;
        }
        out_conn[q] = (int32_t)finite_index[conn];
    }
done:
    free(node_of);
    free(nid);
    free(npar);
    free(nbirth);
    free(nmax);
    free(maxl);
    free(nlab);
    free(anchor_label);
    free(pnode);
    free(pdep);
    free(anchor_of_label);
    return rc;
}
