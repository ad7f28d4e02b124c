/*
 * cuscan_gb300: GB300-native (sm_103a) HDBSCAN fit core behind a plain C ABI.
 *
 * The entry points replace, one for one, the device operations that lega0208/cuscan routes
 * through its Burn/CubeCL backend extension for the exact complete-graph HDBSCAN fit:
 *
 *   cuscan_exact_knn            <- NeighborOps::exact_neighbors
 *                                  (crates/cuscan-common/src/backend.rs:13-20,
 *                                   crates/cuscan-common/src/neighbors.rs:148-165)
 *   cuscan_boruvka_candidates   <- HdbscanOps::boruvka_candidates
 *                                  (crates/hdbscan/src/backend.rs:75-81)
 *   cuscan_component_reduce     <- HdbscanOps::component_reduce
 *                                  (crates/hdbscan/src/backend.rs:90-98)
 *   cuscan_fit_core[_device]    <- core_distances + spanning_tree of the brute-force
 *                                  complete-graph route, fused and device resident
 *                                  (crates/hdbscan/src/estimator.rs:524-874)
 *   cuscan_clusters_from_spanning_tree
 *                               <- hdbscan_core::clusters_from_spanning_tree
 *                                  (crates/hdbscan-core/src/lib.rs:57-97), host code
 *
 * Conventions
 *  - Every function returns a cuscan_status (0 = success). The message of the last failure
 *    on a context is read with cuscan_last_error(); the status values map one to one onto the
 *    reference's HdbscanError variants (crates/hdbscan-core/src/error.rs:8-19).
 *  - Pointers are caller owned. "device" arguments are CUDA device pointers on the context's
 *    device; "host" arguments are ordinary host memory. No function keeps a pointer after it
 *    returns.
 *  - `stream` is a cudaStream_t passed as void*; NULL means the context's own stream. Device
 *    entry points only enqueue work on that stream, except where a function states it
 *    synchronises.
 *  - Row-major float32 data, int32 ids, n < 2^31 rows.
 */
#ifndef CUSCAN_GB300_H
#define CUSCAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cuscan_status {
    CUSCAN_OK = 0,
    CUSCAN_INVALID_CONFIG = 1,      /* HdbscanError::InvalidConfig */
    CUSCAN_INVALID_INPUT = 2,       /* HdbscanError::InvalidInput */
    CUSCAN_BACKEND_UNAVAILABLE = 3, /* HdbscanError::BackendUnavailable (no device, CUDA error) */
    CUSCAN_NUMERICAL = 4,           /* HdbscanError::Numerical */
    CUSCAN_OVERFLOW = 5,            /* HdbscanError::Overflow */
    CUSCAN_CAPACITY = 6,            /* HdbscanError::Capacity */
    CUSCAN_MEMORY = 7,              /* HdbscanError::Memory */
    CUSCAN_PENDING = 8              /* not an error: a server request is still queued or
                                       running (returned only by the cuscan_server_* calls) */
} cuscan_status;

/* Arithmetic used by the distance sweeps of cuscan_fit_core. All give bit-identical results:
 * PLAIN evaluates every pair with exact f32 direct differences on the SIMT cores;
 * BF16_REFINED screens pairs with bf16 tensor-core GEMM tiles (f32 accumulation) and
 * re-evaluates every pair that the proven error bound cannot rule out with the same exact f32
 * direct differences; FP16_REFINED does the same with fp16 operands of x * 2^k (k chosen from
 * the data's largest |x|), whose 8x smaller rounding error leaves fewer pairs to re-evaluate on
 * data whose norms are large against the neighbour distances (falls back to bf16 operands when
 * no such scale exists). Both refined forms run the exact kernels for data whose values could
 * overflow an f32 squared norm or distance (d * max|x|^2 > FLT_MAX / 16). */
typedef enum cuscan_precision {
    CUSCAN_PRECISION_PLAIN = 0,
    CUSCAN_PRECISION_BF16_REFINED = 1,
    CUSCAN_PRECISION_FP16_REFINED = 2
} cuscan_precision;

typedef struct cuscan_ctx cuscan_ctx;

/* Per-fit counters and stage times (milliseconds, CUDA events on the fit stream). */
typedef struct cuscan_fit_stats {
    double core_ms;          /* kNN sweep + core distances ("core_distances" stage) */
    double mst_ms;           /* seed + all Boruvka rounds ("mst" stage) */
    double knn_kernel_ms;    /* the kNN distance-sweep kernels alone */
    double candidate_kernel_ms; /* the Boruvka candidate kernels alone, summed over rounds */
    int64_t rounds;          /* Boruvka rounds after the kNN seed */
    int64_t seed_edges;      /* edges added by the kNN seed */
    int64_t components_after_seed;
    int64_t refined_rows;    /* kNN rows screened on the tensor cores */
    int64_t fallback_rows;   /* kNN rows whose screens were inconclusive and ran exact f32 */
    int64_t boruvka_fallback_rows; /* Borůvka rows (summed over rounds) re-run exact f32 */
    double cross_pairs;      /* sum over rounds of ordered cross-component pairs */
    int64_t rescreened_rows; /* kNN rows screened a second time in threshold mode */
    int64_t screen_tile_pairs; /* 128 x 256 tensor-core tiles the screens computed */
    int64_t boruvka_screened_rows; /* query rows of the Boruvka screens, summed over rounds
                                      (rows whose core exceeds their component's bound skip) */
    double mst_weight;       /* total MST weight: sum of sqrt((double) w_sq) over the edges, the
                                weights finalize_mst forms (mst.rs:501-512), reduced in f64 on
                                the device in a fixed order */
    double knn_screen_ms;    /* the kNN tensor-core screen launch alone (0 when the fit ran
                                the exact kernels only) */
    int64_t symmetric_rounds; /* Borůvka rounds screened with each unordered pair once */
    int64_t operand_format;   /* screen operands the fit ended with: 0 bf16, 1 fp16 (scaled),
                                 2 split bf16 (hi + lo). A bf16-refined fit whose plain bf16
                                 bound leaves too many kNN rows inconclusive switches to split
                                 bf16 (d <= 64) or scaled fp16 (wider rows); -1: no screen ran */
} cuscan_fit_stats;

/* ---- context ---- */
int cuscan_ctx_create(int device, cuscan_ctx **out);
void cuscan_ctx_destroy(cuscan_ctx *ctx);
const char *cuscan_last_error(const cuscan_ctx *ctx);
int cuscan_error_kind(const cuscan_ctx *ctx);
/* The context's own CUDA stream (cudaStream_t as void*). */
void *cuscan_ctx_stream(cuscan_ctx *ctx);
/* Library version string. */
const char *cuscan_version(void);
/* Number of CUDA kernels this library has launched in the process so far (all contexts). */
int64_t cuscan_launch_count(void);

/*
 * Exact k nearest neighbours of `query` rows among `reference` rows (all device pointers),
 * ordered by (squared distance, reference id). With exclude_self, reference row
 * query_offset + i is skipped for query row i. Missing neighbours are padded with id nr and
 * distance +inf (squared) or sqrt(FLT_MAX) (unsquared); unsquared output is the sqrt of the
 * squared value. Replaces NeighborOps::exact_neighbors
 * (crates/cuscan-common/src/kernels/neighbors.rs:17-76 semantics).
 */
int cuscan_exact_knn(cuscan_ctx *ctx, const float *query, int64_t nq, const float *reference,
                     int64_t nr, int32_t d, int32_t k, int32_t exclude_self,
                     int64_t query_offset, int32_t squared, int32_t *ids_out, float *dist_out,
                     void *stream);

/*
 * Per-row Borůvka candidate: for every row i the lexicographically smallest
 * (max(max(d2_ij, core_sq_i), core_sq_j), j) over rows j with components[j] != components[i];
 * rows without a candidate get (+inf, n). Device pointers. Replaces
 * HdbscanOps::boruvka_candidates (crates/hdbscan/src/backend.rs:75-81;
 * crates/hdbscan/src/kernels/boruvka.rs:68-140).
 */
int cuscan_boruvka_candidates(cuscan_ctx *ctx, const float *data, const float *core_sq,
                              const int32_t *components, int64_t n, int32_t d, float *weights_out,
                              int32_t *destinations_out, void *stream);

/*
 * Per-component winner over a stable CSR component plan (device pointers). weights/indices
 * are the per-row candidates; members/tile_starts/tile_ends/partial_offsets are the
 * ComponentReductionPlan arrays (crates/hdbscan-core/src/mst.rs:30-147). Outputs:
 * win_weights[c] (original weight bits of the winner, +inf when absent) and
 * win_meta[c*5] = (source, destination, bad_row, error_kind, bad_destination), exactly as
 * HdbscanOps::component_reduce (crates/hdbscan/src/backend.rs:90-98;
 * crates/hdbscan/src/kernels/component_reduce.rs:28-353).
 * The plan arrays must form a valid plan. A malformed one is not detected, but it cannot make
 * the kernels read outside the buffers: CSR positions are clamped to [0, n), member ids at or
 * above n are skipped, and partial offsets are clamped to [0, p).
 */
int cuscan_component_reduce(cuscan_ctx *ctx, const float *weights, const int32_t *indices,
                            const int32_t *members, const int32_t *tile_starts,
                            const int32_t *tile_ends, const int32_t *partial_offsets, int64_t n,
                            int64_t p, int64_t c, float *win_weights, int32_t *win_meta,
                            void *stream);

/*
 * cuscan_component_reduce without any device allocation (no counterpart in the reference; an
 * addition for callers that cannot allocate device memory, e.g. because another framework's
 * caching pool owns it, or because the implicit synchronisation of cudaMalloc/cudaFree is not
 * acceptable on their path). Same inputs, outputs and results as cuscan_component_reduce; no
 * context is needed. The per-tile scratch is a static device array of
 * CUSCAN_NOALLOC_MAX_TILES entries (1 MiB) that every GPU loading this library holds until
 * exit; plans with more tiles (p) are rejected with CUSCAN_CAPACITY.
 *  - The first call on a device, with that device current, resolves the array's address
 *    (cudaGetSymbolAddress); make that first call before any stream capture.
 *  - Every call shares the one array: calls that overlap on the GPU (different streams, or
 *    different host threads on the same device) race and must be serialised by the caller.
 *  - The address is cached per device for the life of the process: resetting a device
 *    (cudaDeviceReset, or a reset of its primary context) after the first call is not
 *    supported, because the module and its array may then live at another address.
 *  - stream is a cudaStream_t as void* (NULL = the legacy default stream); err (may be NULL)
 *    receives the message of a failure.
 */
#define CUSCAN_NOALLOC_MAX_TILES 65536
int cuscan_component_reduce_noalloc(const float *weights, const int32_t *indices,
                                    const int32_t *members, const int32_t *tile_starts,
                                    const int32_t *tile_ends, const int32_t *partial_offsets,
                                    int64_t n, int64_t p, int64_t c, float *win_weights,
                                    int32_t *win_meta, void *stream, char *err, size_t err_len);

/*
 * Fused exact fit core of the brute-force complete-graph route: kNN core distances
 * (k = min(min_samples, n-1)), kNN seed forest, then Borůvka rounds until one component
 * remains, all on the device. Inputs and outputs are HOST pointers; the function copies the
 * data in, runs the fit on the context stream and synchronises before returning.
 * Outputs: knn_ids[n*k], knn_sq[n*k] (may be NULL), core_sq[n], and the n-1 MST edges
 * (src, dst, squared weight) in the reference's merge order: seed edges by point, then each
 * round's winners by component first appearance (crates/hdbscan/src/estimator.rs:689-874).
 * Callers finalise with sqrt((double) w) and sort by (weight, src, dst)
 * (crates/hdbscan-core/src/mst.rs:501-512). stats may be NULL.
 */
int cuscan_fit_core(cuscan_ctx *ctx, const float *data, int64_t n, int32_t d,
                    int32_t min_samples, int32_t precision, int32_t *knn_ids, float *knn_sq,
                    float *core_sq, uint32_t *mst_src, uint32_t *mst_dst, float *mst_wsq,
                    int64_t *n_edges, cuscan_fit_stats *stats);

/*
 * Same as cuscan_fit_core with every array a DEVICE pointer (data resident in HBM). The call
 * enqueues on `stream`, synchronises it once per Borůvka round to read the component count,
 * and returns when the fit is complete.
 */
int cuscan_fit_core_device(cuscan_ctx *ctx, const float *data, int64_t n, int32_t d,
                           int32_t min_samples, int32_t precision, int32_t *knn_ids,
                           float *knn_sq, float *core_sq, uint32_t *mst_src, uint32_t *mst_dst,
                           float *mst_wsq, int64_t *n_edges, cuscan_fit_stats *stats,
                           void *stream);

/*
 * Packed small fits (no reference counterpart; each fit is the core_distances + spanning_tree
 * body of crates/hdbscan/src/estimator.rs:524-874, as in cuscan_fit_core). Up to
 * CUSCAN_PACK_MAX_FITS independent point sets of at most CUSCAN_PACK_MAX_ROWS rows each are fit
 * together, each step of every fit in one launch: one copy in (every fit's rows), the exact kNN
 * lists, the core column with the kNN seed, the Borůvka rounds (component sort, sorted copy,
 * candidate sweep, merge: four launches per round for the whole pack; a fit whose forest is
 * complete skips the rest on the device), the f64 MST weight, one copy out. The host reads one counter
 * after the first three rounds and after every two more. At these sizes every precision runs
 * the exact f32 kernels, so each item's outputs are bit identical to cuscan_fit_core's for the
 * same input. Host pointers; the call synchronises the context stream before returning.
 * Each item's status is set; the call returns the first failing item's status (message in
 * cuscan_last_error), or CUSCAN_OK. Stats are the pack's: core_ms and knn_kernel_ms cover the
 * copy in and the kNN lists, mst_ms the core column, seed, rounds and weight;
 * candidate_kernel_ms is 0 (the rounds are not timed one by one).
 */
#define CUSCAN_PACK_MAX_FITS 16
#define CUSCAN_PACK_MAX_ROWS 2047
#define CUSCAN_PACK_MAX_FEATURES 256
typedef struct cuscan_fit_item {
    const float *data;      /* host, n x d row-major, finite */
    int64_t n;              /* 2 .. CUSCAN_PACK_MAX_ROWS */
    int32_t d;              /* 1 .. CUSCAN_PACK_MAX_FEATURES */
    int32_t min_samples;
    int32_t precision;      /* a cuscan_precision */
    int32_t status;         /* out: cuscan_status of this fit */
    int32_t *knn_ids;       /* host out, n*k (k = min(min_samples, n-1)); may be NULL */
    float *knn_sq;          /* host out, n*k; may be NULL */
    float *core_sq;         /* host out, n */
    uint32_t *mst_src;      /* host out, n-1 edges in the reference's merge order */
    uint32_t *mst_dst;
    float *mst_wsq;
    int64_t n_edges;        /* out */
    cuscan_fit_stats stats; /* out */
} cuscan_fit_item;
int cuscan_fit_core_packed(cuscan_ctx *ctx, cuscan_fit_item *items, int32_t count);
/*
 * The context's latest pack (no reference counterpart): the kernels it launched and the host
 * reads of its round counter between the copy in and the copy out. Either pointer may be NULL.
 */
int cuscan_fit_core_packed_launch_stats(cuscan_ctx *ctx, int64_t *launches,
                                        int64_t *host_reads);

/*
 * Per Borůvka round of the context's last fit (no reference counterpart; the reference logs
 * the component counts of its rounds only): the query rows the round screened (all n for the
 * plain f32 form), the 128 x 256 tensor-core tiles its screens ran, its candidate-kernel time
 * in ms and the ordered cross-component pairs entering it. Fills at most max_rounds entries of
 * each non-null array and returns the number of rounds (-1 on a null context).
 */
int cuscan_fit_round_stats(const cuscan_ctx *ctx, int32_t max_rounds, int64_t *rows,
                           int64_t *tiles, double *ms, double *cross_pairs);

/*
 * Row shards: one fit split by query rows over ranks (processes, one per GPU), each holding
 * every point. A rank computes the kNN rows and the Borůvka candidates of its own rows
 * [row_begin, row_end); the ranks exchange results on the host and every rank merges the same
 * rounds, so all ranks hold the same forest. The reference runs these steps on one device in
 * HDBSCAN::spanning_tree (crates/hdbscan/src/estimator.rs:689-874) with the per-row rule of
 * crates/hdbscan/src/kernels/boruvka.rs:68-140 over row blocks (boruvka.rs:28-66,147-288).
 *  1. kNN rows of the shard: cuscan_exact_knn with query = data + row_begin * d, nq = the
 *     shard's rows, query_offset = row_begin; then an all-gather of the rows.
 *  2. cuscan_shard_seed: core distances and the kNN seed forest (mst.rs:368-420) from the full
 *     kNN rows; labels[n] receive each point's component (its smallest point), mst_* the seed
 *     edges; returns the edge and component counts.
 *  3. Each round, cuscan_shard_round_keys: row_keys[n] receive, for the shard's rows,
 *     (canonical weight bits << 32) | destination of the row's cheapest cross-component edge,
 *     and ~0 elsewhere; an all-reduce MIN over the ranks' arrays gives every row's key (keys
 *     of non-negative weights are below 2^63, so they order alike as signed integers).
 *  4. cuscan_shard_round_merge: the reduced keys merged exactly as a fit core round (winners,
 *     cycle breaking, emit in merge order, union); mst_* receive the round's edges after the
 *     earlier ones; once one component remains and mst_weight is non-null, it receives the f64
 *     total weight. Repeat 3-4 until one component remains.
 * All pointers are device pointers; data, core_sq and labels are the full arrays in original
 * row order. No counterpart in the reference's surface, which has no multi-device path.
 */
int cuscan_shard_seed(cuscan_ctx *ctx, int64_t n, int32_t d, int32_t min_samples,
                      const int32_t *knn_ids, const float *knn_sq, float *core_sq,
                      int32_t *labels, uint32_t *mst_src, uint32_t *mst_dst, float *mst_wsq,
                      int64_t *n_edges, int64_t *components, void *stream);
int cuscan_shard_round_keys(cuscan_ctx *ctx, const float *data, const float *core_sq,
                            const int32_t *labels, int64_t n, int32_t d, int64_t row_begin,
                            int64_t row_end, uint64_t *row_keys, void *stream);
int cuscan_shard_round_merge(cuscan_ctx *ctx, const float *data, const float *core_sq,
                             int32_t *labels, int64_t n, int32_t d, const uint64_t *row_keys,
                             uint32_t *mst_src, uint32_t *mst_dst, float *mst_wsq,
                             int64_t *n_edges, int64_t *components, double *mst_weight,
                             void *stream);

/*
 * Diagnostic of the bf16 tensor-core screen (no reference counterpart): runs the screening
 * pipeline on `data` (device, n >= 256 rows) and writes the raw fp32 accumulator of the first
 * 128-row query block against the first 256-row reference tile, i.e. the bf16 dot products
 * x_r . x_c for r < 128, c < 256, to tile_out[128*256] (device, row-major). Synchronises.
 */
int cuscan_debug_screen_tile(cuscan_ctx *ctx, const float *data, int64_t n, int32_t d,
                             float *tile_out, void *stream);
/*
 * The same diagnostic for a chosen operand format: operands 0 = bf16 (as above), 1 = fp16 of
 * x * scale with the power-of-two scale the fp16-refined fits choose for this data (written to
 * *scale_out when given; the accumulator is then scale^2 times the dot products), 2 = split
 * bf16 (hi.hi' + hi.lo' + lo.hi', d <= 64). With rows_out (device, float[n][4]) every row's
 * bound terms (ps, pb, cm, m) are written, ps = (1 - C_B) p - abs_c, pb = (1 - C_B) p,
 * cm = C_A m, so that the screen's lower bound of entry (r, c) is
 * fmaf(-cm_r, m_c, fmaf(-2, tile[r][c], pb_c) + ps_r), in screen units. With chunk_out (device,
 * float[128][8]) the screen's phase-1 maxima of the tile's 32-column chunks are written: entry
 * (r, h) is the largest of tile[r][32 h .. 32 h + 31], as the TMEM load returned it.
 */
int cuscan_debug_screen_tile_operands(cuscan_ctx *ctx, const float *data, int64_t n, int32_t d,
                                      int32_t operands, float *tile_out, float *rows_out,
                                      float *chunk_out, float *scale_out, void *stream);

/* ---- host-side extraction (no device work) ---- */

typedef struct cuscan_extract_config {
    int64_t min_cluster_size;
    int32_t selection_leaf;        /* 0 = excess of mass, 1 = leaf */
    int32_t allow_single_cluster;
    int64_t max_cluster_size;      /* <= 0 means unbounded */
    double cluster_selection_epsilon;
    double cluster_selection_persistence;
} cuscan_extract_config;

typedef struct cuscan_clustering cuscan_clustering;

/*
 * Run sort_mst, mst_to_linkage, condense_tree, simplify_hierarchy, select_clusters,
 * labels and membership strengths on an MST of m = n_points - 1 edges (host pointers:
 * src[m], dst[m], weight[m] Euclidean f64). Mirrors hdbscan_core::clusters_from_spanning_tree
 * (crates/hdbscan-core/src/lib.rs:57-97). The result is read with the accessors below and
 * freed with cuscan_clustering_free.
 */
int cuscan_clusters_from_spanning_tree(const uint32_t *src, const uint32_t *dst,
                                       const double *weight, int64_t m,
                                       const cuscan_extract_config *config,
                                       cuscan_clustering **out, char *err, size_t err_len);
int64_t cuscan_clustering_points(const cuscan_clustering *r);
int64_t cuscan_clustering_condensed_rows(const cuscan_clustering *r);
/* labels[n], probabilities[n], linkage[m*4] (left, right, distance, size),
 * sorted_mst[m*3] (src, dst, weight), condensed parent/child/lambda/child_size[rows]. */
void cuscan_clustering_read(const cuscan_clustering *r, int32_t *labels, float *probabilities,
                            double *linkage, double *sorted_mst, int64_t *condensed_parent,
                            int64_t *condensed_child, float *condensed_lambda,
                            float *condensed_child_size);
void cuscan_clustering_free(cuscan_clustering *r);

/*
 * DBSCAN labels at a strict single-linkage distance cut: rows of `linkage` ([rows*4] as
 * above) with distance < cut are merged, groups smaller than min_size are noise (-1), the
 * rest are numbered by their representative. labels_out has rows+1 entries. Mirrors
 * hdbscan_core::labels::dbscan_cut (crates/hdbscan-core/src/labels.rs:154-209).
 */
int cuscan_dbscan_cut(const double *linkage, int64_t rows, double cut, int64_t min_size,
                      int32_t *labels_out);

/* ---------------------------------------------------------------------------------------
 * approximate_predict. A predictor holds the prediction hierarchy of a fitted model
 * (hdbscan_core::prediction::PredictionHierarchy::new, crates/hdbscan-core/src/prediction.rs:
 * 433-700), the prediction core distances and a device copy of the finite training rows.
 * Predictions follow predict_row (prediction.rs:855-925) on exact candidate rows of width
 * 2 * min_samples (crates/hdbscan/src/prediction.rs:1806-1978).
 * ------------------------------------------------------------------------------------- */
typedef struct cuscan_predictor cuscan_predictor;

/*
 * Build a predictor from a fitted model: the raw-id condensed tree (rows of parent, child,
 * lambda, child_size), raw fitted labels[raw_n] and the ascending finite_index[n_finite].
 * train[n_finite * d] (host) are the finite training rows in compact order; they are copied to
 * the context's device. prediction_core[n_finite] (Euclidean, may be NULL when train is given)
 * are the training cores at self-inclusive rank min_samples; when NULL they are computed on the
 * device. With train NULL (ctx may then be NULL) the predictor is host-only: it serves
 * cuscan_predictor_predict_candidates only. Errors are also written to err.
 */
int cuscan_predictor_create(cuscan_ctx *ctx, const float *train, int64_t n_finite, int32_t d,
                            int32_t min_samples, const int64_t *tree_parent,
                            const int64_t *tree_child, const float *tree_lambda,
                            const float *tree_child_size, int64_t tree_rows,
                            const int32_t *labels, int64_t raw_n, const uint32_t *finite_index,
                            const double *prediction_core, cuscan_predictor **out, char *err,
                            size_t err_len);
void cuscan_predictor_destroy(cuscan_predictor *p);
int cuscan_predictor_shape(const cuscan_predictor *p, int64_t *n_finite, int32_t *d,
                           int32_t *min_samples);
/*
 * Portable predictor state: the columns of the reference's PredictionHierarchyState
 * (crates/hdbscan-core/src/prediction.rs:161-272) plus the geometry and the prediction cores,
 * the arrays of its HDF5 predictor schema v1 (python/cuscan/_hdbscan_predictor_serialization_v1.py).
 * The no-cluster-tree state has n_finite = cluster_nodes = 0 and no arrays. Node 0 is the root,
 * its parent index UINT64_MAX. cuscan_predictor_from_state validates every column as
 * PredictionHierarchy::from_state does (prediction.rs:279-433) and copies the geometry
 * ([n_finite * d] f32) to the context's device. A host-only predictor (created without training
 * rows) exports with ctx and geometry NULL, and from_state with geometry NULL (ctx may be NULL)
 * builds one: it runs cuscan_predictor_predict_candidates but not cuscan_predictor_predict.
 */
int cuscan_predictor_state_shape(const cuscan_predictor *p, int64_t *n_finite,
                                 int64_t *cluster_nodes);
int cuscan_predictor_export(cuscan_ctx *ctx, const cuscan_predictor *p, float *geometry,
                            uint32_t *finite_index, uint64_t *node_ids,
                            uint64_t *node_parent_indices, double *node_birth_lambdas,
                            int32_t *node_labels, double *node_max_lambdas,
                            uint64_t *point_node_indices, double *point_departure_lambdas,
                            double *prediction_cores);
int cuscan_predictor_from_state(cuscan_ctx *ctx, const float *geometry, int64_t n_finite,
                                int32_t d, int32_t min_samples, const uint32_t *finite_index,
                                int64_t cluster_nodes, const uint64_t *node_ids,
                                const uint64_t *node_parent_indices,
                                const double *node_birth_lambdas, const int32_t *node_labels,
                                const double *node_max_lambdas,
                                const uint64_t *point_node_indices,
                                const double *point_departure_lambdas,
                                const double *prediction_cores, cuscan_predictor **out,
                                char *err, size_t err_len);
/* Upper bound on the context workspace one cuscan_predictor_predict of m rows allocates. */
int64_t cuscan_predict_workspace_bytes(const cuscan_predictor *p, int64_t m);
/* 1 when the fitted tree has no clusters (every prediction is noise, 0, -1). */
int cuscan_predictor_no_cluster_tree(const cuscan_predictor *p);
int cuscan_predictor_read_cores(const cuscan_predictor *p, double *out);
/* Predict m finite query rows (host, [m * d]): exact candidate search on the context's device,
 * then the host candidate math. labels[m], strengths[m] (f64), connecting_points[m] (raw
 * training rows). */
int cuscan_predictor_predict(cuscan_ctx *ctx, const cuscan_predictor *p, const float *queries,
                             int64_t m, int32_t *labels, double *strengths,
                             int32_t *connecting_points);
/* The candidate math alone on given rows of width 2 * min_samples: compact ids and Euclidean
 * distances, ordered as the exact search orders them. */
int cuscan_predictor_predict_candidates(const cuscan_predictor *p, const int32_t *ids,
                                        const double *distances, int64_t m, int32_t *labels,
                                        double *strengths, int32_t *connecting_points, char *err,
                                        size_t err_len);

/* ---------------------------------------------------------------------------------------
 * Workspace accounting. No reference counterpart: the reference allocates through Burn's
 * memory pool. These let a caller budget device memory around the fit core.
 * ------------------------------------------------------------------------------------- */

/* Upper bound on the device workspace cuscan_fit_core allocates for one fit of n rows. */
int64_t cuscan_fit_workspace_bytes(int64_t n, int32_t d, int32_t min_samples, int32_t precision);
/* Device bytes the context's workspace holds now (buffers are kept between calls). */
int64_t cuscan_ctx_reserved_bytes(const cuscan_ctx *ctx);
/* Synchronise the context's stream and free its workspace. */
int cuscan_ctx_release_workspace(cuscan_ctx *ctx);

/* ---------------------------------------------------------------------------------------
 * Request server: continuous batching of HDBSCAN fits and approximate_predict batches on one
 * GPU. No reference counterpart (the reference serves one call at a time). A fit request runs
 * the estimator flow of crates/hdbscan/src/estimator.rs:1034-1392: finite split,
 * cuscan_fit_core, then cuscan_clusters_from_spanning_tree; a predict request runs
 * cuscan_predictor_predict against a resident predictor.
 *
 * Requests queue in arrival order and are admitted onto `slots` execution slots, each with its
 * own CUDA stream, workspace and host thread, as slots and device memory free up: the sum over
 * slots of max(workspace held, cuscan_fit_workspace_bytes of the running request) stays
 * within `budget_bytes`. Idle slots release retained workspace when the head request needs
 * the room; a request whose own bound exceeds the budget finishes at once with CUSCAN_MEMORY.
 * The fits of different slots overlap on the device. A request's result equals that of the
 * same fit run alone.
 *
 * The caller keeps `data` valid and unchanged until the request has finished. Results stay on
 * the server until cuscan_server_release. All calls are thread safe.
 * ------------------------------------------------------------------------------------- */
typedef struct cuscan_server cuscan_server;

typedef struct cuscan_server_info {
    int64_t request_id;
    int32_t status;          /* outcome once finished; CUSCAN_PENDING while queued or running */
    int32_t slot;            /* slot that ran it, -1 before admission */
    int32_t kind;            /* 0 fit, 1 approximate_predict */
    int32_t pack_size;       /* fits in the pack that ran it (1: run on its own) */
    int64_t n;
    int64_t finite_rows;
    int32_t d;
    int32_t n_clusters;
    int64_t workspace_bound_bytes;
    double submit_ms;        /* since the server was created */
    double queued_ms;        /* submit -> admission */
    double run_ms;           /* admission -> result ready on the host */
    double latency_ms;       /* submit -> result ready on the host */
    double done_ms;          /* since the server was created */
    double prep_ms;          /* host: finite split and compaction */
    double fit_ms;           /* host wall time of cuscan_fit_core (copies included) */
    double extract_ms;       /* host: cuscan_clusters_from_spanning_tree and scatter */
    cuscan_fit_stats stats;
} cuscan_server_info;

typedef struct cuscan_server_stats {
    int32_t slots;
    int32_t pad;
    int64_t budget_bytes;
    int64_t submitted, completed, failed, queued, running;
    int64_t committed_bytes;       /* current sum of slot commitments */
    int64_t peak_committed_bytes;  /* largest sum at any admission */
    int64_t workspace_releases;    /* idle-slot releases ordered by admission */
    int64_t packs;                 /* packs that ran two or more small fits */
    int64_t packed_requests;       /* fit requests those launches ran */
} cuscan_server_stats;

int cuscan_server_create(int device, int32_t slots, int64_t budget_bytes, cuscan_server **out,
                         char *err, size_t err_len);
/* Scheduling test double: the same queue and admission, with slots that run no fit (each
 * request waits us_per_kpoint microseconds per 1000 rows and reports its workspace bound as
 * held). It needs no GPU; cuscan_server_read_fit on it fails. */
int cuscan_server_create_simulated(int32_t slots, int64_t budget_bytes, double us_per_kpoint,
                                   cuscan_server **out, char *err, size_t err_len);
/* Fails queued requests, waits for running ones, stops the slots and frees everything. */
void cuscan_server_destroy(cuscan_server *server);
int cuscan_server_submit_fit(cuscan_server *server, const float *data, int64_t n, int32_t d,
                             int32_t min_samples, int32_t precision,
                             const cuscan_extract_config *config, int64_t *request_id);
/* Queue an approximate_predict of m finite query rows (host, [m * d]) against a resident
 * predictor created on the server's device. The predictor and the queries stay valid and
 * unchanged until the request has finished. */
int cuscan_server_submit_predict(cuscan_server *server, const cuscan_predictor *predictor,
                                 const float *queries, int64_t m, int64_t *request_id);
/* labels[m], strengths[m], connecting_points[m] of a finished predict request. */
int cuscan_server_read_predict(cuscan_server *server, int64_t request_id, int32_t *labels,
                               double *strengths, int32_t *connecting_points);
/* Wait up to timeout_ms (< 0: no limit) for one request; CUSCAN_OK once it has finished
 * (info->status is its outcome), CUSCAN_PENDING if it has not. */
int cuscan_server_wait(cuscan_server *server, int64_t request_id, double timeout_ms,
                       cuscan_server_info *info);
/* Next finished request in completion order (each is returned once, released requests not
 * at all); CUSCAN_PENDING on timeout. */
int cuscan_server_wait_any(cuscan_server *server, double timeout_ms, int64_t *request_id);
/* labels[n] and probabilities[n] over all submitted rows (non-finite rows: -1 and 0),
 * core_distances[finite_rows] (Euclidean), sorted_mst[(finite_rows - 1) * 3]; any may be
 * NULL. Returns the request's failure status if it failed. */
int cuscan_server_read_fit(cuscan_server *server, int64_t request_id, int32_t *labels,
                           float *probabilities, float *core_distances, double *sorted_mst);
int cuscan_server_request_error(cuscan_server *server, int64_t request_id, char *buf,
                                size_t len);
/* Drop a finished request's results. */
int cuscan_server_release(cuscan_server *server, int64_t request_id);
int cuscan_server_get_stats(cuscan_server *server, cuscan_server_stats *out);
/* Most small fits (at most CUSCAN_PACK_MAX_ROWS rows) one slot runs together as one pack
 * (cuscan_fit_core_packed), 1 .. CUSCAN_PACK_MAX_FITS; 1 turns packing off. When a slot admits
 * a small fit at the head of the queue it also takes the small fits queued right behind it, in
 * order, while the pack limit and the memory budget allow (a pack commits the sum of its
 * requests' bounds on top of the workspace the slot holds). Default 8: a pack launches each
 * step once for all of its fits, so eight slots running packs launch and synchronise far less
 * than eight slots running one small fit each. */
int cuscan_server_set_pack_limit(cuscan_server *server, int32_t max_fits);

#ifdef __cplusplus
}
#endif

#endif /* CUSCAN_GB300_H */
