// Device buffers and entry points of the MST integer work (forest.cu).
#pragma once

#include "common.cuh"

namespace cuscan {

// Small status block that the host reads once per Borůvka round.
struct DevStatus {
    unsigned long long components;  // components after the last merge
    unsigned long long edges;       // MST edges emitted so far
    double same_pairs;     // sum of squared component sizes entering the current round
    int err_kind;          // 0 ok, 1 numerical weight, 2 index out of range, 4 no progress
    int pad[3];
    double mst_weight;     // f64 total MST weight, written once after the last round
    // kept on the device by packed fits (no host read after every round): the seed's results,
    // rounds run and ordered cross pairs entering them
    unsigned long long seed_edges;
    unsigned long long components_after_seed;
    unsigned long long rounds;
    double cross_pairs;
};

// Buffers of the bf16 screening path (refined.cu).
struct RefinedBuffers {
    Buffer xt, pnorm, mnorm, tile_mmax, tile_lo, tile_hi, cand_ids, cand_lb, fallback, count;
    Buffer error, cbound, rowcnt, pivots, cells, cell_d, absmax;
    Buffer qthr, xq, pq, mq, cand2, rowcnt2, fallback2;  // threshold re-screen of kNN rows
    Buffer urow, colcnt, colbuf;  // symmetric Borůvka: row bounds, column-side buffers
    Buffer act_flag, act_idx, act_pos;  // Borůvka rows that can hold their component's edge
    Buffer rowlb, lbtmp;  // lower bounds of each row's cheapest cross edge (original order)
    // operand format of the current fit: fp16 of x * scale (scale a power of two), or bf16
    bool want_fp16 = false;  // requested by the caller's precision
    bool fp16 = false;       // in use (the data's range allows a scale)
    Buffer cursor;        // kNN screens: tiles issued, query blocks taken
    Buffer colp, colc, cmin;  // column terms of the running screen (screen_columns_kernel)
    bool split = false;      // split-bf16 operands (hi + lo) in use for the current fit
    bool have_scale = false; // scale computed for the current fit
    float scale = 1.0f;
    float amax_value = 0.0f; // largest |x| of the current fit
    bool range_ok = true;    // the current fit's values keep every screen quantity finite
    int64_t tile_pairs = 0;  // (query block, tile) pairs the screens of the current fit ran
    int64_t screened_rows = 0;  // query rows of the current fit's Borůvka screens
    int64_t symmetric_rounds = 0;  // rounds of the current fit the symmetric screen ran
    bool lb_valid = false;      // rowlb holds bounds of the current fit
    // CUDA events around the kNN list screen's launch (created on first use); screen_timed
    // says they hold the current fit's launch
    cudaEvent_t screen_ev[2] = {nullptr, nullptr};
    bool screen_timed = false;
};

struct ForestBuffers {
    Buffer next, esrc, edst, ew;            // proposals per node
    Buffer jmp_a, mx_a, jmp_b, mx_b;        // pointer doubling
    Buffer keep, pos, parent, minlab, kept_total;
    Buffer cnt, start, fill, perm;          // counting sort by component
    Buffer xp, corep, labp;                 // component-sorted copies
    Buffer row_keys, comp_keys;             // 64-bit candidate keys
    Buffer tile_lo, tile_hi;                // label range per 32-row tile
    Buffer status_buf, scan_tmp;
    Buffer knn_ids_tmp, knn_dist_tmp;       // split-kNN partial lists
    RefinedBuffers refined;
    DevStatus *status = nullptr;
};

int forest_reserve(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int d);
void forest_release(ForestBuffers &b);
// Every device buffer of the forest and of the bf16 screen (out may be null); returns the count.
constexpr int kForestBufferCount = 64;
int forest_buffers(ForestBuffers &b, Buffer **out);
int forest_core(cuscan_ctx *ctx, const float *knn_sq, int64_t n, int k, int min_samples,
                float *core, cudaStream_t s);
// Seed forest (mst.rs:368-420): appends the kept seed edges and labels points by the smallest
// point of their tree; status->components is refreshed. active_bound (default n) bounds the
// nodes of the seed graph for the pointer-doubling step count.
int forest_seed(cuscan_ctx *ctx, ForestBuffers &b, const float *core, const int32_t *ids,
                const float *dsq, int64_t n, int k, int32_t *label, uint32_t *out_src,
                uint32_t *out_dst, float *out_w, cudaStream_t s, int64_t active_bound = -1);
// Group points by label: perm, xp, corep, labp.
int forest_sort_by_component(cuscan_ctx *ctx, ForestBuffers &b, const float *x, const float *core,
                             const int32_t *label, int64_t n, int d, cudaStream_t s);
// Merge one round from the per-row candidate keys in b.row_keys.
// allow_empty: rows may lack a candidate (the bf16 screen appends only pairs that can reach
// their component's cheapest edge).
int forest_round(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int64_t components,
                 int32_t *label, uint32_t *out_src, uint32_t *out_dst, float *out_w,
                 cudaStream_t s, int allow_empty = 0);
// status->mst_weight = sum over the first m edges of sqrt((double) w[i]), reduced in f64 in a
// fixed order (deterministic for a given edge list).
int forest_mst_weight(cuscan_ctx *ctx, ForestBuffers &b, const float *w, int64_t m,
                      cudaStream_t s);
int scan_exclusive(cuscan_ctx *ctx, const int32_t *in, int32_t *out, int64_t n,
                   int32_t *grand_total, Buffer &tmp, cudaStream_t s);

// ---- packed small fits (pack.cu): one launch per step for every fit of a pack ----
// One fit of a pack: its sizes and every device buffer its steps use. An array of these sits
// in device memory; the grouped kernels take fit blockIdx.z (kNN, candidates) or blockIdx.x
// (the one-CTA forest steps) from it.
struct PackFit {
    const float *x;  // n x d rows
    int64_t n;
    int d, k, min_samples, allow_empty;
    int32_t *ids;
    float *dsq, *core;
    int32_t *label;
    uint32_t *src, *dst;
    float *w;
    int32_t *next, *ja, *ma, *jb, *mb, *keep, *pos, *parent, *minlab;
    int32_t *kept_total;  // [0] kept edges of the last merge, [1] this round runs (0/1)
    uint32_t *esrc, *edst;
    float *ew;
    int32_t *cnt, *start, *fill, *perm, *labp;
    float *xp, *corep;
    unsigned long long *row_keys, *comp_keys;
    int32_t *tile_lo, *tile_hi;
    int32_t *part_ids;  // kNN partial lists when the reference range is split
    float *part_dist;
    DevStatus *status;
};
constexpr int kPackMaxRounds = 64;  // the host driver's round limit (api.cu)
constexpr int kPackErrNoConvergence = 8;
// Exact kNN lists of every fit whose k is at most 32 (squared distances, self excluded), the
// reference range of each fit split in `splits` chunks (partial lists merged when > 1).
int pack_knn(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max, int d_max,
             int k_max, int splits, cudaStream_t s, int64_t &launches);
// Core column, kNN seed and its merge (forest_core + forest_seed) of every fit; zeroes the
// fits' status blocks and the pack's per-round counters more[0, kPackMaxRounds + 2).
int pack_seed(cuscan_ctx *ctx, const PackFit *fits, int count, int *more, cudaStream_t s);
// One Borůvka round r of every fit that still has more than one component: the component
// sort, the sorted copy of the rows, the exact candidate sweep, the winners and the merge.
// more[r] counts the fits that need another round after it.
int pack_round(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max, int d_max,
               int splits, int r, int *more, cudaStream_t s);
// status->mst_weight of every fit without an error (forest_mst_weight's order).
int pack_weight(cuscan_ctx *ctx, const PackFit *fits, int count, cudaStream_t s);
// Grouped launches inside other translation units (knn.cu, boruvka.cu).
int launch_pack_knn(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max, int d_max,
                    int k_max, int splits, cudaStream_t s, int64_t &launches);
int launch_pack_candidates(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max,
                           int d_max, int splits, cudaStream_t s);

}  // namespace cuscan
