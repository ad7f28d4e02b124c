// Exact integer work of the MST on the device: the kNN seed forest, per-round component
// winners, cycle breaking that reproduces the reference's sequential merge order, pointer
// jumping union/relabel, component sorting and an exclusive scan.
//
// Why cycle breaking is enough. In both the seed (crates/hdbscan-core/src/mst.rs:368-420) and
// a Borůvka merge (mst.rs:259-277) every node (a point, or a component slot) proposes at most
// one edge, so the proposals form a functional graph: each weakly connected part is a tree
// (one node without a proposal) or has exactly one cycle. The reference walks the proposals in
// slot order and skips an edge whose endpoints are already joined. An edge is skipped only if
// the edges processed before it already connect its endpoints, which closes the part's only
// cycle, so exactly one edge per cycle is skipped: the cycle edge with the largest slot. Slots
// are numbered by first appearance, i.e. by the smallest point of a component; components are
// therefore labelled here by their smallest point, and "largest slot" is "largest label".
// Pointer doubling with a running maximum finds, for every node, a node on its cycle and the
// cycle's largest label, without any sequential pass.
#include "common.cuh"
#include "forest.cuh"

namespace cuscan {
namespace {

__device__ __forceinline__ bool active_node(const int32_t *label, int64_t s) {
    return label == nullptr || label[s] == (int32_t)s;
}

__device__ __forceinline__ void core_at(int64_t i, const float *__restrict__ knn_sq, int64_t n,
                                        int k, int min_samples, float *__restrict__ core) {
    float c;
    if ((int64_t)min_samples >= n)
        c = CUSCAN_INF;
    else if (min_samples == 1)
        c = 0.0f;
    else
        c = knn_sq[i * k + min_samples - 1];
    core[i] = c;
}

__global__ void core_kernel(const float *__restrict__ knn_sq, int64_t n, int k, int min_samples,
                            float *__restrict__ core) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) core_at(i, knn_sq, n, k, min_samples, core);
}

// Seed proposal of point i: the first non-padding neighbour j with core_i >= core_j
// (mst.rs:390-417); next[i] = i when there is none.
__device__ __forceinline__ void seed_at(int64_t i, const float *__restrict__ core,
                                        const int32_t *__restrict__ ids,
                                        const float *__restrict__ dsq, int64_t n, int k,
                                        int32_t *__restrict__ next, uint32_t *__restrict__ esrc,
                                        uint32_t *__restrict__ edst, float *__restrict__ ew,
                                        DevStatus *status) {
    const float ci = core[i];
    int32_t pick = (int32_t)i;
    float w = 0.0f;
    for (int s = 0; s < k; ++s) {
        int32_t j = ids[i * k + s];
        if (j < 0) continue;
        if ((int64_t)j >= n) {
            atomicCAS(&status->err_kind, 0, 2);
            break;
        }
        if (ci >= core[j]) {
            pick = j;
            w = fmaxf(ci, dsq[i * k + s]);
            break;
        }
    }
    next[i] = pick;
    esrc[i] = (uint32_t)i;
    edst[i] = (uint32_t)pick;
    ew[i] = w;
}

__global__ void seed_kernel(const float *__restrict__ core, const int32_t *__restrict__ ids,
                            const float *__restrict__ dsq, int64_t n, int k,
                            int32_t *__restrict__ next, uint32_t *__restrict__ esrc,
                            uint32_t *__restrict__ edst, float *__restrict__ ew,
                            DevStatus *status) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) seed_at(i, core, ids, dsq, n, k, next, esrc, edst, ew, status);
}

__global__ void iota_kernel(int32_t *p, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (int32_t)i;
}

// Per-node steps of the cycle breaking and union (resolve_proposals). Each is run by one
// thread per node, either as a kernel of its own or inside the single-CTA resolve_small_kernel;
// the step order and the barriers between them are the same in both.
__device__ __forceinline__ void dbl_init_at(int64_t s, const int32_t *__restrict__ next,
                                            const int32_t *__restrict__ label,
                                            int32_t *__restrict__ jmp, int32_t *__restrict__ mx) {
    if (!active_node(label, s)) return;
    jmp[s] = next[s];
    mx[s] = (int32_t)s;
}
__device__ __forceinline__ void dbl_step_at(int64_t s, const int32_t *__restrict__ jin,
                                            const int32_t *__restrict__ min_,
                                            const int32_t *__restrict__ label,
                                            int32_t *__restrict__ jout, int32_t *__restrict__ mout) {
    if (!active_node(label, s)) return;
    int32_t j = jin[s];
    jout[s] = jin[j];
    int32_t a = min_[s], b = min_[j];
    mout[s] = a > b ? a : b;
}
// keep[s] = s proposes an edge that is not its cycle's largest-label edge; parent[s] is the
// forest parent after the skipped edges are removed.
__device__ __forceinline__ void keep_at(int64_t s, const int32_t *__restrict__ next,
                                        const int32_t *__restrict__ jmp,
                                        const int32_t *__restrict__ mx,
                                        const int32_t *__restrict__ label,
                                        int32_t *__restrict__ keep, int32_t *__restrict__ parent) {
    if (!active_node(label, s)) {
        keep[s] = 0;
        return;
    }
    int32_t t = next[s];
    bool k = t != (int32_t)s && mx[jmp[s]] != (int32_t)s;
    keep[s] = k ? 1 : 0;
    parent[s] = k ? t : (int32_t)s;
}
__device__ __forceinline__ void emit_at(int64_t s, const int32_t *__restrict__ keep,
                                        const int32_t *__restrict__ pos,
                                        const uint32_t *__restrict__ esrc,
                                        const uint32_t *__restrict__ edst,
                                        const float *__restrict__ ew, int64_t edges,
                                        uint32_t *__restrict__ out_src,
                                        uint32_t *__restrict__ out_dst, float *__restrict__ out_w,
                                        int64_t capacity) {
    if (!keep[s]) return;
    int64_t at = edges + pos[s];
    if (at >= capacity) return;
    out_src[at] = esrc[s];
    out_dst[at] = edst[s];
    out_w[at] = ew[s];
}
// Path halving toward the root (in place).
__device__ __forceinline__ void jump_at(int64_t s, int32_t *__restrict__ parent,
                                        const int32_t *__restrict__ label) {
    if (!active_node(label, s)) return;
    int32_t p = parent[s];
    int32_t pp = parent[p];
    if (pp != p) parent[s] = pp;
}
__device__ __forceinline__ void minlab_init_at(int64_t s, const int32_t *__restrict__ parent,
                                               const int32_t *__restrict__ label,
                                               int32_t *__restrict__ minlab) {
    if (!active_node(label, s)) return;
    if (parent[s] == (int32_t)s) minlab[s] = (int32_t)s;
}
__device__ __forceinline__ void minlab_reduce_at(int64_t s, const int32_t *__restrict__ parent,
                                                 const int32_t *__restrict__ label,
                                                 int32_t *__restrict__ minlab) {
    if (!active_node(label, s)) return;
    atomicMin(&minlab[parent[s]], (int32_t)s);
}
// label[i] <- smallest label of the tree that holds i's old component.
__device__ __forceinline__ void relabel_at(int64_t i, int32_t *__restrict__ label,
                                           const int32_t *__restrict__ parent,
                                           const int32_t *__restrict__ minlab) {
    label[i] = minlab[parent[label[i]]];
}

__global__ void dbl_init_kernel(const int32_t *__restrict__ next, const int32_t *__restrict__ label,
                                int64_t n, int32_t *__restrict__ jmp, int32_t *__restrict__ mx) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) dbl_init_at(s, next, label, jmp, mx);
}

__global__ void dbl_step_kernel(const int32_t *__restrict__ jin, const int32_t *__restrict__ min_,
                                const int32_t *__restrict__ label, int64_t n,
                                int32_t *__restrict__ jout, int32_t *__restrict__ mout) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) dbl_step_at(s, jin, min_, label, jout, mout);
}

__global__ void keep_kernel(const int32_t *__restrict__ next, const int32_t *__restrict__ jmp,
                            const int32_t *__restrict__ mx, const int32_t *__restrict__ label,
                            int64_t n, int32_t *__restrict__ keep, int32_t *__restrict__ parent) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) keep_at(s, next, jmp, mx, label, keep, parent);
}

__global__ void emit_kernel(const int32_t *__restrict__ keep, const int32_t *__restrict__ pos,
                            const uint32_t *__restrict__ esrc, const uint32_t *__restrict__ edst,
                            const float *__restrict__ ew, int64_t n, const DevStatus *status,
                            uint32_t *__restrict__ out_src, uint32_t *__restrict__ out_dst,
                            float *__restrict__ out_w, int64_t capacity) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n)
        emit_at(s, keep, pos, esrc, edst, ew, (int64_t)status->edges, out_src, out_dst, out_w,
                capacity);
}

__global__ void add_edges_kernel(DevStatus *status, const int32_t *kept_total,
                                 int require_progress) {
    status->edges += *kept_total;
    // "Boruvka round made no progress" (mst.rs:279-283)
    if (require_progress && *kept_total == 0) atomicCAS(&status->err_kind, 0, 4);
}

// Path halving toward the root, repeated a fixed number of times by the host.
__global__ void jump_kernel(int32_t *__restrict__ parent, const int32_t *__restrict__ label,
                            int64_t n) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) jump_at(s, parent, label);
}

__global__ void minlab_init_kernel(const int32_t *__restrict__ parent,
                                   const int32_t *__restrict__ label, int64_t n,
                                   int32_t *__restrict__ minlab) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) minlab_init_at(s, parent, label, minlab);
}

__global__ void minlab_reduce_kernel(const int32_t *__restrict__ parent,
                                     const int32_t *__restrict__ label, int64_t n,
                                     int32_t *__restrict__ minlab) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) minlab_reduce_at(s, parent, label, minlab);
}

__global__ void relabel_kernel(int32_t *__restrict__ label, const int32_t *__restrict__ parent,
                               const int32_t *__restrict__ minlab, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) relabel_at(i, label, parent, minlab);
}

__global__ void count_components_kernel(const int32_t *__restrict__ label, int64_t n,
                                        DevStatus *status) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool root = i < n && label[i] == (int32_t)i;
    unsigned m = __ballot_sync(0xffffffffu, root);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(&status->components, (unsigned long long)__popc(m));
}

// Counting sort of points by label: histogram with warp-aggregated atomics.
__global__ void hist_kernel(const int32_t *__restrict__ label, int64_t n, int32_t *__restrict__ cnt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int32_t l = i < n ? label[i] : -1;
    unsigned peers = __match_any_sync(0xffffffffu, l);
    int lane = threadIdx.x & 31;
    if (l >= 0 && lane == __ffs(peers) - 1) atomicAdd(&cnt[l], __popc(peers));
}

// Sum of squared component sizes (ordered same-component pairs) for the work counters.
__global__ void same_pairs_kernel(const int32_t *__restrict__ cnt, int64_t n, DevStatus *status) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        double c = (double)cnt[i];
        v = c * c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(&status->same_pairs, v);
}

__global__ void scatter_kernel(const int32_t *__restrict__ label, int64_t n,
                               const int32_t *__restrict__ start, int32_t *__restrict__ fill,
                               int32_t *__restrict__ perm) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int32_t l = i < n ? label[i] : -1;
    unsigned peers = __match_any_sync(0xffffffffu, l);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int base = 0;
    if (l >= 0 && lane == leader) base = atomicAdd(&fill[l], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    if (l < 0) return;
    int rank = __popc(peers & ((1u << lane) - 1u));
    perm[start[l] + base + rank] = (int32_t)i;
}

__global__ void gather_kernel(const float *__restrict__ x, const float *__restrict__ core,
                              const int32_t *__restrict__ label, const int32_t *__restrict__ perm,
                              int64_t n, int d, float *__restrict__ xp, float *__restrict__ corep,
                              int32_t *__restrict__ labp) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * d) return;
    int64_t pos = e / d;
    int f = (int)(e - pos * d);
    int32_t i = perm[pos];
    xp[e] = x[(int64_t)i * d + f];
    if (f == 0) {
        if (core) corep[pos] = core[i];
        labp[pos] = label[i];
    }
}

// Per-component minimum of (row weight bits << 32 | row) over component-sorted positions:
// segmented warp reduction over the contiguous label runs, one atomic per run.
// Component key of the row at sorted position pos: (weight bits << 32 | row), ~0 for a row
// without a candidate (an error unless allow_empty) or with a non-finite weight (an error).
__device__ __forceinline__ unsigned long long comp_key_at(int64_t pos,
                                                          const int32_t *__restrict__ perm,
                                                          const unsigned long long *__restrict__ row_keys,
                                                          DevStatus *status, int allow_empty) {
    const int32_t i = perm[pos];
    const unsigned long long rk = row_keys[i];
    if (rk == ~0ull) {
        if (!allow_empty) atomicCAS(&status->err_kind, 0, 4);
        return ~0ull;
    }
    const uint32_t wb = (uint32_t)(rk >> 32);
    if (numerical_bits(wb)) {
        atomicCAS(&status->err_kind, 0, 1);
        return ~0ull;
    }
    return ((unsigned long long)wb << 32) | (uint32_t)i;
}

__global__ void component_min_kernel(const int32_t *__restrict__ perm,
                                     const int32_t *__restrict__ labp,
                                     const unsigned long long *__restrict__ row_keys, int64_t n,
                                     unsigned long long *__restrict__ comp_keys,
                                     DevStatus *status, int allow_empty) {
    int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int32_t l = -1;
    unsigned long long v = ~0ull;
    if (pos < n) {
        l = labp[pos];
        v = comp_key_at(pos, perm, row_keys, status, allow_empty);
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long ov = __shfl_down_sync(0xffffffffu, v, o);
        int32_t ol = __shfl_down_sync(0xffffffffu, l, o);
        if (lane + o < 32 && ol == l && ov < v) v = ov;
    }
    int32_t prev = __shfl_up_sync(0xffffffffu, l, 1);
    bool head = l >= 0 && (lane == 0 || prev != l);
    if (head && v != ~0ull) atomicMin(&comp_keys[l], v);
}

// Winner of each active component: source = argmin row, destination = that row's candidate.
__device__ __forceinline__ void winner_at(int64_t s, const int32_t *label,
                                          const unsigned long long *__restrict__ comp_keys,
                                          const unsigned long long *__restrict__ row_keys,
                                          int64_t n, int32_t *__restrict__ next,
                                          uint32_t *__restrict__ esrc, uint32_t *__restrict__ edst,
                                          float *__restrict__ ew, DevStatus *status) {
    if (label[s] != (int32_t)s) return;
    unsigned long long ck = comp_keys[s];
    if (ck == ~0ull) {
        atomicCAS(&status->err_kind, 0, 4);
        next[s] = (int32_t)s;
        return;
    }
    uint32_t src = (uint32_t)ck;
    uint32_t dst = (uint32_t)row_keys[src];
    if ((int64_t)dst >= n) {
        atomicCAS(&status->err_kind, 0, 2);
        next[s] = (int32_t)s;
        return;
    }
    next[s] = label[dst];
    esrc[s] = src;
    edst[s] = dst;
    ew[s] = __uint_as_float((uint32_t)(ck >> 32));
}

__global__ void winner_kernel(const int32_t *__restrict__ label,
                              const unsigned long long *__restrict__ comp_keys,
                              const unsigned long long *__restrict__ row_keys, int64_t n,
                              int32_t *__restrict__ next, uint32_t *__restrict__ esrc,
                              uint32_t *__restrict__ edst, float *__restrict__ ew,
                              DevStatus *status) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) winner_at(s, label, comp_keys, row_keys, n, next, esrc, edst, ew, status);
}

// ---- exclusive scan of int32 (three passes) ----
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int block_exclusive_scan(int v, int *warp_sums, int &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (SCAN_THREADS / 32) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (SCAN_THREADS / 32)) warp_sums[lane] = w;
    }
    __syncthreads();
    int warp_prefix = warp > 0 ? warp_sums[warp - 1] : 0;
    total = warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void scan_tiles_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                  int64_t n, int32_t *__restrict__ tile_sums) {
    __shared__ int warp_sums[SCAN_THREADS / 32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int sum = 0;
#pragma unroll
    for (int t = 0; t < SCAN_ITEMS; ++t) {
        v[t] = base + t < n ? in[base + t] : 0;
        sum += v[t];
    }
    int total;
    int prefix = block_exclusive_scan(sum, warp_sums, total);
#pragma unroll
    for (int t = 0; t < SCAN_ITEMS; ++t) {
        if (base + t < n) out[base + t] = prefix;
        prefix += v[t];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void scan_sums_kernel(int32_t *__restrict__ sums, int64_t tiles,
                                 int32_t *__restrict__ grand_total) {
    __shared__ int warp_sums[SCAN_THREADS / 32];
    int carry = 0;
    for (int64_t b = 0; b < tiles; b += SCAN_THREADS) {
        int64_t i = b + threadIdx.x;
        int v = i < tiles ? sums[i] : 0;
        int total;
        int p = block_exclusive_scan(v, warp_sums, total);
        if (i < tiles) sums[i] = carry + p;
        carry += total;
    }
    if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

__global__ void scan_add_kernel(int32_t *__restrict__ out, int64_t n,
                                const int32_t *__restrict__ sums) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[i / SCAN_TILE];
}

// resolve_proposals of up to SMALL_RESOLVE_ROWS nodes in one CTA: the same per-node steps in
// the same order as the kernel sequence below, with block barriers where the sequence has
// kernel boundaries (global writes of the block are visible to the whole block after
// __syncthreads). One launch instead of about 33 per seed or round of a small fit. In a round
// active_label and point_label are the same array (no __restrict__ on either).
constexpr int64_t SMALL_RESOLVE_ROWS = 2048;
constexpr int SMALL_ITEMS = (int)(SMALL_RESOLVE_ROWS / SCAN_THREADS);
__device__ __forceinline__ void resolve_block(
    const int32_t *__restrict__ next, const int32_t *active_label, int32_t *point_label, int64_t n,
    int steps, int32_t *ja, int32_t *ma, int32_t *jb, int32_t *mb, int32_t *__restrict__ keep,
    int32_t *__restrict__ pos, int32_t *__restrict__ kept_total, const uint32_t *__restrict__ esrc,
    const uint32_t *__restrict__ edst, const float *__restrict__ ew, int32_t *parent,
    int32_t *__restrict__ minlab, DevStatus *status, uint32_t *__restrict__ out_src,
    uint32_t *__restrict__ out_dst, float *__restrict__ out_w, int64_t capacity,
    int require_progress) {
    __shared__ int warp_sums[SCAN_THREADS / 32];
    const int tid = threadIdx.x;
    // cycle breaking: pointer doubling with a running maximum, ping-pong buffers
    for (int64_t s = tid; s < n; s += SCAN_THREADS) dbl_init_at(s, next, active_label, ja, ma);
    __syncthreads();
    for (int t = 0; t < steps; ++t) {
        for (int64_t s = tid; s < n; s += SCAN_THREADS)
            dbl_step_at(s, ja, ma, active_label, jb, mb);
        __syncthreads();
        int32_t *tj = ja, *tm = ma;
        ja = jb;
        ma = mb;
        jb = tj;
        mb = tm;
    }
    for (int64_t s = tid; s < n; s += SCAN_THREADS) keep_at(s, next, ja, ma, active_label, keep, parent);
    __syncthreads();
    // exclusive scan of keep in node order: thread t holds nodes [t SMALL_ITEMS, +SMALL_ITEMS)
    int v[SMALL_ITEMS];
    int sum = 0;
    const int64_t base = (int64_t)tid * SMALL_ITEMS;
#pragma unroll
    for (int u = 0; u < SMALL_ITEMS; ++u) {
        v[u] = base + u < n ? keep[base + u] : 0;
        sum += v[u];
    }
    int total;
    int prefix = block_exclusive_scan(sum, warp_sums, total);
#pragma unroll
    for (int u = 0; u < SMALL_ITEMS; ++u) {
        if (base + u < n) pos[base + u] = prefix;
        prefix += v[u];
    }
    __syncthreads();
    // append the kept edges in node order after the edges emitted so far
    const int64_t edges = (int64_t)status->edges;
    for (int64_t s = tid; s < n; s += SCAN_THREADS)
        emit_at(s, keep, pos, esrc, edst, ew, edges, out_src, out_dst, out_w, capacity);
    __syncthreads();
    if (tid == 0) {
        *kept_total = total;
        status->edges += (unsigned long long)total;
        // "Boruvka round made no progress" (mst.rs:279-283)
        if (require_progress && total == 0) atomicCAS(&status->err_kind, 0, 4);
    }
    // union: path halving, smallest point of every tree, relabel, count the components
    for (int t = 0; t < steps; ++t) {
        for (int64_t s = tid; s < n; s += SCAN_THREADS) jump_at(s, parent, active_label);
        __syncthreads();
    }
    for (int64_t s = tid; s < n; s += SCAN_THREADS) minlab_init_at(s, parent, active_label, minlab);
    __syncthreads();
    for (int64_t s = tid; s < n; s += SCAN_THREADS)
        minlab_reduce_at(s, parent, active_label, minlab);
    __syncthreads();
    for (int64_t i = tid; i < n; i += SCAN_THREADS) relabel_at(i, point_label, parent, minlab);
    __syncthreads();
    int roots = 0;
    for (int64_t i0 = 0; i0 < n; i0 += SCAN_THREADS) {
        const int64_t i = i0 + tid;
        roots += __syncthreads_count(i < n && point_label[i] == (int32_t)i);
    }
    if (tid == 0) status->components = (unsigned long long)roots;
}

__global__ void __launch_bounds__(SCAN_THREADS)
    resolve_small_kernel(const int32_t *__restrict__ next, const int32_t *active_label,
                         int32_t *point_label, int64_t n, int steps, int32_t *ja,
                         int32_t *ma, int32_t *jb, int32_t *mb, int32_t *__restrict__ keep,
                         int32_t *__restrict__ pos, int32_t *__restrict__ kept_total,
                         const uint32_t *__restrict__ esrc, const uint32_t *__restrict__ edst,
                         const float *__restrict__ ew, int32_t *parent,
                         int32_t *__restrict__ minlab, DevStatus *status,
                         uint32_t *__restrict__ out_src, uint32_t *__restrict__ out_dst,
                         float *__restrict__ out_w, int64_t capacity, int require_progress) {
    resolve_block(next, active_label, point_label, n, steps, ja, ma, jb, mb, keep, pos, kept_total,
                  esrc, edst, ew, parent, minlab, status, out_src, out_dst, out_w, capacity,
                  require_progress);
}

// A Borůvka round's winners and merge for at most SMALL_RESOLVE_ROWS points in one CTA: the
// per-component minimum key (component_min_kernel's keys, reduced with block atomics), the
// winners (winner_kernel), then resolve_block. One launch instead of four.
__device__ __forceinline__ void round_block(
    const int32_t *__restrict__ perm, const int32_t *__restrict__ labp,
    const unsigned long long *__restrict__ row_keys, unsigned long long *__restrict__ comp_keys,
    int allow_empty, int32_t *label, int64_t n, int steps, int32_t *next, int32_t *ja,
    int32_t *ma, int32_t *jb, int32_t *mb, int32_t *__restrict__ keep, int32_t *__restrict__ pos,
    int32_t *__restrict__ kept_total, uint32_t *esrc, uint32_t *edst, float *ew, int32_t *parent,
    int32_t *__restrict__ minlab, DevStatus *status, uint32_t *__restrict__ out_src,
    uint32_t *__restrict__ out_dst, float *__restrict__ out_w, int64_t capacity) {
    const int tid = threadIdx.x;
    for (int64_t i = tid; i < n; i += SCAN_THREADS) comp_keys[i] = ~0ull;
    __syncthreads();
    for (int64_t p = tid; p < n; p += SCAN_THREADS) {
        const unsigned long long v = comp_key_at(p, perm, row_keys, status, allow_empty);
        if (v != ~0ull) atomicMin(&comp_keys[labp[p]], v);
    }
    __syncthreads();
    for (int64_t i = tid; i < n; i += SCAN_THREADS)
        winner_at(i, label, comp_keys, row_keys, n, next, esrc, edst, ew, status);
    __syncthreads();
    resolve_block(next, label, label, n, steps, ja, ma, jb, mb, keep, pos, kept_total, esrc, edst,
                  ew, parent, minlab, status, out_src, out_dst, out_w, capacity, 1);
}

__global__ void __launch_bounds__(SCAN_THREADS)
    round_small_kernel(const int32_t *__restrict__ perm, const int32_t *__restrict__ labp,
                       const unsigned long long *__restrict__ row_keys,
                       unsigned long long *__restrict__ comp_keys, int allow_empty,
                       int32_t *label, int64_t n, int steps, int32_t *next, int32_t *ja,
                       int32_t *ma, int32_t *jb, int32_t *mb, int32_t *__restrict__ keep,
                       int32_t *__restrict__ pos, int32_t *__restrict__ kept_total,
                       uint32_t *esrc, uint32_t *edst, float *ew, int32_t *parent,
                       int32_t *__restrict__ minlab, DevStatus *status,
                       uint32_t *__restrict__ out_src, uint32_t *__restrict__ out_dst,
                       float *__restrict__ out_w, int64_t capacity) {
    round_block(perm, labp, row_keys, comp_keys, allow_empty, label, n, steps, next, ja, ma, jb,
                mb, keep, pos, kept_total, esrc, edst, ew, parent, minlab, status, out_src,
                out_dst, out_w, capacity);
}

// Counting sort by label for at most SMALL_RESOLVE_ROWS points in one CTA: histogram, sum of
// squared sizes, exclusive scan and scatter (hist_kernel, same_pairs_kernel, scan_exclusive,
// scatter_kernel). The order of points within a label is free, as in scatter_kernel.
__device__ __forceinline__ void sort_block(const int32_t *__restrict__ label, int64_t n,
                                           int32_t *__restrict__ cnt, int32_t *__restrict__ start,
                                           int32_t *__restrict__ fill, int32_t *__restrict__ perm,
                                           DevStatus *status) {
    __shared__ int warp_sums[SCAN_THREADS / 32];
    __shared__ double pair_sums[SCAN_THREADS / 32];
    const int tid = threadIdx.x;
    for (int64_t i = tid; i < n; i += SCAN_THREADS) {
        cnt[i] = 0;
        fill[i] = 0;
    }
    __syncthreads();
    for (int64_t i = tid; i < n; i += SCAN_THREADS) atomicAdd(&cnt[label[i]], 1);
    __syncthreads();
    // sum of squared sizes (exact in f64: integers below 2^53)
    double v = 0.0;
    for (int64_t i = tid; i < n; i += SCAN_THREADS) {
        const double c = (double)cnt[i];
        v += c * c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) pair_sums[tid >> 5] = v;
    int c[SMALL_ITEMS];
    int sum = 0;
    const int64_t base = (int64_t)tid * SMALL_ITEMS;
#pragma unroll
    for (int u = 0; u < SMALL_ITEMS; ++u) {
        c[u] = base + u < n ? cnt[base + u] : 0;
        sum += c[u];
    }
    int total;
    int prefix = block_exclusive_scan(sum, warp_sums, total);
#pragma unroll
    for (int u = 0; u < SMALL_ITEMS; ++u) {
        if (base + u < n) start[base + u] = prefix;
        prefix += c[u];
    }
    if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < SCAN_THREADS / 32; ++w) t += pair_sums[w];
        status->same_pairs = t;
    }
    __syncthreads();
    for (int64_t i = tid; i < n; i += SCAN_THREADS) {
        const int32_t l = label[i];
        perm[start[l] + atomicAdd(&fill[l], 1)] = (int32_t)i;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS)
    sort_small_kernel(const int32_t *__restrict__ label, int64_t n, int32_t *__restrict__ cnt,
                      int32_t *__restrict__ start, int32_t *__restrict__ fill,
                      int32_t *__restrict__ perm, DevStatus *status) {
    sort_block(label, n, cnt, start, fill, perm, status);
}

inline unsigned blocks(int64_t n, int t = 256) { return (unsigned)ceil_div(n > 0 ? n : 1, t); }

}  // namespace

int scan_exclusive(cuscan_ctx *ctx, const int32_t *in, int32_t *out, int64_t n,
                   int32_t *grand_total, Buffer &tmp, cudaStream_t s) {
    const int64_t tiles = ceil_div(n > 0 ? n : 1, SCAN_TILE);
    int rc = ensure(ctx, tmp, (size_t)tiles * sizeof(int32_t), "scan tile sums");
    if (rc) return rc;
    CUSCAN_KERNEL(scan_tiles_kernel, (unsigned)tiles, SCAN_THREADS, 0, s, in, out, n, as<int32_t>(tmp));
    CUSCAN_KERNEL(scan_sums_kernel, 1, SCAN_THREADS, 0, s, as<int32_t>(tmp), tiles, grand_total);
    CUSCAN_KERNEL(scan_add_kernel, blocks(n), 256, 0, s, out, n, as<int32_t>(tmp));
    CUSCAN_LAUNCH(ctx, "scan_exclusive");
    return CUSCAN_OK;
}

int forest_core(cuscan_ctx *ctx, const float *knn_sq, int64_t n, int k, int min_samples,
                float *core, cudaStream_t s) {
    CUSCAN_KERNEL(core_kernel, blocks(n), 256, 0, s, knn_sq, n, k, min_samples, core);
    CUSCAN_LAUNCH(ctx, "core_kernel");
    return CUSCAN_OK;
}

static int log2_ceil(int64_t c) {
    int l = 0;
    while ((1ll << l) < c) ++l;
    return l;
}

// Common tail of the seed and of every round: break cycles of the proposals next[] over the
// active nodes, append the kept edges in node order, merge and relabel points.
static int resolve_proposals(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int64_t active,
                             const int32_t *active_label, int32_t *point_label,
                             uint32_t *out_src, uint32_t *out_dst, float *out_w,
                             int require_progress, cudaStream_t s) {
    int32_t *next = as<int32_t>(b.next);
    int32_t *ja = as<int32_t>(b.jmp_a), *ma = as<int32_t>(b.mx_a);
    int32_t *jb = as<int32_t>(b.jmp_b), *mb = as<int32_t>(b.mx_b);
    const int steps = log2_ceil(active > 1 ? active : 2) + 1;
    if (n <= SMALL_RESOLVE_ROWS) {
        CUSCAN_KERNEL(resolve_small_kernel, 1, SCAN_THREADS, 0, s, next, active_label,
                      point_label, n, steps, ja, ma, jb, mb, as<int32_t>(b.keep),
                      as<int32_t>(b.pos), as<int32_t>(b.kept_total), as<uint32_t>(b.esrc),
                      as<uint32_t>(b.edst), as<float>(b.ew), as<int32_t>(b.parent),
                      as<int32_t>(b.minlab), b.status, out_src, out_dst, out_w, n - 1,
                      require_progress);
        CUSCAN_LAUNCH(ctx, "resolve_small_kernel");
        return CUSCAN_OK;
    }
    CUSCAN_KERNEL(dbl_init_kernel, blocks(n), 256, 0, s, next, active_label, n, ja, ma);
    for (int t = 0; t < steps; ++t) {
        CUSCAN_KERNEL(dbl_step_kernel, blocks(n), 256, 0, s, ja, ma, active_label, n, jb, mb);
        int32_t *tj = ja, *tm = ma;
        ja = jb;
        ma = mb;
        jb = tj;
        mb = tm;
    }
    int32_t *keep = as<int32_t>(b.keep), *pos = as<int32_t>(b.pos), *parent = as<int32_t>(b.parent);
    CUSCAN_KERNEL(keep_kernel, blocks(n), 256, 0, s, next, ja, ma, active_label, n, keep, parent);
    CUSCAN_LAUNCH(ctx, "cycle breaking");
    int rc = scan_exclusive(ctx, keep, pos, n, as<int32_t>(b.kept_total), b.scan_tmp, s);
    if (rc) return rc;
    CUSCAN_KERNEL(emit_kernel, blocks(n), 256, 0, s, keep, pos, as<uint32_t>(b.esrc), as<uint32_t>(b.edst),
                                           as<float>(b.ew), n, b.status, out_src, out_dst, out_w,
                                           n - 1);
    CUSCAN_KERNEL(add_edges_kernel, 1, 1, 0, s, b.status, as<int32_t>(b.kept_total), require_progress);
    for (int t = 0; t < steps; ++t) CUSCAN_KERNEL(jump_kernel, blocks(n), 256, 0, s, parent, active_label, n);
    int32_t *minlab = as<int32_t>(b.minlab);
    CUSCAN_KERNEL(minlab_init_kernel, blocks(n), 256, 0, s, parent, active_label, n, minlab);
    CUSCAN_KERNEL(minlab_reduce_kernel, blocks(n), 256, 0, s, parent, active_label, n, minlab);
    CUSCAN_KERNEL(relabel_kernel, blocks(n), 256, 0, s, point_label, parent, minlab, n);
    CUSCAN_CUDA(ctx, cudaMemsetAsync(&b.status->components, 0, sizeof(unsigned long long), s));
    CUSCAN_KERNEL(count_components_kernel, blocks(n), 256, 0, s, point_label, n, b.status);
    CUSCAN_LAUNCH(ctx, "union/relabel");
    return CUSCAN_OK;
}

int forest_seed(cuscan_ctx *ctx, ForestBuffers &b, const float *core, const int32_t *ids,
                const float *dsq, int64_t n, int k, int32_t *label, uint32_t *out_src,
                uint32_t *out_dst, float *out_w, cudaStream_t s, int64_t active_bound) {
    CUSCAN_KERNEL(seed_kernel, blocks(n), 256, 0, s, core, ids, dsq, n, k, as<int32_t>(b.next),
                                           as<uint32_t>(b.esrc), as<uint32_t>(b.edst),
                                           as<float>(b.ew), b.status);
    CUSCAN_KERNEL(iota_kernel, blocks(n), 256, 0, s, label, n);
    CUSCAN_LAUNCH(ctx, "seed_kernel");
    // all points are active nodes of the seed graph (active_label == nullptr)
    int rc = resolve_proposals(ctx, b, n, active_bound > 0 ? active_bound : n, nullptr, label,
                               out_src, out_dst, out_w, 0, s);
    if (rc) return rc;
    return CUSCAN_OK;
}

int forest_sort_by_component(cuscan_ctx *ctx, ForestBuffers &b, const float *x, const float *core,
                             const int32_t *label, int64_t n, int d, cudaStream_t s) {
    int32_t *cnt = as<int32_t>(b.cnt), *start = as<int32_t>(b.start), *fill = as<int32_t>(b.fill);
    if (n <= SMALL_RESOLVE_ROWS) {
        CUSCAN_KERNEL(sort_small_kernel, 1, SCAN_THREADS, 0, s, label, n, cnt, start, fill,
                      as<int32_t>(b.perm), b.status);
        CUSCAN_KERNEL(gather_kernel, blocks(n * d), 256, 0, s, x, core, label, as<int32_t>(b.perm),
                      n, d, as<float>(b.xp), as<float>(b.corep), as<int32_t>(b.labp));
        CUSCAN_LAUNCH(ctx, "component sort");
        return CUSCAN_OK;
    }
    CUSCAN_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * n, s));
    CUSCAN_CUDA(ctx, cudaMemsetAsync(fill, 0, sizeof(int32_t) * n, s));
    CUSCAN_KERNEL(hist_kernel, blocks(n), 256, 0, s, label, n, cnt);
    CUSCAN_CUDA(ctx, cudaMemsetAsync(&b.status->same_pairs, 0, sizeof(double), s));
    CUSCAN_KERNEL(same_pairs_kernel, blocks(n), 256, 0, s, cnt, n, b.status);
    CUSCAN_LAUNCH(ctx, "hist_kernel");
    int rc = scan_exclusive(ctx, cnt, start, n, nullptr, b.scan_tmp, s);
    if (rc) return rc;
    CUSCAN_KERNEL(scatter_kernel, blocks(n), 256, 0, s, label, n, start, fill, as<int32_t>(b.perm));
    CUSCAN_KERNEL(gather_kernel, blocks(n * d), 256, 0, s, x, core, label, as<int32_t>(b.perm), n, d,
                                                 as<float>(b.xp), as<float>(b.corep),
                                                 as<int32_t>(b.labp));
    CUSCAN_LAUNCH(ctx, "component sort");
    return CUSCAN_OK;
}

int forest_round(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int64_t components,
                 int32_t *label, uint32_t *out_src, uint32_t *out_dst, float *out_w,
                 cudaStream_t s, int allow_empty) {
    unsigned long long *comp_keys = as<unsigned long long>(b.comp_keys);
    if (n <= SMALL_RESOLVE_ROWS) {
        const int steps = log2_ceil(components > 1 ? components : 2) + 1;
        CUSCAN_KERNEL(round_small_kernel, 1, SCAN_THREADS, 0, s, as<int32_t>(b.perm),
                      as<int32_t>(b.labp), as<unsigned long long>(b.row_keys), comp_keys,
                      allow_empty, label, n, steps, as<int32_t>(b.next), as<int32_t>(b.jmp_a),
                      as<int32_t>(b.mx_a), as<int32_t>(b.jmp_b), as<int32_t>(b.mx_b),
                      as<int32_t>(b.keep), as<int32_t>(b.pos), as<int32_t>(b.kept_total),
                      as<uint32_t>(b.esrc), as<uint32_t>(b.edst), as<float>(b.ew),
                      as<int32_t>(b.parent), as<int32_t>(b.minlab), b.status, out_src, out_dst,
                      out_w, n - 1);
        CUSCAN_LAUNCH(ctx, "round_small_kernel");
        return CUSCAN_OK;
    }
    int rc = launch_fill_u64(ctx, comp_keys, n, ~0ull, s);
    if (rc) return rc;
    CUSCAN_KERNEL(component_min_kernel, blocks(n), 256, 0, s, as<int32_t>(b.perm),
                  as<int32_t>(b.labp), as<unsigned long long>(b.row_keys), n, comp_keys, b.status,
                  allow_empty);
    CUSCAN_KERNEL(winner_kernel, blocks(n), 256, 0, s, label, comp_keys, as<unsigned long long>(b.row_keys),
                                             n, as<int32_t>(b.next), as<uint32_t>(b.esrc),
                                             as<uint32_t>(b.edst), as<float>(b.ew), b.status);
    CUSCAN_LAUNCH(ctx, "component winners");
    return resolve_proposals(ctx, b, n, components, label, label, out_src, out_dst, out_w, 1, s);
}

// Total MST weight in f64: the sum over the emitted edges of sqrt((double) w_sq), the per-edge
// weight that finalize_mst forms (crates/hdbscan-core/src/mst.rs:501-512). Every edge's f64
// weight is exact (IEEE square root of an exactly widened f32); only the order of the sum is
// this kernel's own: a fixed grid-stride assignment and a fixed shared-memory tree per block,
// then one block sums the partials the same way. The result depends only on the edge list.
constexpr int kWeightThreads = 256;
constexpr int kWeightBlocks = 256;

__device__ double block_tree_sum(double v, double *sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
#pragma unroll
    for (int off = kWeightThreads / 2; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    return sh[0];
}

__global__ void __launch_bounds__(kWeightThreads)
mst_weight_partials_kernel(const float *__restrict__ w, int64_t m, int grid,
                           double *__restrict__ partials) {
    __shared__ double sh[kWeightThreads];
    double acc = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kWeightThreads + threadIdx.x; i < m;
         i += (int64_t)grid * kWeightThreads)
        acc += sqrt((double)w[i]);
    const double total = block_tree_sum(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kWeightThreads)
mst_weight_final_kernel(const double *__restrict__ partials, int grid, DevStatus *status) {
    __shared__ double sh[kWeightThreads];
    double acc = 0.0;
    for (int i = threadIdx.x; i < grid; i += kWeightThreads) acc += partials[i];
    const double total = block_tree_sum(acc, sh);
    if (threadIdx.x == 0) status->mst_weight = total;
}

int forest_mst_weight(cuscan_ctx *ctx, ForestBuffers &b, const float *w, int64_t m,
                      cudaStream_t s) {
    if (m <= 0) {
        CUSCAN_CUDA(ctx, cudaMemsetAsync(&b.status->mst_weight, 0, sizeof(double), s));
        return CUSCAN_OK;
    }
    // partials live in the component-key array (n 64-bit slots, idle once the rounds end);
    // the grid never exceeds the edge count, which is below n
    const int grid = (int)std::min<int64_t>(kWeightBlocks, ceil_div(m, kWeightThreads));
    double *partials = as<double>(b.comp_keys);
    CUSCAN_KERNEL(mst_weight_partials_kernel, grid, kWeightThreads, 0, s, w, m, grid, partials);
    CUSCAN_KERNEL(mst_weight_final_kernel, 1, kWeightThreads, 0, s, partials, grid, b.status);
    CUSCAN_LAUNCH(ctx, "MST weight");
    return CUSCAN_OK;
}

int forest_reserve(cuscan_ctx *ctx, ForestBuffers &b, int64_t n, int d) {
    const size_t ni = sizeof(int32_t) * (size_t)n;
    int rc = 0;
#define RES(buf, bytes, what) \
    if ((rc = ensure(ctx, b.buf, (bytes), what))) return rc;
    RES(next, ni, "forest proposals");
    RES(esrc, ni, "forest sources");
    RES(edst, ni, "forest destinations");
    RES(ew, sizeof(float) * (size_t)n, "forest weights");
    RES(jmp_a, ni, "pointer doubling");
    RES(mx_a, ni, "pointer doubling");
    RES(jmp_b, ni, "pointer doubling");
    RES(mx_b, ni, "pointer doubling");
    RES(keep, ni, "kept edges");
    RES(pos, ni, "edge positions");
    RES(parent, ni, "forest parents");
    RES(minlab, ni, "component labels");
    RES(kept_total, 64, "kept total");
    RES(cnt, ni, "component histogram");
    RES(start, ni, "component offsets");
    RES(fill, ni, "component cursors");
    RES(perm, ni, "component order");
    RES(xp, sizeof(float) * (size_t)n * (size_t)d, "component-sorted data");
    RES(corep, sizeof(float) * (size_t)n, "component-sorted core distances");
    RES(labp, ni, "component-sorted labels");
    RES(row_keys, sizeof(unsigned long long) * (size_t)n, "row candidates");
    RES(comp_keys, sizeof(unsigned long long) * (size_t)n, "component candidates");
    RES(tile_lo, sizeof(int32_t) * (size_t)(ceil_div(n, 32) + 1), "tile label ranges");
    RES(tile_hi, sizeof(int32_t) * (size_t)(ceil_div(n, 32) + 1), "tile label ranges");
    RES(status_buf, sizeof(DevStatus), "fit status");
#undef RES
    b.status = as<DevStatus>(b.status_buf);
    return CUSCAN_OK;
}

int forest_buffers(ForestBuffers &b, Buffer **out) {
    RefinedBuffers &r = b.refined;
    Buffer *all[] = {&b.next, &b.esrc, &b.edst, &b.ew, &b.jmp_a, &b.mx_a, &b.jmp_b, &b.mx_b,
                     &b.keep, &b.pos, &b.parent, &b.minlab, &b.kept_total, &b.cnt, &b.start,
                     &b.fill, &b.perm, &b.xp, &b.corep, &b.labp, &b.row_keys, &b.comp_keys,
                     &b.tile_lo, &b.tile_hi, &b.status_buf, &b.scan_tmp, &b.knn_ids_tmp,
                     &b.knn_dist_tmp, &r.xt, &r.pnorm, &r.mnorm, &r.tile_mmax, &r.tile_lo,
                     &r.tile_hi, &r.cand_ids, &r.cand_lb, &r.fallback, &r.count, &r.error,
                     &r.cbound, &r.rowcnt, &r.pivots, &r.cells, &r.cell_d, &r.absmax,
                     &r.qthr, &r.xq, &r.pq, &r.mq, &r.cand2, &r.rowcnt2, &r.fallback2,
                     &r.urow, &r.colcnt, &r.colbuf, &r.act_flag, &r.act_idx, &r.act_pos,
                     &r.rowlb, &r.lbtmp, &r.cursor, &r.colp, &r.colc, &r.cmin};
    static_assert(sizeof(all) / sizeof(all[0]) == kForestBufferCount, "buffer list");
    const int count = (int)(sizeof(all) / sizeof(all[0]));
    if (out)
        for (int i = 0; i < count; ++i) out[i] = all[i];
    return count;
}

void forest_release(ForestBuffers &b) {
    Buffer *all[kForestBufferCount];
    const int count = forest_buffers(b, all);
    for (int i = 0; i < count; ++i) release(*all[i]);
    b.status = nullptr;
}

// ---- packed small fits: the one-CTA steps of every fit of a pack, one launch each ----
namespace {

constexpr int kPackRowTile = 32;  // rows per label-range tile of the candidate sweep

__device__ __forceinline__ int log2_ceil_dev(int64_t c) {
    int l = 0;
    while ((1ll << l) < c) ++l;
    return l;
}

// Fit blockIdx.x: core column, seed proposals, labels 0..n-1 and the seed's merge; the kernels
// core_kernel, seed_kernel, iota_kernel and resolve_small_kernel of the fit alone, with its
// step count. Block 0 also clears the pack's per-round counters.
__global__ void __launch_bounds__(SCAN_THREADS)
    pack_seed_kernel(const PackFit *__restrict__ fits, int *more) {
    const PackFit &f = fits[blockIdx.x];
    const int tid = threadIdx.x;
    const int64_t n = f.n;
    DevStatus *st = f.status;
    if (blockIdx.x == 0)
        for (int r = tid; r < kPackMaxRounds + 2; r += SCAN_THREADS) more[r] = 0;
    if (tid == 0) {
        *st = DevStatus{};
        f.kept_total[1] = 0;
    }
    for (int64_t i = tid; i < n; i += SCAN_THREADS) core_at(i, f.dsq, n, f.k, f.min_samples, f.core);
    __syncthreads();
    for (int64_t i = tid; i < n; i += SCAN_THREADS) {
        seed_at(i, f.core, f.ids, f.dsq, n, f.k, f.next, f.esrc, f.edst, f.ew, st);
        f.label[i] = (int32_t)i;
    }
    __syncthreads();
    resolve_block(f.next, nullptr, f.label, n, log2_ceil_dev(n > 1 ? n : 2) + 1, f.ja, f.ma,
                  f.jb, f.mb, f.keep, f.pos, f.kept_total, f.esrc, f.edst, f.ew, f.parent,
                  f.minlab, st, f.src, f.dst, f.w, n - 1, 0);
    if (tid == 0) {
        st->seed_edges = st->edges;
        st->components_after_seed = st->components;
    }
}

// Start of round r of fit blockIdx.x: whether it runs (more than one component, no error,
// within the round limit: the host driver's checks), then the component sort, the sorted labels
// and core distances (gather_kernel; pack_gather_kernel copies the rows), cleared row keys and
// the label range of every 32-row tile (tile_range_kernel).
__global__ void __launch_bounds__(SCAN_THREADS) pack_sort_kernel(const PackFit *__restrict__ fits) {
    const PackFit &f = fits[blockIdx.x];
    const int tid = threadIdx.x;
    const int64_t n = f.n;
    DevStatus *st = f.status;
    __shared__ int run;
    if (tid == 0) {
        int on = st->components > 1 && st->err_kind == 0;
        if (on && st->rounds > (unsigned long long)kPackMaxRounds) {
            st->err_kind = kPackErrNoConvergence;
            on = 0;
        }
        f.kept_total[1] = on;
        run = on;
    }
    __syncthreads();
    if (!run) return;
    sort_block(f.label, n, f.cnt, f.start, f.fill, f.perm, st);
    __syncthreads();
    for (int64_t p = tid; p < n; p += SCAN_THREADS) {
        const int32_t i = f.perm[p];
        f.corep[p] = f.core[i];
        f.labp[p] = f.label[i];
        f.row_keys[p] = ~0ull;
    }
    __syncthreads();
    const int64_t tiles = ceil_div(n, kPackRowTile);
    for (int64_t t = tid; t < tiles; t += SCAN_THREADS) {
        const int64_t a = t * kPackRowTile, b = a + kPackRowTile < n ? a + kPackRowTile : n;
        int32_t mn = f.labp[a], mx = mn;
        for (int64_t i = a + 1; i < b; ++i) {
            const int32_t l = f.labp[i];
            mn = l < mn ? l : mn;
            mx = l > mx ? l : mx;
        }
        f.tile_lo[t] = mn;
        f.tile_hi[t] = mx;
    }
}

// Sorted copy of the rows of fit blockIdx.y whose round runs (gather_kernel's copy), spread over
// the grid's x blocks: a single CTA per fit would wait on one dependent load pair per element.
__global__ void pack_gather_kernel(const PackFit *__restrict__ fits) {
    const PackFit &f = fits[blockIdx.y];
    if (!*(volatile int32_t *)&f.kept_total[1]) return;
    const int64_t n = f.n;
    const int d = f.d;
    const int64_t total = n * d;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = e / d;
        const int c = (int)(e - p * d);
        f.xp[e] = f.x[(int64_t)f.perm[p] * d + c];
    }
}

// End of round r of fit blockIdx.x: winners and merge (round_small_kernel), then the round's
// bookkeeping (rounds run, ordered cross pairs entering it) and whether another round is due.
__global__ void __launch_bounds__(SCAN_THREADS)
    pack_merge_kernel(const PackFit *__restrict__ fits, int r, int *more) {
    const PackFit &f = fits[blockIdx.x];
    if (!*(volatile int32_t *)&f.kept_total[1]) return;
    const int tid = threadIdx.x;
    const int64_t n = f.n;
    DevStatus *st = f.status;
    const int64_t comps = (int64_t)st->components;
    __syncthreads();  // every thread has the count before the merge rewrites it
    round_block(f.perm, f.labp, f.row_keys, f.comp_keys, f.allow_empty, f.label, n,
                log2_ceil_dev(comps > 1 ? comps : 2) + 1, f.next, f.ja, f.ma, f.jb, f.mb, f.keep,
                f.pos, f.kept_total, f.esrc, f.edst, f.ew, f.parent, f.minlab, st, f.src, f.dst,
                f.w, n - 1);
    if (tid == 0) {
        st->rounds += 1;
        st->cross_pairs += (double)n * (double)n - st->same_pairs;
        if (st->components > 1 && st->err_kind == 0) atomicAdd(&more[r], 1);
    }
}

// f64 MST weight of fit blockIdx.x in forest_mst_weight's order: the partial of block b of its
// grid is the tree sum over edges b * 256 + t + i * grid * 256, then the partials' tree sum.
__global__ void __launch_bounds__(kWeightThreads)
    pack_weight_kernel(const PackFit *__restrict__ fits) {
    __shared__ double sh[kWeightThreads];
    __shared__ double partials[kWeightBlocks];
    const PackFit &f = fits[blockIdx.x];
    DevStatus *st = f.status;
    if (st->err_kind) return;
    // a complete forest has n - 1 edges (any other count is reported by the host)
    const int64_t m = (int64_t)st->edges < f.n - 1 ? (int64_t)st->edges : f.n - 1;
    if (m <= 0) {
        if (threadIdx.x == 0) st->mst_weight = 0.0;
        return;
    }
    const int64_t g = ceil_div(m, kWeightThreads);
    const int grid = (int)(g < kWeightBlocks ? g : kWeightBlocks);
    for (int b = 0; b < grid; ++b) {
        double acc = 0.0;
        for (int64_t i = (int64_t)b * kWeightThreads + threadIdx.x; i < m;
             i += (int64_t)grid * kWeightThreads)
            acc += sqrt((double)f.w[i]);
        const double total = block_tree_sum(acc, sh);
        if (threadIdx.x == 0) partials[b] = total;
        __syncthreads();
    }
    double acc = 0.0;
    for (int i = threadIdx.x; i < grid; i += kWeightThreads) acc += partials[i];
    const double total = block_tree_sum(acc, sh);
    if (threadIdx.x == 0) st->mst_weight = total;
}

}  // namespace

int pack_knn(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max, int d_max,
             int k_max, int splits, cudaStream_t s, int64_t &launches) {
    return launch_pack_knn(ctx, fits, count, n_max, d_max, k_max, splits, s, launches);
}

int pack_seed(cuscan_ctx *ctx, const PackFit *fits, int count, int *more, cudaStream_t s) {
    CUSCAN_KERNEL(pack_seed_kernel, count, SCAN_THREADS, 0, s, fits, more);
    CUSCAN_LAUNCH(ctx, "pack_seed_kernel");
    return CUSCAN_OK;
}

int pack_round(cuscan_ctx *ctx, const PackFit *fits, int count, int64_t n_max, int d_max,
               int splits, int r, int *more, cudaStream_t s) {
    CUSCAN_KERNEL(pack_sort_kernel, count, SCAN_THREADS, 0, s, fits);
    CUSCAN_LAUNCH(ctx, "pack_sort_kernel");
    const dim3 gg((unsigned)std::min<int64_t>(ceil_div(n_max * d_max, 256), 128), (unsigned)count);
    CUSCAN_KERNEL(pack_gather_kernel, gg, 256, 0, s, fits);
    CUSCAN_LAUNCH(ctx, "pack_gather_kernel");
    if (int rc = launch_pack_candidates(ctx, fits, count, n_max, d_max, splits, s)) return rc;
    CUSCAN_KERNEL(pack_merge_kernel, count, SCAN_THREADS, 0, s, fits, r, more);
    CUSCAN_LAUNCH(ctx, "pack_merge_kernel");
    return CUSCAN_OK;
}

int pack_weight(cuscan_ctx *ctx, const PackFit *fits, int count, cudaStream_t s) {
    CUSCAN_KERNEL(pack_weight_kernel, count, kWeightThreads, 0, s, fits);
    CUSCAN_LAUNCH(ctx, "pack_weight_kernel");
    return CUSCAN_OK;
}

}  // namespace cuscan
