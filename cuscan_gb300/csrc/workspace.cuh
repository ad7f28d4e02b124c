// Per-context device workspace (buffers are kept between calls and grow on demand).
#pragma once

#include "common.cuh"
#include "forest.cuh"

namespace cuscan {

// Workspace of packed small fits (pack.cu): per-fit buffers, branch streams, pinned staging.
struct PackWorkspace;
int64_t pack_reserved_bytes(const PackWorkspace *p);  // device bytes held
void pack_release(PackWorkspace *p);                 // frees device and pinned buffers
void pack_destroy(PackWorkspace *p);                 // also streams and events

struct FitWorkspace {
    ForestBuffers forest;
    Buffer x, ids, dsq, core, label, src, dst, w;  // device copies for the host-pointer entry
    Buffer op_keys, op_tiles_lo, op_tiles_hi, op_partials, op_knn_ids, op_knn_dist;
    Buffer pred_q, pred_ids, pred_dist;            // approximate_predict queries and candidates
    DevStatus *host_status = nullptr;              // pinned
    cudaEvent_t ev[6] = {};
    PackWorkspace *pack = nullptr;                 // created by the first packed call
    // per Borůvka round of the last fit: query rows screened, tensor-core tiles run, candidate
    // kernel time (ms), ordered cross-component pairs entering the round
    static constexpr int kMaxRoundLog = 64;
    int round_count = 0;
    int64_t round_rows[kMaxRoundLog] = {};
    int64_t round_tiles[kMaxRoundLog] = {};
    double round_ms[kMaxRoundLog] = {};
    double round_cross[kMaxRoundLog] = {};
};
constexpr int kOwnBufferCount = 17;

}  // namespace cuscan
