// bf16 tensor-core screening sweeps with exact f32 re-evaluation (placeholder until the
// tcgen05 kernels land; the fit rejects the refined precision while this reports 0).
#include "common.cuh"
#include "forest.cuh"

namespace cuscan {

int refined_available() { return 0; }

int launch_knn_refined(cuscan_ctx *ctx, ForestBuffers &, const float *, int64_t, int, int,
                       int32_t *, float *, cudaStream_t, int64_t *, int64_t *) {
    return fail(ctx, CUSCAN_BACKEND_UNAVAILABLE, "bf16-refined kNN is not built");
}

int launch_candidates_refined(cuscan_ctx *ctx, ForestBuffers &, int64_t, int, cudaStream_t,
                              int64_t *) {
    return fail(ctx, CUSCAN_BACKEND_UNAVAILABLE, "bf16-refined candidates are not built");
}

}  // namespace cuscan
