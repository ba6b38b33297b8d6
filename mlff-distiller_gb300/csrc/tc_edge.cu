// Tensor-core (tcgen05) fused edge kernels -- placeholder until written.
#include "common.cuh"
#include "workspace.h"
#include "edge_common.cuh"

namespace mlff {

int pack_bf16(const mlff_dims& d, float* out, const PackedOffsets& o, cudaStream_t st) {
    (void)d; (void)out; (void)o; (void)st;
    return MLFF_OK;
}

int launch_edge_fwd_tc(const EdgeArgs& a, int layer, cudaStream_t st) {
    (void)a; (void)layer; (void)st;
    set_error("tensor-core path not built yet");
    return MLFF_ERR_UNSUPPORTED;
}

int launch_edge_bwd_tc(const EdgeArgs& a, int layer, cudaStream_t st) {
    (void)a; (void)layer; (void)st;
    set_error("tensor-core path not built yet");
    return MLFF_ERR_UNSUPPORTED;
}

}  // namespace mlff
