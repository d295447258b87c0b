// adjoint.cu - checkpointed adjoint of the deposit -> decay -> diffuse chain.
#include "ctx.h"

using namespace slime;

namespace slime {
void free_adjoint(slime_ctx* ctx) {
    auto& a = ctx->adj;
    cudaFree(a.ckpt_agents);
    cudaFree(a.ckpt_trail);
    cudaFree(a.seg_trail);
    cudaFree(a.seg_counts);
    cudaFree(a.g[0]);
    cudaFree(a.g[1]);
    cudaFree(a.acc);
    cudaFree(a.agents_tmp);
    cudaFree(a.trail_tmp[0]);
    cudaFree(a.trail_tmp[1]);
    cudaFree(a.counts_tmp);
    a = slime_ctx::Adjoint();
}
} // namespace slime

extern "C" {
int slime_forward_record(slime_ctx* ctx, uint32_t, uint32_t) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    return set_error(ctx->err, SLIME_ERR_STATE, "adjoint not built yet");
}
int slime_backward(slime_ctx* ctx, const float*, SlimeGrads*, float*) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    return set_error(ctx->err, SLIME_ERR_STATE, "adjoint not built yet");
}
}
