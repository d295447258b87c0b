// ensemble.cu - batched ensemble of independent colonies.
#include "ctx.h"

extern "C" {
slime_ensemble* slime_ensemble_create(uint32_t, const uint32_t*, const uint32_t*, const uint64_t*, const SlimeParams*, int* status) {
    if (status) *status = SLIME_ERR_STATE;
    return nullptr;
}
void slime_ensemble_destroy(slime_ensemble*) {}
const char* slime_ensemble_last_error(const slime_ensemble*) { return "ensemble not built yet"; }
int slime_ensemble_set_params(slime_ensemble*, uint32_t, const SlimeParams*) { return SLIME_ERR_STATE; }
int slime_ensemble_upload_agents(slime_ensemble*, uint32_t, const float*, uint64_t) { return SLIME_ERR_STATE; }
int slime_ensemble_download_agents(slime_ensemble*, uint32_t, float*, uint64_t) { return SLIME_ERR_STATE; }
int slime_ensemble_seed_agents(slime_ensemble*, uint32_t, uint64_t, float, float) { return SLIME_ERR_STATE; }
int slime_ensemble_upload_trail(slime_ensemble*, uint32_t, const float*, uint64_t) { return SLIME_ERR_STATE; }
int slime_ensemble_download_trail(slime_ensemble*, uint32_t, float*, uint64_t) { return SLIME_ERR_STATE; }
int slime_ensemble_step(slime_ensemble*, uint32_t) { return SLIME_ERR_STATE; }
int slime_ensemble_sync(slime_ensemble*) { return SLIME_ERR_STATE; }
int slime_ensemble_get_stream(slime_ensemble*, void**) { return SLIME_ERR_STATE; }
int slime_ensemble_autotune(slime_ensemble*, uint32_t) { return SLIME_ERR_STATE; }
int slime_ensemble_launch_count(const slime_ensemble*, uint64_t*) { return SLIME_ERR_STATE; }
}
