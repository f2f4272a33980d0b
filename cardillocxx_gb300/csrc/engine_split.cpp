// Split-precision form (FP32 contact/Delassus/projection, FP64 state): host side.
#include "engine.h"

int Engine::step_split() { return fail(CDX_ERR_UNSUPPORTED, "split precision not built yet"); }
void Engine::destroy_split() {}
int Engine::sync_state_to_fp64() { return CDX_OK; }
int Engine::mark_state_changed() { return CDX_OK; }
int Engine::get_contacts_split(int32_t*, int32_t*, double*, double*, double*, int32_t*) {
    return fail(CDX_ERR_UNSUPPORTED, "split precision not built yet");
}
double Engine::split_bytes_per_iter() const { return 0.0; }
