// bh.cu -- Barnes-Hut on the GPU (placeholder until the tree kernels land).
#include "common.cuh"
#include "engine.h"
#include "plugin_state.h"

namespace pg {
struct BhWorkspace {
    int dummy;
};
int bh_reserve(BhWorkspace *&ws, size_t, int)
{
    if (!ws) ws = new BhWorkspace();
    return PHYSIM_OK;
}
void bh_free(BhWorkspace *ws) { delete ws; }
int bh_accelerations(BhWorkspace *, const DeviceBodies &, const BhParams &, double *, cudaStream_t)
{
    set_error("Barnes-Hut kernels are not built yet");
    return PHYSIM_ERR_ARGUMENT;
}
int bh_launches(const BhWorkspace *) { return 0; }
}  // namespace pg
