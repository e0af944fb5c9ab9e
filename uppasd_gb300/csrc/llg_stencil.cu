// llg_stencil.cu -- structured-lattice mixed-precision LLG path (precision = 1).
// Placeholder until the structured kernels land: every entry reports that the
// path is unavailable so callers fall back to precision = 0.
#include "sim.h"

namespace uppasd {

int structured_init(Sim &, const uppasd_gpu_consts *, const uppasd_gpu_arrays *) {
    set_error("precision = 1 (structured mixed-precision path) is not available in this build");
    return UPPASD_GPU_EUNSUPPORTED;
}
int structured_step(Sim &, int64_t, int) { return UPPASD_GPU_EUNSUPPORTED; }
int structured_sync_state(Sim &) { return UPPASD_GPU_EUNSUPPORTED; }
int structured_load_state(Sim &) { return UPPASD_GPU_EUNSUPPORTED; }
void structured_free(Sim &) {}

}  // namespace uppasd
