// fest_stage_none.cu - fused stage sweeps with the none reconstruction
// (all six flux schemes, FP32 and FP64); see fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_none) { return launch_stage_t<FEST_INTERP_NONE>(prec, flux, occ, grid, s, p, a, tm); }
FEST_BATCH_LAUNCHER(launch_batch_none) { return launch_batch_t<FEST_INTERP_NONE>(prec, flux, ctas, s, e, nb); }
}  // namespace fest
