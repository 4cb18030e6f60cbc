// fest_stage_muscl.cu - fused stage sweeps with the muscl reconstruction
// (all six flux schemes, FP32 and FP64); see fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_muscl) { return launch_stage_t<FEST_INTERP_MUSCL>(prec, flux, occ, grid, s, p, a, tm); }
FEST_BATCH_LAUNCHER(launch_batch_muscl) { return launch_batch_t<FEST_INTERP_MUSCL>(prec, flux, ctas, s, e, nb); }
}  // namespace fest
