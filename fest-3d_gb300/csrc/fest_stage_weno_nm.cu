// fest_stage_weno_nm.cu - fused stage sweeps with the weno_nm reconstruction
// (all six flux schemes, FP32 and FP64); see fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_weno_nm) { return launch_stage_t<FEST_INTERP_WENO_NM>(prec, flux, occ, grid, s, p, a, tm); }
FEST_BATCH_LAUNCHER(launch_batch_weno_nm) { return launch_batch_t<FEST_INTERP_WENO_NM>(prec, flux, ctas, s, e, nb); }
}  // namespace fest
