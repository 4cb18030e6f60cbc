// fest_stage_muscl_visc.cu - laminar-viscous FP32 stage sweeps with the muscl
// reconstruction (all six flux schemes, single-block and batched); see
// fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_muscl_visc) {
  if (prec == FEST_FP64) return launch_stage_muscl_visc64(prec, flux, occ, grid, s, p, a, tm);
  (void)occ;
  return launch_stage_visc_t<FEST_INTERP_MUSCL>(flux, grid, s, p, a, tm);
}
FEST_BATCH_LAUNCHER(launch_batch_muscl_visc) {
  (void)prec;
  return launch_batch_visc_t<FEST_INTERP_MUSCL>(flux, ctas, s, e, nb);
}
}  // namespace fest
