// fest_stage_weno_visc.cu - laminar-viscous FP32 stage sweeps with the weno
// reconstruction (all six flux schemes, single-block and batched); see
// fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_weno_visc) {
  if (prec == FEST_FP64) return launch_stage_weno_visc64(prec, flux, occ, grid, s, p, a, tm);
  (void)occ;
  return launch_stage_visc_t<FEST_INTERP_WENO>(flux, grid, s, p, a, tm);
}
FEST_BATCH_LAUNCHER(launch_batch_weno_visc) {
  (void)prec;
  return launch_batch_visc_t<FEST_INTERP_WENO>(flux, ctas, s, e, nb);
}
}  // namespace fest
