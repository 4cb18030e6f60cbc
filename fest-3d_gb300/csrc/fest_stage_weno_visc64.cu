// fest_stage_weno_visc64.cu - laminar-viscous FP64 stage sweeps with the weno
// reconstruction (all six flux schemes); see fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_weno_visc64) {
  (void)prec;
  (void)occ;
  return launch_stage_visc_t<FEST_INTERP_WENO, double>(flux, grid, s, p, a, tm);
}
}  // namespace fest
