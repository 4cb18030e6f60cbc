// fest_stage_ppm_sst64.cu - k-omega SST FP64 stage sweeps with the ppm
// reconstruction (all six flux schemes); see fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_ppm_sst64) {
  (void)prec;
  (void)occ;
  return launch_stage_sst_t<FEST_INTERP_PPM, double>(flux, grid, s, p, a, tm);
}
}  // namespace fest
