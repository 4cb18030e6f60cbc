// fest_stage_ppm_sst.cu - k-omega SST FP32 stage sweeps with the ppm
// reconstruction (all six flux schemes, single-block and batched); see fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_ppm_sst) {
  if (prec == FEST_FP64) return launch_stage_ppm_sst64(prec, flux, occ, grid, s, p, a, tm);
  (void)occ;
  return launch_stage_sst_t<FEST_INTERP_PPM>(flux, grid, s, p, a, tm);
}
FEST_BATCH_LAUNCHER(launch_batch_ppm_sst) {
  (void)prec;
  return launch_batch_sst_t<FEST_INTERP_PPM>(flux, ctas, s, e, nb);
}
}  // namespace fest
