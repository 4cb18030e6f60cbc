// fest_stage_weno_nm_sst.cu - k-omega SST FP32 stage sweeps with the weno_nm
// reconstruction (all six flux schemes, single-block and batched); see fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_weno_nm_sst) {
  if (prec == FEST_FP64) return launch_stage_weno_nm_sst64(prec, flux, occ, grid, s, p, a, tm);
  (void)occ;
  return launch_stage_sst_t<FEST_INTERP_WENO_NM>(flux, grid, s, p, a, tm);
}
FEST_BATCH_LAUNCHER(launch_batch_weno_nm_sst) {
  (void)prec;
  return launch_batch_sst_t<FEST_INTERP_WENO_NM>(flux, ctas, s, e, nb);
}
}  // namespace fest
