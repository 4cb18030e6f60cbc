// fest_stage_weno_nm_sst64.cu - k-omega SST FP64 stage sweeps with the weno_nm
// reconstruction (all six flux schemes); see fest_stage.cuh.
#include "fest_stage.cuh"

namespace fest {
FEST_STAGE_LAUNCHER(launch_stage_weno_nm_sst64) {
  (void)prec;
  (void)occ;
  return launch_stage_sst_t<FEST_INTERP_WENO_NM, double>(flux, grid, s, p, a, tm);
}
}  // namespace fest
