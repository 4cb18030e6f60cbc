// fest_fused.cu - fused fast path (see fest_fused.cuh).
#include "fest_fused.cuh"

namespace fest {

struct FusedState {
  int dummy;
};

bool fused_supported(const Params&, int) { return false; }
int fused_create(const Params&, const DevBlock&, const BlockRef*, cudaStream_t, FusedState** out) {
  *out = nullptr;
  return FEST_ERR_ARG;
}
void fused_destroy(FusedState* f) { delete f; }
void fused_invalidate(FusedState*) {}
int fused_run(FusedState*, const Params&, const DevBlock&, int, int, int, double, cudaStream_t,
              long long*) {
  return FEST_ERR_ARG;
}
int fused_export_state(FusedState*, double*, cudaStream_t) { return FEST_ERR_ARG; }
int fused_export_residual(FusedState*, const DevBlock&, cudaStream_t) { return FEST_ERR_ARG; }

}  // namespace fest
