// fest_fused.cuh - the fused fast path: one sweep kernel per RK stage that
// reconstructs, evaluates fluxes, sums the residual and updates the state,
// in FP32 (FEST_MIXED) or FP64 arithmetic.
#pragma once
#include <vector>

#include "fest_kernels.cuh"

namespace fest {

struct FusedState;
// true when the fused sweep covers this scheme in this precision
bool fused_supported(const Params& p, int precision);
int fused_create(const Params& p, const DevBlock& b, const BlockRef* table, cudaStream_t s,
                 FusedState** out);
void fused_destroy(FusedState* f);
// the FP64 state in the DevBlock changed: re-seed the fused buffers
void fused_invalidate(FusedState* f);
int fused_run(FusedState* f, const Params& p, const DevBlock& b, int precision, int n_iters,
              int first_iter, double CFL, cudaStream_t s, long long* launches);
// copy the fused path's FP64 state into qp (the reference layout)
int fused_export_state(FusedState* f, double* qp, cudaStream_t s);
// the buffer holding the current state (reference layout), nullptr before
// the first run or after an invalidation; reading it keeps the fused state
const double* fused_current_state(const FusedState* f);
// the interior cells of the current state, and of its FP32 mirror where the
// mixed path keeps one, from a dense (imx-1)(jmx-1)(kmx-1) x n_var array in
// device-readable memory; the buffers, ghost cells and captured graphs stay
// as they are.  FEST_ERR_ARG if the state is not seeded (nothing written).
int fused_import_interior(FusedState* f, const double* src, cudaStream_t s, long long* cnt);
// event timing of the stage-sweep launches
void fused_profile(FusedState* f, bool enable);
int fused_profile_read(FusedState* f, long long* launches, double* total_ms);
// materialise the last stage's residual and boundary fluxes for find_resnorm
int fused_export_residual(FusedState* f, const DevBlock& b, cudaStream_t s);

// Blocks of one multiblock case advanced together, stage by stage, their
// interface ghosts read from each other: mixed precision (same
// reconstruction, flux scheme, integrator and physics) with one ghost launch
// and one sweep launch per stage for all blocks after iteration 2; FP64
// with each block's own launches.  p: the blocks' parameters with
// part_block set to batch indices and self_block to the block's own.
struct FusedBatch;
int fused_batch_create(const std::vector<FusedState*>& f, const std::vector<Params>& p,
                       const std::vector<DevBlock>& b, int precision, FusedBatch** out);
void fused_batch_destroy(FusedBatch* B);
int fused_batch_run(FusedBatch* B, int n_iters, int first_iter, double CFL, cudaStream_t s, long long* cnt);

}  // namespace fest
