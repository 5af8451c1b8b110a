// The 32 fast-arithmetic block-per-tile fused-step variants of the D3Q27 lattice (LBM_ARITH_FAST).
#include "lbm_step.cuh"

namespace lbm {
StepLaunch get_fast_tile_step_d3q27(int method, int f16c, int coll, int les) {
    static const StepLaunch t[32] = LBM_STEP_TABLE(launch_step_tile_fast, D3Q27);
    return t[step_index(method, f16c, coll, les)];
}
}  // namespace lbm
