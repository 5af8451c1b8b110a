// The 32 generic fused-step variants of the D3Q27 lattice (any tile shape, 64-bit offsets).
#include "lbm_step.cuh"

namespace lbm {
StepLaunch get_step_d3q27(int method, int f16c, int coll, int les) {
    static const StepLaunch t[32] = LBM_STEP_TABLE(launch_step, D3Q27);
    return t[step_index(method, f16c, coll, les)];
}
}  // namespace lbm
