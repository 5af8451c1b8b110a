// The 32 double-buffer staged fused-step variants of the D3Q27 lattice (lbm_stage.cuh), exact and
// fast arithmetic.
#include "lbm_stage.cuh"

namespace lbm {
StepLaunch get_staged_step_d3q27(int f16c, int coll, int les, int fast) {
    static const StepLaunch exact[16] = LBM_DB_TABLE(launch_step_staged, D3Q27);
    static const StepLaunch fastt[16] = LBM_DB_TABLE(launch_step_staged_fast, D3Q27);
    return (fast ? fastt : exact)[db_index(f16c, coll, les)];
}
}  // namespace lbm
