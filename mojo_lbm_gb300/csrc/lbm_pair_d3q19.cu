// The 32 double-buffer cell-pair fused-step variants of the D3Q19 lattice (lbm_pair.cuh),
// exact and fast arithmetic.
#include "lbm_pair.cuh"

namespace lbm {
StepLaunch get_pair_step_d3q19(int f16c, int coll, int les, int fast) {
    static const StepLaunch exact[16] = LBM_DB_TABLE(launch_step_pair, D3Q19);
    static const StepLaunch fastt[16] = LBM_DB_TABLE(launch_step_pair_fast, D3Q19);
    return (fast ? fastt : exact)[db_index(f16c, coll, les)];
}
}  // namespace lbm
