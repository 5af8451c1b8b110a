// The 32 double-buffer block-per-tile fused-step variants of the D3Q19 lattice with the
// interpolated bounce-back fused in (lbm_set_links), exact and fast arithmetic.
#include "lbm_step.cuh"

namespace lbm {
StepLaunch get_links_tile_step_d3q19(int f16c, int coll, int les, int fast) {
    static const StepLaunch exact[16] = LBM_DB_TABLE(launch_step_tile_links, D3Q19);
    static const StepLaunch fastt[16] = LBM_DB_TABLE(launch_step_tile_links_fast, D3Q19);
    return (fast ? fastt : exact)[db_index(f16c, coll, les)];
}
}  // namespace lbm
