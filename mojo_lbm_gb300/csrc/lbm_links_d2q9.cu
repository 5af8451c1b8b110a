// The 32 double-buffer block-per-tile fused-step variants of the D2Q9 lattice with the
// interpolated bounce-back fused in (lbm_set_links), exact and fast arithmetic.
#include "lbm_step.cuh"

namespace lbm {
StepLaunch get_links_tile_step_d2q9(int f16c, int coll, int les, int fast) {
    static const StepLaunch exact[16] = LBM_DB_TABLE(launch_step_tile_links, D2Q9);
    static const StepLaunch fastt[16] = LBM_DB_TABLE(launch_step_tile_links_fast, D2Q9);
    return (fast ? fastt : exact)[db_index(f16c, coll, les)];
}
}  // namespace lbm
