// The 16 double-buffer batched persistent-step variants of the D3Q19 lattice with the interpolated
// bounce-back fused in (lbm_batch_set_link_mode).
#include "lbm_batch.cuh"

namespace lbm {
BatchLaunch get_batch_links_step_d3q19(int f16c, int coll, int les) {
    static const BatchLaunch t[16] = LBM_DB_TABLE(launch_step_batch_links, D3Q19);
    return t[db_index(f16c, coll, les)];
}
}  // namespace lbm
