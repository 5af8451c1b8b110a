// The 16 learned-closure LES variants of the D3Q27 lattice (persistent block-per-tile kernel).
#include "lbm_step.cuh"

namespace lbm {
StepLaunch get_learned_step_d3q27(int method, int f16c, int coll) {
    static const StepLaunch t[16] = LBM_LEARNED_TABLE(launch_step_learned, D3Q27);
    return t[learned_index(method, f16c, coll)];
}
}  // namespace lbm
