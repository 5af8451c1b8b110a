// The 32 fused-step variants of the D3Q19 lattice (get_D3Q19, src/lbm/lattice.mojo:221-299).
#include "lbm_step.cuh"

namespace lbm {
StepLaunch get_step_d3q19(int method, int f16c, int coll, int les) {
    return StepTable<D3Q19>::get(method, f16c, coll, les);
}
}  // namespace lbm
