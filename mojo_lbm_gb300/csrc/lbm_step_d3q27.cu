// The 32 fused-step variants of the D3Q27 lattice (get_D3Q27, src/lbm/lattice.mojo:122-218).
#include "lbm_step.cuh"

namespace lbm {
StepLaunch get_step_d3q27(int method, int f16c, int coll, int les) {
    return StepTable<D3Q27>::get(method, f16c, coll, les);
}
}  // namespace lbm
