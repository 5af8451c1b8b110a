// The 32 fused-step variants of the D2Q9 lattice (get_D2Q9, src/lbm/lattice.mojo:302-351).
#include "lbm_step.cuh"

namespace lbm {
StepLaunch get_step_d2q9(int method, int f16c, int coll, int les) {
    return StepTable<D2Q9>::get(method, f16c, coll, les);
}
}  // namespace lbm
