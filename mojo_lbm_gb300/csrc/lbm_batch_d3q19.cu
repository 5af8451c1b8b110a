// The 32 batched persistent-step variants of the D3Q19 lattice and its batched link kernel.
#include "lbm_batch.cuh"

namespace lbm {
BatchLaunch get_batch_step_d3q19(int method, int f16c, int coll, int les) {
    static const BatchLaunch t[32] = LBM_STEP_TABLE(launch_step_batch, D3Q19);
    return t[step_index(method, f16c, coll, les)];
}

cudaError_t launch_link_batch_d3q19(const BatchLinkArgs& b, bool f16c, cudaStream_t s) {
    const uint32_t blocks = (uint32_t)((b.n + 255) / 256);
    if (f16c) link_kernel_batch<D3Q19, true><<<blocks, 256, 0, s>>>(b);
    else link_kernel_batch<D3Q19, false><<<blocks, 256, 0, s>>>(b);
    return cudaGetLastError();
}
}  // namespace lbm
