// Batched persistent step: many domains of different size, one launch.
//
// Each domain is a complete single-domain problem (its own grid, tiled layout, f / bc / flags
// buffers and tau), described by a StepArgs.  The work units are the 256-cell tiles of all
// domains, numbered consecutively domain after domain.  A fixed grid of CTAs (SMs x resident
// CTAs) takes equal contiguous ranges of units; a CTA keeps its current domain's StepArgs in
// shared memory, reloads it when its range crosses into the next domain, and runs the same
// block-per-tile body (tile_step) as the single-domain kernel, so a batched step equals the
// single-domain steps bit for bit.  Two descriptor arrays hold the even and odd step of every
// domain (buffers swapped, esoteric parity), so the kernel only picks one.
#pragma once

#include "lbm_aux.cuh"

namespace lbm {

struct BatchArgs {
    const StepArgs* dom;          // ndom descriptors for this step's parity
    const uint32_t* unit_begin;   // ndom + 1 offsets of the domains' first tile units
    uint32_t ndom, total_units;
};

__device__ __forceinline__ uint32_t find_domain(const uint32_t* begin, uint32_t ndom, uint32_t u) {
    uint32_t lo = 0, hi = ndom;  // begin[lo] <= u < begin[hi]
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(begin + mid) <= u) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Resident CTAs per SM of the batched kernel; LINKS: with the interpolated bounce-back fused in
// (each descriptor's link table; tile_min_blocks of the single-domain kernel).
template <class L, int COLL, bool LINKS>
constexpr int batch_min_blocks() {
    if constexpr (LINKS) return tile_min_blocks<L, COLL, true>();
    else return (L::Q == 9) ? 5 : ((COLL == LBM_KBC || L::Q == 27) ? 3 : 4);
}

template <class L, int METHOD, bool F16C, int COLL, int LES, bool LINKS = false>
__global__ void __launch_bounds__(256, (batch_min_blocks<L, COLL, LINKS>())) step_kernel_batch(const BatchArgs b) {
    __shared__ StepArgs sa;
    // a contiguous, equal share of the units per CTA: the domain changes rarely along it, so the
    // descriptor is reloaded only when it does
    const uint32_t per = (b.total_units + gridDim.x - 1u) / gridDim.x;
    const uint32_t u0 = blockIdx.x * per;
    const uint32_t u1 = min(b.total_units, u0 + per);
    if (u0 >= u1) return;
    uint32_t d = find_domain(b.unit_begin, b.ndom, u0);
    uint32_t loaded = 0xffffffffu;
    uint32_t next_begin = __ldg(b.unit_begin + d + 1);
    for (uint32_t u = u0; u < u1; ++u) {
        while (u >= next_begin) {  // block-uniform
            ++d;
            next_begin = __ldg(b.unit_begin + d + 1);
        }
        if (d != loaded) {  // block-uniform
            __syncthreads();  // every thread is done with the previous descriptor
            const uint32_t* src = reinterpret_cast<const uint32_t*>(b.dom + d);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&sa);
            for (uint32_t i = threadIdx.x; i < sizeof(StepArgs) / 4; i += blockDim.x) dst[i] = __ldg(src + i);
            __syncthreads();
            loaded = d;
        }
        tile_step<L, METHOD, F16C, COLL, LES, false, LINKS>(sa, u - __ldg(b.unit_begin + d), threadIdx.x);
    }
}

// warp_near bit of warp box i (unit i / 8, warp i % 8) from the box summaries of its domain
// (one thread per box; 0 past the last box).
__device__ __forceinline__ uint32_t batch_near_box(const BatchArgs& b, uint32_t i, const uint8_t* box_sum) {
    const uint32_t u = i / kTileWarps;
    if (u >= b.total_units) return 0u;
    const uint32_t d = find_domain(b.unit_begin, b.ndom, u);
    const uint32_t first = b.unit_begin[d];
    return warp_near(box_sum + (size_t)first * kTileWarps, b.dom[d].lay, u - first, i % kTileWarps);
}

// Brings the summary of warp box `box` of the batch (unit box / 8) up to date (update_box_summary;
// flags_seen and box_sum hold 32 cells and one byte per box of the batch).  One thread per box.
__device__ __forceinline__ void batch_box_summary(const BatchArgs& b, uint32_t box, uint8_t* box_sum,
                                                  uint8_t* flags_seen, uint32_t* changed, uint32_t gen, int force) {
    const uint32_t u = box / kTileWarps;
    if (u >= b.total_units) return;
    const uint32_t d = find_domain(b.unit_begin, b.ndom, u);
    const uint32_t first = b.unit_begin[d];
    const StepArgs& a = b.dom[d];
    const uint32_t lb = box - first * kTileWarps;  // box index within the domain
    update_box_summary(a.flags, lb, flags_seen + (size_t)first * kTileCells, box_sum + (size_t)first * kTileWarps, a.lay,
                       changed, gen, force);
}

struct BatchLinkArgs {
    const StepArgs* dom;   // descriptors of the step that just ran: f_out is the lattice to fix
    const int32_t* domain;
    const int32_t* ids;
    const int32_t* dirs;
    const float* dists;
    float* force;
    int64_t n;
    float q_clamp;
    int32_t bouzidi, compute_force, ddf;
};

// linkwise_bounceback_kernel (src/lbm/geometry/interpolated_BB.mojo:46-141) over the links of all
// domains: each link carries its domain, and works on that domain's freshly written lattice.
template <class L, bool F16C>
__global__ void link_kernel_batch(const BatchLinkArgs b) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= b.n) return;
    const StepArgs& a = b.dom[b.domain[t]];
    LinkArgs la;
    la.lay = a.lay;
    la.f = a.f_out;
    la.force = b.force;
    la.ids = b.ids;
    la.dirs = b.dirs;
    la.dists = b.dists;
    la.n = b.n;
    la.q_clamp = b.q_clamp;
    la.bouzidi = b.bouzidi;
    la.compute_force = b.compute_force;
    la.ddf = b.ddf;
    link_one<L, F16C>(la, t);
}

using BatchLaunch = cudaError_t (*)(const BatchArgs&, int sms, cudaStream_t);

template <class L, int METHOD, bool F16C, int COLL, int LES, bool LINKS = false>
cudaError_t launch_step_batch_impl(const BatchArgs& b, int sms, cudaStream_t s) {
    static int per_sm = 0;
    if (per_sm == 0) {
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, step_kernel_batch<L, METHOD, F16C, COLL, LES, LINKS>, (int)kTileCells, 0);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    uint32_t grid = (uint32_t)(sms * per_sm);
    if (grid > b.total_units) grid = b.total_units;
    if (grid == 0) return cudaSuccess;
    step_kernel_batch<L, METHOD, F16C, COLL, LES, LINKS><<<grid, kTileCells, 0, s>>>(b);
    return cudaGetLastError();
}
template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_batch(const BatchArgs& b, int sms, cudaStream_t s) {
    return launch_step_batch_impl<L, METHOD, F16C, COLL, LES, false>(b, sms, s);
}
// The batched step with the links fused in (lbm_batch_set_link_mode, double buffer).
template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_batch_links(const BatchArgs& b, int sms, cudaStream_t s) {
    return launch_step_batch_impl<L, METHOD, F16C, COLL, LES, true>(b, sms, s);
}

}  // namespace lbm
