// The staged block-per-tile step (double buffer): a persistent CTA walks tiles, and while it streams
// and collides one tile from shared memory, bulk asynchronous copies (cp.async.bulk, completing on
// an mbarrier) bring the next tile's pull neighbourhood into the other half of a two-stage buffer.
//
// The neighbourhood is copied as whole 16-byte-aligned tile rows: for each direction q the rows the
// tile's cells pull from (stage_off in lbm_step.cuh: the tile's own x-column of tiles, shifted by
// -c_q.y and -c_q.z across the y/z-neighbour tiles, plus the x-neighbour column for c_q.x != 0).  The
// host builds the list of copy segments once per tile shape (build_stage_segments): consecutive
// rows that are consecutive in both the source tile and the stage merge into one copy, so a D3Q19
// 8x8x4 tile takes about 140 copies.  The copies move no population that the tile does not read
// except the x-neighbour rows (a whole 16-byte row for its one edge cell); those rows come from L2,
// where the neighbouring CTAs' own reads have put them.
//
// The thread then reads its Q populations from shared memory at its own position plus constant
// offsets (three per-thread bases: x, x - 1, x + 1), with none of the per-direction global address
// arithmetic of step_kernel_tile, and runs tile_step's boundary handling, collision and stores.
// Every wait is bounded (kStageWaitNs of global time): on a timeout the CTA raises a.err, waits (as
// long again at most) for the copies it has in flight and returns; the host reports LBM_ETIMEOUT
// (lbm_device_status).  The copies need 16-byte aligned population buffers and tile rows of a
// multiple of 16 bytes (tx >= 8 for Float16C, tx >= 4 for float32); the host checks both.
#pragma once

#include "lbm_step.cuh"

namespace lbm {

// One bulk copy of the stage: `bytes` from element `src` of the population block of the tile at
// offset (dx, dy, dz) = (nbr % 3, nbr / 3 % 3, nbr / 9) - 1 from the current tile, to byte `dst`
// of the stage buffer.
struct StageSeg {
    uint32_t src, dst, bytes, nbr;
};

constexpr uint64_t kStageWaitNs = 500000000ull;  // 0.5 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0u;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Waits for the completion of phase `parity` of the mbarrier, for kStageWaitNs at most.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > kStageWaitNs) return false;
    return true;
}
// Orders this thread's earlier generic-proxy accesses of shared memory before the async-proxy
// writes of the bulk copies it issues next.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Index of the neighbour tile (nbr % 3, nbr / 3 % 3, nbr / 9) - 1 of `tile`, with the periodic wrap.
__device__ __forceinline__ uint32_t stage_nbr_tile(const StepArgs& a, uint32_t tile, uint32_t nbr) {
    const uint32_t ntx = (uint32_t)a.lay.ntx, nty = (uint32_t)a.lay.nty, ntz = (uint32_t)a.lay.ntz;
    const uint32_t byz = a.lay.d_ntx.div(tile);
    const uint32_t bx = tile - byz * ntx;
    const uint32_t bz = a.lay.d_nty.div(byz);
    const uint32_t by = byz - bz * nty;
    const uint32_t ox = nbr % 3u, oy = (nbr / 3u) % 3u, oz = nbr / 9u;  // offset + 1
    const uint32_t x = ox == 0u ? (bx == 0u ? ntx - 1u : bx - 1u) : ox == 2u ? (bx + 1u == ntx ? 0u : bx + 1u) : bx;
    const uint32_t y = oy == 0u ? (by == 0u ? nty - 1u : by - 1u) : oy == 2u ? (by + 1u == nty ? 0u : by + 1u) : by;
    const uint32_t z = oz == 0u ? (bz == 0u ? ntz - 1u : bz - 1u) : oz == 2u ? (bz + 1u == ntz ? 0u : bz + 1u) : bz;
    return x + ntx * (y + nty * z);
}

// The stage's copies into the buffer at shared address `buf`, completing on `bar`, from the tiles
// nbr[0..26]; spread over the CTA's warps (segment i goes to warp i % 8), since the copy
// instruction takes its operands from uniform registers and a warp issues its lanes' copies one
// after another.
template <class L, bool F16C>
__device__ __forceinline__ void stage_copies(const StepArgs& a, const StageSeg* segs, const uint32_t* nbr,
                                             uint32_t buf, uint32_t bar, uint32_t tid) {
    using S = typename Pop<F16C>::T;
    const S* f = static_cast<const S*>(a.f_in);
    fence_proxy_async_smem();
    constexpr uint32_t W = kTileCells / 32u;
    for (uint32_t i = (tid >> 5) + W * (tid & 31u); i < a.nsegs; i += kTileCells) {
        const StageSeg s = segs[i];
        bulk_copy_g2s(buf + s.dst, f + (uint64_t)nbr[s.nbr] * (uint64_t)(kTileCells * L::Q) + s.src, s.bytes, bar);
    }
}

constexpr uint32_t kStageHead = 128;  // two mbarriers, padded

// Dynamic shared memory of the staged kernel: the barriers, the segment list, two stage buffers.
LBM_HD uint32_t stage_smem_bytes(uint32_t nsegs, uint32_t stage_bytes) {
    return kStageHead + ((nsegs * (uint32_t)sizeof(StageSeg) + 127u) & ~127u) + 2u * stage_bytes;
}

// Resident CTAs per SM the register budget is set for: D2Q9 5, KBC and D3Q27 3, others 4 (the
// tile walk and the stage bookkeeping take the registers 5 would leave the D3Q19 collision).
// Shared memory (two stages: 15 KB each for D3Q19 Float16C, 30 KB float32, 45 KB D3Q27 float32)
// allows fewer for the float32 and D3Q27 kernels.
template <class L, int COLL>
constexpr int stage_min_blocks() {
    return (COLL == LBM_KBC || L::Q == 27) ? 3 : (L::Q == 9 ? 5 : 4);
}

template <class L, bool F16C, int COLL, int LES, bool FAST>
__global__ void __launch_bounds__(kTileCells, (stage_min_blocks<L, COLL>())) step_kernel_staged(const StepArgs a) {
    static_assert(LES != kLesLearned, "the learned closure runs in step_kernel_learned");
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ uint32_t nbr[2][27];  // the neighbour tiles of the tile each buffer is staging
    const uint32_t tid = threadIdx.x;
    StageSeg* segs = reinterpret_cast<StageSeg*>(smem + kStageHead);
    uint8_t* const buf0 = smem + kStageHead + ((a.nsegs * (uint32_t)sizeof(StageSeg) + 127u) & ~127u);
    uint8_t* const buf1 = buf0 + a.stage_bytes;
    const uint32_t bar0 = smem_u32(smem), bar1 = bar0 + 8u;
    const uint32_t ntiles = a.lay.ncells / kTileCells;
    const uint32_t G = gridDim.x;
    uint32_t tile = blockIdx.x;
    if (tile >= ntiles) return;

    // prologue: the segment list, the barriers, the stages of the first two tiles
    const uint32_t* src = static_cast<const uint32_t*>(a.stage_segs);
    for (uint32_t i = tid; i < a.nsegs * 4u; i += kTileCells) reinterpret_cast<uint32_t*>(segs)[i] = __ldg(src + i);
    const bool second = tile + G < ntiles;
    if (tid < 27u) {
        nbr[0][tid] = stage_nbr_tile(a, tile, tid);
        if (second) nbr[1][tid] = stage_nbr_tile(a, tile + G, tid);
    }
    if (tid == 0u) {
        mbar_init(bar0, 1u);
        mbar_init(bar1, 1u);
        mbar_fence_init();
        mbar_expect_tx(bar0, a.stage_bytes + a.stage_extra);
        if (second) mbar_expect_tx(bar1, a.stage_bytes + a.stage_extra);
    }
    __syncthreads();
    stage_copies<L, F16C>(a, segs, nbr[0], smem_u32(buf0), bar0, tid);
    if (second) stage_copies<L, F16C>(a, segs, nbr[1], smem_u32(buf1), bar1, tid);

    for (uint32_t k = 0;; ++k) {
        const uint32_t s = k & 1u;
        const uint32_t bar_s = s ? bar1 : bar0, bar_o = s ? bar0 : bar1;
        uint8_t* const buf_s = s ? buf1 : buf0;
        const bool ok = mbar_wait(bar_s, (k >> 1) & 1u);
        if (__syncthreads_or(!ok)) {
            // timed out: report, let the copies in flight land (bounded), leave
            if (tid == 0u) {
                atomicExch(a.err, 1u);
                mbar_wait(bar_s, (k >> 1) & 1u);
                if (tile + G < ntiles) mbar_wait(bar_o, ((k + 1) >> 1) & 1u);
            }
            return;
        }
        tile_step<L, LBM_DOUBLE_BUFFER, F16C, COLL, LES, FAST, false, true>(a, tile, tid, nullptr, nullptr, -1,
                                                                          buf_s);
        // buffer s next stages the tile two ahead, once every thread has read it
        const uint32_t ahead = tile + 2u * G;
        const bool more = ahead < ntiles;
        if (more) {
            if (tid < 27u) nbr[s][tid] = stage_nbr_tile(a, ahead, tid);
            if (tid == 0u) mbar_expect_tx(bar_s, a.stage_bytes + a.stage_extra);
        }
        __syncthreads();
        if (more) stage_copies<L, F16C>(a, segs, nbr[s], smem_u32(buf_s), bar_s, tid);
        if (tile + G >= ntiles) break;
        tile += G;
    }
}

template <class L, int METHOD, bool F16C, int COLL, int LES, bool FAST>
cudaError_t launch_step_staged_impl(const StepArgs& a, cudaStream_t s) {
    static_assert(METHOD == LBM_DOUBLE_BUFFER, "the staged kernel is double-buffer only");
    auto kernel = step_kernel_staged<L, F16C, COLL, LES, FAST>;
    const uint32_t smem = stage_smem_bytes(a.nsegs, a.stage_bytes);
    static int per_sm = 0, sms = 0;
    static uint32_t smem_set = 0;
    if (smem_set != smem) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, (int)kTileCells, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        smem_set = smem;
    }
    const uint32_t ntiles = a.lay.ncells / kTileCells;
    const uint32_t grid = min(ntiles, (uint32_t)(sms * per_sm));
    kernel<<<grid, kTileCells, smem, s>>>(a);
    return cudaGetLastError();
}
template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_staged(const StepArgs& a, int, cudaStream_t s) {
    return launch_step_staged_impl<L, METHOD, F16C, COLL, LES, false>(a, s);
}
template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_staged_fast(const StepArgs& a, int, cudaStream_t s) {
    return launch_step_staged_impl<L, METHOD, F16C, COLL, LES, true>(a, s);
}

}  // namespace lbm
