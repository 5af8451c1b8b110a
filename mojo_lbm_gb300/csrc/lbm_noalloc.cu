// lbm_reduce_mass_momentum_noalloc: the float64 mass/momentum reduction for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs while a memory pool or
// arena owned by someone else is the only allowed source of device memory, plugins loaded into a
// host application that forbids allocation on its hot path, and code that must not synchronise
// the device (cudaMalloc/cudaFree can).  lbm_create allocates handle scratch, so those callers
// cannot use lbm_reduce_mass_momentum.  This entry point needs no handle and allocates nothing:
// its scratch (one float64 x 4 partial per block of 4096 cells, plus the 4 results) lives in the
// file-scope device array below, which every GPU that loads the library holds until the process
// exits.  That bounds the grid to kNoAllocMaxCells cells.  The first call on a device looks the
// array up with cudaGetSymbolAddress, so it should come before any stream capture; the address is
// kept for the rest of the process, so the entry point must not be used on a device after a
// cudaDeviceReset of that device (the array then lives at a new address).  Every call shares the
// array: calls that overlap on the GPU race.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "lbm_aux.cuh"

namespace lbm {
void set_last_error(const char* msg);         // lbm_capi.cu
LayoutDesc make_layout(const lbm_grid_t& g);  // lbm_capi.cu
}

using namespace lbm;

namespace {

constexpr uint32_t kChunkThreads = 256;
constexpr uint32_t kCellsPerThread = 16;
constexpr uint32_t kChunkCells = kChunkThreads * kCellsPerThread;  // cells reduced by one block
constexpr uint32_t kMaxPartials = 32768;                           // 1 MiB of float64 x 4 partials
constexpr uint64_t kNoAllocMaxCells = (uint64_t)kMaxPartials * kChunkCells;  // 2^27 = 512^3

// Scratch of the no-allocation reduction: kMaxPartials partials of 4 doubles, then the 4 results.
// Host code must not use this name as an address; it goes through noalloc_scratch().
static __device__ __align__(256) double g_noalloc_scratch[kMaxPartials * 4 + 4];

// Device address of g_noalloc_scratch on the current device, looked up once per device and kept
// (valid until a cudaDeviceReset of that device).
std::mutex g_noalloc_mutex;
constexpr int kMaxDevices = 64;
double* g_noalloc_ptr[kMaxDevices] = {};

cudaError_t noalloc_scratch(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = (double*)p;
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

struct ChunkArgs {
    LayoutDesc lay;
    const void* f;
    const uint8_t* flags;
    double* partial;
    int32_t ddf, after_odd;
};

// One block reduces cells [blockIdx * kChunkCells, +kChunkCells): the same per-cell sums as
// mass_partial_kernel, with one partial per block instead of a fixed grid.
template <class L, bool F16C, bool ESO>
__global__ void __launch_bounds__(kChunkThreads) mass_chunk_kernel(const ChunkArgs a) {
    using S = typename Pop<F16C>::T;
    constexpr int Q = L::Q, D = L::D;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const uint32_t begin = blockIdx.x * kChunkCells;
    for (uint32_t k = 0; k < kCellsPerThread; ++k) {
        const uint32_t n = begin + k * kChunkThreads + threadIdx.x;
        if (n >= a.lay.ncells) break;
        const uint8_t flag = a.flags[n];
        if ((flag & 0x0F) == LBM_FLAG_SOLID || (flag & LBM_FLAG_EXCLUDE)) continue;
        Nbr nb;
        const Cell c = decode_cell<L>(a.lay, n, nb);
        float f[Q];
        gather_post<L, F16C, ESO>((const S*)a.f, a.lay, c, nb, a.after_odd != 0, f);
        double rho = a.ddf ? 1.0 : 0.0;
        double m[3] = {0.0, 0.0, 0.0};
        static_for<0, Q>([&](auto qc) {
            constexpr int q = qc.value;
            rho += (double)f[q];
            static_for<0, D>([&](auto dc) {
                constexpr int d = dc.value;
                if constexpr (L::c(q, d) > 0) m[d] += (double)f[q];
                else if constexpr (L::c(q, d) < 0) m[d] -= (double)f[q];
            });
        });
        acc[0] += rho;
        acc[1] += m[0];
        acc[2] += m[1];
        acc[3] += m[2];
    }
    block_sum_store<4>(acc, a.partial + (size_t)blockIdx.x * 4);
}

lbm_status nfail(lbm_status s, const std::string& m) {
    lbm::set_last_error(m.c_str());  // reported by lbm_last_error()
    return s;
}

}  // namespace

extern "C" lbm_status lbm_validate(const lbm_config_t* cfg, const lbm_grid_t* grid);
extern "C" const char* lbm_last_error(void);

extern "C" lbm_status lbm_reduce_mass_momentum_noalloc(const lbm_config_t* cfg, const lbm_grid_t* grid, const void* f,
                                                      const uint8_t* flags, int32_t after_odd_step, double out[4],
                                                      void* stream) {
    if (!cfg || !grid) return nfail(LBM_EINVAL, "null config or grid");
    const lbm_status v = lbm_validate(cfg, grid);
    if (v != LBM_OK) return nfail(v, lbm_last_error());
    const uint64_t N = (uint64_t)grid->nx * grid->ny * grid->nz;
    if (N > kNoAllocMaxCells)
        return nfail(LBM_EINVAL, "lbm_reduce_mass_momentum_noalloc: the grid has " + std::to_string(N) +
                                     " cells; its fixed scratch covers at most " + std::to_string(kNoAllocMaxCells) +
                                     " (512^3); use lbm_reduce_mass_momentum for larger grids");
    if (!f || !flags || !out) return nfail(LBM_EINVAL, "null buffer");
    double* scratch = nullptr;
    cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess)
        return nfail(LBM_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));

    ChunkArgs a;
    a.lay = make_layout(*grid);
    a.f = f;
    a.flags = flags;
    a.partial = scratch;
    a.ddf = cfg->DDF_shift;
    a.after_odd = after_odd_step ? 1 : 0;
    const uint32_t nblocks = (uint32_t)((N + kChunkCells - 1) / kChunkCells);
    cudaStream_t s = (cudaStream_t)stream;
    const bool f16 = cfg->use_float16c != 0, eso = cfg->lbm_method == LBM_ESOTERIC_PULL;
    auto go = [&](auto Lt) {
        using L = decltype(Lt);
        if (f16) {
            if (eso) mass_chunk_kernel<L, true, true><<<nblocks, kChunkThreads, 0, s>>>(a);
            else mass_chunk_kernel<L, true, false><<<nblocks, kChunkThreads, 0, s>>>(a);
        } else {
            if (eso) mass_chunk_kernel<L, false, true><<<nblocks, kChunkThreads, 0, s>>>(a);
            else mass_chunk_kernel<L, false, false><<<nblocks, kChunkThreads, 0, s>>>(a);
        }
    };
    if (grid->lattice == LBM_D2Q9) go(D2Q9{});
    else if (grid->lattice == LBM_D3Q19) go(D3Q19{});
    else go(D3Q27{});
    e = cudaGetLastError();
    if (e != cudaSuccess) return nfail(LBM_ECUDA, std::string("mass_chunk_kernel: ") + cudaGetErrorString(e));
    // every partial in [0, nblocks) was just written, so nothing has to be cleared first
    double* res = scratch + (size_t)kMaxPartials * 4;
    final_sum_kernel<4><<<1, kReduceThreads, 0, s>>>(scratch, (int)nblocks, res);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, res, 4 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return nfail(LBM_ECUDA, std::string("lbm_reduce_mass_momentum_noalloc: ") + cudaGetErrorString(e));
    for (int k = 0; k < 4; ++k)
        if (!std::isfinite(out[k])) return nfail(LBM_ENAN, "mass/momentum reduction found a non-finite value");
    return LBM_OK;
}
