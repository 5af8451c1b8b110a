// Autotuner: picks the tile shape of the layout (and, if allowed, pull vs esoteric-pull streaming)
// for a configuration and grid size by timing each candidate's step on the device.  No counterpart
// in the reference, whose block and tile shapes are compile-time choices (grid.mojo:55-107).
//
// The timing workload is the caller's flags and boundary values (given in the untiled layout and
// laid out on the device for each candidate tile), or a periodic box of fluid at rest, stepped
// from a captured CUDA graph through the same entry points a caller uses (lbm_create,
// lbm_init_equilibrium, lbm_run).  Scratch buffers are allocated once and freed before returning.
// The flags matter: a tile that is long in one direction touches walls almost everywhere and
// loses the block-per-tile kernel's all-fluid fast path.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "../../include/lbm_gb300.h"

namespace lbm {
__attribute__((visibility("hidden"))) void set_last_error(const char* msg);
}

namespace {

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

// dst (tiled layout tx, ty, tz; K components per cell) <- src (untiled: x fastest, then y, z, k).
template <class E>
__global__ void relayout_kernel(const E* __restrict__ src, E* __restrict__ dst, int32_t nx, int32_t ny, int32_t nz,
                                int32_t tx, int32_t ty, int32_t tz, int32_t K) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)nx * ny * nz;
    if (i >= n * K) return;
    const int64_t cell = i % n;
    const int32_t k = (int32_t)(i / n);
    const int32_t x = (int32_t)(cell % nx), y = (int32_t)((cell / nx) % ny), z = (int32_t)(cell / ((int64_t)nx * ny));
    const int64_t T = (int64_t)tx * ty * tz;
    const int64_t tile = x / tx + (int64_t)(nx / tx) * (y / ty + (int64_t)(ny / ty) * (z / tz));
    const int64_t loc = x % tx + (int64_t)tx * (y % ty + (int64_t)ty * (z % tz));
    dst[loc + T * (k + (int64_t)K * tile)] = src[i];
}

template <class E>
cudaError_t relayout(const E* src, E* dst, const lbm_grid_t& g, int32_t K, cudaStream_t s) {
    const int64_t n = (int64_t)g.nx * g.ny * g.nz * K;
    relayout_kernel<E><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, g.nx, g.ny, g.nz, g.tx, g.ty, g.tz, K);
    return cudaGetLastError();
}

lbm_status tune_fail(lbm_status s, const char* msg) {
    lbm::set_last_error(msg);
    return s;
}

lbm_status cuda_fail(const char* where, cudaError_t e) {
    static thread_local char buf[256];
    std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
    lbm::set_last_error(buf);
    return LBM_ECUDA;
}

struct Scratch {
    void* fa = nullptr;
    void* fb = nullptr;
    float* bc = nullptr;
    uint8_t* flags = nullptr;
    ~Scratch() {
        if (fa) cudaFree(fa);
        if (fb) cudaFree(fb);
        if (bc) cudaFree(bc);
        if (flags) cudaFree(flags);
    }
};

// Seconds per step of one candidate (graph-replayed), or a negative value with the status set.
lbm_status time_candidate(const lbm_config_t& cfg, const lbm_grid_t& g, Scratch& s, int32_t steps,
                          cudaStream_t stream, double* sec_per_step) {
    lbm_handle* h = nullptr;
    lbm_status st = lbm_create(&cfg, &g, &h);
    if (st != LBM_OK) return st;
    const bool eso = cfg.lbm_method == LBM_ESOTERIC_PULL;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
        lbm_destroy(h);
        return cuda_fail("cudaEventCreate", e);
    }
    st = lbm_init_equilibrium(h, s.fa, 1.f, 0.8f, nullptr, nullptr, stream);
    if (st == LBM_OK && !eso) {
        const size_t bytes = (size_t)lbm_f_elements(&g) * (cfg.use_float16c ? 2 : 4);
        e = cudaMemcpyAsync(s.fb, s.fa, bytes, cudaMemcpyDeviceToDevice, stream);
        if (e != cudaSuccess) st = cuda_fail("cudaMemcpyAsync", e);
    }
    void* fb = eso ? s.fa : s.fb;
    // warm-up (also captures the graph), then the timed replay
    if (st == LBM_OK) st = lbm_run(h, s.fa, fb, s.bc, s.flags, 0.8f, 64, 0, stream);
    if (st == LBM_OK) {
        cudaEventRecord(e0, stream);
        st = lbm_run(h, s.fa, fb, s.bc, s.flags, 0.8f, steps, 0, stream);
        cudaEventRecord(e1, stream);
        e = cudaEventSynchronize(e1);
        if (st == LBM_OK && e != cudaSuccess) st = cuda_fail("cudaEventSynchronize", e);
    }
    if (st == LBM_OK) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        *sec_per_step = 1e-3 * ms / steps;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    lbm_destroy(h);
    return st;
}

}  // namespace

extern "C" {

int32_t lbm_tune_candidates(int32_t lattice, int32_t nx, int32_t ny, int32_t nz, int32_t* tiles, int32_t max) {
    const int d = lbm_lattice_d(lattice);
    if (d < 0 || nx <= 0 || ny <= 0 || nz <= 0) return -1;
    if ((d == 2) != (nz == 1)) return -1;
    int32_t n = 0;
    for (int tx = 1; tx <= 256; tx *= 2)
        for (int ty = 1; ty <= 256; ty *= 2) {
            const int tz = 256 / (tx * ty);
            if (tx * ty > 256 || tx * ty * tz != 256 || !pow2(tz)) continue;
            if (d == 2 && tz != 1) continue;
            if (nx % tx || ny % ty || nz % tz) continue;
            if (tiles && n < max) {
                tiles[3 * n] = tx;
                tiles[3 * n + 1] = ty;
                tiles[3 * n + 2] = tz;
            }
            ++n;
        }
    return n;
}

lbm_status lbm_autotune(const lbm_config_t* cfg, int32_t lattice, int32_t nx, int32_t ny, int32_t nz,
                        const uint8_t* flags, const float* bc, int32_t choose_method, int32_t steps,
                        lbm_tune_result_t* out, void* stream) {
    if (!cfg || !out) return tune_fail(LBM_EINVAL, "null argument");
    if (steps < 1) return tune_fail(LBM_EINVAL, "steps must be positive");
    int32_t tiles[3 * 64];
    const int32_t nt = lbm_tune_candidates(lattice, nx, ny, nz, tiles, 64);
    if (nt < 0) return tune_fail(LBM_EINVAL, "bad lattice or grid shape");
    if (nt == 0)
        return tune_fail(LBM_EUNSUPPORTED, "no 256-cell power-of-two tile divides the grid: the generic kernel "
                                           "runs the caller's layout as given");
    lbm_grid_t g{lattice, nx, ny, nz, tiles[0], tiles[1], tiles[2]};
    lbm_status st = lbm_validate(cfg, &g);
    if (st != LBM_OK) return st;
    const int64_t fe = lbm_f_elements(&g), be = lbm_bc_elements(&g), ne = lbm_flag_elements(&g);
    const size_t fbytes = (size_t)fe * (cfg->use_float16c ? 2 : 4);
    Scratch s;
    cudaError_t e = cudaMalloc(&s.fa, fbytes);
    if (e == cudaSuccess) e = cudaMalloc(&s.fb, fbytes);
    if (e == cudaSuccess) e = cudaMalloc(&s.bc, sizeof(float) * be);
    if (e == cudaSuccess) e = cudaMalloc(&s.flags, ne);
    if (e == cudaSuccess) e = cudaMemset(s.bc, 0, sizeof(float) * be);
    if (e == cudaSuccess) e = cudaMemset(s.flags, 0, ne);
    if (e != cudaSuccess) return cuda_fail("lbm_autotune scratch", e);

    lbm_config_t c = *cfg;
    if (!flags) {
        // a periodic box needs no wall or equilibrium boundary data; the step kernels are the same
        c.include_equilibrium_bc = 0;
        c.capture_density = c.capture_velocity = 0;
    } else if (!bc && (c.include_moving_boundary || c.include_equilibrium_bc || c.capture_density ||
                       c.capture_velocity)) {
        return tune_fail(LBM_EINVAL, "bc is required with these flags and this configuration");
    }
    const int32_t K = lbm_lattice_d(lattice) + 1;
    cudaStream_t cs = (cudaStream_t)stream;
    const int n_methods = choose_method ? 2 : 1;
    double best = -1.0;
    std::memset(out, 0, sizeof(*out));
    for (int m = 0; m < n_methods; ++m) {
        c.lbm_method = choose_method ? m : cfg->lbm_method;
        for (int i = 0; i < nt; ++i) {
            g.tx = tiles[3 * i];
            g.ty = tiles[3 * i + 1];
            g.tz = tiles[3 * i + 2];
            if (flags) {
                e = relayout<uint8_t>(flags, s.flags, g, 1, cs);
                if (e == cudaSuccess && bc) e = relayout<float>(bc, s.bc, g, K, cs);
                if (e != cudaSuccess) return cuda_fail("relayout", e);
            }
            double sec = 0.0;
            st = time_candidate(c, g, s, steps, cs, &sec);
            if (st != LBM_OK) return st;
            ++out->n_candidates;
            if (best < 0.0 || sec < best) {
                best = sec;
                out->tx = g.tx;
                out->ty = g.ty;
                out->tz = g.tz;
                out->lbm_method = c.lbm_method;
                out->mlups = (float)((double)nx * ny * nz / sec / 1e6);
            }
        }
    }
    return LBM_OK;
}

}  // extern "C"
