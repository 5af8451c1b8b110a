// Wall and shape painting on the device: set_exterior_walls / set_exterior_walls_with_func
// (src/lbm/preprocess/boundary_condition.mojo:78-309) and add_sphere / add_circle / add_box
// (src/lbm/geometry/primatives.mojo:110-240), written into caller-owned device arrays in the grid's
// tiled layout.  The reference paints on the host in loops over the wall or the shape's bounding
// box; here one thread paints one cell.  Shape tests are float32 in the reference's operation
// order (the translation unit is built without contraction), so the painted cells are the
// reference's.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/lbm_gb300.h"

namespace lbm {
__attribute__((visibility("hidden"))) void set_last_error(const char* msg);
}

namespace {

struct PaintLayout {
    int32_t n[3], t[3];  // grid and tile extents
    int32_t ntx, nty;    // tiles along x and y
    int32_t K;           // bc components per cell (D + 1)
};

__device__ __forceinline__ void tiled(const PaintLayout& g, const int32_t (&c)[3], int64_t& loc, int64_t& tile) {
    tile = c[0] / g.t[0] + (int64_t)g.ntx * (c[1] / g.t[1] + (int64_t)g.nty * (c[2] / g.t[2]));
    loc = c[0] % g.t[0] + (int64_t)g.t[0] * (c[1] % g.t[1] + (int64_t)g.t[1] * (c[2] % g.t[2]));
}

// One cell of an exterior face: flag, velocity (u_face: component-major per face cell, or the
// uniform u) and density.  Face cells are ordered by the first free axis fastest.
__global__ void wall_kernel(const PaintLayout g, int32_t axis, int32_t fixed, uint8_t* __restrict__ flags,
                            float* __restrict__ bc, uint8_t type, float u0, float u1, float u2, float rho,
                            const float* __restrict__ u_face, int32_t D, int64_t nface) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nface) return;
    const int32_t a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    int32_t c[3];
    c[axis] = fixed;
    c[a1] = (int32_t)(i % g.n[a1]);
    c[a2] = (int32_t)(i / g.n[a1]);
    int64_t loc, tile;
    tiled(g, c, loc, tile);
    const int64_t T = (int64_t)g.t[0] * g.t[1] * g.t[2];
    flags[loc + T * tile] = type;
    const float u[3] = {u0, u1, u2};
    for (int32_t d = 0; d < D; ++d) bc[loc + T * (d + (int64_t)g.K * tile)] = u_face ? u_face[d * nface + i] : u[d];
    bc[loc + T * (D + (int64_t)g.K * tile)] = rho;
}

// SOLID in every cell of the box lo..hi (exclusive) inside the sphere (box = 0) or the
// axis-aligned box (box = 1).  Coordinates are origin + n * dx in float32.
__global__ void shape_kernel(const PaintLayout g, int32_t lo0, int32_t lo1, int32_t lo2, int32_t e0, int32_t e1,
                             int64_t count, int32_t box, float c0, float c1, float c2, float r0, float r1, float r2,
                             float o0, float o1, float o2, float dx, uint8_t* __restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int32_t c[3];
    c[0] = lo0 + (int32_t)(i % e0);
    c[1] = lo1 + (int32_t)((i / e0) % e1);
    c[2] = lo2 + (int32_t)(i / ((int64_t)e0 * e1));
    const float p[3] = {(float)c[0] * dx + o0, (float)c[1] * dx + o1, (float)c[2] * dx + o2};
    const float ctr[3] = {c0, c1, c2}, rad[3] = {r0, r1, r2};
    bool inside;
    if (!box) {
        // ((coord - center)^2).sum() <= radius^2 (primatives.mojo:178-186; Vector.sum is sequential)
        float s = 0.f;
        for (int k = 0; k < 3; ++k) {
            const float d = p[k] - ctr[k];
            s += d * d;
        }
        inside = s <= rad[0] * rad[0];
    } else {
        // check_box_axis (primatives.mojo:247-266): center - r <= p <= center + r on every axis
        inside = true;
        for (int k = 0; k < 3; ++k) inside = inside && (ctr[k] - rad[k] <= p[k]) && (p[k] <= ctr[k] + rad[k]);
    }
    if (!inside) return;
    int64_t loc, tile;
    tiled(g, c, loc, tile);
    flags[loc + (int64_t)g.t[0] * g.t[1] * g.t[2] * tile] = LBM_FLAG_SOLID;
}

lbm_status pfail(lbm_status s, const char* msg) {
    lbm::set_last_error(msg);
    return s;
}

lbm_status layout_of(const lbm_grid_t* grid, PaintLayout& g) {
    if (!grid) return pfail(LBM_EINVAL, "null grid");
    const int32_t D = lbm_lattice_d(grid->lattice);
    if (D < 0) return pfail(LBM_EINVAL, "lattice must be LBM_D2Q9, LBM_D3Q19 or LBM_D3Q27");
    const int32_t n[3] = {grid->nx, grid->ny, grid->nz}, t[3] = {grid->tx, grid->ty, grid->tz};
    for (int k = 0; k < 3; ++k) {
        if (n[k] <= 0 || t[k] <= 0) return pfail(LBM_EINVAL, "grid and tile extents must be positive");
        if (n[k] % t[k]) return pfail(LBM_EINVAL, "Tile size must divide nx, ny and nz");
        g.n[k] = n[k];
        g.t[k] = t[k];
    }
    g.ntx = n[0] / t[0];
    g.nty = n[1] / t[1];
    g.K = D + 1;
    return LBM_OK;
}

// _error_check (preprocess/boundary_condition.mojo:20-69); u NULL = free velocity.
lbm_status check_wall(const lbm_config_t* cfg, int32_t D, int32_t side, uint8_t type, const float* u, float rho,
                      bool u_known_nonzero) {
    if (!cfg) return pfail(LBM_EINVAL, "null config");
    const bool valid_type = type == LBM_FLAG_FLUID || type == LBM_FLAG_SOLID ||
                            (type == LBM_FLAG_EQUILIBRIUM && cfg->include_equilibrium_bc);
    if (!valid_type) return pfail(LBM_EINVAL, "Input Boundary Type is not in the configuration's INCLUDED_BCs");
    if (side < 0 || side > 5) return pfail(LBM_EINVAL, "Side not valid: expects 0..5 for -X, +X, -Y, +Y, -Z, +Z");
    const bool u_free = u == nullptr && !u_known_nonzero;
    if (u_free && std::isnan(rho))
        return pfail(LBM_EINVAL, "Either velocity or density or both have to be specified. Both cant be left as None");
    bool nonzero = u_known_nonzero;
    if (u) {
        for (int32_t d = 0; d < D; ++d) {
            if (std::isnan(u[d]))
                return pfail(LBM_EINVAL, "either all components of velocity must be free or specified (cannot be NaN)");
            nonzero = nonzero || u[d] != 0.f;
        }
    }
    if (type == LBM_FLAG_SOLID) {
        if (u_free || std::isnan(rho)) return pfail(LBM_EINVAL, "For Solid Type you must specify both u and rho");
        if (!cfg->include_moving_boundary && nonzero)
            return pfail(LBM_EINVAL, "include_moving_boundary in config was set to False but a non zero velocity was "
                                     "specified, Please set config.include_moving_boundary to True First");
    }
    if (type == LBM_FLAG_EQUILIBRIUM && !u_free && std::isnan(rho))
        return pfail(LBM_EINVAL, "For Equilibrium BC, if u is specified then the density must also be specified");
    return LBM_OK;
}

lbm_status launch_wall(const PaintLayout& g, int32_t D, int32_t side, uint8_t* flags, float* bc, uint8_t type,
                       const float* u, float rho, const float* u_face, cudaStream_t s) {
    if (!flags || !bc) return pfail(LBM_EINVAL, "null flags or bc");
    const int32_t axis = side / 2;
    const int32_t fixed = (side % 2 == 0) ? 0 : g.n[axis] - 1;
    const int32_t a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    const int64_t nface = (int64_t)g.n[a1] * g.n[a2];
    const float nan = std::nanf("");
    float uu[3] = {nan, nan, nan};
    if (u)
        for (int32_t d = 0; d < D; ++d) uu[d] = u[d];
    wall_kernel<<<(unsigned)((nface + 255) / 256), 256, 0, s>>>(g, axis, fixed, flags, bc, type, uu[0], uu[1], uu[2],
                                                                 rho, u_face, D, nface);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        static thread_local char buf[160];
        std::snprintf(buf, sizeof(buf), "wall painting: %s", cudaGetErrorString(e));
        return pfail(LBM_ECUDA, buf);
    }
    return LBM_OK;
}

// The reference's bounding box along one axis (primatives.mojo:133-138): [max(0, floor((lo -
// origin) / dx)), min(n, floor((hi - origin) / dx) + 1)), float32 arithmetic; [0, 1) beyond D.
void bbox_axis(float center, float r, float origin, float dx, int32_t n, bool active, int32_t& lo, int32_t& hi) {
    if (!active) {
        lo = 0;
        hi = 1;
        return;
    }
    const float a_min = center - r, a_max = center + r;
    const float fmin = std::floor((a_min - origin) / dx), fmax = std::floor((a_max - origin) / dx) + 1.0f;
    lo = fmin > 0.f ? (fmin < (float)n ? (int32_t)fmin : n) : 0;
    hi = fmax < (float)n ? (fmax > 0.f ? (int32_t)fmax : 0) : n;
}

lbm_status paint_shape(const lbm_grid_t* grid, uint8_t* flags, const float center[3], const float rad[3], bool box,
                       const float origin[3], float dx, cudaStream_t s) {
    PaintLayout g;
    lbm_status st = layout_of(grid, g);
    if (st != LBM_OK) return st;
    if (!flags || !center || !rad || !origin) return pfail(LBM_EINVAL, "null argument");
    if (!(dx > 0.f) || !std::isfinite(dx)) return pfail(LBM_EINVAL, "dx must be a positive number");
    const int32_t D = lbm_lattice_d(grid->lattice);
    int32_t lo[3], hi[3];
    for (int k = 0; k < 3; ++k) bbox_axis(center[k], rad[k], origin[k], dx, g.n[k], k < D, lo[k], hi[k]);
    const int32_t e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
    if (e0 <= 0 || e1 <= 0 || e2 <= 0) return LBM_OK;  // the box misses the grid
    const int64_t count = (int64_t)e0 * e1 * e2;
    shape_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(g, lo[0], lo[1], lo[2], e0, e1, count, box ? 1 : 0,
                                                                  center[0], center[1], center[2], rad[0], rad[1],
                                                                  rad[2], origin[0], origin[1], origin[2], dx, flags);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        static thread_local char buf[160];
        std::snprintf(buf, sizeof(buf), "shape painting: %s", cudaGetErrorString(e));
        return pfail(LBM_ECUDA, buf);
    }
    return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_paint_wall(const lbm_config_t* cfg, const lbm_grid_t* grid, uint8_t* flags, float* bc, int32_t side,
                          uint8_t boundary_type, const float* u, float rho, void* stream) {
    PaintLayout g;
    lbm_status st = layout_of(grid, g);
    if (st != LBM_OK) return st;
    const int32_t D = g.K - 1;
    st = check_wall(cfg, D, side, boundary_type, u, rho, false);
    if (st != LBM_OK) return st;
    return launch_wall(g, D, side, flags, bc, boundary_type, u, rho, nullptr, (cudaStream_t)stream);
}

lbm_status lbm_paint_wall_values(const lbm_config_t* cfg, const lbm_grid_t* grid, uint8_t* flags, float* bc,
                                 int32_t side, uint8_t boundary_type, const float* u_face, float rho, void* stream) {
    PaintLayout g;
    lbm_status st = layout_of(grid, g);
    if (st != LBM_OK) return st;
    if (!u_face) return pfail(LBM_EINVAL, "null u_face");
    // set_exterior_walls_with_func checks with a velocity of ones (boundary_condition.mojo:250-251)
    const int32_t D = g.K - 1;
    st = check_wall(cfg, D, side, boundary_type, nullptr, rho, true);
    if (st != LBM_OK) return st;
    return launch_wall(g, D, side, flags, bc, boundary_type, nullptr, rho, u_face, (cudaStream_t)stream);
}

lbm_status lbm_paint_sphere(const lbm_grid_t* grid, uint8_t* flags, const float center[3], float radius,
                            const float origin[3], float dx, void* stream) {
    const float r[3] = {radius, radius, radius};
    return paint_shape(grid, flags, center, r, false, origin, dx, (cudaStream_t)stream);
}

lbm_status lbm_paint_box(const lbm_grid_t* grid, uint8_t* flags, const float center[3], const float half[3],
                         const float origin[3], float dx, void* stream) {
    if (!half) return pfail(LBM_EINVAL, "null argument");
    return paint_shape(grid, flags, center, half, true, origin, dx, (cudaStream_t)stream);
}

}  // extern "C"
