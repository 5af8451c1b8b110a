// C ABI of the GB300 LBM step (include/lbm_gb300.h): configuration checks, handles, dispatch to
// the per-lattice kernel tables, the graph-replayed time loop, and the auxiliary kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "lbm_aux.cuh"
#include "lbm_link_tables.h"
#include "lbm_stage.cuh"

namespace lbm {
StepLaunch get_step_d2q9(int, int, int, int);
StepLaunch get_step_d3q19(int, int, int, int);
StepLaunch get_step_d3q27(int, int, int, int);
StepLaunch get_tile_step_d2q9(int, int, int, int);
StepLaunch get_tile_step_d3q19(int, int, int, int);
StepLaunch get_tile_step_d3q27(int, int, int, int);
StepLaunch get_fast_tile_step_d2q9(int, int, int, int);
StepLaunch get_fast_tile_step_d3q19(int, int, int, int);
StepLaunch get_fast_tile_step_d3q27(int, int, int, int);
StepLaunch get_pair_step_d2q9(int, int, int, int);
StepLaunch get_pair_step_d3q19(int, int, int, int);
StepLaunch get_pair_step_d3q27(int, int, int, int);
StepLaunch get_links_tile_step_d2q9(int, int, int, int);
StepLaunch get_staged_step_d2q9(int, int, int, int);
StepLaunch get_staged_step_d3q19(int, int, int, int);
StepLaunch get_staged_step_d3q27(int, int, int, int);
std::vector<StageSeg> build_stage_segments(int lattice, int tx, int ty, int tz, int esz, uint32_t* stage_bytes);
StepLaunch get_links_tile_step_d3q19(int, int, int, int);
StepLaunch get_links_tile_step_d3q27(int, int, int, int);
StepLaunch get_learned_step_d2q9(int, int, int);
StepLaunch get_learned_step_d3q19(int, int, int);
StepLaunch get_learned_step_d3q27(int, int, int);
void pack_closure(const lbm_closure_t& c, ClosureDev& d, ClosureUniform& u);
}  // namespace lbm

using namespace lbm;

namespace {

// box_sum: the summary byte of every warp box (the 32 cells of one warp of a tile), recomputed only
// for the boxes whose flags differ from flags_seen (the flags of the previous summary; every box
// when force), which takes the new flags.  A recomputed box sets *changed = gen.  One thread per box.
__global__ void __launch_bounds__(256) box_summary_kernel(const uint8_t* __restrict__ flags,
                                                          uint8_t* __restrict__ flags_seen, const LayoutDesc l,
                                                          uint8_t* __restrict__ box_sum, uint32_t* changed,
                                                          uint32_t gen, int force) {
    const uint32_t box = blockIdx.x * blockDim.x + threadIdx.x;
    if (box < l.ncells / 32u) update_box_summary(flags, box, flags_seen, box_sum, l, changed, gen, force);
}

// tile_near: per tile, bit w = warp_near of its warp box w; one thread per warp box.  Skipped
// (every thread returns) unless a box summary changed in this round (*changed == gen).
__global__ void __launch_bounds__(256) tile_near_kernel(const uint8_t* __restrict__ box_sum, const LayoutDesc l,
                                                        uint32_t nboxes, uint8_t* __restrict__ tile_near,
                                                        const uint32_t* changed, uint32_t gen) {
    if (*changed != gen) return;  // the same value for every thread
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t bit = i < nboxes ? warp_near(box_sum, l, i / kTileWarps, i % kTileWarps) : 0u;
    write_near_mask(i, nboxes, bit, tile_near);
}

// The neighbour-solid masks of every cell in a warp with its mask bit set (256 threads per tile,
// blocks striding over the tiles: a launch with nothing to do is one short wave), after a change of
// the flags in this round (*changed == gen).
template <class L>
__global__ void __launch_bounds__(256) cell_mask_kernel(const StepArgs a, uint2* __restrict__ masks,
                                                        const uint32_t* changed, uint32_t gen, uint32_t ntiles) {
    if (*changed != gen) return;  // the same value for every thread
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) tile_cell_masks<L>(a, tile, masks);
}

thread_local std::string g_err;

lbm_status fail(lbm_status s, const std::string& msg) {
    g_err = msg;
    return s;
}

#define LBM_CK(call)                                                                          \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(LBM_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
    } while (0)

int lattice_q(int id) { return id == LBM_D2Q9 ? 9 : id == LBM_D3Q19 ? 19 : id == LBM_D3Q27 ? 27 : -1; }
int lattice_d(int id) { return id == LBM_D2Q9 ? 2 : (id == LBM_D3Q19 || id == LBM_D3Q27) ? 3 : -1; }

// Graph cache key for lbm_run: buffers, tau bits, parity of the first step, chunk length.
using GraphKey = std::tuple<const void*, const void*, const void*, const void*, uint32_t, int, int64_t, int>;

}  // namespace

namespace lbm {
// Sets the message lbm_last_error() returns, for entry points defined in other files.
__attribute__((visibility("hidden"))) void set_last_error(const char* msg) { g_err = msg; }
}  // namespace lbm

struct lbm_handle {
    lbm_config_t cfg;
    lbm_grid_t grid;
    LayoutDesc lay;
    StepLaunch step;       // generic kernel (any tile)
    StepLaunch step_tile;  // block-per-tile kernel, or null when the grid does not qualify
    StepLaunch step_learned;  // block-per-tile kernel with the learned closure (LES handles), or null
    StepLaunch step_pair;  // cell-pair block-per-tile kernel (double buffer, tx >= 2), or null
    int pair_auto;         // the automatic choice takes the cell-pair kernel
    StepLaunch step_links;    // block-per-tile kernel with fused links (double buffer), or null
    StepLaunch step_staged;   // staged block-per-tile kernel (double buffer, 16-byte tile rows), or null
    int path;              // 0 auto, 1 generic only, 2 block-per-tile only, 3 cell-pair, 4 staged
    StageSeg* stage_segs;  // the staged kernel's copy segments (device), or null
    uint32_t nsegs, stage_bytes, stage_extra;
    uint32_t* dev_err;     // device word raised by the staged kernel's bounded waits
    uint8_t* box_sum;      // per warp box (32 cells): summary byte (flags other than 0 inside, on faces)
    uint2* cell_masks;     // per cell: neighbour-solid masks, written for the warps with a mask bit set
    uint8_t* flags_seen;   // the flags the summary was built from
    uint32_t* changed;     // device word: summary round in which a box summary last changed
    uint32_t summary_gen;  // summary rounds issued
    int summary_valid;     // box_sum and flags_seen hold a complete summary
    uint8_t* tile_near;    // per tile: warp_near bits of its 8 warp boxes (block-per-tile kernel)
    uint32_t ntiles;
    uint32_t mx, my, shx, shxy;
    int threads;
    int device;
    int sm_count;
    double* scratch;  // kReduceBlocks*4 partials + 4 results
    ClosureDev* closure;  // device copy of the learned closure's fragments, or null
    ClosureUniform closure_uniform;
    int closure_on;
    cudaStream_t capture_stream;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    // interpolated bounce-back fused into the step (lbm_set_links)
    uint2* link_table;     // per cell, or null
    float* link_dist;
    int32_t* link_id;
    float* link_force;     // caller's, or null
    int64_t n_links;
    float q_clamp;
    int bouzidi;
};

namespace lbm {

// The layout descriptor of a grid (shared with the allocation-free reduction, lbm_noalloc.cu).
__attribute__((visibility("hidden"))) LayoutDesc make_layout(const lbm_grid_t& g) {
    LayoutDesc l;
    l.nx = g.nx; l.ny = g.ny; l.nz = g.nz;
    l.tx = g.tx; l.ty = g.ty; l.tz = g.tz;
    l.ntx = g.nx / g.tx; l.nty = g.ny / g.ty; l.ntz = g.nz / g.tz;
    l.T = (uint32_t)(g.tx * g.ty * g.tz);
    l.ncells = (uint32_t)((int64_t)g.nx * g.ny * g.nz);
    l.d_tx = FastDiv((uint32_t)g.tx);
    l.d_ty = FastDiv((uint32_t)g.ty);
    l.d_T = FastDiv(l.T);
    l.d_ntx = FastDiv((uint32_t)l.ntx);
    l.d_nty = FastDiv((uint32_t)l.nty);
    return l;
}

}  // namespace lbm

namespace {

StepArgs step_args(const lbm_handle* h, const void* f_in, void* f_out, float* bc, const uint8_t* flags, float tau,
                   int even) {
    StepArgs a;
    a.lay = h->lay;
    a.f_in = f_in;
    a.f_out = f_out;
    a.bc = bc;
    a.flags = flags;
    a.tau = tau;
    a.inv_tau = 1.f / tau;  // IEEE float32 quotient, as the kernel would compute it
    a.Cs = h->cfg.Cs;
    a.trt_lambda = h->cfg.trt_lambda;
    a.ddf = h->cfg.DDF_shift;
    a.moving = h->cfg.include_moving_boundary;
    a.eqbc = h->cfg.include_equilibrium_bc;
    a.cap_rho = h->cfg.capture_density;
    a.cap_u = h->cfg.capture_velocity;
    a.even = even;
    a.closure = h->closure_on ? h->closure : nullptr;
    a.cl = h->closure_uniform;
    a.tile_near = h->tile_near;
    a.cell_masks = h->cell_masks;
    a.mx = h->mx;
    a.my = h->my;
    a.shx = h->shx;
    a.shxy = h->shxy;
    a.link_table = h->link_table;
    a.link_dist = h->link_dist;
    a.link_id = h->link_id;
    a.link_force = h->link_force;
    a.link_stride = h->n_links;
    a.q_clamp = h->q_clamp;
    a.bouzidi = h->bouzidi;
    a.stage_segs = h->stage_segs;
    a.nsegs = h->nsegs;
    a.stage_bytes = h->stage_bytes;
    a.err = h->dev_err;
    a.stage_extra = h->stage_extra;
    return a;
}

bool use_tile(const lbm_handle* h) { return h->step_tile != nullptr && h->path != 1; }

// Two waves of the cell-pair kernel's CTAs (8 per SM) on the 152 SMs of a GB300.
constexpr uint32_t kPairAutoMinTiles = 2u * 8u * 152u;

// The staged kernel is chosen (path 4) and can run: no learned closure, no fused links.
bool use_staged(const lbm_handle* h) {
    return h->path == 4 && h->step_staged != nullptr && !h->closure_on && !h->link_table;
}

// The cell-pair kernel is chosen (path 3) and can run: no learned closure, no fused links.
// The automatic choice (path 0) takes it where it measured faster than the per-cell kernel: the
// double-buffer D2Q9 / D3Q19 configurations other than KBC (whose larger register demand halves the
// pair kernel's occupancy) on grids of at least kPairAutoMinTiles tiles.  On fewer tiles the step
// is latency-bound, and the per-cell kernel, which gives each pair two threads, finishes sooner
// (the 256^2 D2Q9 cavity, 256 tiles: 3.2 against 4.3 us a step).
bool use_pair(const lbm_handle* h) {
    return (h->path == 3 || (h->path == 0 && h->pair_auto)) && h->step_pair != nullptr && !h->closure_on &&
           !h->link_table;
}

// The kernel the next step with these arguments runs.  The cell-pair kernel moves 8-byte
// (float32) or 4-byte (Float16C) words, so it needs 8-byte aligned population buffers; others
// take the per-cell block-per-tile kernel.
StepLaunch step_fn(const lbm_handle* h, const StepArgs& a) {
    if (!use_tile(h)) return h->step;
    if (h->closure_on) return h->step_learned;
    if (h->link_table) return h->step_links;
    const uintptr_t al = reinterpret_cast<uintptr_t>(a.f_in) | reinterpret_cast<uintptr_t>(a.f_out);
    if (use_staged(h) && (al & 15u) == 0u) return h->step_staged;  // bulk copies: 16-byte aligned rows
    if (use_pair(h) && ((reinterpret_cast<uintptr_t>(a.f_in) | reinterpret_cast<uintptr_t>(a.f_out)) & 7u) == 0u)
        return h->step_pair;
    return h->step_tile;
}

// Brings the per-tile warp masks of the block-per-tile kernel up to date with `flags`: the boxes
// whose flags changed since the previous call are summarised again, and the masks are rebuilt
// only if one did (every step of a run with fixed flags costs one pass over the flags).
lbm_status tile_summary(lbm_handle* h, const uint8_t* flags, cudaStream_t s) {
    if (++h->summary_gen == 0u) ++h->summary_gen;  // 0 is the initial value of *changed
    const uint32_t gen = h->summary_gen;
    const uint32_t nboxes = h->ntiles * kTileWarps;
    box_summary_kernel<<<(nboxes + 255u) / 256u, 256, 0, s>>>(flags, h->flags_seen, h->lay, h->box_sum, h->changed,
                                                              gen, h->summary_valid ? 0 : 1);
    LBM_CK(cudaGetLastError());
    h->summary_valid = 1;
    tile_near_kernel<<<(nboxes + 255u) / 256u, 256, 0, s>>>(h->box_sum, h->lay, nboxes, h->tile_near, h->changed,
                                                             gen);
    LBM_CK(cudaGetLastError());
    const StepArgs a = step_args(h, nullptr, nullptr, nullptr, flags, 1.f, 0);
    const uint32_t grid = std::min<uint32_t>(h->ntiles, (uint32_t)h->sm_count * 8u);
    switch (h->grid.lattice) {
        case LBM_D2Q9: cell_mask_kernel<D2Q9><<<grid, kTileCells, 0, s>>>(a, h->cell_masks, h->changed, gen, h->ntiles); break;
        case LBM_D3Q19: cell_mask_kernel<D3Q19><<<grid, kTileCells, 0, s>>>(a, h->cell_masks, h->changed, gen, h->ntiles); break;
        default: cell_mask_kernel<D3Q27><<<grid, kTileCells, 0, s>>>(a, h->cell_masks, h->changed, gen, h->ntiles); break;
    }
    LBM_CK(cudaGetLastError());
    return LBM_OK;
}

uint32_t blocks_for(uint32_t n, int threads) { return (n + (uint32_t)threads - 1u) / (uint32_t)threads; }

lbm_status check_handle(const lbm_handle* h) {
    if (!h) return fail(LBM_EINVAL, "null handle");
    return LBM_OK;
}

// One step.  with_summary: rebuild the tile summary from `flags` first (single-step calls; a
// multi-step run builds it once, since flags cannot change inside the run).
lbm_status step_once(lbm_handle* h, const void* f_in, void* f_out, float* bc, const uint8_t* flags, float tau,
                     int even, cudaStream_t s, bool with_summary = true) {
    const StepArgs a = step_args(h, f_in, f_out, bc, flags, tau, even);
    if (use_tile(h)) {
        if (with_summary) {
            const lbm_status st = tile_summary(h, flags, s);
            if (st != LBM_OK) return st;
        }
    }
    LBM_CK(step_fn(h, a)(a, h->threads, s));
    return LBM_OK;
}

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
int ilog2(int v) { int r = 0; while ((1 << r) < v) ++r; return r; }

template <class F>
lbm_status dispatch_lattice(int lattice, F&& f) {
    switch (lattice) {
        case LBM_D2Q9: return f(D2Q9{});
        case LBM_D3Q19: return f(D3Q19{});
        case LBM_D3Q27: return f(D3Q27{});
    }
    return fail(LBM_EINVAL, "unknown lattice");
}

}  // namespace

extern "C" {

const char* lbm_last_error(void) { return g_err.c_str(); }

const char* lbm_version(void) { return "mojo_lbm_gb300 0.1 (sm_103a)"; }

int32_t lbm_lattice_q(int32_t lattice) { return lattice_q(lattice); }
int32_t lbm_lattice_d(int32_t lattice) { return lattice_d(lattice); }

int64_t lbm_f_elements(const lbm_grid_t* g) {
    return g ? (int64_t)lattice_q(g->lattice) * g->nx * g->ny * g->nz : -1;
}
int64_t lbm_bc_elements(const lbm_grid_t* g) {
    return g ? (int64_t)(lattice_d(g->lattice) + 1) * g->nx * g->ny * g->nz : -1;
}
int64_t lbm_flag_elements(const lbm_grid_t* g) { return g ? (int64_t)g->nx * g->ny * g->nz : -1; }

lbm_status lbm_config_default(lbm_config_t* cfg, int32_t lbm_method) {
    if (!cfg) return fail(LBM_EINVAL, "null config");
    if (lbm_method != LBM_DOUBLE_BUFFER && lbm_method != LBM_ESOTERIC_PULL)
        return fail(LBM_EINVAL, "lbm_method must be LBM_DOUBLE_BUFFER or LBM_ESOTERIC_PULL");
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->lbm_method = lbm_method;
    cfg->collision_op = LBM_SRT;
    cfg->include_moving_boundary = 1;
    cfg->Cs = 0.1f;
    cfg->trt_lambda = 3.0f / 16.0f;
    return LBM_OK;
}

lbm_status lbm_validate(const lbm_config_t* c, const lbm_grid_t* g) {
    if (!c || !g) return fail(LBM_EINVAL, "null config or grid");
    if (c->lbm_method != LBM_DOUBLE_BUFFER && c->lbm_method != LBM_ESOTERIC_PULL)
        return fail(LBM_EINVAL, "lbm_method not valid");
    /* Collisions.valid_set (constants.mojo:53) */
    if (c->collision_op < LBM_SRT || c->collision_op > LBM_RLBM)
        return fail(LBM_EINVAL, "Invalid Collision Operator specified: must be SRT, TRT, KBC or RLBM");
    const int D = lattice_d(g->lattice);
    if (D < 0) return fail(LBM_EINVAL, "lattice must be LBM_D2Q9, LBM_D3Q19 or LBM_D3Q27");
    if (g->nx <= 0 || g->ny <= 0 || g->nz <= 0) return fail(LBM_EINVAL, "grid extents must be positive");
    /* check_model_match_dim (grid.mojo:345-365) */
    const int gridD = (g->nx > 1) + (g->ny > 1) + (g->nz > 1);
    if (gridD != D)
        return fail(LBM_EINVAL,
                    "The given dimension of the Lattice does not match that of the dimension of the grid");
    if (g->tx <= 0 || g->ty <= 0 || g->tz <= 0) return fail(LBM_EINVAL, "tile extents must be positive");
    /* set_block_shape_and_grid_dim / set_grid_dims (grid.mojo:301-305,434-438) */
    if (g->nx % g->tx || g->ny % g->ty || g->nz % g->tz)
        return fail(LBM_EINVAL, "Tile size must divide nx, ny and nz");
    const int64_t N = (int64_t)g->nx * g->ny * g->nz;
    if (N >= (int64_t)1 << 32) return fail(LBM_EINVAL, "grid has 2^32 or more cells");
    if (c->LES && !(c->Cs == c->Cs)) return fail(LBM_EINVAL, "Cs is NaN");
    if (c->LES && !(c->Cs >= 0.0f)) return fail(LBM_EINVAL, "Cs must be non-negative");
    if (c->arithmetic != LBM_ARITH_EXACT && c->arithmetic != LBM_ARITH_FAST)
        return fail(LBM_EINVAL, "arithmetic must be LBM_ARITH_EXACT or LBM_ARITH_FAST");
    return LBM_OK;
}

lbm_status lbm_create(const lbm_config_t* cfg, const lbm_grid_t* grid, lbm_handle** out) {
    if (!out) return fail(LBM_EINVAL, "null output handle pointer");
    *out = nullptr;
    lbm_status s = lbm_validate(cfg, grid);
    if (s != LBM_OK) return s;
    lbm_handle* h = new lbm_handle();
    h->cfg = *cfg;
    h->grid = *grid;
    h->lay = make_layout(*grid);
    const int m = cfg->lbm_method, f16 = cfg->use_float16c ? 1 : 0, co = cfg->collision_op, les = cfg->LES ? 1 : 0;
    h->step = grid->lattice == LBM_D2Q9 ? get_step_d2q9(m, f16, co, les)
            : grid->lattice == LBM_D3Q19 ? get_step_d3q19(m, f16, co, les)
                                         : get_step_d3q27(m, f16, co, les);
    // block-per-tile kernel: 256-cell tiles with power-of-two sides and 32-bit offsets
    const int64_t Q = lattice_q(grid->lattice);
    const bool tile_ok = (int64_t)grid->tx * grid->ty * grid->tz == (int64_t)kTileCells && pow2(grid->tx) &&
                         pow2(grid->ty) && pow2(grid->tz) && Q * h->lay.ncells < ((int64_t)1 << 31);
    const bool fast = cfg->arithmetic == LBM_ARITH_FAST;
    h->step_tile = !tile_ok ? nullptr
                 : fast ? (grid->lattice == LBM_D2Q9 ? get_fast_tile_step_d2q9(m, f16, co, les)
                           : grid->lattice == LBM_D3Q19 ? get_fast_tile_step_d3q19(m, f16, co, les)
                                                        : get_fast_tile_step_d3q27(m, f16, co, les))
                 : grid->lattice == LBM_D2Q9 ? get_tile_step_d2q9(m, f16, co, les)
                 : grid->lattice == LBM_D3Q19 ? get_tile_step_d3q19(m, f16, co, les)
                                              : get_tile_step_d3q27(m, f16, co, les);
    h->step_learned = !(tile_ok && les) ? nullptr
                    : grid->lattice == LBM_D2Q9 ? get_learned_step_d2q9(m, f16, co)
                    : grid->lattice == LBM_D3Q19 ? get_learned_step_d3q19(m, f16, co)
                                                 : get_learned_step_d3q27(m, f16, co);
    h->step_pair = !(tile_ok && m == LBM_DOUBLE_BUFFER && grid->tx >= 2) ? nullptr
                 : grid->lattice == LBM_D2Q9 ? get_pair_step_d2q9(f16, co, les, fast)
                 : grid->lattice == LBM_D3Q19 ? get_pair_step_d3q19(f16, co, les, fast)
                                              : get_pair_step_d3q27(f16, co, les, fast);
    h->step_links = !(tile_ok && m == LBM_DOUBLE_BUFFER) ? nullptr
                  : grid->lattice == LBM_D2Q9 ? get_links_tile_step_d2q9(f16, co, les, fast)
                  : grid->lattice == LBM_D3Q19 ? get_links_tile_step_d3q19(f16, co, les, fast)
                                               : get_links_tile_step_d3q27(f16, co, les, fast);
    const int esz = f16 ? 2 : 4;
    std::vector<StageSeg> segs;
    h->stage_bytes = 0;
    if (tile_ok && m == LBM_DOUBLE_BUFFER)
        segs = build_stage_segments(grid->lattice, grid->tx, grid->ty, grid->tz, esz, &h->stage_bytes);
    h->nsegs = (uint32_t)segs.size();
    h->stage_extra = 0;
    h->stage_segs = nullptr;
    h->dev_err = nullptr;
    h->step_staged = segs.empty() ? nullptr
                   : grid->lattice == LBM_D2Q9 ? get_staged_step_d2q9(f16, co, les, fast)
                   : grid->lattice == LBM_D3Q19 ? get_staged_step_d3q19(f16, co, les, fast)
                                                : get_staged_step_d3q27(f16, co, les, fast);
    h->pair_auto = h->step_pair != nullptr && co != LBM_KBC && grid->lattice != LBM_D3Q27 &&
                   h->lay.ncells / h->lay.T >= kPairAutoMinTiles;
    h->path = 0;
    h->ntiles = h->lay.ncells / h->lay.T;
    h->mx = (uint32_t)grid->tx - 1u;
    h->my = (uint32_t)grid->ty - 1u;
    h->shx = (uint32_t)ilog2(grid->tx);
    h->shxy = (uint32_t)(ilog2(grid->tx) + ilog2(grid->ty));
    h->box_sum = nullptr;
    h->cell_masks = nullptr;
    h->flags_seen = nullptr;
    h->changed = nullptr;
    h->summary_gen = 0;
    h->summary_valid = 0;
    h->tile_near = nullptr;
    h->threads = 256;
    h->scratch = nullptr;
    h->closure = nullptr;
    std::memset(&h->closure_uniform, 0, sizeof(h->closure_uniform));
    h->closure_on = 0;
    h->capture_stream = nullptr;
    h->link_table = nullptr;
    h->link_dist = nullptr;
    h->link_id = nullptr;
    h->link_force = nullptr;
    h->n_links = 0;
    h->q_clamp = 0.f;
    h->bouzidi = 0;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device);
    if (e == cudaSuccess) e = cudaMalloc(&h->scratch, sizeof(double) * (kReduceBlocks * kReduceWidth + 8));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->capture_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess && h->step_tile) e = cudaMalloc(&h->box_sum, (size_t)h->ntiles * kTileWarps);
    if (e == cudaSuccess && h->step_tile) e = cudaMalloc(&h->flags_seen, (size_t)h->lay.ncells);
    if (e == cudaSuccess && h->step_tile) e = cudaMalloc(&h->cell_masks, sizeof(uint2) * (size_t)h->lay.ncells);
    if (e == cudaSuccess && h->step_tile) e = cudaMalloc(&h->changed, sizeof(uint32_t));
    if (e == cudaSuccess && h->step_tile) e = cudaMemset(h->changed, 0, sizeof(uint32_t));
    if (e == cudaSuccess && h->step_tile) e = cudaMalloc(&h->tile_near, h->ntiles);
    if (e == cudaSuccess) e = cudaMalloc(&h->dev_err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(h->dev_err, 0, sizeof(uint32_t));
    if (e == cudaSuccess && !segs.empty()) e = cudaMalloc(&h->stage_segs, sizeof(StageSeg) * segs.size());
    if (e == cudaSuccess && !segs.empty())
        e = cudaMemcpy(h->stage_segs, segs.data(), sizeof(StageSeg) * segs.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        lbm_destroy(h);
        return fail(LBM_ECUDA, std::string("lbm_create: ") + cudaGetErrorString(e));
    }
    *out = h;
    return LBM_OK;
}

lbm_status lbm_destroy(lbm_handle* h) {
    if (!h) return LBM_OK;
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    if (h->scratch) cudaFree(h->scratch);
    if (h->box_sum) cudaFree(h->box_sum);
    if (h->flags_seen) cudaFree(h->flags_seen);
    if (h->cell_masks) cudaFree(h->cell_masks);
    if (h->changed) cudaFree(h->changed);
    if (h->tile_near) cudaFree(h->tile_near);
    if (h->closure) cudaFree(h->closure);
    if (h->link_table) cudaFree(h->link_table);
    if (h->link_dist) cudaFree(h->link_dist);
    if (h->link_id) cudaFree(h->link_id);
    if (h->stage_segs) cudaFree(h->stage_segs);
    if (h->dev_err) cudaFree(h->dev_err);
    if (h->capture_stream) cudaStreamDestroy(h->capture_stream);
    delete h;
    return LBM_OK;
}

lbm_status lbm_set_links(lbm_handle* h, const int32_t* fluid_ids, const int32_t* dirs, const float* dists,
                         int64_t n_links, int32_t method, float q_clamp, float* link_force, void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (n_links < 0 || n_links >= ((int64_t)1 << 31)) return fail(LBM_EINVAL, "n_links must be in [0, 2^31)");
    if (n_links > 0 && h->cfg.lbm_method != LBM_DOUBLE_BUFFER)
        return fail(LBM_EUNSUPPORTED, "interpolated bounce-back needs the double-buffer method");
    if (method != LBM_BB_MID_GRID && method != LBM_BB_BOUZIDI) return fail(LBM_EINVAL, "unknown bounce-back method");
    if (n_links > 0 && (!h->step_links || h->path == 1))
        return fail(LBM_EUNSUPPORTED, "links fused into the step need the block-per-tile kernel: 256-cell "
                                      "power-of-two tiles, Q*N < 2^31, kernel path not forced to generic");
    if (n_links > 0 && h->closure_on)
        return fail(LBM_EUNSUPPORTED, "links fused into the step and the learned closure are not built together");
    if (n_links > 0 && (!fluid_ids || !dirs || !dists)) return fail(LBM_EINVAL, "null link array");
    cudaStream_t s = (cudaStream_t)stream;
    LinkTables lt;
    if (n_links > 0) {
        std::vector<int32_t> ids(n_links), dv(n_links);
        std::vector<float> qv(n_links);
        LBM_CK(cudaMemcpyAsync(ids.data(), fluid_ids, sizeof(int32_t) * n_links, cudaMemcpyDeviceToHost, s));
        LBM_CK(cudaMemcpyAsync(dv.data(), dirs, sizeof(int32_t) * n_links, cudaMemcpyDeviceToHost, s));
        LBM_CK(cudaMemcpyAsync(qv.data(), dists, sizeof(float) * n_links, cudaMemcpyDeviceToHost, s));
        LBM_CK(cudaStreamSynchronize(s));
        const std::string err = build_link_tables(h->lay.ncells, lattice_q(h->grid.lattice), n_links, nullptr, nullptr,
                                                  nullptr, 1, ids.data(), dv.data(), qv.data(), lt);
        if (!err.empty()) return fail(LBM_EINVAL, "lbm_set_links: " + err);
    }
    // steps in flight may read the current tables; cached graphs hold the old arguments
    LBM_CK(cudaDeviceSynchronize());
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    if (h->link_table) cudaFree(h->link_table);
    if (h->link_dist) cudaFree(h->link_dist);
    if (h->link_id) cudaFree(h->link_id);
    h->link_table = nullptr;
    h->link_dist = nullptr;
    h->link_id = nullptr;
    h->link_force = nullptr;
    h->n_links = 0;
    if (n_links == 0) return LBM_OK;
    LBM_CK(cudaMalloc(&h->link_table, sizeof(uint2) * lt.table.size()));
    LBM_CK(cudaMalloc(&h->link_dist, sizeof(float) * n_links));
    LBM_CK(cudaMalloc(&h->link_id, sizeof(int32_t) * n_links));
    LBM_CK(cudaMemcpy(h->link_table, lt.table.data(), sizeof(uint2) * lt.table.size(), cudaMemcpyHostToDevice));
    LBM_CK(cudaMemcpy(h->link_dist, lt.dist.data(), sizeof(float) * n_links, cudaMemcpyHostToDevice));
    LBM_CK(cudaMemcpy(h->link_id, lt.id.data(), sizeof(int32_t) * n_links, cudaMemcpyHostToDevice));
    h->link_force = link_force;
    h->n_links = n_links;
    h->q_clamp = q_clamp;
    h->bouzidi = method == LBM_BB_BOUZIDI;
    return LBM_OK;
}

lbm_status lbm_set_closure(lbm_handle* h, const lbm_closure_t* closure) {
    if (check_handle(h)) return LBM_EINVAL;
    if (closure && !h->cfg.LES)
        return fail(LBM_EUNSUPPORTED, "the learned closure replaces Smagorinsky: the configuration needs LES");
    if (closure && h->link_table)
        return fail(LBM_EUNSUPPORTED, "links fused into the step and the learned closure are not built together");
    if (closure && (!h->step_learned || h->path == 1))
        return fail(LBM_EUNSUPPORTED, "the learned closure runs in the block-per-tile kernel: 256-cell "
                                      "power-of-two tiles, Q*N < 2^31, kernel path not forced to generic");
    if (closure) {
        const float* p = reinterpret_cast<const float*>(closure);
        for (size_t i = 0; i < sizeof(lbm_closure_t) / sizeof(float); ++i)
            if (!std::isfinite(p[i])) return fail(LBM_EINVAL, "closure parameters must be finite");
        if (!(closure->nu_scale >= 0.f)) return fail(LBM_EINVAL, "nu_scale must be non-negative");
    }
    // steps in flight may read the current fragments; graphs hold the old descriptor
    LBM_CK(cudaDeviceSynchronize());
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    if (!closure) {
        h->closure_on = 0;
        return LBM_OK;
    }
    ClosureDev d;
    pack_closure(*closure, d, h->closure_uniform);
    if (!h->closure) LBM_CK(cudaMalloc(&h->closure, sizeof(ClosureDev)));
    LBM_CK(cudaMemcpy(h->closure, &d, sizeof(ClosureDev), cudaMemcpyHostToDevice));
    h->closure_on = 1;
    return LBM_OK;
}

lbm_status lbm_set_block_threads(lbm_handle* h, int32_t threads) {
    if (check_handle(h)) return LBM_EINVAL;
    if (threads == 0) threads = 256;
    if (threads < 32 || threads > 256 || threads % 32)
        return fail(LBM_EINVAL, "threads per block must be a multiple of 32 in [32, 256]");
    h->threads = threads;
    return LBM_OK;
}

lbm_status lbm_set_kernel_path(lbm_handle* h, int32_t path) {
    if (check_handle(h)) return LBM_EINVAL;
    if (path < 0 || path > 4)
        return fail(LBM_EINVAL, "path must be 0 (auto), 1 (generic), 2 (block-per-tile), 3 (cell-pair) or 4 (staged)");
    if (path == 4 && !h->step_staged)
        return fail(LBM_EUNSUPPORTED, "the staged kernel needs the double-buffer method, 256-cell power-of-two tiles "
                                      "whose rows are multiples of 16 bytes (tx >= 8 Float16C, tx >= 4 float32) and "
                                      "Q*N < 2^31");
    if (path == 2 && !h->step_tile)
        return fail(LBM_EUNSUPPORTED, "the block-per-tile kernel needs 256-cell power-of-two tiles and Q*N < 2^31");
    if (path == 3 && !h->step_pair)
        return fail(LBM_EUNSUPPORTED, "the cell-pair kernel needs the double-buffer method, 256-cell power-of-two "
                                      "tiles with tx >= 2 and Q*N < 2^31");
    if (path == 1 && h->closure_on)
        return fail(LBM_EUNSUPPORTED, "the learned closure runs in the block-per-tile kernel only");
    if (path == 1 && h->link_table)
        return fail(LBM_EUNSUPPORTED, "links fused into the step (lbm_set_links) run in the block-per-tile kernel only");
    h->path = path;
    return LBM_OK;
}

int32_t lbm_kernel_path(const lbm_handle* h) {
    return h ? (use_tile(h) ? (use_staged(h) ? 4 : use_pair(h) ? 3 : 2) : 1) : -1;
}

lbm_status lbm_device_status(lbm_handle* h) {
    if (check_handle(h)) return LBM_EINVAL;
    LBM_CK(cudaDeviceSynchronize());
    uint32_t v = 0;
    LBM_CK(cudaMemcpy(&v, h->dev_err, sizeof(v), cudaMemcpyDeviceToHost));
    if (v == 0u) return LBM_OK;
    LBM_CK(cudaMemset(h->dev_err, 0, sizeof(uint32_t)));
    return fail(LBM_ETIMEOUT, "a staged step's wait for its bulk copies ran out of time; the tiles it had not "
                              "reached were not stepped");
}

lbm_status lbm_debug_stage_extra_bytes(lbm_handle* h, uint32_t bytes) {
    if (check_handle(h)) return LBM_EINVAL;
    if (bytes % 16u) return fail(LBM_EINVAL, "extra bytes must be a multiple of 16");
    h->stage_extra = bytes;
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    return LBM_OK;
}

lbm_status lbm_double_buffer_step(lbm_handle* h, void* f_out, const void* f_in, float* bc, const uint8_t* flags,
                                  float tau, void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (h->cfg.lbm_method != LBM_DOUBLE_BUFFER)
        return fail(LBM_EINVAL, "This function is only valid if the lbm method is Double Buffer");
    if (!f_out || !f_in || !flags) return fail(LBM_EINVAL, "null buffer");
    if (f_out == f_in) return fail(LBM_EINVAL, "double buffer step needs distinct f_in and f_out");
    if (!bc && (h->cfg.include_moving_boundary || h->cfg.include_equilibrium_bc || h->cfg.capture_density ||
                h->cfg.capture_velocity))
        return fail(LBM_EINVAL, "bc is required by this configuration");
    return step_once(h, f_in, f_out, bc, flags, tau, 0, (cudaStream_t)stream);
}

lbm_status lbm_esoteric_pull_step(lbm_handle* h, void* f, float* bc, const uint8_t* flags, float tau,
                                  int32_t is_even_step, void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (h->cfg.lbm_method != LBM_ESOTERIC_PULL)
        return fail(LBM_EINVAL, "This function is only valid if the lbm method is Esoteric Pull");
    if (!f || !flags) return fail(LBM_EINVAL, "null buffer");
    if (!bc && (h->cfg.include_moving_boundary || h->cfg.include_equilibrium_bc || h->cfg.capture_density ||
                h->cfg.capture_velocity))
        return fail(LBM_EINVAL, "bc is required by this configuration");
    return step_once(h, f, f, bc, flags, tau, is_even_step ? 1 : 0, (cudaStream_t)stream);
}

lbm_status lbm_run(lbm_handle* h, void* f_a, void* f_b, float* bc, const uint8_t* flags, float tau, int64_t n_steps,
                   int64_t first_step, void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (n_steps < 0 || first_step < 0) return fail(LBM_EINVAL, "n_steps and first_step must be non-negative");
    const bool eso = h->cfg.lbm_method == LBM_ESOTERIC_PULL;
    if (!f_a || !flags || (!eso && (!f_b || f_a == f_b))) return fail(LBM_EINVAL, "bad buffers for lbm_run");
    if (!bc && (h->cfg.include_moving_boundary || h->cfg.include_equilibrium_bc || h->cfg.capture_density ||
                h->cfg.capture_velocity))
        return fail(LBM_EINVAL, "bc is required by this configuration");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_steps == 0) return LBM_OK;
    if (use_tile(h)) {
        const lbm_status st = tile_summary(h, flags, s);
        if (st != LBM_OK) return st;
    }
    auto launch_k = [&](int64_t k) -> lbm_status {
        const bool a_is_src = ((first_step + k) % 2) == 0;
        if (eso) return step_once(h, f_a, f_a, bc, flags, tau, a_is_src ? 1 : 0, s, false);
        return a_is_src ? step_once(h, f_a, f_b, bc, flags, tau, 0, s, false)
                        : step_once(h, f_b, f_a, bc, flags, tau, 0, s, false);
    };
    // Chunks of an even number of steps keep the buffer/parity pattern of every replay identical.
    const int64_t chunk = 64;
    int64_t done = 0;
    if (n_steps >= chunk) {
        uint32_t tau_bits;
        std::memcpy(&tau_bits, &tau, 4);
        const GraphKey key{f_a, f_b, bc, flags, tau_bits, (int)(first_step % 2), chunk, use_tile(h) ? (use_staged(h) ? 4 : use_pair(h) ? 3 : 2) : 1};
        auto it = h->graphs.find(key);
        if (it == h->graphs.end()) {
            cudaGraph_t g = nullptr;
            LBM_CK(cudaStreamBeginCapture(h->capture_stream, cudaStreamCaptureModeThreadLocal));
            lbm_status st = LBM_OK;
            for (int64_t k = 0; k < chunk && st == LBM_OK; ++k) {
                const bool a_is_src = ((first_step + k) % 2) == 0;
                const StepArgs a = eso ? step_args(h, f_a, f_a, bc, flags, tau, a_is_src ? 1 : 0)
                                       : (a_is_src ? step_args(h, f_a, f_b, bc, flags, tau, 0)
                                                   : step_args(h, f_b, f_a, bc, flags, tau, 0));
                const StepLaunch fn = step_fn(h, a);
                if (fn(a, h->threads, h->capture_stream) != cudaSuccess) st = LBM_ECUDA;
            }
            cudaError_t e = cudaStreamEndCapture(h->capture_stream, &g);
            if (st != LBM_OK || e != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return fail(LBM_ECUDA, "lbm_run: graph capture failed");
            }
            cudaGraphExec_t ge = nullptr;
            e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(LBM_ECUDA, std::string("lbm_run: ") + cudaGetErrorString(e));
            it = h->graphs.emplace(key, ge).first;
        }
        for (; done + chunk <= n_steps; done += chunk) LBM_CK(cudaGraphLaunch(it->second, s));
    }
    for (; done < n_steps; ++done) {
        const lbm_status st = launch_k(done);
        if (st != LBM_OK) return st;
    }
    return LBM_OK;
}

lbm_status lbm_init_equilibrium(lbm_handle* h, void* f, float rho, float tau, const float* u, const float* grad,
                                void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (!f) return fail(LBM_EINVAL, "null f");
    InitArgs a;
    a.lay = h->lay;
    a.f = f;
    a.u = u;
    a.grad = grad;
    a.rho = rho;
    a.tau = tau;
    a.ddf = h->cfg.DDF_shift;
    a.esoteric = h->cfg.lbm_method == LBM_ESOTERIC_PULL;
    const bool f16 = h->cfg.use_float16c != 0;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t nb = blocks_for(h->lay.ncells, 256);
    return dispatch_lattice(h->grid.lattice, [&](auto Lt) -> lbm_status {
        using L = decltype(Lt);
        if (f16) init_kernel<L, true><<<nb, 256, 0, s>>>(a);
        else init_kernel<L, false><<<nb, 256, 0, s>>>(a);
        LBM_CK(cudaGetLastError());
        return LBM_OK;
    });
}

lbm_status lbm_q_criterion(lbm_handle* h, float* q, const void* f, const float* bc, const uint8_t* flags,
                           const float* u, float tau, int32_t after_odd_step, void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (!q || !u || !f || !bc || !flags) return fail(LBM_EINVAL, "null buffer");
    RhoUArgs a;
    a.lay = h->lay;
    a.f = f;
    a.bc = bc;
    a.flags = flags;
    a.rho = nullptr;
    a.u = const_cast<float*>(u);  // read only in this pass
    a.q = q;
    a.tau = tau;
    a.ddf = h->cfg.DDF_shift;
    a.moving = h->cfg.include_moving_boundary;
    a.eqbc = h->cfg.include_equilibrium_bc;
    a.even = after_odd_step ? 1 : 0;
    const bool f16 = h->cfg.use_float16c != 0, eso = h->cfg.lbm_method == LBM_ESOTERIC_PULL;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t nb = blocks_for(h->lay.ncells, 256);
    return dispatch_lattice(h->grid.lattice, [&](auto Lt) -> lbm_status {
        using L = decltype(Lt);
        if (f16) {
            if (eso) rho_u_kernel<L, true, true, true><<<nb, 256, 0, s>>>(a);
            else rho_u_kernel<L, true, false, true><<<nb, 256, 0, s>>>(a);
        } else {
            if (eso) rho_u_kernel<L, false, true, true><<<nb, 256, 0, s>>>(a);
            else rho_u_kernel<L, false, false, true><<<nb, 256, 0, s>>>(a);
        }
        LBM_CK(cudaGetLastError());
        return LBM_OK;
    });
}

lbm_status lbm_compute_rho_u(lbm_handle* h, float* rho, float* u, const void* f, const float* bc,
                             const uint8_t* flags, int32_t after_odd_step, void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (!rho || !u || !f || !bc || !flags) return fail(LBM_EINVAL, "null buffer");
    RhoUArgs a;
    a.lay = h->lay;
    a.f = f;
    a.bc = bc;
    a.flags = flags;
    a.rho = rho;
    a.u = u;
    a.q = nullptr;
    a.tau = 0.f;
    a.ddf = h->cfg.DDF_shift;
    a.moving = h->cfg.include_moving_boundary;
    a.eqbc = h->cfg.include_equilibrium_bc;
    a.even = after_odd_step ? 1 : 0;
    const bool f16 = h->cfg.use_float16c != 0, eso = h->cfg.lbm_method == LBM_ESOTERIC_PULL;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t nb = blocks_for(h->lay.ncells, 256);
    return dispatch_lattice(h->grid.lattice, [&](auto Lt) -> lbm_status {
        using L = decltype(Lt);
        if (f16) {
            if (eso) rho_u_kernel<L, true, true><<<nb, 256, 0, s>>>(a);
            else rho_u_kernel<L, true, false><<<nb, 256, 0, s>>>(a);
        } else {
            if (eso) rho_u_kernel<L, false, true><<<nb, 256, 0, s>>>(a);
            else rho_u_kernel<L, false, false><<<nb, 256, 0, s>>>(a);
        }
        LBM_CK(cudaGetLastError());
        return LBM_OK;
    });
}

lbm_status lbm_reduce_mass_momentum(lbm_handle* h, const void* f, const uint8_t* flags, int32_t after_odd_step,
                                    double out[4], void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (!f || !flags || !out) return fail(LBM_EINVAL, "null buffer");
    MassArgs a;
    a.lay = h->lay;
    a.f = f;
    a.flags = flags;
    a.partial = h->scratch;
    a.ddf = h->cfg.DDF_shift;
    a.even = after_odd_step ? 1 : 0;
    const bool f16 = h->cfg.use_float16c != 0, eso = h->cfg.lbm_method == LBM_ESOTERIC_PULL;
    cudaStream_t s = (cudaStream_t)stream;
    lbm_status st = dispatch_lattice(h->grid.lattice, [&](auto Lt) -> lbm_status {
        using L = decltype(Lt);
        if (f16) {
            if (eso) mass_partial_kernel<L, true, true><<<kReduceBlocks, kReduceThreads, 0, s>>>(a);
            else mass_partial_kernel<L, true, false><<<kReduceBlocks, kReduceThreads, 0, s>>>(a);
        } else {
            if (eso) mass_partial_kernel<L, false, true><<<kReduceBlocks, kReduceThreads, 0, s>>>(a);
            else mass_partial_kernel<L, false, false><<<kReduceBlocks, kReduceThreads, 0, s>>>(a);
        }
        LBM_CK(cudaGetLastError());
        return LBM_OK;
    });
    if (st != LBM_OK) return st;
    double* res = h->scratch + kReduceBlocks * kReduceWidth;
    final_sum_kernel<4><<<1, kReduceThreads, 0, s>>>(h->scratch, kReduceBlocks, res);
    LBM_CK(cudaGetLastError());
    LBM_CK(cudaMemcpyAsync(out, res, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    LBM_CK(cudaStreamSynchronize(s));
    for (int k = 0; k < 4; ++k)
        if (!std::isfinite(out[k])) return fail(LBM_ENAN, "mass/momentum reduction found a non-finite value");
    return LBM_OK;
}

lbm_status lbm_linkwise_bounceback(lbm_handle* h, void* f, float* link_force, const int32_t* fluid_ids,
                                   const int32_t* dirs, const float* dists, int64_t n_links, int32_t method,
                                   int32_t compute_force, float q_clamp, void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (h->cfg.lbm_method != LBM_DOUBLE_BUFFER)
        return fail(LBM_EUNSUPPORTED, "linkwise bounce-back needs the double-buffer method");
    if (method != LBM_BB_MID_GRID && method != LBM_BB_BOUZIDI) return fail(LBM_EINVAL, "unknown bounce-back method");
    if (n_links < 0) return fail(LBM_EINVAL, "n_links must be non-negative");
    if (n_links == 0) return LBM_OK;
    if (!f || !fluid_ids || !dirs || !dists || (compute_force && !link_force)) return fail(LBM_EINVAL, "null buffer");
    LinkArgs a;
    a.lay = h->lay;
    a.f = f;
    a.force = link_force;
    a.ids = fluid_ids;
    a.dirs = dirs;
    a.dists = dists;
    a.n = n_links;
    a.q_clamp = q_clamp;
    a.bouzidi = method == LBM_BB_BOUZIDI;
    a.compute_force = compute_force;
    a.ddf = h->cfg.DDF_shift;
    const bool f16 = h->cfg.use_float16c != 0;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t nb = (uint32_t)((n_links + 255) / 256);
    return dispatch_lattice(h->grid.lattice, [&](auto Lt) -> lbm_status {
        using L = decltype(Lt);
        if (f16) link_kernel<L, true><<<nb, 256, 0, s>>>(a);
        else link_kernel<L, false><<<nb, 256, 0, s>>>(a);
        LBM_CK(cudaGetLastError());
        return LBM_OK;
    });
}

lbm_status lbm_sum_link_force(lbm_handle* h, const float* link_force, int64_t n_links, double out[3], void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (!out || (n_links > 0 && !link_force)) return fail(LBM_EINVAL, "null buffer");
    if (n_links < 0) return fail(LBM_EINVAL, "n_links must be non-negative");
    out[0] = out[1] = out[2] = 0.0;
    if (n_links == 0) return LBM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int D = lattice_d(h->grid.lattice);
    colsum_partial_kernel<<<kReduceBlocks, kReduceThreads, 0, s>>>(link_force, n_links, D, h->scratch);
    LBM_CK(cudaGetLastError());
    double* res = h->scratch + kReduceBlocks * kReduceWidth;
    final_sum_kernel<4><<<1, kReduceThreads, 0, s>>>(h->scratch, kReduceBlocks, res);
    LBM_CK(cudaGetLastError());
    double tmp[4];
    LBM_CK(cudaMemcpyAsync(tmp, res, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    LBM_CK(cudaStreamSynchronize(s));
    for (int k = 0; k < 3; ++k) out[k] = tmp[k];
    return LBM_OK;
}

lbm_status lbm_drag_force(lbm_handle* h, float* node_force, const void* f, const uint8_t* flags,
                          const int32_t* fluid_ids, int64_t n_nodes, void* stream) {
    if (check_handle(h)) return LBM_EINVAL;
    if (n_nodes < 0) return fail(LBM_EINVAL, "n_nodes must be non-negative");
    if (n_nodes == 0) return LBM_OK;
    if (!node_force || !f || !flags || !fluid_ids) return fail(LBM_EINVAL, "null buffer");
    DragArgs a;
    a.lay = h->lay;
    a.f = f;
    a.flags = flags;
    a.ids = fluid_ids;
    a.force = node_force;
    a.n = n_nodes;
    a.ddf = h->cfg.DDF_shift;
    const bool f16 = h->cfg.use_float16c != 0;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t nb = (uint32_t)((n_nodes + 255) / 256);
    return dispatch_lattice(h->grid.lattice, [&](auto Lt) -> lbm_status {
        using L = decltype(Lt);
        if (f16) drag_kernel<L, true><<<nb, 256, 0, s>>>(a);
        else drag_kernel<L, false><<<nb, 256, 0, s>>>(a);
        LBM_CK(cudaGetLastError());
        return LBM_OK;
    });
}

}  // extern "C"

namespace {
__global__ void f16c_encode_kernel(const float* in, uint16_t* out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint16_t)f16c_encode(in[i]);
}
__global__ void f16c_decode_kernel(const uint16_t* in, float* out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = f16c_decode(in[i]);
}
}  // namespace

extern "C" {

lbm_status lbm_float16c_encode(const float* in, uint16_t* out, int64_t n, void* stream) {
    if (n < 0 || (n > 0 && (!in || !out))) return fail(LBM_EINVAL, "bad codec arguments");
    if (n == 0) return LBM_OK;
    f16c_encode_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(in, out, n);
    LBM_CK(cudaGetLastError());
    return LBM_OK;
}

lbm_status lbm_float16c_decode(const uint16_t* in, float* out, int64_t n, void* stream) {
    if (n < 0 || (n > 0 && (!in || !out))) return fail(LBM_EINVAL, "bad codec arguments");
    if (n == 0) return LBM_OK;
    f16c_decode_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(in, out, n);
    LBM_CK(cudaGetLastError());
    return LBM_OK;
}

}  // extern "C"
