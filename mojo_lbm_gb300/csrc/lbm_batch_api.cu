// C ABI of the batched persistent step (lbm_batch_* in include/lbm_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>

#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "lbm_batch.cuh"
#include "lbm_link_tables.h"

namespace lbm {
void set_last_error(const char* msg);  // lbm_capi.cu
BatchLaunch get_batch_step_d2q9(int, int, int, int);
BatchLaunch get_batch_step_d3q19(int, int, int, int);
BatchLaunch get_batch_step_d3q27(int, int, int, int);
BatchLaunch get_batch_links_step_d2q9(int, int, int);
BatchLaunch get_batch_links_step_d3q19(int, int, int);
BatchLaunch get_batch_links_step_d3q27(int, int, int);
cudaError_t launch_link_batch_d2q9(const BatchLinkArgs&, bool, cudaStream_t);
cudaError_t launch_link_batch_d3q19(const BatchLinkArgs&, bool, cudaStream_t);
cudaError_t launch_link_batch_d3q27(const BatchLinkArgs&, bool, cudaStream_t);
}  // namespace lbm

using namespace lbm;

extern "C" lbm_status lbm_validate(const lbm_config_t* cfg, const lbm_grid_t* grid);
extern "C" const char* lbm_last_error(void);

struct lbm_batch {
    lbm_config_t cfg;
    int32_t lattice;
    int32_t ndom;
    std::vector<lbm_grid_t> grids;
    std::vector<StepArgs> even, odd;   // host descriptors per parity
    std::vector<uint8_t> set;          // domain has buffers
    std::vector<uint32_t> unit_begin;  // ndom + 1
    StepArgs* d_even = nullptr;
    StepArgs* d_odd = nullptr;
    uint32_t* d_begin = nullptr;
    uint8_t* d_box_sum = nullptr;
    uint8_t* d_tile_near = nullptr;
    uint8_t* d_flags_seen = nullptr;  // the flags of the last summary, 256 cells per unit
    uint2* d_cell_masks = nullptr;    // neighbour-solid masks per cell, 256 cells per unit
    uint32_t* d_changed = nullptr;    // summary round in which a box summary last changed
    uint32_t summary_gen = 0;
    bool summary_valid = false;
    bool dirty = true;
    BatchLaunch step = nullptr;
    BatchLaunch step_links = nullptr;  // the step with the links fused in (double buffer), or null
    // links (caller-owned device arrays, concatenated over domains)
    const int32_t *l_dom = nullptr, *l_ids = nullptr, *l_dirs = nullptr;
    const float* l_dists = nullptr;
    float* l_force = nullptr;
    int64_t n_links = 0;
    int32_t l_method = LBM_BB_BOUZIDI;
    float l_qclamp = 0.f;
    int32_t link_mode = LBM_LINKS_SEPARATE;
    bool tables_stale = true;          // the fused tables do not hold the current links
    uint2* d_link_table = nullptr;     // fused: per cell of the batch (256 cells per unit)
    float* d_link_dist = nullptr;
    int32_t* d_link_id = nullptr;
    int sms = 1;
    cudaStream_t capture_stream = nullptr;
    std::map<int, cudaGraphExec_t> graphs;  // keyed by the parity of the first step
};

namespace {

lbm_status bfail(lbm_status s, const std::string& m) {
    set_last_error(m.c_str());
    return s;
}

#define LBM_BCK(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) return bfail(LBM_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
int ilog2(int v) { int r = 0; while ((1 << r) < v) ++r; return r; }

void drop_graphs(lbm_batch* b) {
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

// tile_near: per unit, the warp_near bits of its 8 warp boxes; one thread per box.  Skipped unless
// a box summary changed in this round (*changed == gen).
__global__ void batch_near_kernel(const BatchArgs b, const uint8_t* box_sum, uint8_t* tile_near,
                                  const uint32_t* changed, uint32_t gen) {
    if (*changed != gen) return;  // the same value for every thread
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    write_near_mask(i, b.total_units * kTileWarps, batch_near_box(b, i, box_sum), tile_near);
}

// The neighbour-solid masks of the cells of every warp with its mask bit set, one block per unit,
// after a change of the flags in this round (*changed == gen).
template <class L>
__global__ void __launch_bounds__(256) batch_cell_mask_kernel(const BatchArgs b, const uint32_t* changed,
                                                              uint32_t gen) {
    if (*changed != gen) return;  // the same value for every thread
    for (uint32_t u = blockIdx.x; u < b.total_units; u += gridDim.x) {  // blocks stride over the units
        const uint32_t d = find_domain(b.unit_begin, b.ndom, u);
        const StepArgs& a = b.dom[d];
        tile_cell_masks<L>(a, u - b.unit_begin[d], const_cast<uint2*>(a.cell_masks));
    }
}

// The summary byte of every warp box of the batch whose flags changed; one thread per box.
__global__ void batch_summary_kernel(const BatchArgs b, uint8_t* box_sum, uint8_t* flags_seen, uint32_t* changed,
                                     uint32_t gen, int force) {
    batch_box_summary(b, blockIdx.x * blockDim.x + threadIdx.x, box_sum, flags_seen, changed, gen, force);
}

lbm_status launch_links(lbm_batch* b, const StepArgs* dom, cudaStream_t s) {
    if (b->n_links == 0) return LBM_OK;
    BatchLinkArgs la;
    la.dom = dom;
    la.domain = b->l_dom;
    la.ids = b->l_ids;
    la.dirs = b->l_dirs;
    la.dists = b->l_dists;
    la.force = b->l_force;
    la.n = b->n_links;
    la.q_clamp = b->l_qclamp;
    la.bouzidi = b->l_method == LBM_BB_BOUZIDI;
    la.compute_force = b->l_force != nullptr;
    la.ddf = b->cfg.DDF_shift;
    const bool f16 = b->cfg.use_float16c != 0;
    cudaError_t e = b->lattice == LBM_D2Q9 ? launch_link_batch_d2q9(la, f16, s)
                  : b->lattice == LBM_D3Q19 ? launch_link_batch_d3q19(la, f16, s)
                                            : launch_link_batch_d3q27(la, f16, s);
    LBM_BCK(e);
    return LBM_OK;
}

bool fused_links(const lbm_batch* b) { return b->link_mode == LBM_LINKS_FUSED && b->n_links > 0; }

// One step of every domain: the persistent step kernel, then the link-wise bounce-back (or the
// step kernel with the links fused in).
lbm_status batch_step(lbm_batch* b, bool parity_odd, cudaStream_t s) {
    BatchArgs a;
    a.dom = parity_odd ? b->d_odd : b->d_even;
    a.unit_begin = b->d_begin;
    a.ndom = (uint32_t)b->ndom;
    a.total_units = b->unit_begin.back();
    if (fused_links(b)) {
        LBM_BCK(b->step_links(a, b->sms, s));
        return LBM_OK;
    }
    LBM_BCK(b->step(a, b->sms, s));
    return launch_links(b, a.dom, s);
}

void free_tables(lbm_batch* b) {
    cudaFree(b->d_link_table);
    cudaFree(b->d_link_dist);
    cudaFree(b->d_link_id);
    b->d_link_table = nullptr;
    b->d_link_dist = nullptr;
    b->d_link_id = nullptr;
}

// The fused mode's per-cell link table from the caller's link arrays (the batch's cells numbered
// unit after unit, 256 per unit), and the descriptors' pointers into it.
lbm_status build_tables(lbm_batch* b, cudaStream_t s) {
    const int64_t n = b->n_links;
    const uint64_t cells = (uint64_t)b->unit_begin.back() * kTileCells;
    std::vector<int32_t> dom(n), ids(n), dirs(n);
    std::vector<float> dists(n);
    LBM_BCK(cudaMemcpyAsync(dom.data(), b->l_dom, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    LBM_BCK(cudaMemcpyAsync(ids.data(), b->l_ids, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    LBM_BCK(cudaMemcpyAsync(dirs.data(), b->l_dirs, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    LBM_BCK(cudaMemcpyAsync(dists.data(), b->l_dists, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    LBM_BCK(cudaStreamSynchronize(s));
    std::vector<uint64_t> cell0(b->ndom), ncells(b->ndom);
    for (int32_t d = 0; d < b->ndom; ++d) {
        cell0[d] = (uint64_t)b->unit_begin[d] * kTileCells;
        ncells[d] = (uint64_t)(b->unit_begin[d + 1] - b->unit_begin[d]) * kTileCells;
    }
    LinkTables lt;
    const int Q = b->lattice == LBM_D2Q9 ? 9 : b->lattice == LBM_D3Q19 ? 19 : 27;
    const std::string err = build_link_tables((int64_t)cells, Q, n, dom.data(), cell0.data(), ncells.data(), b->ndom,
                                              ids.data(), dirs.data(), dists.data(), lt);
    if (!err.empty()) return bfail(LBM_EINVAL, "lbm_batch_run (fused links): " + err);
    free_tables(b);
    LBM_BCK(cudaMalloc(&b->d_link_table, sizeof(uint2) * lt.table.size()));
    LBM_BCK(cudaMalloc(&b->d_link_dist, sizeof(float) * n));
    LBM_BCK(cudaMalloc(&b->d_link_id, sizeof(int32_t) * n));
    LBM_BCK(cudaMemcpy(b->d_link_table, lt.table.data(), sizeof(uint2) * lt.table.size(), cudaMemcpyHostToDevice));
    LBM_BCK(cudaMemcpy(b->d_link_dist, lt.dist.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    LBM_BCK(cudaMemcpy(b->d_link_id, lt.id.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    for (int32_t d = 0; d < b->ndom; ++d) {
        for (StepArgs* a : {&b->even[d], &b->odd[d]}) {
            a->link_table = b->d_link_table + cell0[d];
            a->link_dist = b->d_link_dist;
            a->link_id = b->d_link_id;
            a->link_force = b->l_force;
            a->link_stride = n;
            a->q_clamp = b->l_qclamp;
            a->bouzidi = b->l_method == LBM_BB_BOUZIDI;
        }
    }
    b->tables_stale = false;
    b->dirty = true;
    return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_batch_create(const lbm_config_t* cfg, int32_t n_domains, const lbm_grid_t* grids, lbm_batch** out) {
    if (!out) return bfail(LBM_EINVAL, "null output pointer");
    *out = nullptr;
    if (!cfg || !grids || n_domains <= 0) return bfail(LBM_EINVAL, "need a config and at least one grid");
    const int32_t lat = grids[0].lattice;
    uint64_t units = 0;
    std::vector<uint32_t> begin(n_domains + 1, 0);
    for (int32_t i = 0; i < n_domains; ++i) {
        const lbm_grid_t& g = grids[i];
        const lbm_status v = lbm_validate(cfg, &g);
        if (v != LBM_OK) return bfail(v, "domain " + std::to_string(i) + ": " + lbm_last_error());
        if (g.lattice != lat) return bfail(LBM_EINVAL, "all domains of a batch must use the same lattice");
        const int64_t Q = lat == LBM_D2Q9 ? 9 : lat == LBM_D3Q19 ? 19 : 27;
        const int64_t N = (int64_t)g.nx * g.ny * g.nz;
        if ((int64_t)g.tx * g.ty * g.tz != (int64_t)kTileCells || !pow2(g.tx) || !pow2(g.ty) || !pow2(g.tz) ||
            Q * N >= ((int64_t)1 << 31))
            return bfail(LBM_EUNSUPPORTED, "domain " + std::to_string(i) +
                                               ": batched domains need 256-cell tiles with power-of-two sides "
                                               "and Q*N < 2^31");
        begin[i] = (uint32_t)units;
        units += (uint64_t)(N / kTileCells);
    }
    // (warp boxes, 8 per tile, are numbered in 32 bits)
    if (units >= ((uint64_t)1 << 29)) return bfail(LBM_EINVAL, "too many tiles in the batch");
    begin[n_domains] = (uint32_t)units;

    lbm_batch* b = new lbm_batch();
    b->cfg = *cfg;
    b->lattice = lat;
    b->ndom = n_domains;
    b->grids.assign(grids, grids + n_domains);
    b->unit_begin = begin;
    b->even.resize(n_domains);
    b->odd.resize(n_domains);
    b->set.assign(n_domains, 0);
    const int m = cfg->lbm_method, f16 = cfg->use_float16c ? 1 : 0, co = cfg->collision_op, les = cfg->LES ? 1 : 0;
    b->step = lat == LBM_D2Q9 ? get_batch_step_d2q9(m, f16, co, les)
            : lat == LBM_D3Q19 ? get_batch_step_d3q19(m, f16, co, les)
                               : get_batch_step_d3q27(m, f16, co, les);
    b->step_links = m != LBM_DOUBLE_BUFFER ? nullptr
                  : lat == LBM_D2Q9 ? get_batch_links_step_d2q9(f16, co, les)
                  : lat == LBM_D3Q19 ? get_batch_links_step_d3q19(f16, co, les)
                                     : get_batch_links_step_d3q27(f16, co, les);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_even, sizeof(StepArgs) * n_domains);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_odd, sizeof(StepArgs) * n_domains);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_begin, sizeof(uint32_t) * (n_domains + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_box_sum, units > 0 ? units * kTileWarps : 1);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tile_near, units > 0 ? units : 1);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_flags_seen, units > 0 ? units * kTileCells : 1);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_cell_masks, sizeof(uint2) * (units > 0 ? units * kTileCells : 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_changed, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(b->d_changed, 0, sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_begin, begin.data(), sizeof(uint32_t) * (n_domains + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        lbm_batch_destroy(b);
        return bfail(LBM_ECUDA, std::string("lbm_batch_create: ") + cudaGetErrorString(e));
    }
    *out = b;
    return LBM_OK;
}

lbm_status lbm_batch_destroy(lbm_batch* b) {
    if (!b) return LBM_OK;
    drop_graphs(b);
    cudaFree(b->d_even);
    cudaFree(b->d_odd);
    cudaFree(b->d_begin);
    cudaFree(b->d_box_sum);
    cudaFree(b->d_tile_near);
    cudaFree(b->d_flags_seen);
    cudaFree(b->d_cell_masks);
    cudaFree(b->d_changed);
    free_tables(b);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    delete b;
    return LBM_OK;
}

lbm_status lbm_batch_set_domain(lbm_batch* b, int32_t i, void* f_a, void* f_b, float* bc, const uint8_t* flags,
                                float tau) {
    if (!b) return bfail(LBM_EINVAL, "null batch");
    if (i < 0 || i >= b->ndom) return bfail(LBM_EINVAL, "domain index out of range");
    const bool eso = b->cfg.lbm_method == LBM_ESOTERIC_PULL;
    if (!f_a || !flags || (!eso && (!f_b || f_a == f_b))) return bfail(LBM_EINVAL, "bad buffers for the domain");
    if (!bc && (b->cfg.include_moving_boundary || b->cfg.include_equilibrium_bc || b->cfg.capture_density ||
                b->cfg.capture_velocity))
        return bfail(LBM_EINVAL, "bc is required by this configuration");
    const lbm_grid_t& g = b->grids[i];
    StepArgs a;
    std::memset(&a, 0, sizeof(a));
    a.lay.nx = g.nx; a.lay.ny = g.ny; a.lay.nz = g.nz;
    a.lay.tx = g.tx; a.lay.ty = g.ty; a.lay.tz = g.tz;
    a.lay.ntx = g.nx / g.tx; a.lay.nty = g.ny / g.ty; a.lay.ntz = g.nz / g.tz;
    a.lay.T = kTileCells;
    a.lay.ncells = (uint32_t)((int64_t)g.nx * g.ny * g.nz);
    a.lay.d_tx = FastDiv((uint32_t)g.tx);
    a.lay.d_ty = FastDiv((uint32_t)g.ty);
    a.lay.d_T = FastDiv(kTileCells);
    a.lay.d_ntx = FastDiv((uint32_t)a.lay.ntx);
    a.lay.d_nty = FastDiv((uint32_t)a.lay.nty);
    a.bc = bc;
    a.flags = flags;
    a.tau = tau;
    a.inv_tau = 1.f / tau;  // IEEE float32 quotient, as the kernel would compute it
    a.Cs = b->cfg.Cs;
    a.trt_lambda = b->cfg.trt_lambda;
    a.ddf = b->cfg.DDF_shift;
    a.moving = b->cfg.include_moving_boundary;
    a.eqbc = b->cfg.include_equilibrium_bc;
    a.cap_rho = b->cfg.capture_density;
    a.cap_u = b->cfg.capture_velocity;
    a.tile_near = b->d_tile_near + b->unit_begin[i];
    a.cell_masks = b->d_cell_masks + (size_t)b->unit_begin[i] * kTileCells;
    a.mx = (uint32_t)g.tx - 1u;
    a.my = (uint32_t)g.ty - 1u;
    a.shx = (uint32_t)ilog2(g.tx);
    a.shxy = (uint32_t)(ilog2(g.tx) + ilog2(g.ty));
    StepArgs ev = a, od = a;
    if (eso) {
        ev.f_in = ev.f_out = f_a;
        od.f_in = od.f_out = f_a;
        ev.even = 1;
        od.even = 0;
    } else {
        ev.f_in = f_a; ev.f_out = f_b;
        od.f_in = f_b; od.f_out = f_a;
    }
    b->even[i] = ev;
    b->odd[i] = od;
    b->tables_stale = true;  // the descriptors' link pointers are set when the tables are built
    b->set[i] = 1;
    b->dirty = true;
    return LBM_OK;
}

lbm_status lbm_batch_set_links(lbm_batch* b, const int32_t* domain, const int32_t* fluid_ids, const int32_t* dirs,
                               const float* dists, int64_t n_links, int32_t method, float q_clamp, float* link_force) {
    if (!b) return bfail(LBM_EINVAL, "null batch");
    if (n_links < 0) return bfail(LBM_EINVAL, "n_links must be non-negative");
    if (n_links > 0 && b->cfg.lbm_method != LBM_DOUBLE_BUFFER)
        return bfail(LBM_EUNSUPPORTED, "linkwise bounce-back needs the double-buffer method");
    if (n_links > 0 && (!domain || !fluid_ids || !dirs || !dists)) return bfail(LBM_EINVAL, "null link array");
    if (method != LBM_BB_MID_GRID && method != LBM_BB_BOUZIDI) return bfail(LBM_EINVAL, "unknown bounce-back method");
    b->l_dom = domain;
    b->l_ids = fluid_ids;
    b->l_dirs = dirs;
    b->l_dists = dists;
    b->l_force = link_force;
    b->n_links = n_links;
    b->l_method = method;
    b->l_qclamp = q_clamp;
    b->tables_stale = true;
    drop_graphs(b);
    return LBM_OK;
}

lbm_status lbm_batch_set_link_mode(lbm_batch* b, int32_t mode) {
    if (!b) return bfail(LBM_EINVAL, "null batch");
    if (mode != LBM_LINKS_SEPARATE && mode != LBM_LINKS_FUSED)
        return bfail(LBM_EINVAL, "link mode must be LBM_LINKS_SEPARATE or LBM_LINKS_FUSED");
    if (mode == LBM_LINKS_FUSED && !b->step_links)
        return bfail(LBM_EUNSUPPORTED, "fused links need the double-buffer method");
    if (mode != b->link_mode) {
        b->link_mode = mode;
        b->tables_stale = true;
        drop_graphs(b);
    }
    return LBM_OK;
}

lbm_status lbm_batch_run(lbm_batch* b, int64_t n_steps, int64_t first_step, void* stream) {
    if (!b) return bfail(LBM_EINVAL, "null batch");
    if (n_steps < 0 || first_step < 0) return bfail(LBM_EINVAL, "n_steps and first_step must be non-negative");
    for (int32_t i = 0; i < b->ndom; ++i)
        if (!b->set[i]) return bfail(LBM_EINVAL, "domain " + std::to_string(i) + " has no buffers");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_steps == 0) return LBM_OK;
    if (fused_links(b) && b->tables_stale) {
        const lbm_status st = build_tables(b, s);
        if (st != LBM_OK) return st;
        drop_graphs(b);
    }
    if (b->dirty) {
        LBM_BCK(cudaMemcpyAsync(b->d_even, b->even.data(), sizeof(StepArgs) * b->ndom, cudaMemcpyHostToDevice, s));
        LBM_BCK(cudaMemcpyAsync(b->d_odd, b->odd.data(), sizeof(StepArgs) * b->ndom, cudaMemcpyHostToDevice, s));
        LBM_BCK(cudaStreamSynchronize(s));  // the host descriptors may change after return
        b->dirty = false;
    }
    {
        BatchArgs a;
        a.dom = b->d_even;
        a.unit_begin = b->d_begin;
        a.ndom = (uint32_t)b->ndom;
        a.total_units = b->unit_begin.back();
        const uint32_t nboxes = a.total_units * kTileWarps;  // < 2^32: fewer than 2^29 units
        if (++b->summary_gen == 0u) ++b->summary_gen;  // 0 is the initial value of *d_changed
        if (nboxes)
            batch_summary_kernel<<<(nboxes + 255u) / 256u, 256, 0, s>>>(a, b->d_box_sum, b->d_flags_seen,
                                                                         b->d_changed, b->summary_gen,
                                                                         b->summary_valid ? 0 : 1);
        LBM_BCK(cudaGetLastError());
        b->summary_valid = true;
        if (nboxes)
            batch_near_kernel<<<(nboxes + 255u) / 256u, 256, 0, s>>>(a, b->d_box_sum, b->d_tile_near, b->d_changed,
                                                                    b->summary_gen);
        LBM_BCK(cudaGetLastError());
        if (nboxes) {
            const uint32_t grid = std::min<uint32_t>(a.total_units, (uint32_t)b->sms * 8u);
            if (b->lattice == LBM_D2Q9)
                batch_cell_mask_kernel<D2Q9><<<grid, kTileCells, 0, s>>>(a, b->d_changed, b->summary_gen);
            else if (b->lattice == LBM_D3Q19)
                batch_cell_mask_kernel<D3Q19><<<grid, kTileCells, 0, s>>>(a, b->d_changed, b->summary_gen);
            else
                batch_cell_mask_kernel<D3Q27><<<grid, kTileCells, 0, s>>>(a, b->d_changed, b->summary_gen);
        }
        LBM_BCK(cudaGetLastError());
    }
    const int64_t chunk = 64;
    int64_t done = 0;
    if (n_steps >= chunk) {
        const int key = (int)(first_step % 2);
        auto it = b->graphs.find(key);
        if (it == b->graphs.end()) {
            cudaGraph_t g = nullptr;
            LBM_BCK(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal));
            lbm_status st = LBM_OK;
            for (int64_t k = 0; k < chunk && st == LBM_OK; ++k)
                st = batch_step(b, ((first_step + k) % 2) != 0, b->capture_stream);
            cudaError_t e = cudaStreamEndCapture(b->capture_stream, &g);
            if (st != LBM_OK || e != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return st != LBM_OK ? st : bfail(LBM_ECUDA, "lbm_batch_run: graph capture failed");
            }
            cudaGraphExec_t ge = nullptr;
            e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return bfail(LBM_ECUDA, std::string("lbm_batch_run: ") + cudaGetErrorString(e));
            it = b->graphs.emplace(key, ge).first;
        }
        for (; done + chunk <= n_steps; done += chunk) LBM_BCK(cudaGraphLaunch(it->second, s));
    }
    for (; done < n_steps; ++done) {
        const lbm_status st = batch_step(b, ((first_step + done) % 2) != 0, s);
        if (st != LBM_OK) return st;
    }
    return LBM_OK;
}

int64_t lbm_batch_cells(const lbm_batch* b) {
    if (!b) return -1;
    int64_t n = 0;
    for (const auto& g : b->grids) n += (int64_t)g.nx * g.ny * g.nz;
    return n;
}

}  // extern "C"
