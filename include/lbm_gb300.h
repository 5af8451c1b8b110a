/*
 * lbm_gb300.h — C ABI of the GB300 (sm_103a) fused lattice-Boltzmann stream–collide step.
 *
 * This library replaces the compute path of JohnCSu/mojo_lbm: the comptime-specialised Mojo
 * GPU kernels `double_buffer_kernel` (src/lbm/kernels/double_buffer.mojo:25-99) and
 * `esoteric_pull_kernel` (src/lbm/kernels/esoteric_pull.mojo:24-111), the host launch wrappers
 * `Solver.double_buffer_step` / `Solver.esoteric_pull_step` (src/lbm/solver.mojo:81-154), the
 * link-wise interpolated bounce-back kernel (src/lbm/geometry/interpolated_BB.mojo:46-141) and
 * the output kernels that read the step's populations (src/lbm/output/velocity.mojo:25,
 * src/lbm/output/drag.mojo:16).
 *
 * Conventions
 *  - Every buffer argument is a caller-owned DEVICE pointer, laid out exactly as the reference's
 *    tiled TileTensor layouts (src/lbm/layoutstruct.mojo:37-92):
 *        f[x,y,z,q]  at  lx + tx*(ly + ty*(lz + tz*(q + Q*(bx + ntx*(by + nty*bz)))))
 *        bc[x,y,z,k] at  the same formula with Q -> D+1 (k = 0..D-1 velocity, k = D density)
 *        flags[x,y,z] at lx + tx*(ly + ty*lz) + tx*ty*tz*(bx + ntx*(by + nty*bz))
 *    with lx = x % tx, bx = x / tx (same for y, z).  A tile equal to the whole grid
 *    (tx,ty,tz) = (nx,ny,nz) is the reference's untiled column-major layout.
 *  - Populations are float32, or uint16 Float16C codes when use_float16c is set.  The boundary
 *    tensor bc is always float32.  Arithmetic is float32.
 *  - `stream` is a cudaStream_t passed as void*; NULL is the legacy default stream.  All compute
 *    calls are asynchronous on that stream unless they return a host value.
 *  - Functions return an lbm_status; the message of the last failure on the calling thread is
 *    returned by lbm_last_error().  Nothing traps or aborts on the device.
 *  - A handle is not thread-safe; distinct handles are independent.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference raises Error strings, src/lbm/assembly.mojo:115-189) ---- */
typedef enum lbm_status {
    LBM_OK = 0,
    LBM_EINVAL = 1,       /* invalid argument or configuration                               */
    LBM_ECUDA = 2,        /* a CUDA runtime call failed                                      */
    LBM_ENAN = 3,         /* a reduction found a non-finite value                            */
    LBM_ETIMEOUT = 4,     /* a bounded device wait gave up (the staged kernel's wait for its  */
                          /* bulk copies; reported by lbm_device_status)                     */
    LBM_ENOMEM = 5,       /* a handle-owned allocation failed                                */
    LBM_EUNSUPPORTED = 6  /* the combination is not built (e.g. IBB with esoteric pull)      */
} lbm_status;

/* LBM_method (src/lbm/constants.mojo:20-31) */
enum { LBM_DOUBLE_BUFFER = 0, LBM_ESOTERIC_PULL = 1 };

/* Collisions (src/lbm/constants.mojo:41-55) */
enum { LBM_SRT = 0, LBM_TRT = 1, LBM_KBC = 2, LBM_RLBM = 3 };

/* lattices: get_D2Q9 / get_D3Q19 / get_D3Q27 (src/lbm/lattice.mojo:122,221,302) */
enum { LBM_D2Q9 = 0, LBM_D3Q19 = 1, LBM_D3Q27 = 2 };

/* Flags (src/lbm/constants.mojo:58-116): low nibble is an enum, high bits a bitmask */
enum {
    LBM_FLAG_FLUID = 0,
    LBM_FLAG_SOLID = 1,
    LBM_FLAG_EQUILIBRIUM = 2,
    LBM_FLAG_FLUID_SOLID_BOUNDARY = 3,
    LBM_FLAG_CAPTURE_VELOCITY = 0x20,
    LBM_FLAG_CAPTURE_DENSITY = 0x40,
    LBM_FLAG_EXCLUDE = 0x80
};

/* Bounceback_method (src/lbm/constants.mojo:120-123) */
enum { LBM_BB_MID_GRID = 0, LBM_BB_BOUZIDI = 1 };

/* Arithmetic of the step (no counterpart in the reference, whose step has one float32 form).
 * LBM_ARITH_EXACT: every float32 operation in the reference's order, bit-identical to the
 *   float32 CPU restatement of the reference step (the default).
 * LBM_ARITH_FAST: the same operators rearranged for fused multiply-add (moments from opposite
 *   pairs, one equilibrium evaluation per pair, approximate reciprocals and square roots,
 *   Float16C codes handled in a scaled form), held to a float32 tolerance of the exact step:
 *   after one step every float32 population within 1e-6 of it (plus 2e-6 relative for KBC and
 *   LES), every Float16C code within 1 unit in the last place.  Used by the block-per-tile and
 *   batched kernels; a grid those kernels do not take runs the exact arithmetic. */
enum { LBM_ARITH_EXACT = 0, LBM_ARITH_FAST = 1 };

/*
 * lbm_config_t mirrors LBM_Config (src/lbm/config.mojo:50-153).  The reference fixes these at
 * compile time; here they select a template instantiation at lbm_create.
 *   include_equilibrium_bc  <=>  Flags.EQUILIBRIUM in config.INCLUDED_BCs (config.mojo:141-151)
 *   Cs          Smagorinsky constant; the reference hard-codes 0.1 (steps/collide.mojo:200)
 *   trt_lambda  TRT magic parameter; the reference hard-codes 3/16 (steps/collide.mojo:214)
 *   arithmetic  LBM_ARITH_EXACT (default) or LBM_ARITH_FAST
 * Fill with lbm_config_default() before changing fields.
 */
typedef struct lbm_config_t {
    int32_t lbm_method;
    int32_t collision_op;
    int32_t LES;
    int32_t DDF_shift;
    int32_t use_float16c;
    int32_t include_moving_boundary;
    int32_t include_equilibrium_bc;
    int32_t capture_density;
    int32_t capture_velocity;
    float Cs;
    float trt_lambda;
    int32_t arithmetic;
} lbm_config_t;

/* lbm_grid_t mirrors LBM_Grid's comptime shape and tile (src/lbm/grid.mojo:55-107). */
typedef struct lbm_grid_t {
    int32_t lattice;           /* LBM_D2Q9 / LBM_D3Q19 / LBM_D3Q27                 */
    int32_t nx, ny, nz;        /* nz == 1 for D2Q9                                  */
    int32_t tx, ty, tz;        /* tile shape; each must divide its extent           */
} lbm_grid_t;

typedef struct lbm_handle lbm_handle;

/* ---- configuration ---- */

/* LBM_Config.__init__ defaults (config.mojo:85-99) for the given method. */
lbm_status lbm_config_default(lbm_config_t* cfg, int32_t lbm_method);

/* Host-only validation of a (config, grid) pair; needs no GPU.  The reference enforces the
 * same rules with comptime asserts (config.mojo:153, grid.mojo:301-305,345-365,434-438,
 * kernels/esoteric_pull.mojo:76-78).  Also refused here: fewer than 1 or 2^32 or more cells
 * (cell indices are 32-bit), a NaN or negative Cs with LES, and an arithmetic other than
 * LBM_ARITH_EXACT or LBM_ARITH_FAST. */
lbm_status lbm_validate(const lbm_config_t* cfg, const lbm_grid_t* grid);

/* Number of populations / spatial dimension of a lattice id, or -1. */
int32_t lbm_lattice_q(int32_t lattice);
int32_t lbm_lattice_d(int32_t lattice);

/* Element count of f / bc / flags for the grid (Q*N, (D+1)*N, N). */
int64_t lbm_f_elements(const lbm_grid_t* grid);
int64_t lbm_bc_elements(const lbm_grid_t* grid);
int64_t lbm_flag_elements(const lbm_grid_t* grid);

/* ---- handle ---- */

/* Solver.__init__ (solver.mojo:63-76): validates and selects the kernel for the current device. */
lbm_status lbm_create(const lbm_config_t* cfg, const lbm_grid_t* grid, lbm_handle** out);
lbm_status lbm_destroy(lbm_handle* h);

/* Solver(block_dim=...) override (solver.mojo:63-76): threads per block of the generic kernel
 * (multiple of 32, 32..256) or 0 for the built-in choice. */
lbm_status lbm_set_block_threads(lbm_handle* h, int32_t threads);

/* Kernel choice (no counterpart in the reference, which compiles one kernel per layout):
 * 0 = automatic (default), 1 = the generic kernel (any tile), 2 = the block-per-tile kernel,
 * which needs 256-cell tiles with power-of-two sides and Q*N < 2^31, 3 = the cell-pair
 * block-per-tile kernel (one thread per two cells along x, word-wide population accesses), which
 * also needs the double-buffer method and tx >= 2, 4 = the staged block-per-tile kernel (persistent
 * CTAs; bulk asynchronous copies stage the next tile's pull neighbourhood in shared memory while
 * the current tile is stepped), which needs the double-buffer method and tile rows of a multiple of
 * 16 bytes (tx >= 8 Float16C, tx >= 4 float32) (LBM_EUNSUPPORTED otherwise).  A step whose
 * population buffers are not 8-byte (path 3) or 16-byte (path 4) aligned, or a handle with the
 * learned closure or fused links, runs the block-per-tile kernel (or its variant) instead.  The
 * automatic choice is the cell-pair kernel for double-buffer D2Q9 / D3Q19 configurations other than
 * KBC with at least 2432 tiles (two waves of the pair kernel's CTAs on a 152-SM GPU; below that the
 * step is latency-bound and the per-cell kernel, with two threads per pair, finishes sooner), the
 * block-per-tile kernel for the other qualifying grids, the generic kernel otherwise.  With LBM_ARITH_EXACT all produce identical populations; the
 * generic kernel always computes the exact arithmetic. */
lbm_status lbm_set_kernel_path(lbm_handle* h, int32_t path);

/* The kernel lbm_*_step will use (aligned buffers): 1 generic, 2 block-per-tile, 3 cell-pair,
 * 4 staged, -1 for a null handle. */
int32_t lbm_kernel_path(const lbm_handle* h);

/* Waits for the device and reports the errors the kernels raised on the device since the last
 * call (no counterpart in the reference, whose kernels report nothing): LBM_ETIMEOUT when a wait of
 * the staged kernel for its bulk copies ran out (0.5 s); the steps it had not finished are lost
 * and the error is cleared.  LBM_OK otherwise. */
lbm_status lbm_device_status(lbm_handle* h);

/* Test hook (no counterpart in the reference): adds `bytes` (a multiple of 16) to the byte count
 * each stage of the staged kernel waits for, so that its bounded wait runs out; 0 restores it. */
lbm_status lbm_debug_stage_extra_bytes(lbm_handle* h, uint32_t bytes);

/* Test hook (no counterpart in the reference): the staged kernel's copy segments for a tile shape
 * (lattice, tx, ty, tz, bytes per population esz) as (source element, destination byte, bytes,
 * neighbour code) quadruples in out (at most max_segs); returns their count and the bytes of one
 * stage in *stage_bytes, 0 for a shape whose tile rows are not 16-byte multiples. */
int32_t lbm_stage_segments(int32_t lattice, int32_t tx, int32_t ty, int32_t tz, int32_t esz, uint32_t* out,
                           int32_t max_segs, uint32_t* stage_bytes);

/* ---- the step ---- */

/* Solver.double_buffer_step (solver.mojo:81-111) -> double_buffer_kernel
 * (kernels/double_buffer.mojo:25-99): one pull step f_in -> f_out.  bc is written only when
 * capture_density / capture_velocity are set. */
lbm_status lbm_double_buffer_step(lbm_handle* h, void* f_out, const void* f_in, float* bc,
                                  const uint8_t* flags, float tau, void* stream);

/* Solver.esoteric_pull_step[is_even_step] (solver.mojo:115-154) -> esoteric_pull_kernel
 * (kernels/esoteric_pull.mojo:24-111): one in-place step.  The initial state is stored with
 * the odd-step pattern, so the first step after initialisation is even. */
lbm_status lbm_esoteric_pull_step(lbm_handle* h, void* f, float* bc, const uint8_t* flags,
                                  float tau, int32_t is_even_step, void* stream);

/* The host time loop of examples/LDC.mojo:133-135 as one call: n_steps steps replayed from a
 * CUDA graph captured per (buffers, tau, parity).  Double buffer: step k reads f_a when
 * (first_step + k) is even, else f_b.  Esoteric pull: f_b is ignored and step k is even when
 * (first_step + k) is even. */
lbm_status lbm_run(lbm_handle* h, void* f_a, void* f_b, float* bc, const uint8_t* flags,
                   float tau, int64_t n_steps, int64_t first_step, void* stream);

/* ---- set-up and outputs ---- */

/* initialize_f_from_func / initialize_fluid_at_rest (preprocess/initial_condition.mojo:47-234):
 * f = f_eq(rho, u) (+ f_neq from the velocity gradient when grad != NULL), stored with the
 * double-buffer pattern or, for esoteric pull, the odd-step pattern.
 * u: [D][nx][ny][nz] floats (row-major, as the reference's velocity_layout, examples/LDC.mojo:48),
 * lattice units (NULL = at rest).  grad: [D*D][nx][ny][nz] floats, du_a/dx_b at component a*D+b
 * (NULL = no non-equilibrium part). */
lbm_status lbm_init_equilibrium(lbm_handle* h, void* f, float rho, float tau, const float* u,
                                const float* grad, void* stream);

/* calculate_rho_and_velocity (output/velocity.mojo:25-125).  rho: [nx][ny][nz] floats and
 * u: [D][nx][ny][nz] floats, row-major as the reference's density_layout / velocity_layout
 * (examples/LDC.mojo:47-48).  For esoteric pull, after_odd_step selects the load pattern
 * (ignored for double buffer). */
lbm_status lbm_compute_rho_u(lbm_handle* h, float* rho, float* u, const void* f, const float* bc,
                             const uint8_t* flags, int32_t after_odd_step, void* stream);

/* calculate_Q_criterion (output/Q_criterion.mojo:90-216): Q = |omega|^2 / 4 - |S|^2 / 2 into
 * q ([nx][ny][nz] floats, row-major), at every cell whose flag is not SOLID (raw compare; other
 * cells are left untouched).  S is the strain rate from the non-equilibrium second moment of the
 * next step's streamed populations (with boundary conditions) and `tau`; omega the curl of u
 * ([D][nx][ny][nz], as lbm_compute_rho_u writes it) by the reference's finite differences:
 * one-sided over 1 cell, or 1/2 toward a SOLID neighbour, weighted by the other side's spacing,
 * which makes a derivative across a non-periodic domain edge 0. */
lbm_status lbm_q_criterion(lbm_handle* h, float* q, const void* f, const float* bc, const uint8_t* flags,
                           const float* u, float tau, int32_t after_odd_step, void* stream);

/* Mass and momentum of all non-solid, non-excluded cells, reduced in float64 on the device:
 * out = {sum rho, sum rho*u_x, sum rho*u_y, sum rho*u_z}.  Synchronises the stream.
 * Returns LBM_ENAN if any reduced value is not finite. */
lbm_status lbm_reduce_mass_momentum(lbm_handle* h, const void* f, const uint8_t* flags,
                                    int32_t after_odd_step, double out[4], void* stream);

/* No counterpart in the reference.  The mass/momentum reduction above for callers that cannot
 * allocate device memory (an application-owned pool is their only allowed source, or the call
 * sits where cudaMalloc/cudaFree must not run): it needs no handle and allocates nothing.  Its
 * scratch is a fixed 1 MiB device array in the library, held by every GPU that loads it until the
 * process exits, so grids above 2^27 cells (512^3) are rejected with LBM_EINVAL.  The first call
 * on a device looks that array up (cudaGetSymbolAddress); make it before any stream capture.  The
 * address is kept for the life of the process: do not call this on a device after a
 * cudaDeviceReset of that device.
 * Calls share the array: calls that overlap on the GPU (other streams, other threads) race.
 * Same arguments and results as lbm_reduce_mass_momentum, with (cfg, grid) in place of a handle;
 * synchronises the stream. */
lbm_status lbm_reduce_mass_momentum_noalloc(const lbm_config_t* cfg, const lbm_grid_t* grid,
                                            const void* f, const uint8_t* flags,
                                            int32_t after_odd_step, double out[4], void* stream);

/* linkwise_bounceback_kernel (geometry/interpolated_BB.mojo:46-141) as launched by
 * RigidStationaryObject.bounceback (geometry/rigidstationary.mojo:127-153): per link, in place
 * on the lattice the last double-buffer step wrote.  fluid_ids are linear flag-layout indices,
 * dirs the direction pointing into the wall, dists the wall distance q in [0,1].
 * link_force (n_links*D floats, link fastest) is written when compute_force != 0.
 * method: LBM_BB_MID_GRID or LBM_BB_BOUZIDI. */
lbm_status lbm_linkwise_bounceback(lbm_handle* h, void* f, float* link_force,
                                   const int32_t* fluid_ids, const int32_t* dirs,
                                   const float* dists, int64_t n_links, int32_t method,
                                   int32_t compute_force, float q_clamp, void* stream);

/* Interpolated bounce-back fused into the step: the node-wise form of the reference's WIP kernel
 * nodewise_bounceback_kernel (geometry/nodewise_interpolated_BB.mojo:46-185), with the
 * interpolation of its link-wise kernel (geometry/interpolated_BB.mojo:102-141).  Registers the links
 * (device arrays as lbm_linkwise_bounceback takes them; copied into a per-cell table, so the caller
 * may free them) with the handle: from the next step on, every double-buffer step applies them
 * inside the step kernel, in place of a link-wise pass after it.  A fluid cell with a link (x, i)
 * whose wall node x + c_i is a raw SOLID flag replaces its mid-grid bounce-back value of direction
 * opp(i) by the value the link-wise kernel would have stored at (x, i) after the previous step, and
 * writes that link's force (c_i (f_into + f_bb), n_links*D floats, link fastest, in the caller's link
 * order) into link_force when it is not NULL.  The lattice therefore holds the step's own values in
 * the link slots (x, i): one lbm_linkwise_bounceback pass (method, q_clamp, no force) turns it into
 * the lattice the link-wise path has after the same steps, and the forces written by step k are
 * the link-wise path's of step k-1.  n_links = 0 removes the links.  Needs the block-per-tile
 * kernel (LBM_EUNSUPPORTED otherwise); waits for the device to be idle: call it between steps.
 * LBM_EINVAL for an id outside the grid, a direction outside [1, Q), a NaN distance or two links
 * with the same cell and direction. */
lbm_status lbm_set_links(lbm_handle* h, const int32_t* fluid_ids, const int32_t* dirs, const float* dists,
                         int64_t n_links, int32_t method, float q_clamp, float* link_force, void* stream);

/* RigidStationaryObject.sum_force (geometry/rigidstationary.mojo:155-169): column sums of a
 * link-force array, reduced in float64 on the device.  Synchronises the stream. */
lbm_status lbm_sum_link_force(lbm_handle* h, const float* link_force, int64_t n_links,
                              double out[3], void* stream);

/* calculate_drag_around_object (output/drag.mojo:16-105): momentum-exchange force per listed
 * fluid node (n_nodes*D floats, node fastest). */
lbm_status lbm_drag_force(lbm_handle* h, float* node_force, const void* f, const uint8_t* flags,
                          const int32_t* fluid_ids, int64_t n_nodes, void* stream);

/* ---- batched persistent step ----
 * No counterpart in the reference, whose grid sizes are compile-time parameters
 * (src/lbm/grid.mojo:55-66), so one kernel launch steps one domain.  A batch steps many domains
 * of different sizes (same lattice and config) in one persistent launch: every 256-cell tile of
 * every domain is a work unit, and each domain is stepped exactly as lbm_*_step would step it
 * (identical results).  Each grid needs a 256-cell tile with power-of-two sides and Q*N < 2^31. */
typedef struct lbm_batch lbm_batch;

lbm_status lbm_batch_create(const lbm_config_t* cfg, int32_t n_domains, const lbm_grid_t* grids,
                            lbm_batch** out);
lbm_status lbm_batch_destroy(lbm_batch* b);

/* Buffers and tau of domain i (device pointers, the domain's own layout).  Double buffer: step k
 * of lbm_batch_run reads f_a when (first_step + k) is even, else f_b.  Esoteric pull: f_b unused. */
lbm_status lbm_batch_set_domain(lbm_batch* b, int32_t i, void* f_a, void* f_b, float* bc,
                                const uint8_t* flags, float tau);

/* Link-wise bounce-back after every batched step (interpolated_BB.mojo:46-141): device arrays of
 * n_links entries, each link naming its domain; fluid_ids are flag-layout indices within that
 * domain.  link_force (n_links*D floats, link fastest) may be NULL.  Double buffer only. */
lbm_status lbm_batch_set_links(lbm_batch* b, const int32_t* domain, const int32_t* fluid_ids,
                               const int32_t* dirs, const float* dists, int64_t n_links,
                               int32_t method, float q_clamp, float* link_force);

/* How lbm_batch_run applies the links of lbm_batch_set_links: LBM_LINKS_SEPARATE (default) runs the
 * link-wise kernel over all links after every batched step; LBM_LINKS_FUSED applies them inside the
 * batched step kernel as lbm_set_links does for one domain (one kernel per step; the link slots hold
 * the step's own values and the forces lag one step, as described there).  The fused tables are
 * built from the link arrays at the next lbm_batch_run (the arrays must still hold the links then).
 * Double buffer only (LBM_EUNSUPPORTED otherwise). */
enum { LBM_LINKS_SEPARATE = 0, LBM_LINKS_FUSED = 1 };
lbm_status lbm_batch_set_link_mode(lbm_batch* b, int32_t mode);

/* n_steps steps of every domain, replayed from a CUDA graph of 64 steps. */
lbm_status lbm_batch_run(lbm_batch* b, int64_t n_steps, int64_t first_step, void* stream);

/* Total cells of the batch (-1 for a null batch). */
int64_t lbm_batch_cells(const lbm_batch* b);

/* ---- learned subgrid closure ----
 * No counterpart in the reference, whose LES is Smagorinsky with Cs = 0.1
 * (ops/turbulence.mojo:12-38).  A per-cell MLP 8 -> 32 -> 32 -> 1 (ReLU hidden layers, softplus
 * output) maps invariants of the non-equilibrium strain, rho and |u| to an eddy viscosity
 * nu_t = softplus(y) * nu_scale; tau_eddy = 3 nu_t replaces Smagorinsky's.  Cells whose
 * normalised features leave [feat_lo, feat_hi] (the training range) keep Smagorinsky.  Inference
 * runs inside the collision of LES configurations on the tensor cores (BF16 weights and
 * activations, FP32 accumulation).  Features, with S the strain rate from the non-equilibrium
 * stress (moment.mojo:154-176), s2 its squared norm (off-diagonals twice), q = 2 s2 + 1e-24:
 *   x0 ln(q) / 2                 x1 tr(S) / sqrt(q)
 *   x2 det(S - tr(S)/D I) / q^(3/2)   x3 rho - 1
 *   x4 |u|                       x5 2 (Sxy^2 + Sxz^2 + Syz^2) / s2 (as 4 (...) / q)
 *   x6 ln(tau - 0.5)             x7 |u|^2 / sqrt(q)
 * (the kernel evaluates them with approximate rsqrt, sqrt and log2), normalised as
 * fma(x, feat_scale, -feat_mean * feat_scale).  Weights are stored input-major:
 * w1[k*32 + j] links input k to hidden unit j, w2[k*32 + j] likewise, w3[k] hidden k to y. */
typedef struct lbm_closure_t {
    float w1[8 * 32];
    float b1[32];
    float w2[32 * 32];
    float b2[32];
    float w3[32];
    float b3;
    float nu_scale;
    float feat_mean[8];
    float feat_scale[8];
    float feat_lo[8];
    float feat_hi[8];
} lbm_closure_t;

/* Use the learned closure in an LES handle (copied; NULL returns to Smagorinsky).  Waits for the
 * device to be idle first: call it between steps. */
lbm_status lbm_set_closure(lbm_handle* h, const lbm_closure_t* closure);

/* Training kernels of the closure (float32).  theta: the 1377 parameters packed as
 * w1, b1, w2, b2, w3, b3.  x: n rows of 8 normalised features; nu: n outputs
 * softplus(y) * nu_scale.  lbm_mlp_backward writes d(sum_i g_i nu_i)/d theta into grad_theta
 * (summed in a fixed order: repeatable).  lbm_mlp_adam applies one Adam step to n_params
 * parameters with moments m, v (t = step count from 1). */
lbm_status lbm_mlp_forward(const float* theta, const float* x, int64_t n, float nu_scale, float* nu,
                           void* stream);
lbm_status lbm_mlp_backward(const float* theta, const float* x, const float* g, int64_t n,
                            float nu_scale, float* grad_theta, void* stream);
lbm_status lbm_mlp_adam(float* theta, const float* grad, float* m, float* v, int32_t n_params,
                        float lr, float beta1, float beta2, float eps, int32_t t, void* stream);

/* ---- autotuner ----
 * No counterpart in the reference (its tile and block shapes are compile-time choices,
 * grid.mojo:55-107).  lbm_tune_candidates lists the 256-cell power-of-two tiles (tx, ty, tz)
 * that divide the grid (the layouts the block-per-tile kernel runs), writing at most max triples
 * into tiles (may be NULL); it returns their number, or -1 for a bad lattice or shape.  No GPU is
 * used.  lbm_autotune times every candidate tile (and both streaming methods when choose_method
 * is non-zero) for the configuration, `steps` graph-replayed steps each from rest, and returns
 * the fastest.  flags and bc are the caller's device arrays in the untiled layout (x fastest,
 * then y, z, and the bc component slowest); they are laid out for each candidate.  NULL flags
 * time a periodic box of fluid instead, which favours tiles a walled domain would not.  It
 * allocates scratch buffers of the grid's size and frees them before returning.
 * LBM_EUNSUPPORTED when no candidate tile divides the grid. */
typedef struct lbm_tune_result_t {
    int32_t tx, ty, tz;       /* fastest tile */
    int32_t lbm_method;       /* its streaming method (the configuration's unless chosen) */
    float mlups;              /* its measured throughput */
    int32_t n_candidates;     /* candidates timed */
} lbm_tune_result_t;

int32_t lbm_tune_candidates(int32_t lattice, int32_t nx, int32_t ny, int32_t nz, int32_t* tiles,
                            int32_t max);
lbm_status lbm_autotune(const lbm_config_t* cfg, int32_t lattice, int32_t nx, int32_t ny, int32_t nz,
                        const uint8_t* flags, const float* bc, int32_t choose_method, int32_t steps,
                        lbm_tune_result_t* out, void* stream);

/* ---- wall and shape painting on the device ----
 * Flags and boundary values painted straight into the caller's device arrays (grid layout), for
 * set-ups too large to paint on the host (the 512^3 run, 512 batched channels).
 *
 * lbm_paint_wall replaces set_exterior_walls (src/lbm/preprocess/boundary_condition.mojo:78-183):
 * every cell of the exterior face `side` (0..5 = "-X", "+X", "-Y", "+Y", "-Z", "+Z") gets flag
 * boundary_type and bc (u[0..D-1], rho).  u = NULL leaves the velocity free (NaN); rho NaN leaves
 * the density free.  It checks what the reference's _error_check checks (boundary_condition.mojo:
 * 20-69) against cfg: the type must be FLUID, SOLID or (with include_equilibrium_bc) EQUILIBRIUM;
 * u and rho cannot both be free; a given u has no NaN component; SOLID needs u and rho, and a
 * non-zero u needs include_moving_boundary; EQUILIBRIUM with u needs rho.  Values are lattice
 * units (a unit system converts on the host first).
 * lbm_paint_wall_values replaces set_exterior_walls_with_func (:186-309): u_face holds D device
 * arrays of the face's cell count, component-major, cells ordered by the face's first free axis
 * fastest (y then z for an X face, x then z for Y, x then y for Z).
 * lbm_paint_sphere / lbm_paint_box replace add_sphere / add_circle / add_box
 * (src/lbm/geometry/primatives.mojo:110-240): SOLID in every cell of the reference's bounding box
 * whose coordinate origin + n dx lies inside, tested in float32 in the reference's operation
 * order (sphere: ((x-cx)^2 + (y-cy)^2) + (z-cz)^2 <= r^2; box: |coordinate - centre| <= half
 * extent on every axis). */
lbm_status lbm_paint_wall(const lbm_config_t* cfg, const lbm_grid_t* grid, uint8_t* flags, float* bc,
                          int32_t side, uint8_t boundary_type, const float* u, float rho, void* stream);
lbm_status lbm_paint_wall_values(const lbm_config_t* cfg, const lbm_grid_t* grid, uint8_t* flags, float* bc,
                                 int32_t side, uint8_t boundary_type, const float* u_face, float rho,
                                 void* stream);
lbm_status lbm_paint_sphere(const lbm_grid_t* grid, uint8_t* flags, const float center[3], float radius,
                            const float origin[3], float dx, void* stream);
lbm_status lbm_paint_box(const lbm_grid_t* grid, uint8_t* flags, const float center[3], const float half[3],
                         const float origin[3], float dx, void* stream);

/* Float16C codec (src/utils/custom_fp.mojo:36-101) over device arrays. */
lbm_status lbm_float16c_encode(const float* in, uint16_t* out, int64_t n, void* stream);
lbm_status lbm_float16c_decode(const uint16_t* in, float* out, int64_t n, void* stream);

/* Message of the last failed call on this thread ("" if none). */
const char* lbm_last_error(void);

/* Library version string. */
const char* lbm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
