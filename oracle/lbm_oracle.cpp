/*
 * TEST INFRASTRUCTURE — CPU oracle for the fused LBM stream–collide step.
 *
 * Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library, and
 * only as the values the tests compare against or as the timed CPU baseline.  The product
 * (mojo_lbm_gb300, the CUDA library) never calls it.
 *
 * It restates, scalar and cell by cell, the algorithm of JohnCSu/mojo_lbm's GPU step in the
 * same operation order (sequential sums over q = 0..Q-1, src/utils/vector.mojo:205-224).  It is
 * built twice through templates: R = float (parity with the float32 kernels) and R = double
 * (the float64 oracle used to state the error of the float32 and Float16C paths).
 *
 * PARITY UNPINNED: the reference is Mojo 1.0 / MAX 26.5, which is not installed here, and its
 * repository holds no golden vectors for this path (its tests are compile-and-run scripts,
 * compiletest.py:21-80).  The oracle is checked against the fixtures the reference holds for the
 * path — the Ghia et al. lid-driven-cavity centre lines (benchmarks/LDC/) and the DFG Re = 20
 * cylinder drag the reference recorded at three resolutions
 * (benchmarks/Cylinder2D/CylinderFlow_Re20.mojo) — against the velocity sets, stress-component
 * order, node flags and configuration defaults extracted from the reference's sources, and against
 * conservation and symmetry invariants.
 *
 * Deviations from the reference, each deliberate:
 *  - capture_density/capture_velocity store rho into bc[x,y,z,D] and u into bc[x,y,z,0..D-1];
 *    the reference indexes index[3] there (kernels/utils/index.mojo:121), out of range.
 *  - linkwise bounce-back decodes Float16C when use_float16c is set; the reference passes
 *    DDF_shift as load_f's use_float16c argument (geometry/interpolated_BB.mojo:119,123,129),
 *    which does not compile for float32 storage with DDF shift.  Its link force adds the weight
 *    under DDF shift, as output/drag.mojo:88-93 does.
 *  - KBC for D3Q19/D3Q27 (the reference asserts D2Q9 only, ops/collisions/KBC_.mojo:220) uses
 *    the shear part of the deviatoric non-equilibrium stress (Karlin, Bösch, Chikatamarla,
 *    PRE 90, 031302, 2014): faces (2N_xz - N_yz)/6, (-N_xz + 2N_yz)/6, (-N_xz - N_yz)/6 with
 *    N_xz = P_xx - P_zz, N_yz = P_yy - P_zz; edges s_a s_b P_ab / 4; corners and rest 0.
 *    For D2Q9 this reduces exactly to get_shear_D2Q9 (KBC_.mojo:137-175).
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/lbm_gb300.h"

namespace {

/* ------------------------------------------------------------------------------------------
 * Lattices: exact direction order and weights of get_D2Q9 / get_D3Q19 / get_D3Q27
 * (src/lbm/lattice.mojo:122-352).  Opposites are adjacent: q odd, q+1 = opposite.
 * ---------------------------------------------------------------------------------------- */
struct LatticeDef {
    int D, Q;
    int c[27][3];
    double w[27];
    int opp[27];
};

const int kC27[27][3] = {
    {0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0},  {0, 0, 1},  {0, 0, -1},
    {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},  {-1, 1, 0},  {1, 0, 1},   {-1, 0, -1}, {1, 0, -1},
    {-1, 0, 1},  {0, 1, 1},   {0, -1, -1}, {0, 1, -1},  {0, -1, 1},  {1, 1, 1},   {-1, -1, -1},
    {1, 1, -1},  {-1, -1, 1}, {1, -1, 1},  {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}};

const int kC9[9][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0}, {0, -1, 0},
                       {1, 1, 0},  {-1, -1, 0}, {-1, 1, 0}, {1, -1, 0}};

LatticeDef make_lattice(int id) {
    LatticeDef L{};
    if (id == LBM_D2Q9) {
        L.D = 2; L.Q = 9;
        for (int q = 0; q < 9; ++q) for (int d = 0; d < 3; ++d) L.c[q][d] = kC9[q][d];
        const double w[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                             1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
        for (int q = 0; q < 9; ++q) L.w[q] = w[q];
    } else {
        const bool q27 = (id == LBM_D3Q27);
        L.D = 3; L.Q = q27 ? 27 : 19;
        for (int q = 0; q < L.Q; ++q) for (int d = 0; d < 3; ++d) L.c[q][d] = kC27[q][d];
        for (int q = 0; q < L.Q; ++q) {
            const int nnz = (L.c[q][0] != 0) + (L.c[q][1] != 0) + (L.c[q][2] != 0);
            if (q27) L.w[q] = nnz == 0 ? 8.0 / 27.0 : nnz == 1 ? 2.0 / 27.0 : nnz == 2 ? 1.0 / 54.0 : 1.0 / 216.0;
            else     L.w[q] = nnz == 0 ? 1.0 / 3.0 : nnz == 1 ? 1.0 / 18.0 : 1.0 / 36.0;
        }
    }
    /* Lattice._get_opposite_indices (lattice.mojo:76-91) */
    for (int i = 0; i < L.Q; ++i)
        for (int k = 0; k < L.Q; ++k)
            if (L.c[k][0] == -L.c[i][0] && L.c[k][1] == -L.c[i][1] && L.c[k][2] == -L.c[i][2]) { L.opp[i] = k; break; }
    return L;
}

/* get_stress_indices (lattice.mojo:354-398) */
const int kStress2[3][2] = {{0, 0}, {0, 1}, {1, 1}};
const int kStress3[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};

/* ------------------------------------------------------------------------------------------
 * Float16C (src/utils/custom_fp.mojo:36-101; FluidX3D, Lehmann et al. PRE 106, 015308, 2022).
 * 1 sign, 4 exponent, 11 mantissa bits; exponent offset 112 relative to float32.
 * ---------------------------------------------------------------------------------------- */
inline uint32_t f2u(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
inline float u2f(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }

float f16c_to_f32(uint16_t h) {
    const uint32_t e = (uint32_t)(h & 0x7800u) >> 11;
    const uint32_t m = (uint32_t)(h & 0x07FFu) << 12;
    uint32_t r = (uint32_t)(h & 0x8000u) << 16;
    if (e != 0) r |= ((e + 112u) << 23) | m;
    if (e == 0 && m != 0) {
        /* renormalise a denormal code: v is the biased exponent of float(m) */
        const uint32_t v = f2u((float)m) >> 23;
        r |= ((v - 37u) << 23) | ((m << (150u - v)) & 0x007FF000u);
    }
    return u2f(r);
}

uint16_t f32_to_f16c(float x) {
    const uint32_t b = f2u(x) + 0x00000800u; /* round half up on the 12th dropped bit */
    const uint32_t e = (b & 0x7F800000u) >> 23;
    const uint32_t m = b & 0x007FFFFFu;
    uint32_t r = (b & 0x80000000u) >> 16;
    if (e > 112u) r |= (((e - 112u) << 11) & 0x7800u) | (m >> 12);
    if (e < 113u && e > 100u) r |= (((0x007FF800u + m) >> (124u - e)) + 1u) >> 1;
    if (e > 127u) r |= 0x7FFFu;
    return (uint16_t)(r & 0xFFFFu); /* the low 16 bits, as bitcast[uint16,2](...)[0] */
}

/* ------------------------------------------------------------------------------------------
 * Tiled layout (src/lbm/layoutstruct.mojo:37-92): blocked_product(col_major tile, col_major
 * tiler); per mode the coordinate is (local, tile).
 * ---------------------------------------------------------------------------------------- */
struct Layout {
    int64_t nx, ny, nz, tx, ty, tz, ntx, nty, ntz, T;
    int64_t cell(int64_t x, int64_t y, int64_t z, int64_t q, int64_t K) const {
        const int64_t tile = x / tx + ntx * (y / ty + nty * (z / tz));
        return (x % tx) + tx * ((y % ty) + ty * (z % tz)) + T * (q + K * tile);
    }
    int64_t flag(int64_t x, int64_t y, int64_t z) const { return cell(x, y, z, 0, 1); }
};

Layout make_layout(const lbm_grid_t* g) {
    Layout l;
    l.nx = g->nx; l.ny = g->ny; l.nz = g->nz; l.tx = g->tx; l.ty = g->ty; l.tz = g->tz;
    l.ntx = l.nx / l.tx; l.nty = l.ny / l.ty; l.ntz = l.nz / l.tz; l.T = l.tx * l.ty * l.tz;
    return l;
}

/* get_adjacent_idx (kernels/utils/index.mojo:44-64): floor-mod wrap per active axis. */
inline int64_t wrap(int64_t i, int64_t n) { int64_t r = i % n; return r < 0 ? r + n : r; }

/* Storage access: load_f / store_f (kernels/utils/load_and_store.mojo:17-110). */
template <class S> struct Store;
template <> struct Store<float> {
    static double ld(const float* p, int64_t i) { return p[i]; }
    static void st(float* p, int64_t i, double v) { p[i] = (float)v; }
};
template <> struct Store<double> {
    static double ld(const double* p, int64_t i) { return p[i]; }
    static void st(double* p, int64_t i, double v) { p[i] = v; }
};
template <> struct Store<uint16_t> {
    static double ld(const uint16_t* p, int64_t i) { return f16c_to_f32(p[i]); }
    static void st(uint16_t* p, int64_t i, double v) { p[i] = f32_to_f16c((float)v); }
};

inline bool flag_is(uint8_t f, uint8_t e) { return (f & 0x0F) == e; } /* Flags.is (constants.mojo:88) */

/* ------------------------------------------------------------------------------------------
 * The step.  R is the arithmetic type; every intermediate is rounded to R exactly where the
 * reference's Scalar[float_dtype] arithmetic rounds (compiled with -ffp-contract=off).
 * ---------------------------------------------------------------------------------------- */
/* ---- learned subgrid closure (no counterpart in the reference; the GPU evaluates it on the
 * tensor cores).  BF16 rounding of weights and activations is emulated, products and sums are
 * taken in R, so the GPU matches this within the order of its FP32 accumulation. */
bool g_closure_on = false;
lbm_closure_t g_closure;

float bf16_round(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7FFFFFFFu) > 0x7F800000u) return x;
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

/* Features x0..x7 of the cell (the lbm_closure_t comment in include/lbm_gb300.h lists them).
 * S in stress order (2D xx, xy, yy; 3D xx, xy, xz, yy, yz, zz). */
template <class R>
void closure_features(int D, const R* S, R s2, R rho, R uu, R tau, R* x) {
    R tr, det, off;
    if (D == 3) {
        tr = S[0] + S[3] + S[5];
        const R m = tr / (R)3;
        const R a = S[0] - m, b = S[3] - m, c = S[5] - m;
        det = a * (b * c - S[4] * S[4]) - S[1] * (S[1] * c - S[4] * S[2]) + S[2] * (S[1] * S[4] - b * S[2]);
        off = (R)2 * (S[1] * S[1] + S[2] * S[2] + S[4] * S[4]);
    } else {
        tr = S[0] + S[2];
        const R m = tr / (R)2;
        const R a = S[0] - m, b = S[2] - m;
        det = a * b - S[1] * S[1];
        off = (R)2 * (S[1] * S[1]);
    }
    const R q = (R)2 * s2 + (R)1e-24;
    const R sq = std::sqrt(q);
    x[0] = std::log(q) / (R)2;
    x[1] = tr / sq;
    x[2] = det / (q * sq);
    x[3] = rho - (R)1;
    x[4] = std::sqrt(uu);
    x[5] = (R)2 * off / q;
    x[6] = std::log(tau - (R)0.5);
    x[7] = uu / sq;
}

/* nu_t of the learned closure, or -1 when a normalised feature leaves the training range. */
template <class R>
R closure_nu(const R* x) {
    const lbm_closure_t& c = g_closure;
    float xn[8];
    for (int k = 0; k < 8; ++k) {
        const float shift = -(c.feat_mean[k] * c.feat_scale[k]);
        const float v = std::fma((float)x[k], c.feat_scale[k], shift);
        if (!(v >= c.feat_lo[k] && v <= c.feat_hi[k])) return (R)-1;
        xn[k] = bf16_round(v);
    }
    R h1[32], h2[32];
    for (int j = 0; j < 32; ++j) {
        R a = (R)c.b1[j];
        for (int k = 0; k < 8; ++k) a += (R)xn[k] * (R)bf16_round(c.w1[k * 32 + j]);
        h1[j] = (R)bf16_round((float)(a > 0 ? a : 0));
    }
    for (int j = 0; j < 32; ++j) {
        R a = (R)c.b2[j];
        for (int k = 0; k < 32; ++k) a += h1[k] * (R)bf16_round(c.w2[k * 32 + j]);
        h2[j] = (R)bf16_round((float)(a > 0 ? a : 0));
    }
    R y = (R)c.b3;
    for (int k = 0; k < 32; ++k) y += h2[k] * (R)bf16_round(c.w3[k]);
    const R sp = y > (R)20 ? y : std::log1p(std::exp(y));
    return sp * (R)c.nu_scale;
}

template <class R, class S> struct Stepper {
    const lbm_config_t& cfg;
    const LatticeDef& L;
    const Layout& lay;
    R w[27];       /* weights as Scalar[float_dtype] */
    R six_w[27];   /* 2.*3.*weight  (ops/boundary_condition.mojo:83) */
    R rl_k[27];    /* weights[q]/(2*cs_squared*cs_squared) (ops/collisions/collision.mojo:219) */
    R cs2;         /* cs_squared as Scalar[float_dtype] */

    Stepper(const lbm_config_t& c, const LatticeDef& l, const Layout& y) : cfg(c), L(l), lay(y) {
        for (int q = 0; q < L.Q; ++q) {
            w[q] = (R)L.w[q];
            six_w[q] = (R)((R)6 * w[q]);
            rl_k[q] = (R)(w[q] / (R)(2.0 / 9.0));
        }
        cs2 = (R)(1.0 / 3.0);
    }

    int nstress() const { return L.D == 2 ? 3 : 6; }
    int sa(int n) const { return L.D == 2 ? kStress2[n][0] : kStress3[n][0]; }
    int sb(int n) const { return L.D == 2 ? kStress2[n][1] : kStress3[n][1]; }

    /* dot(velocity, direction) (kernels/utils/equilibrium.mojo:36 -> vector.mojo:205) */
    R edot(const R* u, int q) const {
        R o = 0;
        for (int d = 0; d < L.D; ++d) o = o + u[d] * (R)L.c[q][d];
        return o;
    }
    R udot(const R* u) const {
        R o = 0;
        for (int d = 0; d < L.D; ++d) o = o + u[d] * u[d];
        return o;
    }

    /* f_eq (kernels/utils/equilibrium.mojo:10-39) */
    R feq(int q, R rho, const R* u, R uu, bool ddf) const {
        const R eu = edot(u, q);
        if (ddf) return w[q] * rho * ((R)3 * eu + (R)4.5 * eu * eu - (R)1.5 * uu) + w[q] * (rho - (R)1);
        return w[q] * rho * ((R)1 + (R)3 * eu + (R)4.5 * eu * eu - (R)1.5 * uu);
    }

    /* get_density / get_velocity (kernels/utils/moment.mojo:17-76) */
    R density(const R* f) const {
        R s = 0;
        for (int q = 0; q < L.Q; ++q) s = s + f[q];
        if (cfg.DDF_shift) s = s + (R)1;
        return s;
    }
    void velocity(const R* f, R rho, R* u) const {
        R acc[3] = {0, 0, 0};
        for (int q = 0; q < L.Q; ++q)
            for (int d = 0; d < L.D; ++d) acc[d] = acc[d] + f[q] * (R)L.c[q][d];
        for (int d = 0; d < L.D; ++d) u[d] = acc[d] / rho;
    }

    /* KBC shear part s_q as a linear map of the stress vector (see the header comment). */
    R shear(int q, const R* P) const {
        const int* c = L.c[q];
        const int nnz = (c[0] != 0) + (c[1] != 0) + (c[2] != 0);
        if (L.D == 2) {
            /* get_shear_D2Q9 (ops/collisions/KBC_.mojo:137-175): N = P_xx - P_yy */
            const R N = P[0] - P[2];
            if (nnz == 1) return c[0] != 0 ? N * (R)0.25 : -N * (R)0.25;
            if (nnz == 2) return (c[0] * c[1] > 0) ? P[1] * (R)0.25 : -P[1] * (R)0.25;
            return 0;
        }
        if (nnz == 1) {
            const R Nxz = P[0] - P[5], Nyz = P[3] - P[5];
            const R sixth = (R)(1.0 / 6.0);
            if (c[0] != 0) return ((R)2 * Nxz - Nyz) * sixth;
            if (c[1] != 0) return ((R)2 * Nyz - Nxz) * sixth;
            return (-Nxz - Nyz) * sixth;
        }
        if (nnz == 2) {
            const R quarter = (R)0.25;
            if (c[2] == 0) return (R)(c[0] * c[1]) * P[1] * quarter;
            if (c[1] == 0) return (R)(c[0] * c[2]) * P[2] * quarter;
            return (R)(c[1] * c[2]) * P[4] * quarter;
        }
        return 0;
    }

    /* collide (kernels/steps/collide.mojo:23-90) */
    void collide(R* f, R tau, R* bc, int64_t cell_bc_x, int64_t cell_bc_y, int64_t cell_bc_z, uint8_t own_flag) const {
        const bool ddf = cfg.DDF_shift != 0;
        const R rho = density(f);
        R u[3] = {0, 0, 0};
        velocity(f, rho, u);
        R tau_local = tau;
        if (cfg.capture_density && (own_flag & LBM_FLAG_CAPTURE_DENSITY))
            bc[lay.cell(cell_bc_x, cell_bc_y, cell_bc_z, L.D, L.D + 1)] = rho;
        if (cfg.capture_velocity && (own_flag & LBM_FLAG_CAPTURE_VELOCITY))
            for (int d = 0; d < L.D; ++d) bc[lay.cell(cell_bc_x, cell_bc_y, cell_bc_z, d, L.D + 1)] = u[d];

        const bool need_neq = cfg.LES || cfg.collision_op == LBM_KBC || cfg.collision_op == LBM_RLBM;
        if (need_neq) {
            const R uu = udot(u);
            R fneq[27], P[6];
            for (int q = 0; q < L.Q; ++q) fneq[q] = f[q] - feq(q, rho, u, uu, ddf);
            /* get_non_eq_second_order_moment (moment.mojo:111-150) */
            for (int n = 0; n < nstress(); ++n) {
                R s = 0;
                for (int q = 0; q < L.Q; ++q) s = s + fneq[q] * (R)L.c[q][sa(n)] * (R)L.c[q][sb(n)];
                P[n] = s;
            }
            if (cfg.LES) {
                /* get_strain_rate_tensor (moment.mojo:154-176), norm (:182-215),
                 * get_Smagorinsky_LES_tau (ops/turbulence.mojo:12-38) */
                const R k = (R)-1 / ((R)2 * rho * cs2 * tau_local);
                R s2 = 0, Sv[6];
                for (int n = 0; n < nstress(); ++n) {
                    const R Sn = P[n] * k;
                    Sv[n] = Sn;
                    const R ss = Sn * Sn;
                    s2 = (sa(n) != sb(n)) ? s2 + ss * (R)2 : s2 + ss;
                }
                const R Cs = (R)cfg.Cs;
                R v_eddy = (Cs * Cs) * (R)std::sqrt((R)2 * s2);
                if (g_closure_on) {  /* learned closure; Smagorinsky outside the training range */
                    R x[8];
                    closure_features<R>(L.D, Sv, s2, rho, uu, tau_local, x);
                    const R nu = closure_nu<R>(x);
                    if (nu >= 0) v_eddy = nu;
                }
                tau_local = tau_local + (R)3 * v_eddy;
            }
            if (cfg.collision_op == LBM_RLBM) {
                /* RLBM (ops/collisions/collision.mojo:168-223) */
                const R inv_tau = (R)1 / tau_local;
                for (int q = 0; q < L.Q; ++q) {
                    R dot = 0;
                    for (int n = 0; n < nstress(); ++n) {
                        const int a = sa(n), b = sb(n);
                        R Qn = (R)L.c[q][a] * (R)L.c[q][b];
                        Qn = (a == b) ? Qn - cs2 : Qn * (R)2; /* get_kbc_Qiab (:121-166) */
                        dot = dot + Qn * P[n];
                    }
                    const R fneq_reg = rl_k[q] * dot;
                    f[q] = feq(q, rho, u, uu, ddf) + ((R)1 - inv_tau) * fneq_reg;
                }
            } else if (cfg.collision_op == LBM_KBC) {
                /* KBC (ops/collisions/KBC_.mojo:180-238) */
                const R beta = (R)1 / ((R)2 * tau_local);
                const R inv_beta = (R)2 * tau_local;
                R feq0[27], ds[27], dh[27];
                for (int q = 0; q < L.Q; ++q) feq0[q] = feq(q, rho, u, uu, false);
                for (int q = 0; q < L.Q; ++q) { ds[q] = shear(q, P); dh[q] = fneq[q] - ds[q]; }
                R sp1 = 0, sp2 = 0;
                for (int q = 0; q < L.Q; ++q) sp1 = sp1 + ds[q] * dh[q] / feq0[q];
                for (int q = 0; q < L.Q; ++q) sp2 = sp2 + dh[q] * dh[q] / feq0[q];
                const R gamma = inv_beta - ((R)2 - inv_beta) * sp1 / (sp2 + (R)1e-32);
                for (int q = 0; q < L.Q; ++q) f[q] = f[q] - beta * ((R)2 * ds[q] + gamma * dh[q]);
            }
        }
        if (cfg.collision_op == LBM_SRT) {
            /* SRT (ops/collisions/collision.mojo:12-46) */
            const R uu = udot(u);
            const R inv_tau = (R)1 / tau_local;
            for (int q = 0; q < L.Q; ++q) f[q] = f[q] - inv_tau * (f[q] - feq(q, rho, u, uu, ddf));
        } else if (cfg.collision_op == LBM_TRT) {
            /* TRT (ops/collisions/collision.mojo:49-113), tau_asymm from steps/collide.mojo:214-215 */
            const R tau_asym = (R)0.5 + (R)cfg.trt_lambda / (tau_local - (R)0.5);
            const R is = (R)1 / tau_local, ia = (R)1 / tau_asym;
            const R uu = udot(u);
            f[0] = f[0] - is * (f[0] - feq(0, rho, u, uu, ddf));
            for (int q = 1; q < L.Q; q += 2) {
                const int o = q + 1;
                const R fs = (f[q] + f[o]) * (R)0.5, fa = (f[q] - f[o]) * (R)0.5;
                const R eq = feq(q, rho, u, uu, ddf), eo = feq(o, rho, u, uu, ddf);
                const R es = (eq + eo) * (R)0.5, ea = (eq - eo) * (R)0.5;
                f[q] = f[q] - (is * (fs - es) + ia * (fa - ea));
                f[o] = f[o] - (is * (fs - es) + ia * ((-fa) - (-ea)));
            }
        }
    }

    /* One cell of the step.  f_out == f_in for esoteric pull (in place). */
    void cell(int64_t x, int64_t y, int64_t z, S* f_out, const S* f_in, R* bc, const uint8_t* flags,
              R tau, bool even) const {
        const uint8_t flag = flags[lay.flag(x, y, z)];
        /* is_valid_thread (kernels/utils/checks.mojo:55-60) */
        if (flag_is(flag, LBM_FLAG_SOLID) || (flag & LBM_FLAG_EXCLUDE)) return;
        const int Q = L.Q, D = L.D, K = L.D + 1;
        const int64_t n[3] = {lay.nx, lay.ny, lay.nz};
        const int64_t p[3] = {x, y, z};
        int64_t pull[27][3];
        for (int q = 0; q < Q; ++q)
            for (int d = 0; d < 3; ++d) pull[q][d] = d < D ? wrap(p[d] - L.c[q][d], n[d]) : 0;

        R f[27];
        uint8_t pf[27];
        pf[0] = flag; /* set_f_vector_and_flags (steps/stream.mojo:78) */
        const bool esoteric = cfg.lbm_method == LBM_ESOTERIC_PULL;
        const bool adj = !esoteric || cfg.include_moving_boundary; /* config.mojo:162-163 */
        if (adj)
            for (int q = 1; q < Q; ++q) pf[q] = flags[lay.flag(pull[q][0], pull[q][1], pull[q][2])];
        else
            for (int q = 1; q < Q; ++q) pf[q] = 0;

        if (!esoteric) {
            /* double_buffer_pull_load_f_vec (ops/load_and_store.mojo:164-221): raw compare */
            for (int q = 0; q < Q; ++q) {
                if (pf[q] == LBM_FLAG_SOLID) f[q] = (R)Store<S>::ld(f_in, lay.cell(x, y, z, L.opp[q], Q));
                else f[q] = (R)Store<S>::ld(f_in, lay.cell(pull[q][0], pull[q][1], pull[q][2], q, Q));
            }
        } else {
            /* esoteric_pull_load_f_vec (ops/load_and_store.mojo:11-86) */
            f[0] = (R)Store<S>::ld(f_in, lay.cell(x, y, z, 0, Q));
            for (int pos = 1; pos < Q - 1; pos += 2) {
                const int neg = pos + 1;
                /* neighbour x - c_neg = x + c_pos (even) and x + c_pos (odd) coincide */
                int64_t nb[3];
                for (int d = 0; d < 3; ++d) nb[d] = d < D ? wrap(p[d] + L.c[pos][d], n[d]) : 0;
                if (even) {
                    f[pos] = (R)Store<S>::ld(f_in, lay.cell(x, y, z, pos, Q));
                    f[neg] = (R)Store<S>::ld(f_in, lay.cell(nb[0], nb[1], nb[2], neg, Q));
                } else {
                    f[pos] = (R)Store<S>::ld(f_in, lay.cell(x, y, z, neg, Q));
                    f[neg] = (R)Store<S>::ld(f_in, lay.cell(nb[0], nb[1], nb[2], pos, Q));
                }
            }
        }

        /* apply_boundary_conditions (steps/apply_boundary_condition.mojo:10-41) */
        if (cfg.include_moving_boundary) {
            /* moving_wall_bc (ops/boundary_condition.mojo:17-83): Flags.is compare */
            for (int q = 1; q < Q; ++q) {
                if (!flag_is(pf[q], LBM_FLAG_SOLID)) continue;
                R uw[3];
                for (int d = 0; d < D; ++d) uw[d] = bc[lay.cell(pull[q][0], pull[q][1], pull[q][2], d, K)];
                const R rw = bc[lay.cell(pull[q][0], pull[q][1], pull[q][2], D, K)];
                R cu = 0;
                for (int d = 0; d < D; ++d) cu = cu + (R)L.c[q][d] * uw[d];
                f[q] = f[q] + six_w[q] * rw * cu;
            }
        }
        if (cfg.include_equilibrium_bc && flag_is(flag, LBM_FLAG_EQUILIBRIUM)) {
            /* equilibrium_bc + get_density_and_velocity_for_eq_BC (ops/boundary_condition.mojo:87-205) */
            R ub[3];
            for (int d = 0; d < D; ++d) ub[d] = bc[lay.cell(x, y, z, d, K)];
            const R rb = bc[lay.cell(x, y, z, D, K)];
            R rl = 0, ul[3] = {0, 0, 0};
            for (int q = 0; q < Q; ++q) {
                bool oob = false;
                for (int d = 0; d < D; ++d) {
                    const int64_t pi = p[d] - L.c[q][d];
                    oob = oob || pi < 0 || pi >= n[d];
                }
                const R fq = oob ? (cfg.DDF_shift ? (R)0 : w[q]) : f[q];
                rl = rl + fq;
                for (int d = 0; d < D; ++d) ul[d] = ul[d] + fq * (R)L.c[q][d];
            }
            if (cfg.DDF_shift) rl = rl + (R)1;
            for (int d = 0; d < D; ++d) ul[d] = ul[d] / rl;
            const R* uuse = std::isnan(ub[0]) ? ul : ub;
            const R ruse = std::isnan(rb) ? rl : rb;
            const R uu = udot(uuse);
            for (int q = 0; q < Q; ++q) f[q] = feq(q, ruse, uuse, uu, cfg.DDF_shift != 0);
        }

        collide(f, tau, bc, x, y, z, flag);

        if (!esoteric) {
            for (int q = 0; q < Q; ++q) Store<S>::st(f_out, lay.cell(x, y, z, q, Q), f[q]);
        } else {
            /* esoteric_pull_store_f_vec (ops/load_and_store.mojo:89-159) */
            Store<S>::st(f_out, lay.cell(x, y, z, 0, Q), f[0]);
            for (int neg = 2; neg < Q; neg += 2) {
                const int pos = neg - 1;
                int64_t nb[3];
                for (int d = 0; d < 3; ++d) nb[d] = d < D ? wrap(p[d] + L.c[pos][d], n[d]) : 0;
                if (even) {
                    Store<S>::st(f_out, lay.cell(nb[0], nb[1], nb[2], neg, Q), f[pos]);
                    Store<S>::st(f_out, lay.cell(x, y, z, pos, Q), f[neg]);
                } else {
                    Store<S>::st(f_out, lay.cell(nb[0], nb[1], nb[2], pos, Q), f[pos]);
                    Store<S>::st(f_out, lay.cell(x, y, z, neg, Q), f[neg]);
                }
            }
        }
    }
};

template <class R, class S>
void run_step(const lbm_config_t* cfg, const lbm_grid_t* g, void* f_out, const void* f_in, void* bc,
              const uint8_t* flags, double tau, int even, int nthreads, int64_t begin, int64_t end) {
    const LatticeDef L = make_lattice(g->lattice);
    const Layout lay = make_layout(g);
    Stepper<R, S> st(*cfg, L, lay);
    S* fo = (S*)f_out;
    const S* fi = (const S*)f_in;
    R* b = (R*)bc;
    const int64_t N = lay.nx * lay.ny * lay.nz;
    if (end < 0 || end > N) end = N;
    if (begin < 0) begin = 0;
#ifdef _OPENMP
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nt)
#endif
    for (int64_t i = begin; i < end; ++i) {
        const int64_t x = i % lay.nx, y = (i / lay.nx) % lay.ny, z = i / (lay.nx * lay.ny);
        st.cell(x, y, z, fo, fi, b, flags, (R)tau, even != 0);
    }
    (void)nthreads;
}

/* initialize_f_from_func (preprocess/initial_condition.mojo:86-179) with fi_neq (:182-234). */
template <class R, class S>
void run_init(const lbm_config_t* cfg, const lbm_grid_t* g, void* f, double rho_d, double tau_d,
              const double* u, const double* grad) {
    const LatticeDef L = make_lattice(g->lattice);
    const Layout lay = make_layout(g);
    Stepper<R, S> st(*cfg, L, lay);
    const int Q = L.Q, D = L.D;
    const int64_t N = lay.nx * lay.ny * lay.nz;
    const R rho = (R)rho_d, tau = (R)tau_d;
    S* fs = (S*)f;
    for (int64_t i = 0; i < N; ++i) {
        const int64_t x = i % lay.nx, y = (i / lay.nx) % lay.ny, z = i / (lay.nx * lay.ny);
        const int64_t r = (x * lay.ny + y) * lay.nz + z; /* row-major [nx, ny, nz] */
        R vel[3] = {0, 0, 0};
        if (u) for (int d = 0; d < D; ++d) vel[d] = (R)u[r + N * d];
        const R uu = st.udot(vel);
        R fv[27];
        for (int q = 0; q < Q; ++q) {
            R fi = st.feq(q, rho, vel, uu, cfg->DDF_shift != 0);
            if (grad) {
                R neq = 0;
                for (int a = 0; a < D; ++a)
                    for (int b = 0; b < D; ++b) {
                        /* calculate_Sab: symmetric part of the gradient */
                        const R Sab = (R)0.5 * ((R)grad[r + N * (a * D + b)] + (R)grad[r + N * (b * D + a)]);
                        R Qiab = (R)L.c[q][a] * (R)L.c[q][b];
                        if (a == b) Qiab = Qiab - st.cs2;
                        neq = neq + Qiab * Sab;
                    }
                neq = neq * ((-st.w[q] * rho * tau * (R)3) * ((tau - (R)1) / tau));
                fi = fi + neq;
            }
            fv[q] = fi;
        }
        if (cfg->lbm_method == LBM_ESOTERIC_PULL) {
            /* esoteric_pull_store_f_vec with is_even_time_step = False (:172-174) */
            const int64_t p[3] = {x, y, z}, n[3] = {lay.nx, lay.ny, lay.nz};
            Store<S>::st(fs, lay.cell(x, y, z, 0, Q), fv[0]);
            for (int neg = 2; neg < Q; neg += 2) {
                const int pos = neg - 1;
                int64_t nb[3];
                for (int d = 0; d < 3; ++d) nb[d] = d < D ? wrap(p[d] + L.c[pos][d], n[d]) : 0;
                Store<S>::st(fs, lay.cell(nb[0], nb[1], nb[2], pos, Q), fv[pos]);
                Store<S>::st(fs, lay.cell(x, y, z, neg, Q), fv[neg]);
            }
        } else {
            for (int q = 0; q < Q; ++q) Store<S>::st(fs, lay.cell(x, y, z, q, Q), fv[q]);
        }
    }
}

/* Post-collision populations a cell owns after the last completed step (before streaming).
 * Double buffer: its own slots.  Esoteric pull: the slots the last step stored them to
 * (esoteric_pull_store_f_vec, ops/load_and_store.mojo:89-159). */
template <class R, class S>
void gather_post(const LatticeDef& L, const Layout& lay, const S* f, int64_t x, int64_t y, int64_t z,
                 bool esoteric, bool after_odd, R* out) {
    const int Q = L.Q;
    if (!esoteric) {
        for (int q = 0; q < Q; ++q) out[q] = (R)Store<S>::ld(f, lay.cell(x, y, z, q, Q));
        return;
    }
    const int64_t p[3] = {x, y, z}, n[3] = {lay.nx, lay.ny, lay.nz};
    out[0] = (R)Store<S>::ld(f, lay.cell(x, y, z, 0, Q));
    for (int pos = 1; pos < Q - 1; pos += 2) {
        const int neg = pos + 1;
        int64_t nb[3];
        for (int d = 0; d < 3; ++d) nb[d] = d < L.D ? wrap(p[d] + L.c[pos][d], n[d]) : 0;
        if (after_odd) {
            out[pos] = (R)Store<S>::ld(f, lay.cell(nb[0], nb[1], nb[2], pos, Q));
            out[neg] = (R)Store<S>::ld(f, lay.cell(x, y, z, neg, Q));
        } else {
            out[pos] = (R)Store<S>::ld(f, lay.cell(nb[0], nb[1], nb[2], neg, Q));
            out[neg] = (R)Store<S>::ld(f, lay.cell(x, y, z, pos, Q));
        }
    }
}

/* calculate_rho_and_velocity (output/velocity.mojo:25-125): stream + BC, then moments. */
/* get_velocity_gradient (kernels/utils/finite_difference.mojo:14-140) with dx = 1: component
 * comp of u ([D][nx][ny][nz]) along axis at p.  Spacing 1 to an in-grid neighbour, 1/2 when it is
 * SOLID (raw compare), 0 (no term) outside the grid; weights 1 - own spacing / total. */
template <class R>
R velocity_gradient(const Layout& lay, const uint8_t* flags, const R* u, const int64_t* p, int comp, int axis) {
    const int64_t n[3] = {lay.nx, lay.ny, lay.nz};
    const int64_t N = lay.nx * lay.ny * lay.nz;
    auto U = [&](const int64_t* q) { return u[N * comp + (q[0] * lay.ny + q[1]) * lay.nz + q[2]]; };
    const R u2 = U(p);
    R lg = 0, ldx = 0, rg = 0, rdx = 0;
    int64_t a[3] = {p[0], p[1], p[2]};
    a[axis] = p[axis] - 1;
    const bool vl = a[axis] >= 0;
    if (vl) {
        const R gdx = flags[lay.flag(a[0], a[1], a[2])] == LBM_FLAG_SOLID ? (R)0.5 : (R)1;
        lg = (u2 - U(a)) * ((R)1 / gdx);
        ldx = gdx;
    }
    a[axis] = p[axis] + 1;
    const bool vr = a[axis] < n[axis];
    if (vr) {
        const R gdx = flags[lay.flag(a[0], a[1], a[2])] == LBM_FLAG_SOLID ? (R)0.5 : (R)1;
        rg = (U(a) - u2) * ((R)1 / gdx);
        rdx = gdx;
    }
    if (!vl && !vr) return 0;
    const R total = ldx + rdx;
    const R lw = (R)1 - ldx / total;
    const R rw = (R)1 - lw;
    return rg * rw + lg * lw;
}

/* QCRIT: calculate_Q_criterion (output/Q_criterion.mojo:90-216) into q_out ([nx][ny][nz]) from
 * the same streamed populations, u_in ([D][nx][ny][nz]) and tau; cells with a raw SOLID flag are
 * skipped. */
template <class R, class S, bool QCRIT = false>
void run_rho_u(const lbm_config_t* cfg, const lbm_grid_t* g, const void* fv, const void* bcv,
               const uint8_t* flags, void* rho_out, void* u_out, int after_odd, const void* u_in = nullptr,
               void* q_out = nullptr, double tau = 1.0) {
    const LatticeDef L = make_lattice(g->lattice);
    const Layout lay = make_layout(g);
    lbm_config_t c2 = *cfg;
    Stepper<R, S> st(c2, L, lay);
    const int Q = L.Q, D = L.D, K = L.D + 1;
    const int64_t N = lay.nx * lay.ny * lay.nz;
    const S* f = (const S*)fv;
    const R* bc = (const R*)bcv;
    R* ro = (R*)rho_out;
    R* uo = (R*)u_out;
    for (int64_t i = 0; i < N; ++i) {
        const int64_t x = i % lay.nx, y = (i / lay.nx) % lay.ny, z = i / (lay.nx * lay.ny);
        const int64_t r = (x * lay.ny + y) * lay.nz + z; /* row-major [nx, ny, nz] */
        const uint8_t flag = flags[lay.flag(x, y, z)];
        if (flag == LBM_FLAG_SOLID) {
            if (!QCRIT) {
                for (int d = 0; d < D; ++d) uo[r + N * d] = bc[lay.cell(x, y, z, d, K)];
                ro[r] = bc[lay.cell(x, y, z, D, K)];
            }
            continue;
        }
        /* stream + apply_boundary_conditions with the next step's load pattern */
        const int64_t p[3] = {x, y, z}, n[3] = {lay.nx, lay.ny, lay.nz};
        int64_t pull[27][3];
        for (int q = 0; q < Q; ++q)
            for (int d = 0; d < 3; ++d) pull[q][d] = d < D ? wrap(p[d] - L.c[q][d], n[d]) : 0;
        R fq[27];
        uint8_t pf[27];
        pf[0] = flag;
        const bool esoteric = cfg->lbm_method == LBM_ESOTERIC_PULL;
        for (int q = 1; q < Q; ++q) pf[q] = flags[lay.flag(pull[q][0], pull[q][1], pull[q][2])];
        if (!esoteric) {
            for (int q = 0; q < Q; ++q) {
                if (pf[q] == LBM_FLAG_SOLID) fq[q] = (R)Store<S>::ld(f, lay.cell(x, y, z, L.opp[q], Q));
                else fq[q] = (R)Store<S>::ld(f, lay.cell(pull[q][0], pull[q][1], pull[q][2], q, Q));
            }
        } else {
            const bool even = after_odd != 0; /* is_even_time_step = after_odd_step */
            fq[0] = (R)Store<S>::ld(f, lay.cell(x, y, z, 0, Q));
            for (int pos = 1; pos < Q - 1; pos += 2) {
                const int neg = pos + 1;
                int64_t nb[3];
                for (int d = 0; d < 3; ++d) nb[d] = d < D ? wrap(p[d] + L.c[pos][d], n[d]) : 0;
                if (even) {
                    fq[pos] = (R)Store<S>::ld(f, lay.cell(x, y, z, pos, Q));
                    fq[neg] = (R)Store<S>::ld(f, lay.cell(nb[0], nb[1], nb[2], neg, Q));
                } else {
                    fq[pos] = (R)Store<S>::ld(f, lay.cell(x, y, z, neg, Q));
                    fq[neg] = (R)Store<S>::ld(f, lay.cell(nb[0], nb[1], nb[2], pos, Q));
                }
            }
        }
        if (cfg->include_moving_boundary) {
            for (int q = 1; q < Q; ++q) {
                if (!flag_is(pf[q], LBM_FLAG_SOLID)) continue;
                R cu = 0;
                for (int d = 0; d < D; ++d) cu = cu + (R)L.c[q][d] * bc[lay.cell(pull[q][0], pull[q][1], pull[q][2], d, K)];
                fq[q] = fq[q] + st.six_w[q] * bc[lay.cell(pull[q][0], pull[q][1], pull[q][2], D, K)] * cu;
            }
        }
        if (cfg->include_equilibrium_bc && flag_is(flag, LBM_FLAG_EQUILIBRIUM)) {
            R ub[3];
            for (int d = 0; d < D; ++d) ub[d] = bc[lay.cell(x, y, z, d, K)];
            const R rb = bc[lay.cell(x, y, z, D, K)];
            R rl = 0, ul[3] = {0, 0, 0};
            for (int q = 0; q < Q; ++q) {
                bool oob = false;
                for (int d = 0; d < D; ++d) { const int64_t pi = p[d] - L.c[q][d]; oob = oob || pi < 0 || pi >= n[d]; }
                const R v = oob ? (cfg->DDF_shift ? (R)0 : st.w[q]) : fq[q];
                rl = rl + v;
                for (int d = 0; d < D; ++d) ul[d] = ul[d] + v * (R)L.c[q][d];
            }
            if (cfg->DDF_shift) rl = rl + (R)1;
            for (int d = 0; d < D; ++d) ul[d] = ul[d] / rl;
            const R* uuse = std::isnan(ub[0]) ? ul : ub;
            const R ruse = std::isnan(rb) ? rl : rb;
            const R uu = st.udot(uuse);
            for (int q = 0; q < Q; ++q) fq[q] = st.feq(q, ruse, uuse, uu, cfg->DDF_shift != 0);
        }
        const R rho = st.density(fq);
        R u[3];
        st.velocity(fq, rho, u);
        if (!QCRIT) {
            ro[r] = rho;
            for (int d = 0; d < D; ++d) uo[r + N * d] = u[d];
            continue;
        }
        /* get_f_noneq_vec, get_non_eq_second_order_moment, get_strain_rate_tensor and its norm
         * (kernels/utils/equilibrium.mojo:81-120, moment.mojo:111-215), as collide */
        const R uu = st.udot(u);
        R P[6];
        for (int m = 0; m < st.nstress(); ++m) {
            R acc = 0;
            for (int q = 0; q < Q; ++q)
                acc = acc + (fq[q] - st.feq(q, rho, u, uu, cfg->DDF_shift != 0)) * (R)L.c[q][st.sa(m)] * (R)L.c[q][st.sb(m)];
            P[m] = acc;
        }
        const R kk = (R)-1 / ((R)2 * rho * st.cs2 * (R)tau);
        R s2 = 0;
        for (int m = 0; m < st.nstress(); ++m) {
            const R Sm = P[m] * kk;
            const R ss = Sm * Sm;
            s2 = (st.sa(m) != st.sb(m)) ? s2 + ss * (R)2 : s2 + ss;
        }
        /* calculate_vorticity (Q_criterion.mojo:26-85), Vector.norm_squared (sequential sum) */
        const R* ui = (const R*)u_in;
        R w2 = 0;
        if (D == 2) {
            const R wz = velocity_gradient<R>(lay, flags, ui, p, 1, 0) - velocity_gradient<R>(lay, flags, ui, p, 0, 1);
            w2 = w2 + wz * wz;
        } else {
            const R wx = velocity_gradient<R>(lay, flags, ui, p, 2, 1) - velocity_gradient<R>(lay, flags, ui, p, 1, 2);
            const R wy = velocity_gradient<R>(lay, flags, ui, p, 0, 2) - velocity_gradient<R>(lay, flags, ui, p, 2, 0);
            const R wz = velocity_gradient<R>(lay, flags, ui, p, 1, 0) - velocity_gradient<R>(lay, flags, ui, p, 0, 1);
            w2 = w2 + wx * wx;
            w2 = w2 + wy * wy;
            w2 = w2 + wz * wz;
        }
        ((R*)q_out)[r] = (R)0.25 * w2 - (R)0.5 * s2;
    }
}

/* linkwise_bounceback_kernel (geometry/interpolated_BB.mojo:46-141), sequential over links. */
template <class R, class S>
void run_links(const lbm_config_t* cfg, const lbm_grid_t* g, void* fv, void* force, const int32_t* ids,
               const int32_t* dirs, const void* dists, int64_t n_links, int method, int compute_force,
               double q_clamp) {
    const LatticeDef L = make_lattice(g->lattice);
    const Layout lay = make_layout(g);
    const int Q = L.Q, D = L.D;
    S* f = (S*)fv;
    R* fo = (R*)force;
    const R* qd = (const R*)dists;
    for (int64_t t = 0; t < n_links; ++t) {
        /* idx_to_ijk (interpolated_BB.mojo:24-43): decode a linear flag-layout index */
        const int64_t li = ids[t];
        const int64_t T = lay.T;
        const int64_t loc = li % T, tile = li / T;
        const int64_t lx = loc % lay.tx, ly = (loc / lay.tx) % lay.ty, lz = loc / (lay.tx * lay.ty);
        const int64_t bx = tile % lay.ntx, by = (tile / lay.ntx) % lay.nty, bz = tile / (lay.ntx * lay.nty);
        const int64_t x = bx * lay.tx + lx, y = by * lay.ty + ly, z = bz * lay.tz + lz;
        if (x >= lay.nx || y >= lay.ny || z >= lay.nz) continue;
        const int i = dirs[t], oi = L.opp[i];
        R q = qd[t];
        if (q < (R)q_clamp) q = (R)q_clamp;
        const R f_into = (R)Store<S>::ld(f, lay.cell(x, y, z, i, Q));
        R f_bb = f_into;
        if (method == LBM_BB_BOUZIDI) {
            if (q > (R)0.5) {
                const R f_out = (R)Store<S>::ld(f, lay.cell(x, y, z, oi, Q));
                f_bb = (R)0.5 / q * f_into + ((R)2 * q - (R)1) / ((R)2 * q) * f_out;
            } else {
                const int64_t p[3] = {x, y, z}, n[3] = {lay.nx, lay.ny, lay.nz};
                int64_t xf[3];
                for (int d = 0; d < 3; ++d) xf[d] = d < D ? wrap(p[d] - L.c[i][d], n[d]) : 0;
                const R f_xff = (R)Store<S>::ld(f, lay.cell(xf[0], xf[1], xf[2], oi, Q));
                f_bb = (R)2 * q * f_into + ((R)1 - (R)2 * q) * f_xff;
            }
            Store<S>::st(f, lay.cell(x, y, z, i, Q), f_bb);
        }
        if (compute_force) {
            R a = f_into, b = f_bb;
            if (cfg->DDF_shift) { a = a + (R)L.w[i]; b = b + (R)L.w[i]; }
            for (int d = 0; d < D; ++d) fo[t + n_links * d] = (R)L.c[i][d] * (a + b);
        }
    }
}

/* calculate_drag_around_object (output/drag.mojo:16-105) */
template <class R, class S>
void run_drag(const lbm_config_t* cfg, const lbm_grid_t* g, void* force, const void* fv, const uint8_t* flags,
              const int32_t* ids, int64_t n_nodes) {
    const LatticeDef L = make_lattice(g->lattice);
    const Layout lay = make_layout(g);
    const int Q = L.Q, D = L.D;
    const S* f = (const S*)fv;
    R* fo = (R*)force;
    for (int64_t t = 0; t < n_nodes; ++t) {
        const int64_t li = ids[t];
        const int64_t loc = li % lay.T, tile = li / lay.T;
        const int64_t x = (tile % lay.ntx) * lay.tx + loc % lay.tx;
        const int64_t y = ((tile / lay.ntx) % lay.nty) * lay.ty + (loc / lay.tx) % lay.ty;
        const int64_t z = (tile / (lay.ntx * lay.nty)) * lay.tz + loc / (lay.tx * lay.ty);
        if (x >= lay.nx || y >= lay.ny || z >= lay.nz) continue;
        const int64_t p[3] = {x, y, z}, n[3] = {lay.nx, lay.ny, lay.nz};
        R acc[3] = {0, 0, 0};
        for (int q = 0; q < Q; ++q) {
            int64_t nb[3];
            for (int d = 0; d < 3; ++d) nb[d] = d < D ? wrap(p[d] + L.c[q][d], n[d]) : 0;
            if (flags[lay.flag(nb[0], nb[1], nb[2])] != LBM_FLAG_SOLID) continue;
            R fl = (R)Store<S>::ld(f, lay.cell(x, y, z, q, Q));
            if (cfg->DDF_shift) fl = fl + (R)L.w[q];
            for (int d = 0; d < D; ++d) acc[d] = acc[d] + ((R)2 * fl) * (R)L.c[q][d];
        }
        for (int d = 0; d < D; ++d) fo[t + n_nodes * d] = acc[d];
    }
}

}  // namespace

extern "C" {

/* prec: 32 = float32 arithmetic (storage float32, or Float16C when cfg->use_float16c);
 *       64 = float64 arithmetic and storage (Float16C not applicable). */
int oracle_step(const lbm_config_t* cfg, const lbm_grid_t* g, int prec, void* f_out, const void* f_in,
                void* bc, const uint8_t* flags, double tau, int is_even, int nthreads) {
    if (prec == 64) run_step<double, double>(cfg, g, f_out, f_in, bc, flags, tau, is_even, nthreads, 0, -1);
    else if (cfg->use_float16c) run_step<float, uint16_t>(cfg, g, f_out, f_in, bc, flags, tau, is_even, nthreads, 0, -1);
    else run_step<float, float>(cfg, g, f_out, f_in, bc, flags, tau, is_even, nthreads, 0, -1);
    return 0;
}

/* The step restricted to cells whose index x + nx*(y + ny*z) lies in [begin, end): a bounded
 * sample of a full step, used to time the CPU path on large grids. */
int oracle_step_range(const lbm_config_t* cfg, const lbm_grid_t* g, int prec, void* f_out, const void* f_in,
                      void* bc, const uint8_t* flags, double tau, int is_even, int nthreads, int64_t begin,
                      int64_t end) {
    if (prec == 64) run_step<double, double>(cfg, g, f_out, f_in, bc, flags, tau, is_even, nthreads, begin, end);
    else if (cfg->use_float16c) run_step<float, uint16_t>(cfg, g, f_out, f_in, bc, flags, tau, is_even, nthreads, begin, end);
    else run_step<float, float>(cfg, g, f_out, f_in, bc, flags, tau, is_even, nthreads, begin, end);
    return 0;
}

int oracle_init(const lbm_config_t* cfg, const lbm_grid_t* g, int prec, void* f, double rho, double tau,
                const double* u, const double* grad) {
    if (prec == 64) run_init<double, double>(cfg, g, f, rho, tau, u, grad);
    else if (cfg->use_float16c) run_init<float, uint16_t>(cfg, g, f, rho, tau, u, grad);
    else run_init<float, float>(cfg, g, f, rho, tau, u, grad);
    return 0;
}

int oracle_rho_u(const lbm_config_t* cfg, const lbm_grid_t* g, int prec, const void* f, const void* bc,
                 const uint8_t* flags, void* rho, void* u, int after_odd) {
    if (prec == 64) run_rho_u<double, double>(cfg, g, f, bc, flags, rho, u, after_odd);
    else if (cfg->use_float16c) run_rho_u<float, uint16_t>(cfg, g, f, bc, flags, rho, u, after_odd);
    else run_rho_u<float, float>(cfg, g, f, bc, flags, rho, u, after_odd);
    return 0;
}

int oracle_q_criterion(const lbm_config_t* cfg, const lbm_grid_t* g, int prec, const void* f, const void* bc,
                       const uint8_t* flags, const void* u, double tau, int after_odd, void* q) {
    if (prec == 64) run_rho_u<double, double, true>(cfg, g, f, bc, flags, nullptr, nullptr, after_odd, u, q, tau);
    else if (cfg->use_float16c) run_rho_u<float, uint16_t, true>(cfg, g, f, bc, flags, nullptr, nullptr, after_odd, u, q, tau);
    else run_rho_u<float, float, true>(cfg, g, f, bc, flags, nullptr, nullptr, after_odd, u, q, tau);
    return 0;
}

int oracle_links(const lbm_config_t* cfg, const lbm_grid_t* g, int prec, void* f, void* force,
                 const int32_t* ids, const int32_t* dirs, const void* dists, int64_t n, int method,
                 int compute_force, double q_clamp) {
    if (prec == 64) run_links<double, double>(cfg, g, f, force, ids, dirs, dists, n, method, compute_force, q_clamp);
    else if (cfg->use_float16c) run_links<float, uint16_t>(cfg, g, f, force, ids, dirs, dists, n, method, compute_force, q_clamp);
    else run_links<float, float>(cfg, g, f, force, ids, dirs, dists, n, method, compute_force, q_clamp);
    return 0;
}

int oracle_drag(const lbm_config_t* cfg, const lbm_grid_t* g, int prec, void* force, const void* f,
                const uint8_t* flags, const int32_t* ids, int64_t n) {
    if (prec == 64) run_drag<double, double>(cfg, g, force, f, flags, ids, n);
    else if (cfg->use_float16c) run_drag<float, uint16_t>(cfg, g, force, f, flags, ids, n);
    else run_drag<float, float>(cfg, g, force, f, flags, ids, n);
    return 0;
}

/* Post-collision populations of every cell (gather_post), out[r + N*q], r = (x*ny + y)*nz + z. */
int oracle_gather(const lbm_config_t* cfg, const lbm_grid_t* g, int prec, const void* f, void* out, int after_odd) {
    const LatticeDef L = make_lattice(g->lattice);
    const Layout lay = make_layout(g);
    const int64_t N = lay.nx * lay.ny * lay.nz;
    const bool eso = cfg->lbm_method == LBM_ESOTERIC_PULL;
    for (int64_t i = 0; i < N; ++i) {
        const int64_t x = i % lay.nx, y = (i / lay.nx) % lay.ny, z = i / (lay.nx * lay.ny);
        const int64_t r = (x * lay.ny + y) * lay.nz + z;
        if (prec == 64) {
            double v[27];
            gather_post<double, double>(L, lay, (const double*)f, x, y, z, eso, after_odd != 0, v);
            for (int q = 0; q < L.Q; ++q) ((double*)out)[r + N * q] = v[q];
        } else {
            float v[27];
            if (cfg->use_float16c) gather_post<float, uint16_t>(L, lay, (const uint16_t*)f, x, y, z, eso, after_odd != 0, v);
            else gather_post<float, float>(L, lay, (const float*)f, x, y, z, eso, after_odd != 0, v);
            for (int q = 0; q < L.Q; ++q) ((float*)out)[r + N * q] = v[q];
        }
    }
    return 0;
}

void oracle_f16c_encode(const float* in, uint16_t* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = f32_to_f16c(in[i]);
}
void oracle_f16c_decode(const uint16_t* in, float* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = f16c_to_f32(in[i]);
}

int64_t oracle_layout_offset(const lbm_grid_t* g, int64_t x, int64_t y, int64_t z, int64_t k, int64_t K) {
    return make_layout(g).cell(x, y, z, k, K);
}

int oracle_lattice(int id, int32_t* c_out /* Q*3 */, double* w_out, int32_t* opp_out) {
    const LatticeDef L = make_lattice(id);
    for (int q = 0; q < L.Q; ++q) {
        for (int d = 0; d < 3; ++d) c_out[3 * q + d] = L.c[q][d];
        w_out[q] = L.w[q];
        opp_out[q] = L.opp[q];
    }
    return L.Q;
}

/* The stress-component pairs (alpha, beta) the step uses for dimension D (2 or 3); returns their
 * count (get_stress_indices, lattice.mojo:352-398). */
int oracle_stress_pairs(int D, int32_t* out /* n*2 */) {
    const int n = D == 2 ? 3 : 6;
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < 2; ++j) out[2 * k + j] = D == 2 ? kStress2[k][j] : kStress3[k][j];
    return n;
}

/* Learned closure for the LES steps that follow (copied; NULL returns to Smagorinsky). */
void oracle_set_closure(const lbm_closure_t* c) {
    g_closure_on = c != nullptr;
    if (c) g_closure = *c;
}

/* The closure's features and nu_t for explicit strain tensors: n rows of S (D=2: 3, D=3: 6
 * components), s2, rho, uu and tau; x_out (n*8) and nu_out (n; -1 outside the training range).
 * prec 32 or 64 as for oracle_step. */
void oracle_closure_eval(int D, int prec, int64_t n, const double* S, const double* s2, const double* rho,
                         const double* uu, const double* tau, double* x_out, double* nu_out) {
    const int ns = D == 3 ? 6 : 3;
    for (int64_t i = 0; i < n; ++i) {
        if (prec == 64) {
            double x[8];
            closure_features<double>(D, S + i * ns, s2[i], rho[i], uu[i], tau[i], x);
            for (int k = 0; k < 8; ++k) x_out[i * 8 + k] = x[k];
            nu_out[i] = g_closure_on ? closure_nu<double>(x) : -1.0;
        } else {
            float Sf[6], x[8];
            for (int k = 0; k < ns; ++k) Sf[k] = (float)S[i * ns + k];
            closure_features<float>(D, Sf, (float)s2[i], (float)rho[i], (float)uu[i], (float)tau[i], x);
            for (int k = 0; k < 8; ++k) x_out[i * 8 + k] = x[k];
            nu_out[i] = g_closure_on ? (double)closure_nu<float>(x) : -1.0;
        }
    }
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
