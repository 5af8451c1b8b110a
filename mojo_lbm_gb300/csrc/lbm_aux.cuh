// Auxiliary kernels around the step: initial state, macroscopic outputs, float64 conservation
// reductions, link-wise interpolated bounce-back, momentum-exchange drag, Float16C codec.
#pragma once

#include "lbm_step.cuh"

namespace lbm {

// Decoded cell position and neighbour tables, shared by the auxiliary kernels.
struct Cell {
    uint32_t n, loc, tile, lx, ly, lz, bx, by, bz;
    int32_t x, y, z;
    uint32_t r;  // row-major output index (x*ny + y)*nz + z
};

template <class L>
__device__ __forceinline__ Cell decode_cell(const LayoutDesc& lay, uint32_t n, Nbr& nb) {
    Cell c;
    c.n = n;
    c.tile = lay.d_T.div(n);
    c.loc = n - c.tile * lay.T;
    const uint32_t lyz = lay.d_tx.div(c.loc);
    c.lx = c.loc - lyz * (uint32_t)lay.tx;
    c.lz = lay.d_ty.div(lyz);
    c.ly = lyz - c.lz * (uint32_t)lay.ty;
    const uint32_t byz = lay.d_ntx.div(c.tile);
    c.bx = c.tile - byz * (uint32_t)lay.ntx;
    c.bz = lay.d_nty.div(byz);
    c.by = byz - c.bz * (uint32_t)lay.nty;
    c.x = (int32_t)(c.bx * lay.tx + c.lx);
    c.y = (int32_t)(c.by * lay.ty + c.ly);
    c.z = (int32_t)(c.bz * lay.tz + c.lz);
    c.r = ((uint32_t)c.x * (uint32_t)lay.ny + (uint32_t)c.y) * (uint32_t)lay.nz + (uint32_t)c.z;
    nb.ax.init(c.lx, c.bx, lay.tx, lay.ntx, 1u, 1u);
    nb.ay.init(c.ly, c.by, lay.ty, lay.nty, (uint32_t)lay.tx, (uint32_t)lay.ntx);
    if constexpr (L::D == 3)
        nb.az.init(c.lz, c.bz, lay.tz, lay.ntz, (uint32_t)(lay.tx * lay.ty), (uint32_t)(lay.ntx * lay.nty));
    else {
        nb.az.loc[0] = nb.az.loc[1] = nb.az.loc[2] = 0u;
        nb.az.til[0] = nb.az.til[1] = nb.az.til[2] = 0u;
    }
    return c;
}

struct InitArgs {
    LayoutDesc lay;
    void* f;
    const float* u;     // D * ncells, row-major per component, or null
    const float* grad;  // D*D * ncells, or null
    float rho, tau;
    int32_t ddf, esoteric;
};

// initialize_f_from_func (src/lbm/preprocess/initial_condition.mojo:86-179) with fi_neq
// (:182-234); esoteric pull stores with the odd-step pattern (:172-174).
template <class L, bool F16C>
__global__ void init_kernel(const InitArgs a) {
    using P = Pop<F16C>;
    using S = typename P::T;
    constexpr int Q = L::Q, D = L::D;
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.lay.ncells) return;
    Nbr nb;
    const Cell c = decode_cell<L>(a.lay, n, nb);
    const uint32_t N = a.lay.ncells, T = a.lay.T;
    float u[3] = {0.f, 0.f, 0.f};
    if (a.u) static_for<0, D>([&](auto dc) { u[dc.value] = a.u[(size_t)N * dc.value + c.r]; });
    float uu = 0.f;
    static_for<0, D>([&](auto dc) { uu += u[dc.value] * u[dc.value]; });
    float S_[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    if (a.grad)
        static_for<0, D>([&](auto ac) {
            static_for<0, D>([&](auto bc) {
                constexpr int A = ac.value, B = bc.value;
                S_[A][B] = 0.5f * (a.grad[(size_t)N * (A * D + B) + c.r] + a.grad[(size_t)N * (B * D + A) + c.r]);
            });
        });
    float f[Q];
    static_for<0, Q>([&](auto qc) {
        constexpr int q = qc.value;
        float fi = feq<L, q>(a.rho, u, uu, a.ddf != 0);
        if (a.grad) {
            float neq = 0.f;
            static_for<0, D>([&](auto ac) {
                static_for<0, D>([&](auto bc) {
                    constexpr int A = ac.value, B = bc.value;
                    constexpr float Qab = (float)(L::c(q, A) * L::c(q, B)) - (A == B ? (float)(1.0 / 3.0) : 0.f);
                    neq += Qab * S_[A][B];
                });
            });
            neq *= (-wf<L>(q) * a.rho * a.tau * 3.f) * ((a.tau - 1.f) / a.tau);
            fi += neq;
        }
        f[q] = fi;
    });
    S* fs = (S*)a.f;
    const uint64_t TQ = (uint64_t)T * Q;
    const uint64_t own = c.loc + TQ * c.tile;
    if (!a.esoteric) {
        static_for<0, Q>([&](auto qc) { P::st(fs + own + (uint64_t)T * qc.value, f[qc.value]); });
    } else {
        P::st(fs + own, f[0]);
        static_for<1, Q - 1, 2>([&](auto qc) {
            constexpr int pos = qc.value, neg = pos + 1;
            constexpr int sx = L::c(pos, 0), sy = L::c(pos, 1), sz = L::c(pos, 2);
            const uint64_t nbase = nb.template loc<sx, sy, sz>() + TQ * nb.template til<sx, sy, sz>();
            P::st(fs + nbase + (uint64_t)T * pos, f[pos]);
            P::st(fs + own + (uint64_t)T * neg, f[neg]);
        });
    }
}

// Populations that the next step would load at a cell, before any boundary treatment
// (load_single_f, src/lbm/kernels/steps/load_f.mojo:11-33, for every q).
template <class L, bool F16C, bool ESO>
__device__ __forceinline__ void gather_next(const typename Pop<F16C>::T* f, const LayoutDesc& lay, const Cell& c,
                                            const Nbr& nb, bool even, float (&out)[L::Q]) {
    using P = Pop<F16C>;
    constexpr int Q = L::Q;
    const uint32_t T = lay.T;
    const uint64_t TQ = (uint64_t)T * Q;
    const uint64_t own = c.loc + TQ * c.tile;
    if constexpr (!ESO) {
        static_for<0, Q>([&](auto qc) { out[qc.value] = P::ld(f + own + (uint64_t)T * qc.value); });
    } else {
        out[0] = P::ld(f + own);
        static_for<1, Q - 1, 2>([&](auto qc) {
            constexpr int pos = qc.value, neg = pos + 1;
            constexpr int sx = L::c(pos, 0), sy = L::c(pos, 1), sz = L::c(pos, 2);
            const uint64_t nbase = nb.template loc<sx, sy, sz>() + TQ * nb.template til<sx, sy, sz>();
            out[pos] = P::ld(f + own + (uint64_t)T * (even ? pos : neg));
            out[neg] = P::ld(f + nbase + (uint64_t)T * (even ? neg : pos));
        });
    }
}

// Post-collision populations a cell owns after the last completed step, before streaming:
// its own slots (double buffer) or the slots esoteric_pull_store_f_vec wrote them to
// (src/lbm/kernels/ops/load_and_store.mojo:89-159).
template <class L, bool F16C, bool ESO>
__device__ __forceinline__ void gather_post(const typename Pop<F16C>::T* f, const LayoutDesc& lay, const Cell& c,
                                            const Nbr& nb, bool after_odd, float (&out)[L::Q]) {
    using P = Pop<F16C>;
    constexpr int Q = L::Q;
    const uint32_t T = lay.T;
    const uint64_t TQ = (uint64_t)T * Q;
    const uint64_t own = c.loc + TQ * c.tile;
    if constexpr (!ESO) {
        static_for<0, Q>([&](auto qc) { out[qc.value] = P::ld(f + own + (uint64_t)T * qc.value); });
    } else {
        out[0] = P::ld(f + own);
        static_for<1, Q - 1, 2>([&](auto qc) {
            constexpr int pos = qc.value, neg = pos + 1;
            constexpr int sx = L::c(pos, 0), sy = L::c(pos, 1), sz = L::c(pos, 2);
            const uint64_t nbase = nb.template loc<sx, sy, sz>() + TQ * nb.template til<sx, sy, sz>();
            out[pos] = P::ld(f + nbase + (uint64_t)T * (after_odd ? pos : neg));
            out[neg] = P::ld(f + own + (uint64_t)T * (after_odd ? neg : pos));
        });
    }
}

struct RhoUArgs {
    LayoutDesc lay;
    const void* f;
    const float* bc;
    const uint8_t* flags;
    float* rho;
    float* u;        // [D][nx][ny][nz]: written by the rho/u pass, read by the Q-criterion pass
    float* q;        // [nx][ny][nz]: Q-criterion output
    float tau;       // Q-criterion: the tau of the strain-rate reconstruction
    int32_t ddf, moving, eqbc, even;
};

// get_velocity_gradient (src/lbm/kernels/utils/finite_difference.mojo:14-90), dx = 1: component
// `comp` of the stored velocity differentiated along `axis` at (x, y, z).  Each neighbour inside
// the grid gives a one-sided difference over a spacing of 1, or 1/2 when it is SOLID (raw flag
// compare), weighted (1 - own spacing / sum of spacings).  A neighbour outside the grid gives
// spacing 0, which gives the other side weight 0: the reference's weighting, kept as it is,
// returns 0 across a non-periodic domain edge.
template <int D>
__device__ __forceinline__ float velocity_gradient(const RhoUArgs& a, int32_t x, int32_t y, int32_t z, int comp,
                                                   int axis) {
    const LayoutDesc& l = a.lay;
    const uint32_t N = l.ncells;
    auto u_at = [&](int32_t i, int32_t j, int32_t k) {
        return a.u[(size_t)N * comp + ((uint32_t)i * (uint32_t)l.ny + (uint32_t)j) * (uint32_t)l.nz + (uint32_t)k];
    };
    auto flag_at = [&](int32_t i, int32_t j, int32_t k) {
        const uint32_t tile = (uint32_t)(i / l.tx) + (uint32_t)l.ntx * ((uint32_t)(j / l.ty) + (uint32_t)l.nty * (uint32_t)(k / l.tz));
        const uint32_t loc = (uint32_t)(i % l.tx) + (uint32_t)l.tx * ((uint32_t)(j % l.ty) + (uint32_t)l.ty * (uint32_t)(k % l.tz));
        return a.flags[loc + l.T * tile];
    };
    const int32_t g[3] = {x, y, z}, ng[3] = {l.nx, l.ny, l.nz};
    const float u2 = u_at(x, y, z);
    float lgrad = 0.f, ldx = 0.f, rgrad = 0.f, rdx = 0.f;
    int32_t p[3] = {g[0], g[1], g[2]};
    p[axis] = g[axis] - 1;
    const bool vl = p[axis] >= 0;
    if (vl) {
        const float gdx = flag_at(p[0], p[1], p[2]) == LBM_FLAG_SOLID ? 0.5f : 1.f;
        lgrad = (u2 - u_at(p[0], p[1], p[2])) * (1.f / gdx);
        ldx = gdx;
    }
    p[axis] = g[axis] + 1;
    const bool vr = p[axis] < ng[axis];
    if (vr) {
        const float gdx = flag_at(p[0], p[1], p[2]) == LBM_FLAG_SOLID ? 0.5f : 1.f;
        rgrad = (u_at(p[0], p[1], p[2]) - u2) * (1.f / gdx);
        rdx = gdx;
    }
    if (!vl && !vr) return 0.f;
    const float total = ldx + rdx;
    const float lw = 1.f - ldx / total;
    const float rw = 1.f - lw;
    return rgrad * rw + lgrad * lw;
}

// calculate_rho_and_velocity (src/lbm/output/velocity.mojo:25-125): the next step's stream and
// boundary conditions, then density and velocity; SOLID cells (raw compare) report their bc.
// With QCRIT, calculate_Q_criterion (src/lbm/output/Q_criterion.mojo:90-216) instead: the same
// stream and boundary conditions, the strain rate from the non-equilibrium second moment (tau of
// the call), the vorticity from finite differences of the stored velocity a.u, and
// Q = |omega|^2 / 4 - |S|^2 / 2 at every cell whose raw flag is not SOLID (others untouched).
template <class L, bool F16C, bool ESO, bool QCRIT = false>
__global__ void rho_u_kernel(const RhoUArgs a) {
    using P = Pop<F16C>;
    using S = typename P::T;
    constexpr int Q = L::Q, D = L::D, K = D + 1;
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.lay.ncells) return;
    Nbr nb;
    const Cell c = decode_cell<L>(a.lay, n, nb);
    const uint32_t N = a.lay.ncells, T = a.lay.T;
    const uint8_t flag = a.flags[n];
    const uint64_t own_bc = c.loc + (uint64_t)T * K * c.tile;
    if (flag == LBM_FLAG_SOLID) {
        if constexpr (!QCRIT) {
            static_for<0, D>([&](auto dc) { a.u[(size_t)N * dc.value + c.r] = a.bc[own_bc + (uint64_t)T * dc.value]; });
            a.rho[c.r] = a.bc[own_bc + (uint64_t)T * D];
        }
        return;
    }
    const S* fin = (const S*)a.f;
    const uint64_t TQ = (uint64_t)T * Q;
    const uint64_t own = c.loc + TQ * c.tile;
    uint32_t raw_solid = 0u, nib_solid = 0u;
    static_for<1, Q>([&](auto qc) {
        constexpr int q = qc.value;
        constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
        const uint8_t pf = a.flags[nb.template loc<sx, sy, sz>() + T * nb.template til<sx, sy, sz>()];
        if (pf == LBM_FLAG_SOLID) raw_solid |= 1u << q;
        if ((pf & 0x0F) == LBM_FLAG_SOLID) nib_solid |= 1u << q;
    });
    float f[Q];
    if constexpr (!ESO) {
        static_for<0, Q>([&](auto qc) {
            constexpr int q = qc.value;
            constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
            const uint64_t pull = nb.template loc<sx, sy, sz>() + TQ * nb.template til<sx, sy, sz>() + (uint64_t)T * q;
            const uint64_t bounce = own + (uint64_t)T * opp<L>(q);
            f[q] = P::ld(fin + ((raw_solid >> q) & 1u ? bounce : pull));
        });
    } else {
        gather_next<L, F16C, true>(fin, a.lay, c, nb, a.even != 0, f);
    }
    if (a.moving && nib_solid) {
        const uint64_t TK = (uint64_t)T * K;
        static_for<1, Q>([&](auto qc) {
            constexpr int q = qc.value;
            if ((nib_solid >> q) & 1u) {
                constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
                const uint64_t b = nb.template loc<sx, sy, sz>() + TK * nb.template til<sx, sy, sz>();
                float cu = 0.f;
                static_for<0, D>([&](auto dc) {
                    constexpr int d = dc.value;
                    if constexpr (L::c(q, d) > 0) cu += a.bc[b + (uint64_t)T * d];
                    else if constexpr (L::c(q, d) < 0) cu -= a.bc[b + (uint64_t)T * d];
                });
                constexpr float six_w = 6.f * wf<L>(q);
                f[q] += six_w * a.bc[b + (uint64_t)T * D] * cu;
            }
        });
    }
    const bool ddf = a.ddf != 0;
    if (a.eqbc && (flag & 0x0F) == LBM_FLAG_EQUILIBRIUM) {
        float ub[3] = {0.f, 0.f, 0.f};
        static_for<0, D>([&](auto dc) { ub[dc.value] = a.bc[own_bc + (uint64_t)T * dc.value]; });
        const float rb = a.bc[own_bc + (uint64_t)T * D];
        const int32_t g[3] = {c.x, c.y, c.z}, ng[3] = {a.lay.nx, a.lay.ny, a.lay.nz};
        float rl = 0.f, ul[3] = {0.f, 0.f, 0.f};
        static_for<0, Q>([&](auto qc) {
            constexpr int q = qc.value;
            bool oob = false;
            static_for<0, D>([&](auto dc) {
                const int32_t pi = g[dc.value] - L::c(q, dc.value);
                oob = oob || pi < 0 || pi >= ng[dc.value];
            });
            const float fq = oob ? (ddf ? 0.f : wf<L>(q)) : f[q];
            rl += fq;
            static_for<0, D>([&](auto dc) {
                constexpr int d = dc.value;
                if constexpr (L::c(q, d) > 0) ul[d] += fq;
                else if constexpr (L::c(q, d) < 0) ul[d] -= fq;
            });
        });
        if (ddf) rl += 1.f;
        static_for<0, D>([&](auto dc) { ul[dc.value] = ul[dc.value] / rl; });
        const bool ufree = isnan(ub[0]);
        float us[3];
        static_for<0, D>([&](auto dc) { us[dc.value] = ufree ? ul[dc.value] : ub[dc.value]; });
        const float rs = isnan(rb) ? rl : rb;
        float uu = 0.f;
        static_for<0, D>([&](auto dc) { uu += us[dc.value] * us[dc.value]; });
        static_for<0, Q>([&](auto qc) { f[qc.value] = feq<L, qc.value>(rs, us, uu, ddf); });
    }
    float rho = 0.f;
    static_for<0, Q>([&](auto qc) { rho += f[qc.value]; });
    if (ddf) rho += 1.f;
    float mom[3] = {0.f, 0.f, 0.f};
    static_for<0, Q>([&](auto qc) {
        constexpr int q = qc.value;
        static_for<0, D>([&](auto dc) {
            constexpr int d = dc.value;
            if constexpr (L::c(q, d) > 0) mom[d] += f[q];
            else if constexpr (L::c(q, d) < 0) mom[d] -= f[q];
        });
    });
    if constexpr (!QCRIT) {
        a.rho[c.r] = rho;
        static_for<0, D>([&](auto dc) { a.u[(size_t)N * dc.value + c.r] = mom[dc.value] / rho; });
    } else {
        // get_f_noneq_vec (post_collision False), get_non_eq_second_order_moment,
        // get_strain_rate_tensor and its norm (kernels/utils/{equilibrium,moment}.mojo), as collide
        float u[3] = {0.f, 0.f, 0.f};
        static_for<0, D>([&](auto dc) { u[dc.value] = mom[dc.value] / rho; });
        float uu = 0.f;
        static_for<0, D>([&](auto dc) { uu += u[dc.value] * u[dc.value]; });
        float P[L::NS];
        static_for<0, L::NS>([&](auto nc) { P[nc.value] = 0.f; });
        for_each_feq<L>(rho, u, uu, ddf, [&](auto qc, float e) {
            constexpr int q = decltype(qc)::value;
            const float fn = f[q] - e;
            static_for<0, L::NS>([&](auto nc) {
                constexpr int n = nc.value;
                constexpr int cc = L::c(q, sa<L>(n)) * L::c(q, sb<L>(n));
                if constexpr (cc > 0) P[n] += fn;
                else if constexpr (cc < 0) P[n] -= fn;
            });
        });
        const float k = -1.f / (2.f * rho * (float)(1.0 / 3.0) * a.tau);
        float s2 = 0.f;
        static_for<0, L::NS>([&](auto nc) {
            constexpr int n = nc.value;
            const float Sn = P[n] * k;
            if constexpr (sa<L>(n) != sb<L>(n)) s2 += (Sn * Sn) * 2.f;
            else s2 += Sn * Sn;
        });
        // calculate_vorticity (Q_criterion.mojo:26-85) and Vector.norm_squared (sequential sum)
        float w2 = 0.f;
        if constexpr (D == 2) {
            const float wz = velocity_gradient<D>(a, c.x, c.y, c.z, 1, 0) - velocity_gradient<D>(a, c.x, c.y, c.z, 0, 1);
            w2 += wz * wz;
        } else {
            const float wx = velocity_gradient<D>(a, c.x, c.y, c.z, 2, 1) - velocity_gradient<D>(a, c.x, c.y, c.z, 1, 2);
            const float wy = velocity_gradient<D>(a, c.x, c.y, c.z, 0, 2) - velocity_gradient<D>(a, c.x, c.y, c.z, 2, 0);
            const float wz = velocity_gradient<D>(a, c.x, c.y, c.z, 1, 0) - velocity_gradient<D>(a, c.x, c.y, c.z, 0, 1);
            w2 += wx * wx;
            w2 += wy * wy;
            w2 += wz * wz;
        }
        a.q[c.r] = 0.25f * w2 - 0.5f * s2;
    }
}

// ---- float64 reductions ---------------------------------------------------------------------
// Deterministic two-pass sums: a fixed grid of kReduceBlocks blocks writes one partial per block
// into scratch, and one block adds the partials in a fixed order.
constexpr int kReduceBlocks = 1024;
constexpr int kReduceThreads = 256;
constexpr int kReduceWidth = 4;

template <int W>
__device__ __forceinline__ void block_sum_store(double (&v)[W], double* dst) {
    __shared__ double sm[kReduceThreads / 32][W];
    static_for<0, W>([&](auto kc) {
        double x = v[kc.value];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        v[kc.value] = x;
    });
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) static_for<0, W>([&](auto kc) { sm[warp][kc.value] = v[kc.value]; });
    __syncthreads();
    if (threadIdx.x < 32) {
        static_for<0, W>([&](auto kc) {
            double x = (lane < (int)(blockDim.x >> 5)) ? sm[lane][kc.value] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) dst[kc.value] = x;
        });
    }
}

struct MassArgs {
    LayoutDesc lay;
    const void* f;
    const uint8_t* flags;
    double* partial;  // kReduceBlocks * 4
    int32_t ddf, even;
};

// Mass and momentum of the post-collision populations of every cell the step updates
// (not SOLID, not EXCLUDE); `even` carries after_odd_step.
template <class L, bool F16C, bool ESO>
__global__ void __launch_bounds__(kReduceThreads) mass_partial_kernel(const MassArgs a) {
    using S = typename Pop<F16C>::T;
    constexpr int Q = L::Q, D = L::D;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < a.lay.ncells; n += gridDim.x * blockDim.x) {
        const uint8_t flag = a.flags[n];
        if ((flag & 0x0F) == LBM_FLAG_SOLID || (flag & LBM_FLAG_EXCLUDE)) continue;
        Nbr nb;
        const Cell c = decode_cell<L>(a.lay, n, nb);
        float f[Q];
        gather_post<L, F16C, ESO>((const S*)a.f, a.lay, c, nb, a.even != 0, f);
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

// Adds `nparts` partials of width W in a fixed order; one block.
template <int W>
__global__ void __launch_bounds__(kReduceThreads) final_sum_kernel(const double* partial, int nparts, double* out) {
    double acc[W];
    static_for<0, W>([&](auto kc) { acc[kc.value] = 0.0; });
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
        static_for<0, W>([&](auto kc) { acc[kc.value] += partial[(size_t)i * W + kc.value]; });
    block_sum_store<W>(acc, out);
}

// Column sums of an n x D float array (link fastest), partials of width 4.
static __global__ void __launch_bounds__(kReduceThreads) colsum_partial_kernel(const float* v, int64_t n, int D,
                                                                        double* partial) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        acc[0] += (double)v[i];
        acc[1] += (double)v[i + n];
        if (D == 3) acc[2] += (double)v[i + 2 * n];
    }
    block_sum_store<4>(acc, partial + (size_t)blockIdx.x * 4);
}

// ---- interpolated bounce-back --------------------------------------------------------------
struct LinkArgs {
    LayoutDesc lay;
    void* f;
    float* force;
    const int32_t* ids;
    const int32_t* dirs;
    const float* dists;
    int64_t n;
    float q_clamp;
    int32_t bouzidi, compute_force, ddf;
};

// linkwise_bounceback_kernel (src/lbm/geometry/interpolated_BB.mojo:46-141); fluid ids are
// decoded as idx_to_ijk does (:24-43).  Float16C is decoded with use_float16c and the force adds
// the weight under DDF shift (output/drag.mojo:88-93).
template <class L, bool F16C>
__device__ __forceinline__ void link_one(const LinkArgs& a, const int64_t t) {
    using P = Pop<F16C>;
    using S = typename P::T;
    constexpr int Q = L::Q, D = L::D;
    const uint32_t li = (uint32_t)a.ids[t];
    if (li >= a.lay.ncells) return;
    Nbr nb;
    const Cell c = decode_cell<L>(a.lay, li, nb);
    const int i = a.dirs[t];
    if (i < 0 || i >= Q) return;
    const int oi = (i == 0) ? 0 : ((i & 1) ? i + 1 : i - 1);
    const uint32_t T = a.lay.T;
    const uint64_t TQ = (uint64_t)T * Q;
    const uint64_t own = c.loc + TQ * c.tile;
    S* f = (S*)a.f;
    float q = a.dists[t];
    q = q < a.q_clamp ? a.q_clamp : q;
    const float f_into = P::ld_rw(f + own + (uint64_t)T * i);
    float f_bb = f_into;
    if (a.bouzidi) {
        if (q > 0.5f) {
            const float f_out = P::ld_rw(f + own + (uint64_t)T * oi);
            f_bb = 0.5f / q * f_into + (2.f * q - 1.f) / (2.f * q) * f_out;
        } else {
            // x_f - c_i, one of the lattice's neighbour shifts
            uint64_t xff = 0;
            static_for<0, Q>([&](auto qc) {
                constexpr int qq = qc.value;
                constexpr int sx = -L::c(qq, 0), sy = -L::c(qq, 1), sz = -L::c(qq, 2);
                if (qq == i) xff = nb.template loc<sx, sy, sz>() + TQ * nb.template til<sx, sy, sz>();
            });
            const float f_xff = P::ld_rw(f + xff + (uint64_t)T * oi);
            f_bb = 2.f * q * f_into + (1.f - 2.f * q) * f_xff;
        }
        P::st(f + own + (uint64_t)T * i, f_bb);
    }
    if (a.compute_force) {
        float w = 0.f;
        static_for<0, Q>([&](auto qc) { if (qc.value == i) w = wf<L>(qc.value); });
        const float fa = a.ddf ? f_into + w : f_into, fb = a.ddf ? f_bb + w : f_bb;
        static_for<0, D>([&](auto dc) {
            int cd = 0;
            static_for<0, Q>([&](auto qc) { if (qc.value == i) cd = L::c(qc.value, dc.value); });
            a.force[t + a.n * dc.value] = (float)cd * (fa + fb);
        });
    }
}

template <class L, bool F16C>
__global__ void link_kernel(const LinkArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    link_one<L, F16C>(a, t);
}

struct DragArgs {
    LayoutDesc lay;
    const void* f;
    const uint8_t* flags;
    const int32_t* ids;
    float* force;
    int64_t n;
    int32_t ddf;
};

// calculate_drag_around_object (src/lbm/output/drag.mojo:16-105): push-neighbour flags, raw
// SOLID compare, F = sum 2 f_q c_q (+ weight under DDF shift).
template <class L, bool F16C>
__global__ void drag_kernel(const DragArgs a) {
    using P = Pop<F16C>;
    using S = typename P::T;
    constexpr int Q = L::Q, D = L::D;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    const uint32_t li = (uint32_t)a.ids[t];
    if (li >= a.lay.ncells) return;
    Nbr nb;
    const Cell c = decode_cell<L>(a.lay, li, nb);
    const uint32_t T = a.lay.T;
    const uint64_t own = c.loc + (uint64_t)T * Q * c.tile;
    const S* f = (const S*)a.f;
    float acc[3] = {0.f, 0.f, 0.f};
    static_for<0, Q>([&](auto qc) {
        constexpr int q = qc.value;
        constexpr int sx = L::c(q, 0), sy = L::c(q, 1), sz = L::c(q, 2);
        const uint8_t pf = a.flags[nb.template loc<sx, sy, sz>() + T * nb.template til<sx, sy, sz>()];
        if (pf == LBM_FLAG_SOLID) {
            float fl = P::ld(f + own + (uint64_t)T * q);
            if (a.ddf) fl += wf<L>(q);
            static_for<0, D>([&](auto dc) {
                constexpr int d = dc.value;
                if constexpr (L::c(q, d) > 0) acc[d] += 2.f * fl;
                else if constexpr (L::c(q, d) < 0) acc[d] -= 2.f * fl;
            });
        }
    });
    static_for<0, D>([&](auto dc) { a.force[t + a.n * dc.value] = acc[dc.value]; });
}

}  // namespace lbm
