// The fused stream–collide step for sm_103a.
//
// One thread per lattice cell, threads in the memory order of the reference's tiled layout
// (src/lbm/layoutstruct.mojo:37-92), so every own-cell population access of a warp is a
// contiguous 128-byte (float32) or 64-byte (Float16C) run.  A cell does, in order:
//   stream   — double_buffer_pull_load_f_vec / esoteric_pull_load_f_vec
//              (src/lbm/kernels/ops/load_and_store.mojo:11-86,164-221)
//   BC       — moving_wall_bc, equilibrium_bc (src/lbm/kernels/ops/boundary_condition.mojo:17-205)
//   collide  — SRT / TRT / RLBM / KBC with optional Smagorinsky LES
//              (src/lbm/kernels/steps/collide.mojo:23-90)
//   store    — store_f_vec_to_global (src/lbm/kernels/steps/store_f.mojo:13-40)
// The kernel is bound by HBM traffic (Q loads + Q stores per cell); all arithmetic stays in
// registers, unrolled at compile time over q as the reference does with `comptime for`.
#pragma once

#include "lbm_closure.cuh"
#include "lbm_device.cuh"

namespace lbm {

// LES template argument of the step kernels.
constexpr int kLesOff = 0, kLesSmagorinsky = 1, kLesLearned = 2;


struct StepArgs {
    LayoutDesc lay;
    const void* f_in;
    void* f_out;          // == f_in for esoteric pull
    float* bc;
    const uint8_t* flags;
    float tau, Cs, trt_lambda;
    float inv_tau;             // 1 / tau, rounded as the step would round it (SRT, RLBM without LES)
    int32_t ddf, moving, eqbc, cap_rho, cap_u, even;
    // block-per-tile path (256-cell tiles with power-of-two sides)
    const ClosureDev* closure; // learned LES closure's fragments (learned-closure kernels only)
    ClosureUniform cl;         // and its warp-uniform part
    const uint8_t* tile_near;  // per tile: bit w set if a cell of warp w or a cell it pulls from
                               // holds a flag other than plain FLUID (warp_near)
    const uint2* cell_masks;   // per cell of such a warp: (raw_solid, nib_solid), cell_solid_masks
    uint32_t mx, my, shx, shxy; // lx = t & mx, ly = (t >> shx) & my, lz = t >> shxy
    // interpolated bounce-back fused into the step (block-per-tile kernels, double buffer): per
    // cell, (bit i set for each link whose wall node is x + c_i, index of its first link in the
    // links' order: by cell, then by direction); per link in that order its wall distance and its
    // index in the caller's arrays (for link_force, link_stride floats per component)
    const uint2* link_table;   // null: no fused links
    const float* link_dist;
    const int32_t* link_id;
    float* link_force;         // or null
    int64_t link_stride;
    float q_clamp;
    int32_t bouzidi;
    // staged kernel (lbm_stage.cuh): its copy segments, the bytes they move per tile, the device
    // word its bounded waits raise on a timeout, and bytes added to each stage's expected count
    // (0; a test raises it to make the wait run out)
    const void* stage_segs;
    uint32_t nsegs, stage_bytes;
    uint32_t* err;
    uint32_t stage_extra;
};

// Storage traits: float32, or Float16C codes decoded to float32 (load_f / store_f,
// src/lbm/kernels/utils/load_and_store.mojo:17-110).
template <bool F16C> struct Pop;
template <> struct Pop<false> {
    using T = float;
    static __device__ __forceinline__ float ld(const float* p) { return __ldg(p); }
    static __device__ __forceinline__ float ld_rw(const float* p) { return *p; }
    static __device__ __forceinline__ void st(float* p, float v) { *p = v; }
    // float32 storage has no scaled form (the fast build scales Float16C codes only)
    static __device__ __forceinline__ float ld_scaled(const float* p) { return __ldg(p); }
    static __device__ __forceinline__ float ld_rw_scaled(const float* p) { return *p; }
    static __device__ __forceinline__ void st_scaled(float* p, float v) { *p = v; }
};
template <> struct Pop<true> {
    using T = uint16_t;
    // signed 16-bit loads: the codes arrive sign-extended, as f16c_decode_sx wants them
    static __device__ __forceinline__ float ld(const uint16_t* p) {
        return f16c_decode_sx(__ldg(reinterpret_cast<const int16_t*>(p)));
    }
    static __device__ __forceinline__ float ld_rw(const uint16_t* p) {
        return f16c_decode_sx(*reinterpret_cast<const int16_t*>(p));
    }
    static __device__ __forceinline__ void st(uint16_t* p, float v) { *p = (uint16_t)f16c_encode(v); }
    // the fast build's scaled codes: population * 2^-112 (lbm_fast.cuh)
    static __device__ __forceinline__ float ld_scaled(const uint16_t* p) {
        return f16c_decode_scaled_sx(__ldg(reinterpret_cast<const int16_t*>(p)));
    }
    static __device__ __forceinline__ float ld_rw_scaled(const uint16_t* p) {
        return f16c_decode_scaled_sx(*reinterpret_cast<const int16_t*>(p));
    }
    static __device__ __forceinline__ void st_scaled(uint16_t* p, float v) { *p = (uint16_t)f16c_encode_scaled(v); }
};

// Neighbour offsets along one axis for shifts -1, 0, +1 with the periodic wrap of
// get_adjacent_idx (src/lbm/kernels/utils/index.mojo:44-64): the local part (already scaled by
// the in-tile stride) and the tile part (scaled by the tile stride of the tiler).
struct Axis {
    uint32_t loc[3], til[3];
    __device__ __forceinline__ void init(uint32_t l, uint32_t b, uint32_t t, uint32_t nt, uint32_t lstride,
                                         uint32_t tstride) {
        loc[1] = l * lstride;
        til[1] = b * tstride;
        if (l > 0u) { loc[0] = (l - 1u) * lstride; til[0] = til[1]; }
        else { loc[0] = (t - 1u) * lstride; til[0] = (b > 0u ? b - 1u : nt - 1u) * tstride; }
        if (l + 1u < t) { loc[2] = (l + 1u) * lstride; til[2] = til[1]; }
        else { loc[2] = 0u; til[2] = (b + 1u < nt ? b + 1u : 0u) * tstride; }
    }
};

struct Nbr {
    Axis ax, ay, az;
    // neighbour at (x + sx, y + sy, z + sz), sx..sz in {-1,0,1}: (loc, tile)
    template <int SX, int SY, int SZ>
    __device__ __forceinline__ uint32_t loc() const { return ax.loc[SX + 1] + ay.loc[SY + 1] + az.loc[SZ + 1]; }
    template <int SX, int SY, int SZ>
    __device__ __forceinline__ uint32_t til() const { return ax.til[SX + 1] + ay.til[SY + 1] + az.til[SZ + 1]; }
};

template <class L>
__device__ __forceinline__ float edot(const float* u, int q) {
    // dot(velocity, direction) in d order, zero terms skipped (they add +-0)
    float o = 0.f;
    if (L::c(q, 0)) o = L::c(q, 0) > 0 ? o + u[0] : o - u[0];
    if (L::c(q, 1)) o = L::c(q, 1) > 0 ? o + u[1] : o - u[1];
    if constexpr (L::D == 3) if (L::c(q, 2)) o = L::c(q, 2) > 0 ? o + u[2] : o - u[2];
    return o;
}

// f_eq (src/lbm/kernels/utils/equilibrium.mojo:10-39)
template <class L, int q>
__device__ __forceinline__ float feq(float rho, const float* u, float uu, bool ddf) {
    constexpr float w = wf<L>(q);
    const float eu = edot<L>(u, q);
    if (ddf) return w * rho * (3.f * eu + 4.5f * eu * eu - 1.5f * uu) + w * (rho - 1.f);
    return w * rho * (1.f + 3.f * eu + 4.5f * eu * eu - 1.5f * uu);
}

// Visits f_eq of every direction in order q = 0..Q-1, computing each opposite pair (q, q+1) from
// one dot product: e_{q+1}.u is exactly -(e_q.u) (IEEE sums are sign-symmetric), so 3 e.u and
// 4.5 (e.u)^2 of the pair follow exactly from those of q, and every value equals feq<L, q>.
// fn(qc, feq_with_ddf) is called; with BOTH, fn(qc, feq_with_ddf, feq_unshifted).
template <class L, bool DDF, bool BOTH, class F>
__device__ __forceinline__ void feq_visit(float rho, const float* u, float uu, F&& fn) {
    constexpr int Q = L::Q;
    const float c15 = 1.5f * uu;
    auto emit = [&](auto qc, float wr, float wm, float t3, float t45) {
        [[maybe_unused]] const float plain = (!DDF || BOTH) ? wr * (((1.f + t3) + t45) - c15) : 0.f;
        if constexpr (DDF) {
            const float shifted = wr * ((t3 + t45) - c15) + wm;
            if constexpr (BOTH) fn(qc, shifted, plain);
            else fn(qc, shifted);
        } else {
            if constexpr (BOTH) fn(qc, plain, plain);
            else fn(qc, plain);
        }
    };
    {
        constexpr float w0 = wf<L>(0);
        emit(std::integral_constant<int, 0>{}, w0 * rho, w0 * (rho - 1.f), 0.f, 0.f);
    }
    static_for<1, Q, 2>([&](auto qc) {
        constexpr int q = qc.value;
        constexpr float w = wf<L>(q);
        const float eu = edot<L>(u, q);
        const float t3 = 3.f * eu;
        const float t45 = 4.5f * eu * eu;
        const float wr = w * rho, wm = w * (rho - 1.f);
        emit(qc, wr, wm, t3, t45);
        emit(std::integral_constant<int, q + 1>{}, wr, wm, -t3, t45);
    });
}

template <class L, bool BOTH = false, class F>
__device__ __forceinline__ void for_each_feq(float rho, const float* u, float uu, bool ddf, F&& fn) {
    if (ddf) feq_visit<L, true, BOTH>(rho, u, uu, fn);
    else feq_visit<L, false, BOTH>(rho, u, uu, fn);
}

// KBC shear part of the deviatoric non-equilibrium stress.  D2Q9 is get_shear_D2Q9
// (src/lbm/kernels/ops/collisions/KBC_.mojo:137-175); the 3D form is the same projection for
// D3Q19/D3Q27 (Karlin, Bösch, Chikatamarla, PRE 90, 031302, 2014).
template <class L, int q>
__device__ __forceinline__ float kbc_shear(const float* P) {
    constexpr int cx = L::c(q, 0), cy = L::c(q, 1), cz = L::c(q, 2);
    constexpr int nnz = (cx != 0) + (cy != 0) + (cz != 0);
    if constexpr (L::D == 2) {
        const float N = P[0] - P[2];
        if constexpr (nnz == 1) return cx != 0 ? N * 0.25f : -N * 0.25f;
        else if constexpr (nnz == 2) return (cx * cy > 0) ? P[1] * 0.25f : -P[1] * 0.25f;
        else return 0.f;
    } else {
        if constexpr (nnz == 1) {
            const float Nxz = P[0] - P[5], Nyz = P[3] - P[5];
            constexpr float sixth = (float)(1.0 / 6.0);
            if constexpr (cx != 0) return (2.f * Nxz - Nyz) * sixth;
            else if constexpr (cy != 0) return (2.f * Nyz - Nxz) * sixth;
            else return (-Nxz - Nyz) * sixth;
        } else if constexpr (nnz == 2) {
            if constexpr (cz == 0) return (float)(cx * cy) * P[1] * 0.25f;
            else if constexpr (cy == 0) return (float)(cx * cz) * P[2] * 0.25f;
            else return (float)(cy * cz) * P[4] * 0.25f;
        } else {
            return 0.f;
        }
    }
}

// collide (src/lbm/kernels/steps/collide.mojo:23-90).  LES: 0 off, kLesSmagorinsky, or
// kLesLearned: the closure `cl` in shared memory, evaluated by every lane of the warp (`active`
// is false for the lanes kept alive only for it, which write nothing); the populations wait in
// `stash` (this warp's (Q+3)/4 x 32 float4 of shared memory, lane-fastest) across the features
// and the network, and `stash_holds_f` says the stash already holds them.
template <class L, int COLL, int LES>
__device__ __forceinline__ void collide(float (&f)[L::Q], float tau, const StepArgs& a, float* bc_own_base,
                                        uint32_t T, uint8_t own_flag, bool active = true,
                                        const ClosureDev* cl = nullptr, float4* stash = nullptr,
                                        bool stash_holds_f = false) {
    constexpr int Q = L::Q, D = L::D;
    const bool ddf = a.ddf != 0;
    float rho = 0.f;
    float mom[3] = {0.f, 0.f, 0.f};
    [[maybe_unused]] float Praw[L::NS];  // learned closure: the raw second moment of f
    if constexpr (LES == kLesLearned) {
        // The learned-closure kernels are held to a tolerance (the network is BF16): the moments
        // come from the sums and differences of opposite pairs (q, q+1), c_{q+1} = -c_q, as in the
        // fast arithmetic (lbm_fast.cuh), in place of the reference's sums over q one by one.
        constexpr int NP = (Q - 1) / 2;
        float ps[NP], pd[NP];
        static_for<0, NP>([&](auto pc) {
            constexpr int p = pc.value, q = 2 * p + 1;
            ps[p] = f[q] + f[q + 1];
            pd[p] = f[q] - f[q + 1];
        });
        rho = f[0];
        static_for<0, NP>([&](auto pc) { rho += ps[pc.value]; });
        static_for<0, D>([&](auto dc) {
            constexpr int d = dc.value;
            static_for<0, NP>([&](auto pc) {
                constexpr int p = pc.value, q = 2 * p + 1;
                if constexpr (L::c(q, d) > 0) mom[d] += pd[p];
                else if constexpr (L::c(q, d) < 0) mom[d] -= pd[p];
            });
        });
        static_for<0, L::NS>([&](auto nc) {
            constexpr int n = nc.value;
            Praw[n] = 0.f;
            static_for<0, NP>([&](auto pc) {
                constexpr int p = pc.value, q = 2 * p + 1;
                constexpr int cc = L::c(q, sa<L>(n)) * L::c(q, sb<L>(n));
                if constexpr (cc > 0) Praw[n] += ps[p];
                else if constexpr (cc < 0) Praw[n] -= ps[p];
            });
        });
    } else {
        static_for<0, Q>([&](auto qc) { rho += f[qc.value]; });
        static_for<0, Q>([&](auto qc) {
            constexpr int q = qc.value;
            static_for<0, D>([&](auto dc) {
                constexpr int d = dc.value;
                if constexpr (L::c(q, d) > 0) mom[d] += f[q];
                else if constexpr (L::c(q, d) < 0) mom[d] -= f[q];
            });
        });
    }
    if (ddf) rho += 1.f;
    float u[3] = {0.f, 0.f, 0.f};
    [[maybe_unused]] float ir = 0.f;  // learned closure: 1 / rho
    // A cell with zero momentum (a fluid at rest) takes the signed zeros the divisions would give
    // (rho finite and not zero) without dividing: a zero numerator sends the IEEE division to its
    // special-case path, a third of its usual rate on this GPU.  The learned-closure kernels (held
    // to a tolerance) multiply by one reciprocal of rho instead.
    bool at_rest = LES != kLesLearned && fabsf(rho) < __int_as_float(0x7f800000) && rho != 0.f;
    static_for<0, D>([&](auto dc) { at_rest = at_rest && mom[dc.value] == 0.f; });
    if constexpr (LES == kLesLearned) {
        ir = 1.f / rho;
        static_for<0, D>([&](auto dc) { u[dc.value] = mom[dc.value] * ir; });
    } else if (at_rest) {
        static_for<0, D>([&](auto dc) {
            u[dc.value] = __uint_as_float((__float_as_uint(mom[dc.value]) ^ __float_as_uint(rho)) & 0x80000000u);
        });
    } else {
        static_for<0, D>([&](auto dc) { u[dc.value] = mom[dc.value] / rho; });
    }
    float uu = 0.f;
    static_for<0, D>([&](auto dc) { uu += u[dc.value] * u[dc.value]; });

    if (active && a.cap_rho && (own_flag & LBM_FLAG_CAPTURE_DENSITY)) bc_own_base[(size_t)T * D] = rho;
    if (active && a.cap_u && (own_flag & LBM_FLAG_CAPTURE_VELOCITY))
        static_for<0, D>([&](auto dc) { bc_own_base[(size_t)T * dc.value] = u[dc.value]; });

    float tau_local = tau;
    constexpr bool NEED_NEQ = LES || COLL == LBM_KBC || COLL == LBM_RLBM;
    if constexpr (NEED_NEQ) {
        float P[L::NS];
        static_for<0, L::NS>([&](auto nc) { P[nc.value] = 0.f; });
        if constexpr (LES != kLesLearned) {
            // get_non_eq_second_order_moment (src/lbm/kernels/utils/moment.mojo:111-150)
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
        } else {
            // The same moment from the raw second moment of f less the equilibrium's, which is
            // rho u_a u_b + cs^2 rho delta_ab on these lattices (cs^2 (rho - 1) delta_ab for the
            // DDF-shifted populations): algebraically equal, without f_eq per direction.  The
            // learned-closure kernels are held to a tolerance, not to bit parity.
            static_for<0, L::NS>([&](auto nc) { P[nc.value] = Praw[nc.value]; });
            const float rho_cs2 = (ddf ? rho - 1.f : rho) * (float)(1.0 / 3.0);
            static_for<0, L::NS>([&](auto nc) {
                constexpr int n = nc.value, A = sa<L>(n), B = sb<L>(n);
                P[n] = __fmaf_rn(-mom[A], u[B], P[n]);  // rho u_a = the momentum
                if constexpr (A == B) P[n] -= rho_cs2;
            });
        }
        constexpr int NW = (Q + 3) / 4;
        if constexpr (LES == kLesLearned) {
            // 128-bit words, lane-fastest (conflict-free); explicit shared-memory instructions, so
            // the values leave the registers
            if (!stash_holds_f) {
                const uint32_t lane = threadIdx.x & 31u;
                static_for<0, NW>([&](auto jc) {
                    constexpr int j = jc.value;
                    sts128(stash + j * 32 + lane, f[4 * j], 4 * j + 1 < Q ? f[(4 * j + 1) % Q] : 0.f,
                           4 * j + 2 < Q ? f[(4 * j + 2) % Q] : 0.f, 4 * j + 3 < Q ? f[(4 * j + 3) % Q] : 0.f);
                });
            }
        }
        if constexpr (LES) {
            // get_strain_rate_tensor / _norm_squared (moment.mojo:154-215),
            // get_Smagorinsky_LES_tau (src/lbm/kernels/ops/turbulence.mojo:12-38)
            // k = -1 / (2 rho cs^2 tau); the learned closure's from 1/rho and the host's 1/tau
            const float k = LES == kLesLearned ? (-1.5f * a.inv_tau) * ir
                                               : -1.f / (2.f * rho * (float)(1.0 / 3.0) * tau_local);
            float s2 = 0.f;
            float S[L::NS];
            static_for<0, L::NS>([&](auto nc) {
                constexpr int n = nc.value;
                S[n] = P[n] * k;
                if constexpr (sa<L>(n) != sb<L>(n)) s2 += (S[n] * S[n]) * 2.f;
                else s2 += S[n] * S[n];
            });
            if constexpr (LES == kLesLearned) {
                // learned closure (every lane of the warp), Smagorinsky outside the training range
                __shared__ uint4 stage[8][32];
                __shared__ float ys[8][32];
                const uint32_t w = threadIdx.x >> 5;
                float x[8];
                closure_features<D>(S, s2, rho, uu, tau_local, x);
                bool in_range;
                const float nu = warp_closure_nu(cl, a.cl, x, stage[w], ys[w], in_range);
                if (in_range) tau_local += 3.f * nu;
                else tau_local += 3.f * ((a.Cs * a.Cs) * sqrtf(2.f * s2));  // Smagorinsky (rare)
            } else {
                // sqrt(+0) is +0 (s2 is +0 for a fluid at rest), taken without the square root's
                // special-case path
                const float two_s2 = 2.f * s2;
                tau_local += 3.f * ((a.Cs * a.Cs) * (two_s2 == 0.f ? two_s2 : sqrtf(two_s2)));
            }
        }
        if constexpr (LES == kLesLearned) {
            const uint32_t lane = threadIdx.x & 31u;
            static_for<0, NW>([&](auto jc) {
                constexpr int j = jc.value;
                const float4 v = lds128(stash + j * 32 + lane);
                f[4 * j] = v.x;
                if constexpr (4 * j + 1 < Q) f[4 * j + 1] = v.y;
                if constexpr (4 * j + 2 < Q) f[4 * j + 2] = v.z;
                if constexpr (4 * j + 3 < Q) f[4 * j + 3] = v.w;
            });
        }
        if constexpr (COLL == LBM_RLBM) {
            // RLBM (src/lbm/kernels/ops/collisions/collision.mojo:168-223)
            float inv_tau;
            if constexpr (LES) inv_tau = 1.f / tau_local;
            else inv_tau = a.inv_tau;
            const float one_m = 1.f - inv_tau;
            for_each_feq<L>(rho, u, uu, ddf, [&](auto qc, float e) {
                constexpr int q = decltype(qc)::value;
                float dot = 0.f;
                static_for<0, L::NS>([&](auto nc) {
                    constexpr int n = nc.value, A = sa<L>(n), B = sb<L>(n);
                    constexpr float Qn = (A == B) ? (float)(L::c(q, A) * L::c(q, B)) - (float)(1.0 / 3.0)
                                                  : (float)(2 * L::c(q, A) * L::c(q, B));
                    if constexpr (Qn != 0.f) dot += Qn * P[n];
                });
                constexpr float k = (float)(L::wd(q) / (2.0 / 9.0));
                f[q] = e + one_m * (k * dot);
            });
        } else if constexpr (COLL == LBM_KBC) {
            // KBC (src/lbm/kernels/ops/collisions/KBC_.mojo:180-238); gamma is not clamped
            const float beta = 1.f / (2.f * tau_local);
            const float inv_beta = 2.f * tau_local;
            float sp1 = 0.f, sp2 = 0.f;
            // A zero dh (a population at its equilibrium: every direction of a fluid at rest) makes
            // both numerators zero; with fe0 a number other than zero the quotients are zeros, and
            // adding a zero leaves these sums, which start at +0, unchanged.  Such terms are skipped
            // rather than divided: a zero numerator sends IEEE division to its special-case path, a
            // third of its usual rate on this GPU.  (dh = 0 also means ds is finite.)
            // dh of every direction waits in shared memory (lane-fastest) for the update, which
            // then needs no third f_eq per direction
            __shared__ float dh_keep[Q][256];
            for_each_feq<L, true>(rho, u, uu, ddf, [&](auto qc, float e, float fe0) {
                constexpr int q = decltype(qc)::value;
                const float ds = kbc_shear<L, q>(P);
                const float dh = (f[q] - e) - ds;
                dh_keep[q][threadIdx.x] = dh;
                if (!(dh == 0.f && fe0 == fe0 && fe0 != 0.f)) {
                    sp1 += ds * dh / fe0;
                    sp2 += dh * dh / fe0;
                }
            });
            // The same for gamma's quotient: a zero numerator over a positive finite denominator
            // is the numerator itself.
            const float g_num = (2.f - inv_beta) * sp1, g_den = sp2 + 1e-32f;
            const float g_q = (g_num == 0.f && g_den > 0.f && g_den < __int_as_float(0x7f800000)) ? g_num : g_num / g_den;
            const float gamma = inv_beta - g_q;
            static_for<0, Q>([&](auto qc) {
                constexpr int q = qc.value;
                const float ds = kbc_shear<L, q>(P);
                f[q] -= beta * (2.f * ds + gamma * dh_keep[q][threadIdx.x]);
            });
        }
    }
    if constexpr (COLL == LBM_SRT && LES == kLesLearned) {
        // SRT after the learned closure.  Its kernels are held to a tolerance (the network is
        // BF16), so the relaxation takes the multiply-add form f' = (1 - w) f + w f_eq, with the
        // equilibria of each opposite pair from one e.u: w f_eq(q, q+1) = w_q (a0 + 4.5 r0 (e.u)^2)
        // +- 3 w_q r0 (e.u), a0 = w (rho (1 - 1.5 u.u) - ddf), r0 = w rho
        // (src/lbm/kernels/utils/equilibrium.mojo:10-39, ops/collisions/collision.mojo:12-46).
        const float om = 1.f / tau_local, om1 = 1.f - om;
        const float a0 = om * (rho * (1.f - 1.5f * uu) - (ddf ? 1.f : 0.f)), r0 = om * rho;
        f[0] = om1 * f[0] + wf<L>(0) * a0;
        static_for<1, Q, 2>([&](auto qc) {
            constexpr int q = qc.value;
            constexpr float w = wf<L>(q);
            const float eu = edot<L>(u, q);
            const float c3 = (3.f * w) * r0;
            const float base = ((4.5f * w) * r0) * (eu * eu) + w * a0;
            f[q] = om1 * f[q] + (base + c3 * eu);
            f[q + 1] = om1 * f[q + 1] + (base - c3 * eu);
        });
    } else if constexpr (COLL == LBM_SRT) {
        // SRT (src/lbm/kernels/ops/collisions/collision.mojo:12-46)
        float inv_tau;
        if constexpr (LES) inv_tau = 1.f / tau_local;
        else inv_tau = a.inv_tau;  // the same IEEE quotient, taken once on the host
        for_each_feq<L>(rho, u, uu, ddf, [&](auto qc, float e) {
            constexpr int q = decltype(qc)::value;
            f[q] -= inv_tau * (f[q] - e);
        });
    } else if constexpr (COLL == LBM_TRT) {
        // TRT (collision.mojo:49-113) with tau_asymm of steps/collide.mojo:214-215
        const float tau_a = 0.5f + a.trt_lambda / (tau_local - 0.5f);
        const float is = 1.f / tau_local, ia = 1.f / tau_a;
        float eqv[Q];
        for_each_feq<L>(rho, u, uu, ddf, [&](auto qc, float e) { eqv[decltype(qc)::value] = e; });
        f[0] -= is * (f[0] - eqv[0]);
        static_for<1, Q, 2>([&](auto qc) {
            constexpr int q = qc.value, o = q + 1;
            const float fs = (f[q] + f[o]) * 0.5f, fa = (f[q] - f[o]) * 0.5f;
            const float eq = eqv[q], eo = eqv[o];
            const float es = (eq + eo) * 0.5f, ea = (eq - eo) * 0.5f;
            const float sym = is * (fs - es);
            f[q] -= (sym + ia * (fa - ea));
            f[o] -= (sym + ia * ((-fa) - (-ea)));
        });
    }
}

}  // namespace lbm

#include "lbm_fast.cuh"

namespace lbm {

// moving_wall_bc (src/lbm/kernels/ops/boundary_condition.mojo:17-83): for pulls from a SOLID
// (enum) node, f_q += 6 w_q rho_w (c_q . u_w) with u_w, rho_w read at the solid node.
// bc_base(q) returns the element offset of component 0 of the pull neighbour's bc.  SCALED: f holds
// populations times 2^-112 (the fast build's scaled Float16C codes), and so does the added term.
template <class L, bool SCALED = false, class BcBase>
__device__ __forceinline__ void moving_wall(float (&f)[L::Q], uint32_t nib_solid, const float* bc, uint32_t T,
                                            BcBase&& bc_base) {
    constexpr int Q = L::Q, D = L::D;
    static_for<1, Q>([&](auto qc) {
        constexpr int q = qc.value;
        if ((nib_solid >> q) & 1u) {
            const uint64_t b = bc_base(qc);
            float cu = 0.f;
            static_for<0, D>([&](auto dc) {
                constexpr int d = dc.value;
                if constexpr (L::c(q, d) > 0) cu += bc[b + (uint64_t)T * d];
                else if constexpr (L::c(q, d) < 0) cu -= bc[b + (uint64_t)T * d];
            });
            constexpr float six_w = 6.f * wf<L>(q);
            if constexpr (SCALED) f[q] = __fmaf_rn((six_w * 0x1p-112f) * bc[b + (uint64_t)T * D], cu, f[q]);
            else f[q] += six_w * bc[b + (uint64_t)T * D] * cu;
        }
    });
}

// equilibrium_bc + get_density_and_velocity_for_eq_BC (ops/boundary_condition.mojo:87-205):
// populations pulled across the domain edge count as their rest value; NaN bc components are
// free and come from the node itself.
template <class L>
__device__ __forceinline__ void equilibrium_bc(float (&f)[L::Q], const float* bc, uint64_t own_bc, uint32_t T,
                                               int32_t gx, int32_t gy, int32_t gz, const LayoutDesc& lay, bool ddf) {
    constexpr int Q = L::Q, D = L::D;
    float ub[3] = {0.f, 0.f, 0.f};
    static_for<0, D>([&](auto dc) { ub[dc.value] = bc[own_bc + (uint64_t)T * dc.value]; });
    const float rb = bc[own_bc + (uint64_t)T * D];
    const int32_t g[3] = {gx, gy, gz}, ng[3] = {lay.nx, lay.ny, lay.nz};
    float rl = 0.f, ul[3] = {0.f, 0.f, 0.f};
    static_for<0, Q>([&](auto qc) {
        constexpr int q = qc.value;
        bool oob = false;
        static_for<0, D>([&](auto dc) {
            constexpr int d = dc.value;
            const int32_t pi = g[d] - L::c(q, d);
            oob = oob || pi < 0 || pi >= ng[d];
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
    for_each_feq<L>(rs, us, uu, ddf, [&](auto qc, float e) { f[decltype(qc)::value] = e; });
}

template <class L, int METHOD, bool F16C, int COLL, int LES>
__global__ void __launch_bounds__(256) step_kernel(const StepArgs a) {
    using P = Pop<F16C>;
    using S = typename P::T;
    constexpr int Q = L::Q, D = L::D, K = D + 1;
    constexpr bool ESO = METHOD == LBM_ESOTERIC_PULL;

    static_assert(LES != kLesLearned, "the learned closure runs in the block-per-tile kernel");
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.lay.ncells) return;
    const uint8_t flag = __ldg(a.flags + n);
    // is_valid_thread (src/lbm/kernels/utils/checks.mojo:55-60)
    if ((flag & 0x0F) == LBM_FLAG_SOLID || (flag & LBM_FLAG_EXCLUDE)) return;

    const uint32_t T = a.lay.T;
    const uint32_t tile = a.lay.d_T.div(n);
    const uint32_t loc = n - tile * T;
    const uint32_t lyz = a.lay.d_tx.div(loc);
    const uint32_t lx = loc - lyz * (uint32_t)a.lay.tx;
    const uint32_t lz = a.lay.d_ty.div(lyz);
    const uint32_t ly = lyz - lz * (uint32_t)a.lay.ty;
    const uint32_t byz = a.lay.d_ntx.div(tile);
    const uint32_t bx = tile - byz * (uint32_t)a.lay.ntx;
    const uint32_t bz = a.lay.d_nty.div(byz);
    const uint32_t by = byz - bz * (uint32_t)a.lay.nty;

    Nbr nb;
    const uint32_t txy = (uint32_t)(a.lay.tx * a.lay.ty);
    const uint32_t ntxy = (uint32_t)(a.lay.ntx * a.lay.nty);
    nb.ax.init(lx, bx, a.lay.tx, a.lay.ntx, 1u, 1u);
    nb.ay.init(ly, by, a.lay.ty, a.lay.nty, (uint32_t)a.lay.tx, (uint32_t)a.lay.ntx);
    if constexpr (D == 3) nb.az.init(lz, bz, a.lay.tz, a.lay.ntz, txy, ntxy);
    else { nb.az.loc[0] = nb.az.loc[1] = nb.az.loc[2] = 0u; nb.az.til[0] = nb.az.til[1] = nb.az.til[2] = 0u; }

    const uint64_t TQ = (uint64_t)T * Q;
    const S* fin = (const S*)a.f_in;
    S* fout = (S*)a.f_out;
    const uint64_t own = loc + TQ * tile;

    // ---- stream.  The pull loads are issued first and do not wait for the neighbour flags; the
    // few populations whose pull neighbour is SOLID are re-loaded afterwards from the cell's own
    // opposite slot (mid-grid bounce-back on a raw SOLID compare, ops/load_and_store.mojo:210-219,
    // which also loads the pull value first).
    float f[Q];
    if constexpr (!ESO) {
        static_for<0, Q>([&](auto qc) {
            constexpr int q = qc.value;
            constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
            f[q] = P::ld(fin + nb.template loc<sx, sy, sz>() + TQ * nb.template til<sx, sy, sz>() + (uint64_t)T * q);
        });
    } else {
        const bool ev = a.even != 0;
        f[0] = P::ld_rw(fin + own);
        static_for<1, Q - 1, 2>([&](auto qc) {
            constexpr int pos = qc.value, neg = pos + 1;
            constexpr int sx = L::c(pos, 0), sy = L::c(pos, 1), sz = L::c(pos, 2);
            const uint64_t nbase = nb.template loc<sx, sy, sz>() + TQ * nb.template til<sx, sy, sz>();
            const uint32_t sA = ev ? pos : neg, sB = ev ? neg : pos;
            f[pos] = P::ld_rw(fin + own + (uint64_t)T * sA);
            f[neg] = P::ld_rw(fin + nbase + (uint64_t)T * sB);
        });
    }

    // ---- neighbour flags at x - c_q (set_adjacent_flags, ops/load_and_store.mojo:270-291)
    uint32_t raw_solid = 0u, nib_solid = 0u;
    const bool need_flags = !ESO || a.moving;
    if (need_flags) {
        static_for<1, Q>([&](auto qc) {
            constexpr int q = qc.value;
            constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
            const uint32_t m = nb.template loc<sx, sy, sz>() + T * nb.template til<sx, sy, sz>();
            const uint8_t pf = __ldg(a.flags + m);
            if (pf == LBM_FLAG_SOLID) raw_solid |= 1u << q;
            if ((pf & 0x0F) == LBM_FLAG_SOLID) nib_solid |= 1u << q;
        });
    }
    if constexpr (!ESO) {
        if (raw_solid) {
            static_for<1, Q>([&](auto qc) {
                constexpr int q = qc.value;
                if ((raw_solid >> q) & 1u) f[q] = P::ld(fin + own + (uint64_t)T * opp<L>(q));
            });
        }
    }

    // ---- boundary conditions (steps/apply_boundary_condition.mojo:10-41)
    if (a.moving && nib_solid) {
        const uint64_t TK = (uint64_t)T * K;
        moving_wall<L>(f, nib_solid, a.bc, T, [&](auto qc) -> uint64_t {
            constexpr int q = decltype(qc)::value;
            constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
            return nb.template loc<sx, sy, sz>() + TK * nb.template til<sx, sy, sz>();
        });
    }
    const uint64_t own_bc = loc + (uint64_t)T * K * tile;
    if (a.eqbc && (flag & 0x0F) == LBM_FLAG_EQUILIBRIUM)
        equilibrium_bc<L>(f, a.bc, own_bc, T, (int32_t)(bx * a.lay.tx + lx), (int32_t)(by * a.lay.ty + ly),
                          (int32_t)(bz * a.lay.tz + lz), a.lay, a.ddf != 0);

    collide<L, COLL, LES>(f, a.tau, a, a.bc + own_bc, T, flag);

    // ---- store
    if constexpr (!ESO) {
        static_for<0, Q>([&](auto qc) { P::st(fout + own + (uint64_t)T * qc.value, f[qc.value]); });
    } else {
        // esoteric_pull_store_f_vec (ops/load_and_store.mojo:89-159): the same slots as loaded
        const bool ev = a.even != 0;
        P::st(fout + own, f[0]);
        static_for<1, Q - 1, 2>([&](auto qc) {
            constexpr int pos = qc.value, neg = pos + 1;
            constexpr int sx = L::c(pos, 0), sy = L::c(pos, 1), sz = L::c(pos, 2);
            const uint64_t nbase = nb.template loc<sx, sy, sz>() + TQ * nb.template til<sx, sy, sz>();
            const uint32_t sA = ev ? pos : neg, sB = ev ? neg : pos;
            P::st(fout + nbase + (uint64_t)T * sB, f[pos]);
            P::st(fout + own + (uint64_t)T * sA, f[neg]);
        });
    }
}

// ---------------------------------------------------------------------------------------------
// Block-per-tile path.  One CTA of 256 threads is one 256-cell tile with power-of-two sides, so
// the in-tile coordinates are shifts of threadIdx, the tile coordinates are block-uniform, the
// population offsets q*T are immediates and every neighbour offset is the own offset plus three
// per-axis deltas computed once per thread (32-bit: requires Q*N < 2^31).  Before touching any
// flag, a warp reads its bit of the tile's mask byte: when it is clear, every cell the warp owns
// and every cell it pulls from is plain FLUID, so the neighbour-flag gather and every boundary
// branch are skipped (the common case away from walls).  Results are identical to step_kernel.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kTileCells = 256;

// Per-axis neighbour deltas of a cell of the block-per-tile layout, in cells (dc: flags, bc) and
// in population elements (dp), with periodic wrap across the tile grid.
template <int D>
__device__ __forceinline__ void tile_deltas(const StepArgs& a, uint32_t bx, uint32_t by, uint32_t bz, uint32_t lx,
                                            uint32_t ly, uint32_t lz, int32_t TQ, int32_t (&dc)[3][3],
                                            int32_t (&dp)[3][3]) {
    constexpr int32_t T = (int32_t)kTileCells;
    const int32_t tx = a.lay.tx, ty = a.lay.ty, tz = a.lay.tz, txy = tx * ty;
    const int32_t ntx = a.lay.ntx, nty = a.lay.nty, ntz = a.lay.ntz;
    const int32_t jxm = bx > 0 ? -1 : ntx - 1, jxp = (int32_t)bx + 1 < ntx ? 1 : 1 - ntx;
    const int32_t jym = by > 0 ? -ntx : (nty - 1) * ntx, jyp = (int32_t)by + 1 < nty ? ntx : (1 - nty) * ntx;
    dc[0][1] = dp[0][1] = dc[1][1] = dp[1][1] = dc[2][1] = dp[2][1] = 0;
    if (lx > 0) dc[0][0] = dp[0][0] = -1;
    else { dc[0][0] = (tx - 1) + T * jxm; dp[0][0] = (tx - 1) + TQ * jxm; }
    if ((int32_t)lx + 1 < tx) dc[0][2] = dp[0][2] = 1;
    else { dc[0][2] = (1 - tx) + T * jxp; dp[0][2] = (1 - tx) + TQ * jxp; }
    if (ly > 0) dc[1][0] = dp[1][0] = -tx;
    else { dc[1][0] = (ty - 1) * tx + T * jym; dp[1][0] = (ty - 1) * tx + TQ * jym; }
    if ((int32_t)ly + 1 < ty) dc[1][2] = dp[1][2] = tx;
    else { dc[1][2] = (1 - ty) * tx + T * jyp; dp[1][2] = (1 - ty) * tx + TQ * jyp; }
    if constexpr (D == 3) {
        const int32_t ntxy = ntx * nty;
        const int32_t jzm = bz > 0 ? -ntxy : (ntz - 1) * ntxy, jzp = (int32_t)bz + 1 < ntz ? ntxy : (1 - ntz) * ntxy;
        if (lz > 0) dc[2][0] = dp[2][0] = -txy;
        else { dc[2][0] = (tz - 1) * txy + T * jzm; dp[2][0] = (tz - 1) * txy + TQ * jzm; }
        if ((int32_t)lz + 1 < tz) dc[2][2] = dp[2][2] = txy;
        else { dc[2][2] = (1 - tz) * txy + T * jzp; dp[2][2] = (1 - tz) * txy + TQ * jzp; }
    } else {
        dc[2][0] = dc[2][2] = dp[2][0] = dp[2][2] = 0;
    }
}

// Warp boxes.  Warp w of a 256-cell tile with power-of-two sides owns the cells tid = 32w..32w+31
// of the tile, x fastest: a box of wx x wy x wz cells (wx = min(tx, 32), wy = min(ty, 32 / wx),
// wz = 32 / (wx wy)), lane = ix + wx (iy + wy iz), and these boxes tile the whole grid.  A cell
// pulls from its 26 neighbours at most one cell away: those outside its box lie on the faces of the
// 26 neighbouring boxes that face it (on the intersection of two or three such faces for an edge
// or corner neighbour).
constexpr uint32_t kTileWarps = kTileCells / 32;

// Summary byte of a warp box: bit 0 = a flag of its 32 cells is not 0; bits 1..6 = a flag of its
// -x, +x, -y, +y, -z, +z face layer is not 0.
constexpr uint32_t kBoxAny = 1u;
__host__ __device__ constexpr uint32_t box_face_bit(int axis, int side) { return 1u << (1 + 2 * axis + (side > 0)); }

// 1 if a cell of warp box (tile, w) or a cell it pulls from holds a flag byte other than 0, from the
// box summaries (tile-major: index tile * 8 + w): the box's own bit 0, and for each of the 26
// neighbouring boxes (periodic) the bits of its faces that face the box, all of them set.  When 0,
// every cell of the warp is plain FLUID with plain FLUID pull neighbours, and the step skips every
// flag load.  Exact for walls along the axes; elsewhere it may only report 1 where 0 would do.
__device__ __forceinline__ uint32_t warp_near(const uint8_t* __restrict__ box_sum, const LayoutDesc& l,
                                              uint32_t tile, uint32_t w) {
    // tile sides and box sides are powers of two: shifts and masks; tile-grid sides are not
    const int32_t tx = l.tx, ty = l.ty, tz = l.tz;
    const int32_t wx = min(tx, 32), wy = min(ty, 32 / wx), wz = 32 / (wx * wy);
    const int32_t stx = __ffs(tx) - 1, sty = __ffs(ty) - 1, stz = __ffs(tz) - 1;
    const int32_t swx = __ffs(wx) - 1, swy = __ffs(wy) - 1, swz = __ffs(wz) - 1;
    const uint32_t byz = l.d_ntx.div(tile);
    const int32_t bx = (int32_t)(tile - byz * (uint32_t)l.ntx);
    const int32_t bz = (int32_t)l.d_nty.div(byz), by = (int32_t)byz - bz * l.nty;
    const int32_t t0 = (int32_t)(w * 32u);
    const int32_t gx = ((bx << stx) + (t0 & (tx - 1))) >> swx;
    const int32_t gy = ((by << sty) + ((t0 >> stx) & (ty - 1))) >> swy;
    const int32_t gz = ((bz << stz) + (t0 >> (stx + sty))) >> swz;
    const int32_t nbx = l.nx >> swx, nby = l.ny >> swy, nbz = l.nz >> swz;
    uint32_t r = 0u;
#pragma unroll
    for (int32_t oz = -1; oz <= 1; ++oz) {
        int32_t z = gz + oz;
        z = z < 0 ? nbz - 1 : (z >= nbz ? 0 : z);
        z <<= swz;
#pragma unroll
        for (int32_t oy = -1; oy <= 1; ++oy) {
            int32_t y = gy + oy;
            y = y < 0 ? nby - 1 : (y >= nby ? 0 : y);
            y <<= swy;
            const int32_t tyz = l.ntx * ((y >> sty) + l.nty * (z >> stz));
            const int32_t lyz = ((y & (ty - 1)) << stx) + ((z & (tz - 1)) << (stx + sty));
#pragma unroll
            for (int32_t ox = -1; ox <= 1; ++ox) {
                int32_t x = gx + ox;
                x = x < 0 ? nbx - 1 : (x >= nbx ? 0 : x);
                x <<= swx;
                const uint32_t t = (uint32_t)((x >> stx) + tyz);
                const uint32_t tid = (uint32_t)((x & (tx - 1)) + lyz);
                const uint32_t sum = __ldg(box_sum + t * kTileWarps + (tid >> 5));
                // the neighbour at offset -1 along an axis faces the box with its + face
                uint32_t need = 0u;
                if (ox) need |= box_face_bit(0, -ox);
                if (oy) need |= box_face_bit(1, -oy);
                if (oz) need |= box_face_bit(2, -oz);
                if (!need) need = kBoxAny;
                r |= (sum & need) == need;
            }
        }
    }
    return r;
}

// Cell masks of the six faces of a wx x wy x wz warp box (bit i: cell i = ix + wx (iy + wy iz)):
// -x, +x, -y, +y, -z, +z.
__host__ __device__ __forceinline__ void box_face_masks(uint32_t wx, uint32_t wy, uint32_t wz, uint32_t (&m)[6]) {
    const uint64_t all = 0xFFFFFFFFull;
    const uint64_t every_x = all / ((1ull << wx) - 1ull);            // bit 0 of every row of wx cells
    const uint64_t row = (1ull << wx) - 1ull;                         // one row
    const uint64_t every_layer = all / ((1ull << (wx * wy)) - 1ull);  // bit 0 of every layer
    const uint64_t layer = (1ull << (wx * wy)) - 1ull;                // one layer
    m[0] = (uint32_t)every_x;
    m[1] = (uint32_t)(every_x << (wx - 1u));
    m[2] = (uint32_t)(row * every_layer);
    m[3] = (uint32_t)((row * every_layer) << (wx * (wy - 1u)));
    m[4] = (uint32_t)layer;
    m[5] = (uint32_t)(layer << (wx * wy * (wz - 1u)));
}

// Bit i set where byte i of the 32 bytes w[0..7] (little-endian words) is not 0.
__device__ __forceinline__ uint32_t nonzero_bytes(const uint32_t (&w)[8]) {
    uint32_t m = 0u;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        // bit 7 of each byte: the byte is not 0 (its low 7 bits carry into bit 7, or bit 7 is set)
        const uint32_t t = (((w[k] & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | w[k]) & 0x80808080u;
        m |= ((t * 0x00204081u) >> 28) << (4 * k);  // gathers the four bit 7s into bits 28..31
    }
    return m;
}

// Summary byte of one warp box from its 32 flag bytes (cell order of the box).
__device__ __forceinline__ uint32_t box_summary_of(const uint32_t (&w)[8], const LayoutDesc& l) {
    const uint32_t wx = (uint32_t)min(l.tx, 32), wy = (uint32_t)min(l.ty, 32 / (int32_t)wx), wz = 32u / (wx * wy);
    uint32_t fm[6];
    box_face_masks(wx, wy, wz, fm);
    const uint32_t nz = nonzero_bytes(w);
    uint32_t sum = nz ? kBoxAny : 0u;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (nz & fm[2 * a]) sum |= box_face_bit(a, -1);
        if (nz & fm[2 * a + 1]) sum |= box_face_bit(a, +1);
    }
    return sum;
}

// The 32 flag bytes of warp box `box` (cells 32 box .. 32 box + 31), by 16-byte loads when the
// flags are 16-byte aligned.
__device__ __forceinline__ void load_box_flags(const uint8_t* __restrict__ flags, uint32_t box, uint32_t (&w)[8]) {
    const uint8_t* p = flags + (size_t)box * 32u;
    if ((reinterpret_cast<uintptr_t>(flags) & 15u) == 0u) {
        const uint4 a = __ldg(reinterpret_cast<const uint4*>(p)), b = __ldg(reinterpret_cast<const uint4*>(p) + 1);
        w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w; w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            w[k] = (uint32_t)__ldg(p + 4 * k) | ((uint32_t)__ldg(p + 4 * k + 1) << 8) |
                   ((uint32_t)__ldg(p + 4 * k + 2) << 16) | ((uint32_t)__ldg(p + 4 * k + 3) << 24);
    }
}

// Brings the summary of warp box `box` up to date: if its 32 flags differ from seen (16-byte
// aligned, 32 bytes per box; or force), seen takes them, box_sum[box] is recomputed and *changed
// is set to gen.
__device__ __forceinline__ void update_box_summary(const uint8_t* __restrict__ flags, uint32_t box,
                                                   uint8_t* __restrict__ seen, uint8_t* __restrict__ box_sum,
                                                   const LayoutDesc& l, uint32_t* changed, uint32_t gen, int force) {
    uint32_t w[8];
    load_box_flags(flags, box, w);
    uint4* sp = reinterpret_cast<uint4*>(seen + (size_t)box * 32u);
    const uint4 s0 = sp[0], s1 = sp[1];
    const bool same = s0.x == w[0] && s0.y == w[1] && s0.z == w[2] && s0.w == w[3] && s1.x == w[4] &&
                      s1.y == w[5] && s1.z == w[6] && s1.w == w[7];
    if (same && !force) return;
    sp[0] = make_uint4(w[0], w[1], w[2], w[3]);
    sp[1] = make_uint4(w[4], w[5], w[6], w[7]);
    box_sum[box] = (uint8_t)box_summary_of(w, l);
    *changed = gen;
}

// The per-tile mask byte from the warp_near bits of 8 consecutive threads (thread i: box i of the
// tile-major numbering, i < nboxes); lanes 0, 8, 16, 24 write the byte of their tile.
__device__ __forceinline__ void write_near_mask(uint32_t i, uint32_t nboxes, uint32_t bit, uint8_t* __restrict__ tile_near) {
    const uint32_t m = __ballot_sync(0xffffffffu, i < nboxes && bit != 0u);
    const uint32_t lane = threadIdx.x & 31u;
    if (i < nboxes && (lane & 7u) == 0u) tile_near[i / kTileWarps] = (uint8_t)(m >> lane);
}

// set_adjacent_flags (ops/load_and_store.mojo:270-291) for the cell at flag offset n with cell
// deltas dc: bit q of raw_solid when the flag at x - c_q is SOLID (the raw compare of the
// mid-grid bounce-back, ops/load_and_store.mojo:216), of nib_solid when its enum nibble is SOLID
// (the moving wall, ops/boundary_condition.mojo:77).
template <class L>
__device__ __forceinline__ uint2 cell_solid_masks(const uint8_t* __restrict__ flags, uint32_t n,
                                                  const int32_t (&dc)[3][3]) {
    uint32_t raw_solid = 0u, nib_solid = 0u;
    static_for<1, L::Q>([&](auto qc) {
        constexpr int q = qc.value;
        constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
        const uint8_t pf = __ldg(flags + ((int32_t)n + dc[0][sx + 1] + dc[1][sy + 1] + dc[2][sz + 1]));
        if (pf == LBM_FLAG_SOLID) raw_solid |= 1u << q;
        if ((pf & 0x0F) == LBM_FLAG_SOLID) nib_solid |= 1u << q;
    });
    return make_uint2(raw_solid, nib_solid);
}

// The masks of every cell of the tile's warps whose mask bit is set, for the step to load instead
// of gathering its neighbours' flags (the block of 256 threads of tile `tile`).
template <class L>
__device__ __forceinline__ void tile_cell_masks(const StepArgs& a, uint32_t tile, uint2* __restrict__ masks) {
    const uint32_t tid = threadIdx.x;
    if (((__ldg(a.tile_near + tile) >> (tid >> 5)) & 1u) == 0u) return;  // warp-uniform
    const uint32_t byz = a.lay.d_ntx.div(tile);
    const uint32_t bx = tile - byz * (uint32_t)a.lay.ntx;
    const uint32_t bz = a.lay.d_nty.div(byz);
    const uint32_t by = byz - bz * (uint32_t)a.lay.nty;
    const uint32_t lx = tid & a.mx, ly = (tid >> a.shx) & a.my, lz = tid >> a.shxy;
    int32_t dc[3][3], dp[3][3];
    tile_deltas<L::D>(a, bx, by, bz, lx, ly, lz, (int32_t)(kTileCells * L::Q), dc, dp);
    const uint32_t n = tid + kTileCells * tile;
    masks[n] = cell_solid_masks<L>(a.flags, n, dc);
}

// The shared-memory stage of the staged kernel (lbm_stage.cuh): per direction q, in q order, a region
// of 256 populations (c_q.x = 0) or 512 (c_q.x != 0: the rows of the tile's own column, then those
// of its x-neighbour column).  Position t of a region holds the row the cell t of the tile pulls
// from, shifted by -c_q.y, -c_q.z (from the y/z-neighbour tiles at the tile's faces); along x the
// cell reads position t - c_q.x of the first half, or at the tile's x edge the x-neighbour's cell in
// the second half.
template <class L>
constexpr LBM_HD uint32_t stage_elems(int q) { return L::c(q, 0) == 0 ? kTileCells : 2u * kTileCells; }
template <class L>
constexpr LBM_HD uint32_t stage_off(int q) {
    uint32_t o = 0;
    for (int p = 0; p < q; ++p) o += stage_elems<L>(p);
    return o;
}

// Interpolated bounce-back fused into the step: the node-wise form of the reference's WIP kernel
// (src/lbm/geometry/nodewise_interpolated_BB.mojo:46-185) with the interpolation of its working
// link-wise kernel (geometry/interpolated_BB.mojo:102-141), so that the fused step reproduces the
// link-wise path (step, then linkwise_bounceback_kernel on the lattice it wrote).  For each link
// (x, i) of this cell, i pointing into the wall, the mid-grid bounce-back has just put
// f_in(x, i) into f[j], j = opp(i); with q = max(distance, q_clamp) it becomes Bouzidi's
//   q > 1/2:  f_in(x, i) / (2q) + (2q - 1) / (2q) f_in(x, j)
//   q <= 1/2: 2q f_in(x, i) + (1 - 2q) f_in(x - c_i, j)
// which is the value the link-wise kernel stores in (x, i) for the next step's bounce-back to read;
// the force c_i (f_in(x, i) + f_bb) (+ 2 w_i under DDF shift, output/drag.mojo:88-93) is the link's
// at the step that wrote f_in.  A link whose wall node is not a raw SOLID flag changes nothing here;
// the link-wise path's value in (x, i) is then read by no step either (the wall node is skipped as
// SOLID or pulls its own slot).  The reference's WIP kernel also shifts the interpolation's mass
// change into f_0 (:170,178); the link-wise path does not, nor does this.  SCALED: f holds
// populations times 2^-112, and so do the loaded values.  dp: the cell's element deltas.
template <class L, bool SCALED, class S, class Ld>
__device__ __forceinline__ void fused_links(float (&f)[L::Q], const uint2 lt, const uint32_t raw_solid,
                                            const StepArgs& a, const S* fin, const int32_t own,
                                            const int32_t (&dp)[3][3], Ld&& ld) {
    constexpr int Q = L::Q, D = L::D;
    constexpr uint32_t T = kTileCells;
    uint32_t k = lt.y;
    static_for<1, Q>([&](auto qc) {
        constexpr int i = qc.value, j = opp<L>(i);
        if ((lt.x >> i) & 1u) {
            if ((raw_solid >> j) & 1u) {
                float qd = __ldg(a.link_dist + k);
                qd = qd < a.q_clamp ? a.q_clamp : qd;
                const float f_into = f[j];
                float f_bb = f_into;
                if (a.bouzidi) {
                    if (qd > 0.5f) {
                        const float f_out = ld(fin + own + (int32_t)(T * j));
                        f_bb = 0.5f / qd * f_into + (2.f * qd - 1.f) / (2.f * qd) * f_out;
                    } else {
                        constexpr int sx = L::c(j, 0), sy = L::c(j, 1), sz = L::c(j, 2);  // x - c_i = x + c_j
                        const int32_t o = own + dp[0][sx + 1] + dp[1][sy + 1] + dp[2][sz + 1];
                        const float f_xff = ld(fin + o + (int32_t)(T * j));
                        f_bb = 2.f * qd * f_into + (1.f - 2.f * qd) * f_xff;
                    }
                    f[j] = f_bb;
                }
                if (a.link_force) {
                    constexpr float w = wf<L>(i);
                    float fa = f_into, fb = f_bb;
                    if constexpr (SCALED) { fa *= 0x1p112f; fb *= 0x1p112f; }
                    if (a.ddf) { fa += w; fb += w; }
                    const int64_t id = __ldg(a.link_id + k);
                    static_for<0, D>([&](auto dc) {
                        constexpr int cd = L::c(i, dc.value);
                        a.link_force[id + a.link_stride * dc.value] = (float)cd * (fa + fb);
                    });
                }
            }
            ++k;
        }
    });
}

// The per-thread body of the block-per-tile step: thread `tid` of the CTA that owns tile `tile`.
// Every lane of a warp must call it (the learned closure `cl`, staged in shared memory, is
// evaluated by whole warps).  Learned closure: fbuf is this warp's
// population stash ((Q+3)/4 x 32 float4 of shared memory).
// FAST: the fast-arithmetic collision (collide_fast, lbm_fast.cuh), with scaled Float16C codes
// when the collision is linear in f.  LINKS: the interpolated bounce-back of the links in
// a.link_table fused into the stream (fused_links; double buffer).  It is a separate build because
// its code would raise the register demand of every kernel beyond the budget of 5 CTAs per SM.
// STAGED: the pull loads read the tile's shared-memory stage `stage` (stage_off; double buffer)
// instead of global memory.
// GENERAL = false is the form of a warp whose cells and pull neighbours are all plain FLUID: no
// flag is read and the code is straight-line from the loads to the stores; GENERAL = true reads
// the flags and handles every boundary.
template <class L, int METHOD, bool F16C, int COLL, int LES, bool FAST, bool LINKS, bool STAGED, bool GENERAL>
__device__ __forceinline__ void tile_cell(const StepArgs& a, const uint32_t tile, const uint32_t tid,
                                          const ClosureDev* cl, float4* fbuf, const void* stage) {
    using P = Pop<F16C>;
    using S = typename P::T;
    constexpr int Q = L::Q, D = L::D, K = D + 1;
    constexpr uint32_t T = kTileCells;
    constexpr bool ESO = METHOD == LBM_ESOTERIC_PULL;
    static_assert(!(FAST && LES == kLesLearned), "the learned closure has its own tolerance build");
    static_assert(!(LINKS && ESO), "the fused links are double-buffer only");
    static_assert(!(STAGED && ESO), "the staged kernel is double-buffer only");
    constexpr bool SCALED = FAST && F16C && !LES && COLL != LBM_KBC;
    auto ld = [](const S* p) -> float {
        if constexpr (SCALED) return P::ld_scaled(p);
        else return P::ld(p);
    };
    auto ld_rw = [](const S* p) -> float {
        if constexpr (SCALED) return P::ld_rw_scaled(p);
        else return P::ld_rw(p);
    };
    auto st = [](S* p, float v) {
        if constexpr (SCALED) P::st_scaled(p, v);
        else P::st(p, v);
    };

    const uint32_t n = tid + T * tile;  // cell index = flag offset
    const uint32_t byz = a.lay.d_ntx.div(tile);
    const uint32_t bx = tile - byz * (uint32_t)a.lay.ntx;
    const uint32_t bz = a.lay.d_nty.div(byz);
    const uint32_t by = byz - bz * (uint32_t)a.lay.nty;

    uint8_t flag = 0;
    bool active = true;
    if constexpr (GENERAL) {
        flag = __ldg(a.flags + n);
        // is_valid_thread (src/lbm/kernels/utils/checks.mojo:55-60); the learned closure keeps
        // every lane for its warp-wide products, the invalid ones write nothing
        active = !((flag & 0x0F) == LBM_FLAG_SOLID || (flag & LBM_FLAG_EXCLUDE));
        if constexpr (LES != kLesLearned) {
            if (!active) return;
        }
    }

    // ---- per-axis neighbour deltas, in cells (flags, bc) and in population elements (f)
    const int32_t tx = a.lay.tx, ty = a.lay.ty, tz = a.lay.tz;
    const uint32_t lx = tid & a.mx, ly = (tid >> a.shx) & a.my, lz = tid >> a.shxy;
    const int32_t TQ = (int32_t)(T * Q);
    int32_t dc[3][3], dp[3][3];
    tile_deltas<D>(a, bx, by, bz, lx, ly, lz, TQ, dc, dp);
    const int32_t own = (int32_t)tid + TQ * (int32_t)tile;
    const S* fin = (const S*)a.f_in;
    S* fout = (S*)a.f_out;

    // ---- stream (pull loads first, independent of the flags)
    float f[Q];
    if constexpr (STAGED) {
        // the stage's regions: this cell's position, or along x the neighbour's (stage_off)
        const S* sp = static_cast<const S*>(stage);
        const int32_t t = (int32_t)tid;
        const int32_t bm = lx >= 1u ? t - 1 : t + (int32_t)T + tx - 1;         // source x - 1
        const int32_t bp = (int32_t)lx + 2 <= tx ? t + 1 : t + (int32_t)T - tx + 1;  // source x + 1
        static_for<0, Q>([&](auto qc) {
            constexpr int q = qc.value, cx = L::c(q, 0);
            constexpr uint32_t off = stage_off<L>(q);
            const int32_t b = cx == 0 ? t : (cx > 0 ? bm : bp);
            if constexpr (!F16C) f[q] = sp[off + b];
            else if constexpr (SCALED) f[q] = f16c_decode_scaled_sx(reinterpret_cast<const int16_t*>(sp)[off + b]);
            else f[q] = f16c_decode_sx(reinterpret_cast<const int16_t*>(sp)[off + b]);
        });
    } else if constexpr (!ESO) {
        static_for<0, Q>([&](auto qc) {
            constexpr int q = qc.value;
            constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
            const int32_t o = own + dp[0][sx + 1] + dp[1][sy + 1] + dp[2][sz + 1];
            f[q] = ld(fin + o + (int32_t)(T * q));
        });
    } else {
        // even: pos from (x, pos), neg from (x + c_pos, neg); odd: pos from (x, neg), neg from
        // (x + c_pos, pos).  Slot pos + 1 = neg, so the parity folds into two base pointers.
        const bool ev = a.even != 0;
        const S* finA = fin + (ev ? 0u : T);
        const S* finB = fin + (ev ? T : 0u);
        f[0] = ld_rw(fin + own);
        static_for<1, Q - 1, 2>([&](auto qc) {
            constexpr int pos = qc.value, neg = pos + 1;
            constexpr int sx = L::c(pos, 0), sy = L::c(pos, 1), sz = L::c(pos, 2);
            const int32_t o = own + dp[0][sx + 1] + dp[1][sy + 1] + dp[2][sz + 1];
            f[pos] = ld_rw(finA + own + (int32_t)(T * pos));
            f[neg] = ld_rw(finB + o + (int32_t)(T * pos));
        });
    }

    if constexpr (GENERAL) {
        // ---- neighbour flags at x - c_q, as masks built when the flags last changed
        // (cell_solid_masks: set_adjacent_flags, ops/load_and_store.mojo:270-291)
        uint32_t raw_solid = 0u, nib_solid = 0u;
        if (!ESO || a.moving) {
            const uint2 m = __ldg(a.cell_masks + n);
            raw_solid = m.x;
            nib_solid = m.y;
        }
        if constexpr (!ESO) {
            // mid-grid bounce-back on a raw SOLID compare (ops/load_and_store.mojo:216)
            if (raw_solid)
                static_for<1, Q>([&](auto qc) {
                    constexpr int q = qc.value;
                    if ((raw_solid >> q) & 1u) f[q] = ld(fin + own + (int32_t)(T * opp<L>(q)));
                });
            if constexpr (LINKS) {
                if (raw_solid) {
                    const uint2 lt = __ldg(a.link_table + n);
                    if (lt.x) fused_links<L, SCALED>(f, lt, raw_solid, a, fin, own, dp, ld);
                }
            }
        }
        if (a.moving && nib_solid) {
            moving_wall<L, SCALED>(f, nib_solid, a.bc, T, [&](auto qc) -> uint64_t {
                constexpr int q = decltype(qc)::value;
                constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
                const uint32_t m = (uint32_t)((int32_t)n + dc[0][sx + 1] + dc[1][sy + 1] + dc[2][sz + 1]);
                const uint32_t mt = m / T;
                return (uint64_t)(m - mt * T) + (uint64_t)T * K * mt;
            });
        }
        if (a.eqbc && (flag & 0x0F) == LBM_FLAG_EQUILIBRIUM) {
            if constexpr (SCALED) static_for<0, Q>([&](auto qc) { f[qc.value] *= 0x1p112f; });
            equilibrium_bc<L>(f, a.bc, tid + (uint64_t)T * K * tile, T, (int32_t)(bx * tx + lx),
                              (int32_t)(by * ty + ly), (int32_t)(bz * tz + lz), a.lay, a.ddf != 0);
            if constexpr (SCALED) static_for<0, Q>([&](auto qc) { f[qc.value] *= 0x1p-112f; });
        }
    }

    if constexpr (FAST) collide_fast<L, COLL, LES, SCALED>(f, a, a.bc + (tid + (uint64_t)T * K * tile), T, flag);
    else collide<L, COLL, LES>(f, a.tau, a, a.bc + (tid + (uint64_t)T * K * tile), T, flag, active, cl, fbuf);
    if constexpr (LES == kLesLearned) {
        if (!active) return;
    }

    // ---- store
    if constexpr (!ESO) {
        S* po = fout + own;
        static_for<0, Q>([&](auto qc) { st(po + (int32_t)(T * qc.value), f[qc.value]); });
    } else {
        const bool ev = a.even != 0;
        S* foA = fout + (ev ? 0u : T);
        S* foB = fout + (ev ? T : 0u);
        st(fout + own, f[0]);
        static_for<1, Q - 1, 2>([&](auto qc) {
            constexpr int pos = qc.value, neg = pos + 1;
            constexpr int sx = L::c(pos, 0), sy = L::c(pos, 1), sz = L::c(pos, 2);
            const int32_t o = own + dp[0][sx + 1] + dp[1][sy + 1] + dp[2][sz + 1];
            st(foB + o + (int32_t)(T * pos), f[pos]);
            st(foA + own + (int32_t)(T * pos), f[neg]);
        });
    }
}

template <class L, int METHOD, bool F16C, int COLL, int LES, bool FAST = false, bool LINKS = false,
          bool STAGED = false>
__device__ __forceinline__ void tile_step(const StepArgs& a, const uint32_t tile, const uint32_t tid,
                                          const ClosureDev* cl = nullptr, float4* fbuf = nullptr,
                                          int32_t near = -1, const void* stage = nullptr) {
    // ---- are this warp's cells and their pull neighbours all plain FLUID?  (bit w of the tile's
    // mask byte; the vote makes the choice warp-uniform)
    const uint32_t mask = near >= 0 ? (uint32_t)near : (uint32_t)__ldg(a.tile_near + tile);
    if (__all_sync(0xffffffffu, ((mask >> (tid >> 5)) & 1u) == 0u))
        tile_cell<L, METHOD, F16C, COLL, LES, FAST, LINKS, STAGED, false>(a, tile, tid, cl, fbuf, stage);
    else
        tile_cell<L, METHOD, F16C, COLL, LES, FAST, LINKS, STAGED, true>(a, tile, tid, cl, fbuf, stage);
}

#ifndef LBM_TILE_MIN_BLOCKS
#define LBM_TILE_MIN_BLOCKS 5
#endif
// resident CTAs per SM the KBC and D3Q27 kernels are built for (their register demand is higher)
#ifndef LBM_TILE_MIN_BLOCKS_HEAVY
#define LBM_TILE_MIN_BLOCKS_HEAVY 3
#endif

// Resident CTAs per SM the block-per-tile kernels are built for: D2Q9 5, the KBC and D3Q27 kernels
// LBM_TILE_MIN_BLOCKS_HEAVY, the others LBM_TILE_MIN_BLOCKS (5: 48 registers); the fused-link
// kernels 4 (their interpolation needs 64 registers to run without spilling).
template <class L, int COLL, bool LINKS>
constexpr int tile_min_blocks() {
    constexpr bool heavy = COLL == LBM_KBC || L::Q == 27;
    if constexpr (LINKS) return heavy ? LBM_TILE_MIN_BLOCKS_HEAVY : (L::Q == 9 ? 5 : 4);
    else return (L::Q == 9) ? 5 : (heavy ? LBM_TILE_MIN_BLOCKS_HEAVY : LBM_TILE_MIN_BLOCKS);
}

// Programmatic dependent launch of the step kernels (launch_pdl): wait until the previous grid in
// the stream has completed and its writes are visible, then let the next grid (the next step) be
// scheduled onto the SMs while this one runs, so that its launch latency overlaps this step.  The
// wait comes before any access to the populations, flags or masks; both instructions are no-ops
// for a grid launched without the attribute.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launches a step kernel with programmatic stream serialization allowed (see pdl_enter).
template <class Kernel>
cudaError_t launch_pdl(Kernel kernel, uint32_t grid, uint32_t block, cudaStream_t s, const StepArgs& a) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, a);
}

template <class L, int METHOD, bool F16C, int COLL, int LES, bool FAST = false, bool LINKS = false>
__global__ void __launch_bounds__(256, (tile_min_blocks<L, COLL, LINKS>()))
    step_kernel_tile(const StepArgs a) {
    static_assert(LES != kLesLearned, "the learned closure runs in step_kernel_learned");
    pdl_enter();
    tile_step<L, METHOD, F16C, COLL, LES, FAST, LINKS>(a, blockIdx.x, threadIdx.x);
}

#ifndef LBM_LEARNED_MIN_BLOCKS
#define LBM_LEARNED_MIN_BLOCKS 4
#endif

// The block-per-tile step with the learned closure as a persistent kernel: each CTA stages the
// closure's fragments into shared memory once, then walks the tiles blockIdx.x, + gridDim.x, ...
// (no block barrier inside the time step).
// Shared-memory population stash of the learned-closure kernel: 8 warps x (Q+3)/4 x 32 float4.
template <class L>
struct LearnedStash {
    static constexpr int NW = (L::Q + 3) / 4;
    static constexpr size_t bytes = sizeof(float4) * 8 * NW * 32;  // dynamic shared memory
};

template <class L, int METHOD, bool F16C, int COLL, int LES>
__global__ void __launch_bounds__(256, LBM_LEARNED_MIN_BLOCKS) step_kernel_learned(const StepArgs a) {
    extern __shared__ float4 fbuf[];  // [8 warps][NW][32 lanes]
    const ClosureDev* cl = stage_closure(a.closure);
    __syncthreads();
    const uint32_t ntiles = a.lay.ncells / kTileCells;
    float4* stash = fbuf + (threadIdx.x >> 5) * LearnedStash<L>::NW * 32u;
    // the next tile's neighbourhood byte is loaded one tile ahead
    int32_t near_next = blockIdx.x < ntiles ? __ldg(a.tile_near + blockIdx.x) : 0;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int32_t near = near_next;
        const uint32_t next = tile + gridDim.x;
        near_next = next < ntiles ? __ldg(a.tile_near + next) : 0;
        tile_step<L, METHOD, F16C, COLL, kLesLearned>(a, tile, threadIdx.x, cl, stash, near);
    }
}

// Launcher type used by the dispatch tables.
using StepLaunch = cudaError_t (*)(const StepArgs&, int threads, cudaStream_t);

template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step(const StepArgs& a, int threads, cudaStream_t s) {
    const uint32_t blocks = (a.lay.ncells + (uint32_t)threads - 1u) / (uint32_t)threads;
    step_kernel<L, METHOD, F16C, COLL, LES><<<blocks, threads, 0, s>>>(a);
    return cudaGetLastError();
}

template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_tile(const StepArgs& a, int, cudaStream_t s) {
    return launch_pdl(step_kernel_tile<L, METHOD, F16C, COLL, LES>, a.lay.ncells / kTileCells, kTileCells, s, a);
}

// The fast-arithmetic build of the block-per-tile kernel (LBM_ARITH_FAST).
template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_tile_fast(const StepArgs& a, int, cudaStream_t s) {
    return launch_pdl(step_kernel_tile<L, METHOD, F16C, COLL, LES, true>, a.lay.ncells / kTileCells, kTileCells, s, a);
}

// The block-per-tile kernel with fused links (lbm_set_links), exact and fast arithmetic.
template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_tile_links(const StepArgs& a, int, cudaStream_t s) {
    return launch_pdl(step_kernel_tile<L, METHOD, F16C, COLL, LES, false, true>, a.lay.ncells / kTileCells, kTileCells,
                      s, a);
}
template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_tile_links_fast(const StepArgs& a, int, cudaStream_t s) {
    return launch_pdl(step_kernel_tile<L, METHOD, F16C, COLL, LES, true, true>, a.lay.ncells / kTileCells, kTileCells,
                      s, a);
}

template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_learned(const StepArgs& a, int, cudaStream_t s) {
    constexpr size_t smem = LearnedStash<L>::bytes;
    auto kernel = step_kernel_learned<L, METHOD, F16C, COLL, LES>;
    static int per_sm = 0, sms = 0;
    if (per_sm == 0) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, (int)kTileCells, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    const uint32_t ntiles = a.lay.ncells / kTileCells;
    const uint32_t grid = min(ntiles, (uint32_t)(sms * per_sm));
    kernel<<<grid, kTileCells, smem, s>>>(a);
    return cudaGetLastError();
}

// Tables of the 32 variants of one lattice, indexed by ((method*2 + f16c)*4 + collision)*2 + les.
#define LBM_STEP_ROW(FN, L, M, F)                                                              \
    &FN<L, M, F, LBM_SRT, false>, &FN<L, M, F, LBM_SRT, true>, &FN<L, M, F, LBM_TRT, false>,   \
        &FN<L, M, F, LBM_TRT, true>, &FN<L, M, F, LBM_KBC, false>, &FN<L, M, F, LBM_KBC, true>, \
        &FN<L, M, F, LBM_RLBM, false>, &FN<L, M, F, LBM_RLBM, true>
#define LBM_STEP_TABLE(FN, L)                                                                  \
    {LBM_STEP_ROW(FN, L, LBM_DOUBLE_BUFFER, false), LBM_STEP_ROW(FN, L, LBM_DOUBLE_BUFFER, true), \
     LBM_STEP_ROW(FN, L, LBM_ESOTERIC_PULL, false), LBM_STEP_ROW(FN, L, LBM_ESOTERIC_PULL, true)}

inline int step_index(int method, int f16c, int coll, int les) { return ((method * 2 + f16c) * 4 + coll) * 2 + les; }

// Tables of the 16 double-buffer variants of one lattice (the cell-pair and fused-link kernels),
// indexed by (f16c*4 + collision)*2 + les.
#define LBM_DB_TABLE(FN, L) {LBM_STEP_ROW(FN, L, LBM_DOUBLE_BUFFER, false), LBM_STEP_ROW(FN, L, LBM_DOUBLE_BUFFER, true)}

inline int db_index(int f16c, int coll, int les) { return (f16c * 4 + coll) * 2 + les; }

// Tables of the 16 learned-closure variants of one lattice (block-per-tile kernel), indexed by
// (method*2 + f16c)*4 + collision.
#define LBM_LEARNED_ROW(FN, L, M, F)                                                           \
    &FN<L, M, F, LBM_SRT, kLesLearned>, &FN<L, M, F, LBM_TRT, kLesLearned>,                  \
        &FN<L, M, F, LBM_KBC, kLesLearned>, &FN<L, M, F, LBM_RLBM, kLesLearned>
#define LBM_LEARNED_TABLE(FN, L)                                                               \
    {LBM_LEARNED_ROW(FN, L, LBM_DOUBLE_BUFFER, false), LBM_LEARNED_ROW(FN, L, LBM_DOUBLE_BUFFER, true), \
     LBM_LEARNED_ROW(FN, L, LBM_ESOTERIC_PULL, false), LBM_LEARNED_ROW(FN, L, LBM_ESOTERIC_PULL, true)}

inline int learned_index(int method, int f16c, int coll) { return (method * 2 + f16c) * 4 + coll; }

}  // namespace lbm
