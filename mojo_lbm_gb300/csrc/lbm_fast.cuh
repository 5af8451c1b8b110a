// The collision of the fast-arithmetic build (LBM_ARITH_FAST): the same operators as collide()
// in lbm_step.cuh (src/lbm/kernels/steps/collide.mojo:23-90), rearranged for the FMA pipe and
// held to a float32 tolerance instead of the reference's operation order.
//
//  - Moments from the sums and differences of opposite pairs (q, q+1): rho = f0 + sum s_p,
//    m_d = sum +-d_p, Pi_ab = sum c_a c_b s_p (the reference sums f_q over q one by one,
//    src/utils/vector.mojo:205-224).
//  - One approximate reciprocal of rho (rcp.approx), u = m / rho as three products.
//  - Equilibria per opposite pair: f_eq(q), f_eq(q+1) = (A + C45 (e.u)^2) +- C3 (e.u) with the
//    weight, rho and the relaxation rate folded into A, C3, C45, so SRT is two FMAs per
//    population after three per pair (src/lbm/kernels/ops/collisions/collision.mojo:12-46).
//  - The non-equilibrium stress as the raw second moment less the equilibrium's,
//    rho u_a u_b + cs^2 (rho - ddf) delta_ab (algebraically the reference's sum of
//    (f - f_eq) c_a c_b, src/lbm/kernels/utils/moment.mojo:111-150).
//  - KBC (src/lbm/kernels/ops/collisions/KBC_.mojo:180-238) evaluates each f_eq once per pass and
//    takes 1/f_eq by rcp.approx in place of two IEEE divisions per direction.
//  - Float16C storage with a linear collision (SRT, TRT, RLBM without LES) works on "scaled"
//    populations: a code's bits shifted into float32 position are the population times 2^-112
//    (f16c_decode_sx without its final multiplication), the 2^112 is folded into the
//    coefficients, and the result is encoded straight from its scaled value
//    (f16c_encode_scaled).  Everything linear in f is exact under that scaling up to float32
//    rounding at the scaled magnitudes (float32 denormals below 2^-126, i.e. populations below
//    2^-14, keep an absolute resolution of 2^-37, far below a code's).
//
// Included by lbm_step.cuh after StepArgs, kbc_shear and collide.
#pragma once

#include "lbm_device.cuh"

namespace lbm {

// 1/x to within 1 ulp (PTX rcp.approx; subnormal inputs flush to zero, which rho and f_eq never are)
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// e_q . u with the first non-zero component taken as is (no 0 + x), for the fast build
template <class L, int q>
__device__ __forceinline__ float edot_fast(const float* u) {
    constexpr int d0 = L::c(q, 0) != 0 ? 0 : (L::c(q, 1) != 0 ? 1 : 2);
    float o = L::c(q, d0) > 0 ? u[d0] : -u[d0];
    static_for<d0 + 1, L::D>([&](auto dc) {
        constexpr int d = dc.value;
        if constexpr (L::c(q, d) > 0) o += u[d];
        else if constexpr (L::c(q, d) < 0) o -= u[d];
    });
    return o;
}

template <class L, int q>
constexpr int nnz_of() { return (L::c(q, 0) != 0) + (L::c(q, 1) != 0) + (L::c(q, 2) != 0); }

// The pair (q, q+1) of r * f_eq in units s: (plus, minus) = (A + C45 e2) +- C3 eu with
// A = w a0, C3 = 3 w r0, C45 = 4.5 w r0, where the caller passes a0 = r s (rho (1 - 1.5 uu) - ddf)
// and r0 = r s rho.  With ddf this is the shifted equilibrium
// w rho (3 eu + 4.5 eu^2 - 1.5 uu) + w (rho - 1) (src/lbm/kernels/utils/equilibrium.mojo:10-39).
template <class L, int q>
__device__ __forceinline__ void feq_pair_fast(float a0, float r0, const float* u, const float* uc2, float& plus,
                                              float& minus) {
    constexpr float w = wf<L>(q);
    const float eu = edot_fast<L, q>(u);
    float e2;
    if constexpr (nnz_of<L, q>() == 1) {
        constexpr int d0 = L::c(q, 0) != 0 ? 0 : (L::c(q, 1) != 0 ? 1 : 2);
        e2 = uc2[d0];
    } else {
        e2 = eu * eu;
    }
    const float c3 = (3.f * w) * r0;
    const float base = __fmaf_rn((4.5f * w) * r0, e2, w * a0);
    plus = __fmaf_rn(c3, eu, base);
    minus = __fmaf_rn(-c3, eu, base);
}

// The collision of the fast build, in place on f (in units of 2^-112 when SCALED).
// bc_own_base, T, own_flag: the capture outputs, as collide() writes them.
template <class L, int COLL, int LES, bool SCALED>
__device__ __forceinline__ void collide_fast(float (&f)[L::Q], const StepArgs& a, float* bc_own_base, uint32_t T,
                                             uint8_t own_flag, bool active = true) {
    static_assert(!(SCALED && (LES || COLL == LBM_KBC)), "scaled populations need a collision linear in f");
    constexpr int Q = L::Q, D = L::D, NP = (Q - 1) / 2, NS = L::NS;
    constexpr float S = SCALED ? 0x1p-112f : 1.f;  // stored units per population unit
    constexpr float IS = SCALED ? 0x1p112f : 1.f;
    constexpr float cs2 = (float)(1.0 / 3.0);
    const float ddf = a.ddf ? 1.f : 0.f;

    // ---- moments from opposite pairs
    float ps[NP], pd[NP];
    static_for<0, NP>([&](auto pc) {
        constexpr int p = pc.value, q = 2 * p + 1;
        ps[p] = f[q] + f[q + 1];
        pd[p] = f[q] - f[q + 1];
    });
    float rs = f[0];
    static_for<0, NP>([&](auto pc) { rs += ps[pc.value]; });
    float ms[3] = {0.f, 0.f, 0.f};
    static_for<0, D>([&](auto dc) {
        constexpr int d = dc.value;
        bool first = true;
        static_for<0, NP>([&](auto pc) {
            constexpr int p = pc.value, q = 2 * p + 1;
            if constexpr (L::c(q, d) != 0) {
                const float v = L::c(q, d) > 0 ? pd[p] : -pd[p];
                ms[d] = first ? v : ms[d] + v;
                first = false;
            }
        });
    });
    const float rho = __fmaf_rn(rs, IS, ddf);
    const float k = IS * rcp_approx(rho);
    float u[3] = {0.f, 0.f, 0.f}, uc2[3] = {0.f, 0.f, 0.f};
    static_for<0, D>([&](auto dc) {
        u[dc.value] = ms[dc.value] * k;
        uc2[dc.value] = u[dc.value] * u[dc.value];
    });
    float uu = uc2[0] + uc2[1];
    if constexpr (D == 3) uu += uc2[2];

    if (active && a.cap_rho && (own_flag & LBM_FLAG_CAPTURE_DENSITY)) bc_own_base[(size_t)T * D] = rho;
    if (active && a.cap_u && (own_flag & LBM_FLAG_CAPTURE_VELOCITY))
        static_for<0, D>([&](auto dc) { bc_own_base[(size_t)T * dc.value] = u[dc.value]; });

    // rho (1 - 1.5 uu) - ddf: the part of f_eq / w without e.u
    const float r1 = __fmaf_rn(rho, __fmaf_rn(-1.5f, uu, 1.f), -ddf);

    // ---- non-equilibrium stress and the local relaxation time
    float tau_l = a.tau;
    [[maybe_unused]] float P[NS];
    constexpr bool NEED_NEQ = LES || COLL == LBM_KBC || COLL == LBM_RLBM;
    if constexpr (NEED_NEQ) {
        static_for<0, NS>([&](auto nc) {
            constexpr int n = nc.value, A = sa<L>(n), B = sb<L>(n);
            float raw = 0.f;
            bool first = true;
            static_for<0, NP>([&](auto pc) {
                constexpr int p = pc.value, q = 2 * p + 1;
                constexpr int cc = L::c(q, A) * L::c(q, B);
                if constexpr (cc != 0) {
                    const float v = cc > 0 ? ps[p] : -ps[p];
                    raw = first ? v : raw + v;
                    first = false;
                }
            });
            // Pi_ab = IS (raw - m_a u_b) - cs^2 (rho - ddf) delta_ab, with m_a = IS ms_a = rho u_a
            const float t = __fmaf_rn(-ms[A], u[B], raw);
            if constexpr (A == B) P[n] = __fmaf_rn(t, IS, -cs2 * (rho - ddf));
            else P[n] = t * IS;
        });
        if constexpr (LES) {
            // get_strain_rate_tensor / _norm_squared (moment.mojo:154-215),
            // get_Smagorinsky_LES_tau (src/lbm/kernels/ops/turbulence.mojo:12-38):
            // S = -Pi / (2 rho cs^2 tau), tau_l = tau + 3 Cs^2 sqrt(2 |S|^2)
            const float kS = rcp_approx(2.f * cs2 * rho * a.tau);
            float s2 = 0.f;
            static_for<0, NS>([&](auto nc) {
                constexpr int n = nc.value;
                const float pn = P[n];
                if constexpr (sa<L>(n) != sb<L>(n)) s2 = __fmaf_rn(2.f * pn, pn, s2);
                else s2 = __fmaf_rn(pn, pn, s2);
            });
            // |S| = |Pi| kS
            tau_l = __fmaf_rn(3.f * (a.Cs * a.Cs), sqrt_approx(2.f * s2) * kS, a.tau);
        }
    }

    if constexpr (COLL == LBM_SRT) {
        // SRT: f' = (1 - w) f + w f_eq
        const float om = LES ? rcp_approx(tau_l) : a.inv_tau;
        const float om1 = 1.f - om;
        const float a0 = (om * S) * r1, r0 = (om * S) * rho;
        f[0] = __fmaf_rn(om1, f[0], wf<L>(0) * a0);
        static_for<0, NP>([&](auto pc) {
            constexpr int q = 2 * pc.value + 1;
            float p, m;
            feq_pair_fast<L, q>(a0, r0, u, uc2, p, m);
            f[q] = __fmaf_rn(om1, f[q], p);
            f[q + 1] = __fmaf_rn(om1, f[q + 1], m);
        });
    } else if constexpr (COLL == LBM_TRT) {
        // TRT (collision.mojo:49-113), tau_asymm = 1/2 + Lambda / (tau - 1/2)
        // (steps/collide.mojo:214-215): symmetric part relaxed at 1/tau, antisymmetric at 1/tau_a
        const float os = rcp_approx(tau_l);
        const float tm = tau_l - 0.5f;
        const float oa = tm * rcp_approx(__fmaf_rn(0.5f, tm, a.trt_lambda));  // 1 / (1/2 + Lambda / tm)
        const float a0 = os * S * r1, r0s = os * S * rho, r0a = oa * S * rho;
        const float hs = 0.5f * os, ha = 0.5f * oa;
        f[0] = __fmaf_rn(1.f - os, f[0], wf<L>(0) * a0);
        static_for<0, NP>([&](auto pc) {
            constexpr int q = 2 * pc.value + 1;
            constexpr float w = wf<L>(q);
            const float eu = edot_fast<L, q>(u);
            float e2;
            if constexpr (nnz_of<L, q>() == 1) {
                constexpr int d0 = L::c(q, 0) != 0 ? 0 : (L::c(q, 1) != 0 ? 1 : 2);
                e2 = uc2[d0];
            } else {
                e2 = eu * eu;
            }
            // os (f_s - feq_s) with f_s = (f_q + f_o) / 2, feq_s = w (r1 + 4.5 rho e2);
            // oa (f_a - feq_a) with f_a = (f_q - f_o) / 2, feq_a = 3 w rho eu
            const float sym = __fmaf_rn(hs, ps[pc.value], -__fmaf_rn((4.5f * w) * r0s, e2, w * a0));
            const float asy = __fmaf_rn(ha, pd[pc.value], -((3.f * w) * r0a) * eu);
            f[q] = (f[q] - sym) - asy;
            f[q + 1] = (f[q + 1] - sym) + asy;
        });
    } else if constexpr (COLL == LBM_RLBM) {
        // RLBM (collision.mojo:168-223): f' = f_eq + (1 - 1/tau) w / (2 cs^4) H : Pi_neq
        const float om = LES ? rcp_approx(tau_l) : a.inv_tau;
        const float g = (1.f - om) * S;
        const float a0 = S * r1, r0 = S * rho;
        // rest direction: H = -cs^2 delta: H : Pi = -(Pxx + Pyy (+ Pzz)) / 3
        {
            float tr = P[0] + P[L::D == 2 ? 2 : 3];
            if constexpr (L::D == 3) tr += P[5];
            constexpr float k0 = (float)(L::wd(0) / (2.0 / 9.0));
            f[0] = __fmaf_rn((k0 * g) * (float)(-1.0 / 3.0), tr, wf<L>(0) * a0);
        }
        static_for<0, NP>([&](auto pc) {
            constexpr int q = 2 * pc.value + 1;
            float dot = 0.f;
            bool first = true;
            static_for<0, NS>([&](auto nc) {
                constexpr int n = nc.value, A = sa<L>(n), B = sb<L>(n);
                constexpr float Qn = (A == B) ? (float)(L::c(q, A) * L::c(q, B)) - (float)(1.0 / 3.0)
                                              : (float)(2 * L::c(q, A) * L::c(q, B));
                if constexpr (Qn != 0.f) {
                    dot = first ? Qn * P[n] : __fmaf_rn(Qn, P[n], dot);
                    first = false;
                }
            });
            constexpr float kq = (float)(L::wd(q) / (2.0 / 9.0));
            float p, m;
            feq_pair_fast<L, q>(a0, r0, u, uc2, p, m);
            const float t = (kq * g) * dot;
            f[q] = p + t;
            f[q + 1] = m + t;
        });
    } else if constexpr (COLL == LBM_KBC) {
        // KBC (KBC_.mojo:180-238), gamma not clamped: beta = 1 / (2 tau_l),
        // dh = f - f_eq - ds, gamma = 2 tau_l - (2 - 2 tau_l) <ds, dh> / (<dh, dh> + 1e-32),
        // <x, y> = sum x y / f_eq (unshifted); f' = f - beta (2 ds + gamma dh)
        //       = f_eq + (1 - 2 beta) ds + (1 - beta gamma) dh.
        // One pass over the directions computes f_eq and ds once: dh goes to this thread's
        // lane-fastest slots of shared memory, f_eq + (1 - 2 beta) ds stays in f; once gamma is
        // known the update adds (1 - beta gamma) dh.
        __shared__ float dh_keep[Q][256];
        const uint32_t slot = threadIdx.x;
        const float beta = 0.5f * rcp_approx(tau_l);
        const float inv_beta = 2.f * tau_l;
        const float cds = __fmaf_rn(-2.f, beta, 1.f);
        const float a0u = rho * __fmaf_rn(-1.5f, uu, 1.f);  // unshifted: rho (1 - 1.5 uu)
        float sp1 = 0.f, sp2 = 0.f;
        auto visit = [&](auto qc, float fe0) {
            constexpr int q = decltype(qc)::value;
            constexpr float w = wf<L>(q);
            const float ds = kbc_shear<L, q>(P);
            const float fe = __fmaf_rn(-w, ddf, fe0);  // shifted: f_eq - w
            const float dh = (f[q] - fe) - ds;
            const float t = dh * rcp_approx(fe0);
            sp1 = __fmaf_rn(ds, t, sp1);
            sp2 = __fmaf_rn(dh, t, sp2);
            dh_keep[q][slot] = dh;
            f[q] = __fmaf_rn(cds, ds, fe);
        };
        visit(std::integral_constant<int, 0>{}, wf<L>(0) * a0u);
        static_for<0, NP>([&](auto pc) {
            constexpr int q = 2 * pc.value + 1;
            float p, m;
            feq_pair_fast<L, q>(a0u, rho, u, uc2, p, m);
            visit(std::integral_constant<int, q>{}, p);
            visit(std::integral_constant<int, q + 1>{}, m);
        });
        const float gamma = inv_beta - ((2.f - inv_beta) * sp1) * rcp_approx(sp2 + 1e-32f);
        const float cdh = __fmaf_rn(-beta, gamma, 1.f);
        static_for<0, Q>([&](auto qc) { f[qc.value] = __fmaf_rn(cdh, dh_keep[qc.value][slot], f[qc.value]); });
    }
}

}  // namespace lbm
