// Learned subgrid closure, evaluated inside the LES collision on the tensor cores.
//
// Every warp evaluates the MLP 8 -> 32 -> 32 -> 1 for its 32 cells as three small matrix
// products (cells x features) x (features x units) with mma.sync.m16n8k16 (BF16 inputs, FP32
// accumulation): 2 row tiles of 16 cells x (4 + 8 + 2) tensor instructions.  Biases initialise
// the accumulators, ReLU outputs of one layer are repacked in registers as the next layer's A
// fragments (the accumulator layout of m16n8k16 is the A layout of the next k-slice), and the
// weights sit in device memory pre-arranged per lane as B fragments, so each lane loads exactly
// its own fragment words.  No counterpart in the reference (its LES is Smagorinsky only,
// src/lbm/kernels/ops/turbulence.mojo:12-38).
#pragma once

#include <cuda_bf16.h>

#include "lbm_device.cuh"

namespace lbm {

struct alignas(16) ClosureDev {
    uint2 w1f[4][32];      // [n-tile][lane]: B fragment of W1 (K = 8 features, zero-padded to 16)
    uint2 w2f[4][2][32];   // [n-tile][k-slice][lane]
    uint2 w3f[2][32];      // [k-slice][lane] (output column 0 only)
    float2 b1f[4][32];     // [n-tile][lane]: biases of the lane's two accumulator columns
    float2 b2f[4][32];
    float mean[8], scale[8], lo[8], hi[8];
    float b3, nu_scale, pad_[2];
};
static_assert(sizeof(ClosureDev) % 16 == 0, "ClosureDev is copied in 16-byte words");

// Copies the closure's fragments into this CTA's shared memory (every thread of the block takes
// part; the caller synchronises the block before the first use).  Null stays null.
template <bool LES>
__device__ __forceinline__ const ClosureDev* stage_closure(const ClosureDev* g) {
    if constexpr (!LES) {
        return nullptr;
    } else {
        __shared__ ClosureDev s;
        if (g == nullptr) return nullptr;
        const uint4* src = reinterpret_cast<const uint4*>(g);
        uint4* dst = reinterpret_cast<uint4*>(&s);
        for (uint32_t i = threadIdx.x; i < sizeof(ClosureDev) / 16; i += blockDim.x) dst[i] = __ldg(src + i);
        return &s;
    }
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// The eight closure features of a cell (see lbm_closure_t in the C header).  S: strain-rate
// components in stress order (2D xx, xy, yy; 3D xx, xy, xz, yy, yz, zz), s2 its squared norm.
template <int D>
__device__ __forceinline__ void closure_features(const float* S, float s2, float rho, float uu, float tau,
                                                 float (&x)[8]) {
    const float snorm = sqrtf(2.f * s2);
    float tr, det, off;
    if constexpr (D == 3) {
        tr = S[0] + S[3] + S[5];
        const float m = tr * (1.f / 3.f);
        const float a = S[0] - m, b = S[3] - m, c = S[5] - m;
        det = a * (b * c - S[4] * S[4]) - S[1] * (S[1] * c - S[4] * S[2]) + S[2] * (S[1] * S[4] - b * S[2]);
        off = 2.f * (S[1] * S[1] + S[2] * S[2] + S[4] * S[4]);
    } else {
        tr = S[0] + S[2];
        const float m = tr * 0.5f;
        const float a = S[0] - m, b = S[2] - m;
        det = a * b - S[1] * S[1];
        off = 2.f * (S[1] * S[1]);
    }
    // network inputs need no IEEE rounding: fast log and division (the oracle uses libm's)
    const float inv_s = __fdividef(1.f, snorm + 1e-12f);
    x[0] = __logf(snorm + 1e-12f);
    x[1] = tr * inv_s;
    x[2] = __fdividef(det, snorm * snorm * snorm + 1e-30f);
    x[3] = rho - 1.f;
    x[4] = sqrtf(uu);
    x[5] = __fdividef(off, s2 + 1e-30f);
    x[6] = __logf(tau - 0.5f);
    x[7] = uu * inv_s;
}

// nu_t of the calling lane's cell; every lane of the warp must call it.  stage: 32 x uint4 of
// per-warp shared memory, ys: 32 floats of per-warp shared memory.  in_range reports whether the
// normalised features lie in the training range.
__device__ __forceinline__ float warp_closure_nu(const ClosureDev* __restrict__ c, const float (&x)[8], uint4* stage,
                                                 float* ys, bool& in_range) {
    const uint32_t lane = threadIdx.x & 31u, g = lane >> 2, t = lane & 3u;
    float xn[8];
    in_range = true;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        xn[k] = (x[k] - c->mean[k]) * c->scale[k];
        in_range = in_range && xn[k] >= c->lo[k] && xn[k] <= c->hi[k];
    }
    stage[lane] = make_uint4(pack_bf16x2(xn[0], xn[1]), pack_bf16x2(xn[2], xn[3]), pack_bf16x2(xn[4], xn[5]),
                             pack_bf16x2(xn[6], xn[7]));
    __syncwarp();
    const uint32_t* st = reinterpret_cast<const uint32_t*>(stage);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        // layer 1: rows = cells 16 mt + g (+8), columns = features 2t, 2t+1 (K padded to 16)
        const uint32_t a1[4] = {st[(16 * mt + g) * 4 + t], st[(16 * mt + g + 8) * 4 + t], 0u, 0u};
        float h1[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const float2 bb = c->b1f[nt][lane];
            h1[nt][0] = bb.x; h1[nt][1] = bb.y; h1[nt][2] = bb.x; h1[nt][3] = bb.y;
            mma_bf16_16816(h1[nt], a1, c->w1f[nt][lane]);
        }
        uint32_t a2[2][4];
#pragma unroll
        for (int kc = 0; kc < 2; ++kc) {
            a2[kc][0] = pack_bf16x2(fmaxf(h1[2 * kc][0], 0.f), fmaxf(h1[2 * kc][1], 0.f));
            a2[kc][1] = pack_bf16x2(fmaxf(h1[2 * kc][2], 0.f), fmaxf(h1[2 * kc][3], 0.f));
            a2[kc][2] = pack_bf16x2(fmaxf(h1[2 * kc + 1][0], 0.f), fmaxf(h1[2 * kc + 1][1], 0.f));
            a2[kc][3] = pack_bf16x2(fmaxf(h1[2 * kc + 1][2], 0.f), fmaxf(h1[2 * kc + 1][3], 0.f));
        }
        float h2[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const float2 bb = c->b2f[nt][lane];
            h2[nt][0] = bb.x; h2[nt][1] = bb.y; h2[nt][2] = bb.x; h2[nt][3] = bb.y;
#pragma unroll
            for (int kc = 0; kc < 2; ++kc) mma_bf16_16816(h2[nt], a2[kc], c->w2f[nt][kc][lane]);
        }
        uint32_t a3[2][4];
#pragma unroll
        for (int kc = 0; kc < 2; ++kc) {
            a3[kc][0] = pack_bf16x2(fmaxf(h2[2 * kc][0], 0.f), fmaxf(h2[2 * kc][1], 0.f));
            a3[kc][1] = pack_bf16x2(fmaxf(h2[2 * kc][2], 0.f), fmaxf(h2[2 * kc][3], 0.f));
            a3[kc][2] = pack_bf16x2(fmaxf(h2[2 * kc + 1][0], 0.f), fmaxf(h2[2 * kc + 1][1], 0.f));
            a3[kc][3] = pack_bf16x2(fmaxf(h2[2 * kc + 1][2], 0.f), fmaxf(h2[2 * kc + 1][3], 0.f));
        }
        float y[4] = {c->b3, c->b3, c->b3, c->b3};
#pragma unroll
        for (int kc = 0; kc < 2; ++kc) mma_bf16_16816(y, a3[kc], c->w3f[kc][lane]);
        if (t == 0u) {  // output column 0: rows g and g + 8 of this tile
            ys[16 * mt + g] = y[0];
            ys[16 * mt + g + 8] = y[2];
        }
    }
    __syncwarp();
    const float yo = ys[lane];
    __syncwarp();  // stage / ys are reused by the next call
    const float sp = yo > 20.f ? yo : __logf(1.f + __expf(yo));  // softplus
    return sp * c->nu_scale;
}

}  // namespace lbm
