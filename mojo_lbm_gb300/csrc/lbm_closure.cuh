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
    uint4 w2f[4][32];      // [n-tile][lane]: B fragments of W2, k-slice 0 in .x .y, k-slice 1 in .z .w
    uint4 w3f[32];         // [lane]: B fragments of w3 (output column 0 only), k-slices as W2's
    float4 b1q[4][32];     // [n-tile][lane]: biases of the lane's two accumulator columns laid out as
    float4 b2q[4][32];     // the accumulator quad (c0 c1 | c2 c3 = rows g | g+8): the MMA's C input
    float4 b3q;            // output bias, same layout
};

// The warp-uniform part of the closure, passed by value with the step's arguments (kernel
// parameter space: read as instruction operands, no loads).
struct ClosureUniform {
    float scale[8], shift[8], lo[8], hi[8];  // x_n = fma(x, scale, shift), shift = -mean * scale
    float nu_scale;
};
static_assert(sizeof(ClosureDev) % 16 == 0, "ClosureDev is copied in 16-byte words");

// Copies the closure's fragments into this CTA's shared memory (every thread of the block takes
// part; the caller synchronises the block before the first use).
__device__ __forceinline__ const ClosureDev* stage_closure(const ClosureDev* g) {
    __shared__ ClosureDev s;
    const uint4* src = reinterpret_cast<const uint4*>(g);
    uint4* dst = reinterpret_cast<uint4*>(&s);
    for (uint32_t i = threadIdx.x; i < sizeof(ClosureDev) / 16; i += blockDim.x) dst[i] = __ldg(src + i);
    return &s;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// ReLU and BF16 rounding of two accumulators in one instruction (lo in the low half).
__device__ __forceinline__ uint32_t relu_bf16x2(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

__device__ __forceinline__ void sts128(float4* p, float a, float b, float c, float d) {
    const uint32_t addr = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}
__device__ __forceinline__ float4 lds128(const float4* p) {
    const uint32_t addr = (uint32_t)__cvta_generic_to_shared(p);
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr)
                 : "memory");
    return v;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2_approx(float x) {
    float r;
    asm("lg2.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// d = a b + d
__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// d = a b + c: c is the bias quad (loaded as one 128-bit word, used as is)
__device__ __forceinline__ void mma_bf16_16816_bias(float (&d)[4], const uint32_t (&a)[4], uint2 b, float4 c) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%10,%11,%12,%13};\n"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y), "f"(c.x), "f"(c.y), "f"(c.z), "f"(c.w));
}

// The eight closure features of a cell (definitions in the lbm_closure_t comment of the C
// header), with the hardware's approximate rsqrt / sqrt / log2: network inputs need no IEEE
// rounding.  S: strain-rate components in stress order (2D xx, xy, yy; 3D xx, xy, xz, yy, yz,
// zz), s2 its squared norm (off-diagonals twice).
template <int D>
__device__ __forceinline__ void closure_features(const float* S, float s2, float rho, float uu, float tau,
                                                 float (&x)[8]) {
    float tr, det, off;
    if constexpr (D == 3) {
        tr = S[0] + S[3] + S[5];
        const float m = tr * (1.f / 3.f);
        const float a = S[0] - m, b = S[3] - m, c = S[5] - m;
        const float t1 = __fmaf_rn(b, c, -(S[4] * S[4]));
        const float t2 = __fmaf_rn(-S[4], S[2], S[1] * c);
        const float t3 = __fmaf_rn(-b, S[2], S[1] * S[4]);
        det = __fmaf_rn(S[2], t3, __fmaf_rn(-S[1], t2, a * t1));
        off = 2.f * __fmaf_rn(S[4], S[4], __fmaf_rn(S[2], S[2], S[1] * S[1]));
    } else {
        tr = S[0] + S[2];
        const float m = tr * 0.5f;
        const float a = S[0] - m, b = S[2] - m;
        det = __fmaf_rn(a, b, -(S[1] * S[1]));
        off = 2.f * (S[1] * S[1]);
    }
    const float q = __fmaf_rn(2.f, s2, 1e-24f);  // |S|^2 (+ floor)
    const float r = rsqrt_approx(q);    // 1 / |S|
    constexpr float half_ln2 = 0.34657359027997264f;
    constexpr float ln2 = 0.69314718055994531f;
    x[0] = lg2_approx(q) * half_ln2;
    x[1] = tr * r;
    x[2] = det * (r * r * r);
    x[3] = rho - 1.f;
    x[4] = sqrt_approx(uu);
    x[5] = off * (2.f * (r * r));
    x[6] = lg2_approx(tau - 0.5f) * ln2;
    x[7] = uu * r;
}


// nu_t of the calling lane's cell; every lane of the warp must call it.  c: the per-lane
// fragments in shared memory; u: the uniform part; stage: 32 x uint4 of per-warp shared memory,
// ys: 32 floats of per-warp shared memory.  in_range reports whether the normalised features
// lie in the training range (finite weights assumed: lbm_set_closure rejects others).  Both
// 16-cell row tiles of the warp go through each layer together, so every weight fragment is read
// once and used twice.
__device__ __forceinline__ float warp_closure_nu(const ClosureDev* __restrict__ c, const ClosureUniform& u,
                                                 const float (&x)[8], uint4* stage, float* ys, bool& in_range) {
    const uint32_t lane = threadIdx.x & 31u, g = lane >> 2, t = lane & 3u;
    float xn[8];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        xn[k] = __fmaf_rn(x[k], u.scale[k], u.shift[k]);
        ok = ok & (xn[k] >= u.lo[k]) & (xn[k] <= u.hi[k]);  // no short circuit: predicate chain
    }
    // The verdict rides in the data: a cell outside the training range enters the network as NaN,
    // which stays in its own row of every product, and leaves it as NaN (nothing else stays live
    // across the network).
    xn[0] = ok ? xn[0] : __int_as_float(0x7FC00000);
    stage[lane] = make_uint4(pack_bf16x2(xn[0], xn[1]), pack_bf16x2(xn[2], xn[3]), pack_bf16x2(xn[4], xn[5]),
                             pack_bf16x2(xn[6], xn[7]));
    __syncwarp();
    const uint32_t* st = reinterpret_cast<const uint32_t*>(stage);
    // Layer by layer, each layer's n-tiles in pairs: a pair (2kc, 2kc+1) of one layer's output is
    // k-slice kc of the next layer's input, so it is packed (ReLU, BF16) and consumed before the
    // next pair is computed.  16 accumulators live at a time instead of 32; the products and their
    // accumulation order are those of a layer-at-a-time evaluation.
    uint32_t a1[2][4];  // [mt]: layer-1 A fragments, rows = cells 16 mt + g (+8), K padded to 16
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        a1[mt][0] = st[(16 * mt + g) * 4 + t];
        a1[mt][1] = st[(16 * mt + g + 8) * 4 + t];
        a1[mt][2] = a1[mt][3] = 0u;
    }
    uint32_t a2[2][2][4];  // [mt][k-slice]: layer-2 A fragments
#pragma unroll
    for (int kc = 0; kc < 2; ++kc) {
        float h[2][2][4];  // [mt][j][accumulator] of layer-1 n-tile 2kc + j
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float4 bb = c->b1q[2 * kc + j][lane];
            const uint2 w = c->w1f[2 * kc + j][lane];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) mma_bf16_16816_bias(h[mt][j], a1[mt], w, bb);
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            a2[mt][kc][0] = relu_bf16x2(h[mt][0][0], h[mt][0][1]);
            a2[mt][kc][1] = relu_bf16x2(h[mt][0][2], h[mt][0][3]);
            a2[mt][kc][2] = relu_bf16x2(h[mt][1][0], h[mt][1][1]);
            a2[mt][kc][3] = relu_bf16x2(h[mt][1][2], h[mt][1][3]);
        }
    }
    const uint4 w3 = c->w3f[lane];  // layer 3 (output column 0), k-slice 0 in .x .y, 1 in .z .w
    float y[2][4];
#pragma unroll
    for (int kc = 0; kc < 2; ++kc) {
        float h[2][2][4];  // [mt][j][accumulator] of layer-2 n-tile 2kc + j
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float4 bb = c->b2q[2 * kc + j][lane];
            const uint4 ww = c->w2f[2 * kc + j][lane];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                mma_bf16_16816_bias(h[mt][j], a2[mt][0], make_uint2(ww.x, ww.y), bb);
                mma_bf16_16816(h[mt][j], a2[mt][1], make_uint2(ww.z, ww.w));
            }
        }
        const uint2 w3k = kc == 0 ? make_uint2(w3.x, w3.y) : make_uint2(w3.z, w3.w);
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const uint32_t a3[4] = {relu_bf16x2(h[mt][0][0], h[mt][0][1]), relu_bf16x2(h[mt][0][2], h[mt][0][3]),
                                    relu_bf16x2(h[mt][1][0], h[mt][1][1]), relu_bf16x2(h[mt][1][2], h[mt][1][3])};
            if (kc == 0) mma_bf16_16816_bias(y[mt], a3, w3k, c->b3q);
            else mma_bf16_16816(y[mt], a3, w3k);
        }
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        if (t == 0u) {  // rows g and g + 8 of this tile
            ys[16 * mt + g] = y[mt][0];
            ys[16 * mt + g + 8] = y[mt][2];
        }
    }
    __syncwarp();
    const float yo = ys[lane];
    __syncwarp();  // stage / ys are reused by the next call
    in_range = yo == yo;
    const float sp = yo > 20.f ? yo : __logf(1.f + __expf(yo));  // softplus
    return sp * u.nu_scale;
}

}  // namespace lbm
