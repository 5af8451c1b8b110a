// Device-side building blocks of the fused LBM step for sm_103a: lattice tables, the Float16C
// codec, the reference's tiled memory layout, and fast division for index decoding.
#pragma once

#include <cmath>
#include <cstdint>
#include <type_traits>
#include <utility>

#include "../../include/lbm_gb300.h"

#if defined(__CUDACC__)
#define LBM_HD __host__ __device__ __forceinline__
#else
#define LBM_HD inline
#endif

namespace lbm {

// ---------------------------------------------------------------------------------------------
// Compile-time loops: the reference unrolls every q loop with `comptime for`; here the index is
// a std::integral_constant so every table lookup folds to an immediate.
// ---------------------------------------------------------------------------------------------
template <int B, int E, int S = 1, class F>
LBM_HD void static_for(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + S, E, S>(std::forward<F>(f));
    }
}

// ---------------------------------------------------------------------------------------------
// Lattices.  Direction order and weights are those of get_D2Q9 / get_D3Q19 / get_D3Q27
// (src/lbm/lattice.mojo:122-352): rest first, then opposite pairs (q odd, q+1 = opposite),
// which the esoteric-pull and TRT code rely on (lattice.mojo:93-113).
// ---------------------------------------------------------------------------------------------
struct D2Q9 {
    static constexpr int id = LBM_D2Q9, D = 2, Q = 9, NS = 3;
    static constexpr LBM_HD int c(int q, int d) {
        constexpr int t[9][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                 {1, 1, 0}, {-1, -1, 0}, {-1, 1, 0}, {1, -1, 0}};
        return t[q][d];
    }
    static constexpr LBM_HD double wd(int q) {
        return q == 0 ? 4.0 / 9.0 : (q < 5 ? 1.0 / 9.0 : 1.0 / 36.0);
    }
};

struct D3Q27 {
    static constexpr int id = LBM_D3Q27, D = 3, Q = 27, NS = 6;
    static constexpr LBM_HD int c(int q, int d) {
        constexpr int t[27][3] = {
            {0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0},  {0, 0, 1},
            {0, 0, -1},  {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},  {-1, 1, 0},  {1, 0, 1},
            {-1, 0, -1}, {1, 0, -1},  {-1, 0, 1},  {0, 1, 1},   {0, -1, -1}, {0, 1, -1},
            {0, -1, 1},  {1, 1, 1},   {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
            {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}};
        return t[q][d];
    }
    static constexpr LBM_HD int nnz(int q) { return (c(q, 0) != 0) + (c(q, 1) != 0) + (c(q, 2) != 0); }
    static constexpr LBM_HD double wd(int q) {
        return nnz(q) == 0 ? 8.0 / 27.0 : nnz(q) == 1 ? 2.0 / 27.0 : nnz(q) == 2 ? 1.0 / 54.0 : 1.0 / 216.0;
    }
};

// D3Q19 is the rest, face and edge directions of D3Q27 in the same order.
struct D3Q19 {
    static constexpr int id = LBM_D3Q19, D = 3, Q = 19, NS = 6;
    static constexpr LBM_HD int c(int q, int d) { return D3Q27::c(q, d); }
    static constexpr LBM_HD double wd(int q) {
        return q == 0 ? 1.0 / 3.0 : (q < 7 ? 1.0 / 18.0 : 1.0 / 36.0);
    }
};

template <class L>
constexpr LBM_HD int opp(int q) { return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1); }

template <class L>
constexpr LBM_HD float wf(int q) { return (float)L::wd(q); }

// Stress index pairs of get_stress_indices (lattice.mojo:354-398).
template <class L>
constexpr LBM_HD int sa(int n) {
    if constexpr (L::D == 2) { constexpr int t[3] = {0, 0, 1}; return t[n]; }
    else { constexpr int t[6] = {0, 0, 0, 1, 1, 2}; return t[n]; }
}
template <class L>
constexpr LBM_HD int sb(int n) {
    if constexpr (L::D == 2) { constexpr int t[3] = {0, 1, 1}; return t[n]; }
    else { constexpr int t[6] = {0, 1, 2, 1, 2, 2}; return t[n]; }
}

// ---------------------------------------------------------------------------------------------
// Float16C (src/utils/custom_fp.mojo:36-101; FluidX3D / Lehmann et al., PRE 106, 015308, 2022):
// sign bit, 4-bit exponent offset by 112 from float32, 11-bit mantissa, round half up on the
// first dropped bit, saturation to 0x7FFF, denormal codes renormalised on decode.
// ---------------------------------------------------------------------------------------------
LBM_HD uint32_t as_u32(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u; __builtin_memcpy(&u, &x, 4); return u;
#endif
}
LBM_HD float as_f32(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x; __builtin_memcpy(&x, &u, 4); return x;
#endif
}

// Decode.  The 15 magnitude bits shifted up by 12 are a float32 whose exponent field is the code's
// (offset 0 instead of 112): for a normal code a float of the right mantissa and an exponent 112
// too small, for a denormal code (zero exponent field) the float32 denormal M * 2^-137 of its
// 11-bit mantissa M.  One multiplication by 2^112 (exact: no overflow, denormal operands are
// kept) gives both, the latter being the M * 2^-25 that the reference's renormalisation builds
// bit by bit.  The sign moves from bit 15 to bit 31.
// hs is the code sign-extended to 32 bits (a signed 16-bit load gives it for free): shifted up by
// 12 its sign copies fill bits 27..31, and the mask keeps bit 31 alone.
LBM_HD float f16c_decode_sx(int32_t hs) {
    const uint32_t bits = ((uint32_t)hs << 12) & 0x87FFFFFFu;
#if defined(__CUDA_ARCH__)
    return __fmul_rn(as_f32(bits), 0x1p112f);
#else
    return as_f32(bits) * 0x1p112f;
#endif
}
LBM_HD float f16c_decode(uint32_t h) { return f16c_decode_sx((int32_t)(int16_t)(uint16_t)h); }

// Bits of |x| * 2^-112 rounded toward zero.  For |x| >= 2^-14 the product is a normal float32 whose
// bits are those of |x| less 112 << 23; below, it is the float32 denormal floor(|x| * 2^37) * 2^-149.
LBM_HD uint32_t f16c_scale_down_rz(float x) {
#if defined(__CUDA_ARCH__)
    return as_u32(__fmul_rz(fabsf(x), 0x1p-112f));
#else
    const double v = (double)as_f32(as_u32(x) & 0x7FFFFFFFu) * 0x1p-112;  // exact in double
    if (!(v < 0x1p-126)) return as_u32((float)v);  // normal, inf or NaN: exact, or a NaN (saturates)
    return (uint32_t)(v * 0x1p149);                 // denormal: truncation
#endif
}

// min(a, b, c) of IEEE minNum: a NaN operand is passed over (the result is NaN only if all are).
LBM_HD float fmin3(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fminf(fminf(a, b), c);
#endif
}

// Encode, with the reference's rounding (add 0x800 to the float32 bits, round half up on the first
// dropped bit, saturate to 0x7FFF, sign from the sum).  With y = |x| * 2^-112 rounded toward zero,
// (bits(y) + 0x800) >> 12 is the code for every magnitude: in the normal range it is
// (|b| >> 12) - (112 << 11) with b = bits(x) + 0x800; in the denormal range it is
// floor(|x| * 2^25 + 1/2), which is the reference's (((0x7FF800 + m) >> (124 - e)) + 1) >> 1, and 0
// below 2^-26.
// Saturation and NaN come from one three-way minimum taken before the scaling, of |x|, the
// magnitude of the float whose bits are b, and kSat = 1.999267578125 (0x3FFFE800, the smallest
// float with code 0x7FFF):
//   - finite x: |float(b)| >= |x| (b is x's bits with 0x800 added to the magnitude) or float(b)
//     is NaN, so the minimum is min(|x|, kSat), which saturates exactly where the code does;
//   - infinity, and a NaN whose sum b is still NaN: the minimum is kSat, code 0x7FFF;
//   - a NaN whose mantissa is within 0x800 of all ones: adding 0x800 carries into the sign bit, b
//     is a denormal of at most 0x7FF ulps, the minimum scales to 0, and the code is the signed
//     zero the reference gives.
// (Checked against the oracle's restatement of the reference for all 2^32 inputs.)
// (y + 0x800) >> 12 for y < 2^28, as the high word of the 64-bit y * 2^20 + 2^31: one wide
// multiply-add on the FMA pipe in place of an add and a shift on the integer pipe.
LBM_HD uint32_t round_shift12(uint32_t y) {
#if defined(__CUDA_ARCH__)
    uint64_t d;
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(d) : "r"(y), "r"(1u << 20), "l"(0x80000000ull));
    return (uint32_t)(d >> 32);
#else
    return (y + 0x00000800u) >> 12;
#endif
}

LBM_HD uint32_t f16c_encode(float x) {
    constexpr float kSat = 0x1.ffdp0f;
    const uint32_t b = as_u32(x) + 0x00000800u;
    const float m = fmin3(fabsf(x), fabsf(as_f32(b)), kSat);
    const uint32_t mag = round_shift12(f16c_scale_down_rz(m));  // m <= kSat: the bits are below 2^27
    return ((b >> 16) & 0x8000u) | mag;
}

// The scaled Float16C codec of the fast-arithmetic build (lbm_fast.cuh).
// decode: the population times 2^-112, exact for every code (the code's magnitude bits placed at
// float32 bits 12..26, its sign at bit 31: f16c_decode_sx without its multiplication).
// encode: the code of xs * 2^112 from xs, rounded as the reference rounds (add 0x800 to the
// float32 bits and drop 12 bits: the scaled float32 has the code's exponent field in place),
// |xs| clamped first to the largest value of code 0x7FFF (infinities and NaN saturate: minNum
// passes over a NaN).  Equal to f16c_encode(xs * 2^112) wherever xs is a normal float32; below
// 2^-126 (populations below 2^-14) xs has already been rounded to a float32 denormal, 2^-149,
// which is 2^-12 of a code's last place.
LBM_HD float f16c_decode_scaled_sx(int32_t hs) { return as_f32(((uint32_t)hs << 12) & 0x87FFFFFFu); }

LBM_HD uint32_t f16c_encode_scaled(float xs) {
    constexpr float kSatScaled = 0x1.ffdp-112f;  // 1.999267578125 * 2^-112
    const float m = fminf(fabsf(xs), kSatScaled);
    return ((as_u32(xs) >> 16) & 0x8000u) | round_shift12(as_u32(m));
}

// ---------------------------------------------------------------------------------------------
// Fast unsigned division by a runtime constant (Granlund & Montgomery, PLDI 1994; the
// "round-up" variant valid for every 32-bit numerator).
// ---------------------------------------------------------------------------------------------
struct FastDiv {
    uint32_t d, m, s;  // s = ceil(log2 d); m = floor(2^32 (2^s - d) / d) + 1
    FastDiv() = default;
    explicit FastDiv(uint32_t div) : d(div), m(0), s(0) {
        while ((1ull << s) < div) ++s;
        m = (uint32_t)((((1ull << 32) * ((1ull << s) - div)) / div) + 1ull);
    }
    LBM_HD uint32_t div(uint32_t n) const {
        if (d == 1u) return n;
#if defined(__CUDA_ARCH__)
        const uint32_t t = __umulhi(n, m);
#else
        const uint32_t t = (uint32_t)(((uint64_t)n * m) >> 32);
#endif
        return (t + ((n - t) >> 1)) >> (s - 1u);
    }
};

// ---------------------------------------------------------------------------------------------
// The reference layout (src/lbm/layoutstruct.mojo:37-92): blocked_product(col_major tile,
// col_major tiler).  A cell's linear index n = loc + T*tile is also its flag offset; its
// population q lives at loc + T*(q + Q*tile).
// ---------------------------------------------------------------------------------------------
struct LayoutDesc {
    int32_t nx, ny, nz, tx, ty, tz, ntx, nty, ntz;
    uint32_t T;        // cells per tile
    uint32_t ncells;   // nx*ny*nz
    FastDiv d_tx, d_ty, d_T, d_ntx, d_nty;
};

}  // namespace lbm
