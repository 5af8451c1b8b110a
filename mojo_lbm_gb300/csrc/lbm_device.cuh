// Device-side building blocks of the fused LBM step for sm_103a: lattice tables, the Float16C
// codec, the reference's tiled memory layout, and fast division for index decoding.
#pragma once

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

// Decode.  A code with a non-zero exponent field is a normal float32 whose exponent is 112 larger:
// shifting the 15 magnitude bits up by 12 and adding 112 << 23 produces it.  A code with a zero
// exponent field (denormal) is M * 2^-25 for its 11-bit mantissa M, exact in float32; this is
// the value the reference's renormalisation builds bit by bit.
LBM_HD float f16c_decode(uint32_t h) {
    const uint32_t mag = h & 0x7FFFu;
    const uint32_t nrm = (mag << 12) + 0x38000000u;
    const uint32_t den = as_u32((float)mag * 0x1p-25f);
    return as_f32(((h & 0x8000u) << 16) | (mag >= 0x0800u ? nrm : den));
}

// Encode, with the reference's rounding: add 0x800 to the float32 bits (round half up on the
// first dropped bit), then take the exponent e of the sum:
//   e > 112       normal code ((e - 112) << 11) | (m >> 12), i.e. (|b| >> 12) - (112 << 11),
//                 saturated to 0x7FFF when e > 127;
//   100 < e < 113 denormal code (((0x7FF800 + m) >> (124 - e)) + 1) >> 1;
//   e < 101       zero.
// The sign bit is taken from the sum.  Only the low 16 bits are kept.
LBM_HD uint32_t f16c_encode(float x) {
    const uint32_t b = as_u32(x) + 0x00000800u;
    const uint32_t e = (b >> 23) & 0xFFu;
    const uint32_t m = b & 0x007FFFFFu;
    const uint32_t nrm_raw = ((b & 0x7FFFFFFFu) >> 12) - 0x38000u;
    const uint32_t nrm = nrm_raw < 0x7FFFu ? nrm_raw : 0x7FFFu;
    const uint32_t sh = e > 112u ? 12u : (e < 101u ? 23u : 124u - e);
    const uint32_t den = (((0x007FF800u + m) >> sh) + 1u) >> 1;
    const uint32_t mag = e > 112u ? nrm : (e > 100u ? den : 0u);
    return ((b & 0x80000000u) >> 16) | mag;
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
