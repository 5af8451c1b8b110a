// The cell-pair form of the block-per-tile step (double buffer): one thread streams and collides
// two cells that are neighbours along x, so that half of the population traffic moves as 64-bit
// (float32) or 32-bit (Float16C) words and half of the neighbour address arithmetic is shared.
//
// A 256-cell tile with power-of-two sides and tx >= 2 is one CTA of 128 threads; thread t owns the
// cells tA = 2t and tB = 2t + 1 of the tile, which sit at x_A (even) and x_A + 1 of one tile row.
// For a direction q the pull source of A is x_A - c_q and that of B is one cell further along x:
//   c_q.x =  0: the two sources are the aligned pair (x_A, x_A + 1) of the source row: one word;
//   c_q.x = +1: A from x_A - 1 (the west tile's last cell when x_A = 0), B from x_A;
//   c_q.x = -1: A from x_A + 1, B from x_A + 2 (the east tile's first cell when x_A + 2 = tx).
// The source row (y - c_q.y, z - c_q.z) is shared by up to three directions, so a D3Q19 pair
// computes 9 row addresses and 10 west/east addresses for its 38 populations.  Every own-cell
// access (the stores, the mid-grid bounce-back reload) is one word per direction.
//
// Everything else is the per-cell code of tile_step (lbm_step.cuh), applied to A and B in turn:
// the same mid-grid bounce-back on the cell-solid masks, moving wall, equilibrium boundary,
// collision and capture, so the results are those of step_kernel_tile bit for bit (the exact
// build) or to its tolerance (the fast build).  A warp owns the warp boxes 2w and 2w + 1 of the
// tile (its 64 cells); it takes the all-fluid branch when both boxes' mask bits are clear.
//
// Requirements: the population buffers 8-byte aligned (the host falls back to the per-cell kernel
// otherwise), tx >= 2, the double-buffer method, no learned closure.
#pragma once

#include "lbm_step.cuh"

namespace lbm {

constexpr uint32_t kPairThreads = kTileCells / 2;

// Word access to the aligned pair (A, B) of one population slot.
template <bool F16C, bool SCALED> struct PairWord;
template <bool SCALED> struct PairWord<false, SCALED> {
    static __device__ __forceinline__ void ld(const float* p, float& a, float& b) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(p));
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void st(float* p, float a, float b) {
        *reinterpret_cast<float2*>(p) = make_float2(a, b);
    }
};
template <bool SCALED> struct PairWord<true, SCALED> {
    // low half: A's code, high half: B's (little-endian).  The high code arrives sign-extended by
    // an arithmetic shift; the low one by shifting it to the top first.
    static __device__ __forceinline__ void ld(const uint16_t* p, float& a, float& b) {
        const uint32_t w = __ldg(reinterpret_cast<const uint32_t*>(p));
        const int32_t lo = (int32_t)(w << 16) >> 16, hi = (int32_t)w >> 16;
        if constexpr (SCALED) {
            a = f16c_decode_scaled_sx(lo);
            b = f16c_decode_scaled_sx(hi);
        } else {
            a = f16c_decode_sx(lo);
            b = f16c_decode_sx(hi);
        }
    }
    static __device__ __forceinline__ void st(uint16_t* p, float a, float b) {
        uint32_t w;
        if constexpr (SCALED) {
            // f16c_encode_scaled of both: the two magnitudes side by side, then both signs (the top
            // bytes of a and b moved to bytes 1 and 3, bits 15 and 31 kept) in one bitwise select
            constexpr float kSatScaled = 0x1.ffdp-112f;
            const uint32_t ma = round_shift12(as_u32(fminf(fabsf(a), kSatScaled)));
            const uint32_t mb = round_shift12(as_u32(fminf(fabsf(b), kSatScaled)));
            const uint32_t signs = __byte_perm(as_u32(a), as_u32(b), 0x7430);
            w = (signs & 0x80008000u) | __byte_perm(ma, mb, 0x5410);
        } else {
            w = __byte_perm(f16c_encode(a), f16c_encode(b), 0x5410);
        }
        *reinterpret_cast<uint32_t*>(p) = w;
    }
};

// Element deltas of the pair: y and z as in tile_deltas (shifts -1, 0, +1), and along x the
// delta from A to x_A - 1 and from B to x_B + 1 (-1 / +1 inside the tile, the periodic jump to
// the neighbouring tile at its edge).
template <int D>
__device__ __forceinline__ void pair_deltas(const StepArgs& a, uint32_t bx, uint32_t by, uint32_t bz, uint32_t lxA,
                                            uint32_t ly, uint32_t lz, int32_t TQ, int32_t& dxm, int32_t& dxp,
                                            int32_t (&dy)[3], int32_t (&dz)[3]) {
    const int32_t tx = a.lay.tx, ty = a.lay.ty, tz = a.lay.tz, txy = tx * ty;
    const int32_t ntx = a.lay.ntx, nty = a.lay.nty, ntz = a.lay.ntz;
    const int32_t jxm = bx > 0 ? -1 : ntx - 1, jxp = (int32_t)bx + 1 < ntx ? 1 : 1 - ntx;
    const int32_t jym = by > 0 ? -ntx : (nty - 1) * ntx, jyp = (int32_t)by + 1 < nty ? ntx : (1 - nty) * ntx;
    dxm = lxA > 0 ? -1 : (tx - 1) + TQ * jxm;
    dxp = (int32_t)lxA + 2 < tx ? 1 : (1 - tx) + TQ * jxp;
    dy[1] = dz[1] = 0;
    dy[0] = ly > 0 ? -tx : (ty - 1) * tx + TQ * jym;
    dy[2] = (int32_t)ly + 1 < ty ? tx : (1 - ty) * tx + TQ * jyp;
    if constexpr (D == 3) {
        const int32_t ntxy = ntx * nty;
        const int32_t jzm = bz > 0 ? -ntxy : (ntz - 1) * ntxy, jzp = (int32_t)bz + 1 < ntz ? ntxy : (1 - ntz) * ntxy;
        dz[0] = lz > 0 ? -txy : (tz - 1) * txy + TQ * jzm;
        dz[2] = (int32_t)lz + 1 < tz ? txy : (1 - tz) * txy + TQ * jzp;
    } else {
        dz[0] = dz[2] = 0;
    }
}

// The two cells of one thread.  GENERAL = false is the all-fluid form (the warp's two boxes hold
// no flag and pull from no flagged cell): no flag is read, both cells are active and the code is
// straight-line from the loads to the stores, so the scheduler interleaves the two collisions.
// GENERAL = true reads the flags of the cells whose box bit is set and handles them as tile_step
// does.
template <class L, bool F16C, int COLL, int LES, bool FAST, bool GENERAL>
__device__ __forceinline__ void pair_cells(const StepArgs& a, const uint32_t tile, const uint32_t t,
                                           const uint32_t mask, const uint32_t bx, const uint32_t by,
                                           const uint32_t bz) {
    using P = Pop<F16C>;
    using S = typename P::T;
    constexpr int Q = L::Q, D = L::D, K = D + 1;
    constexpr uint32_t T = kTileCells;
    constexpr bool SCALED = FAST && F16C && !LES && COLL != LBM_KBC;
    using W = PairWord<F16C, SCALED>;
    auto ld = [](const S* p) -> float {
        if constexpr (SCALED) return P::ld_scaled(p);
        else return P::ld(p);
    };
    auto st = [](S* p, float v) {
        if constexpr (SCALED) P::st_scaled(p, v);
        else P::st(p, v);
    };

    const uint32_t tA = 2u * t;         // cell A; B = tA + 1
    const uint32_t nA = tA + T * tile;  // flag offset of A
    const bool flagged = GENERAL && ((mask >> (tA >> 5)) & 1u);  // the pair's box (both cells)

    uint8_t flagA = 0, flagB = 0;
    bool actA = true, actB = true;
    if (flagged) {
        flagA = __ldg(a.flags + nA);
        flagB = __ldg(a.flags + nA + 1u);
        // is_valid_thread (src/lbm/kernels/utils/checks.mojo:55-60), per cell
        actA = !((flagA & 0x0F) == LBM_FLAG_SOLID || (flagA & LBM_FLAG_EXCLUDE));
        actB = !((flagB & 0x0F) == LBM_FLAG_SOLID || (flagB & LBM_FLAG_EXCLUDE));
        if (!actA && !actB) return;
    }

    const uint32_t lxA = tA & a.mx, ly = (tA >> a.shx) & a.my, lz = tA >> a.shxy;
    const int32_t TQ = (int32_t)(T * Q);
    int32_t dxm, dxp, dy[3], dz[3];
    pair_deltas<D>(a, bx, by, bz, lxA, ly, lz, TQ, dxm, dxp, dy, dz);
    const int32_t own = (int32_t)tA + TQ * (int32_t)tile;
    const S* fin = (const S*)a.f_in;
    S* fout = (S*)a.f_out;

    // ---- stream: pull loads of both cells
    float fa[Q], fb[Q];
    static_for<0, Q>([&](auto qc) {
        constexpr int q = qc.value;
        constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
        // the source row at x_A: one 64-bit address per row (shared by its directions, whose q*T
        // are immediate offsets) and one per x edge
        const S* row = fin + (own + dy[sy + 1] + dz[sz + 1]);
        constexpr int32_t qT = (int32_t)(T * q);
        if constexpr (sx == 0) {
            W::ld(row + qT, fa[q], fb[q]);
        } else if constexpr (sx < 0) {
            fa[q] = ld(row + dxm + qT);
            fb[q] = ld(row + qT);
        } else {
            fa[q] = ld(row + (qT + 1));
            fb[q] = ld(row + dxp + (qT + 1));
        }
    });

    if (flagged) {
        // ---- cell-solid masks of both cells (written for every cell of a flagged box): x, z the
        // SOLID pull neighbours of A, B; y, w those with a moving-wall bc.  Loaded after the pulls,
        // whose latency they share.
        const uint4 m = __ldg(reinterpret_cast<const uint4*>(a.cell_masks + nA));
        // mid-grid bounce-back on a raw SOLID compare (ops/load_and_store.mojo:216)
        if (m.x)
            static_for<1, Q>([&](auto qc) {
                constexpr int q = qc.value;
                if ((m.x >> q) & 1u) fa[q] = ld(fin + own + (int32_t)(T * opp<L>(q)));
            });
        if (m.z)
            static_for<1, Q>([&](auto qc) {
                constexpr int q = qc.value;
                if ((m.z >> q) & 1u) fb[q] = ld(fin + own + 1 + (int32_t)(T * opp<L>(q)));
            });
        if (a.moving && (m.y | m.w)) {
            // moving_wall_bc with the bc of each cell's SOLID pull neighbours
            auto wall = [&](float (&f)[Q], uint32_t nib, uint32_t tc) {
                int32_t dc[3][3], dp[3][3];
                tile_deltas<D>(a, bx, by, bz, tc & a.mx, ly, lz, TQ, dc, dp);
                const uint32_t n = tc + T * tile;
                moving_wall<L, SCALED>(f, nib, a.bc, T, [&](auto qc) -> uint64_t {
                    constexpr int q = decltype(qc)::value;
                    constexpr int sx = -L::c(q, 0), sy = -L::c(q, 1), sz = -L::c(q, 2);
                    const uint32_t mm = (uint32_t)((int32_t)n + dc[0][sx + 1] + dc[1][sy + 1] + dc[2][sz + 1]);
                    const uint32_t mt = mm / T;
                    return (uint64_t)(mm - mt * T) + (uint64_t)T * K * mt;
                });
            };
            if (m.y) wall(fa, m.y, tA);
            if (m.w) wall(fb, m.w, tA + 1u);
        }
        if (a.eqbc) {
            const int32_t gx = (int32_t)(bx * (uint32_t)a.lay.tx + lxA), gy = (int32_t)(by * (uint32_t)a.lay.ty + ly),
                          gz = (int32_t)(bz * (uint32_t)a.lay.tz + lz);
            auto eq = [&](float (&f)[Q], uint32_t tc, int32_t x) {
                if constexpr (SCALED) static_for<0, Q>([&](auto qc) { f[qc.value] *= 0x1p112f; });
                equilibrium_bc<L>(f, a.bc, tc + (uint64_t)T * K * tile, T, x, gy, gz, a.lay, a.ddf != 0);
                if constexpr (SCALED) static_for<0, Q>([&](auto qc) { f[qc.value] *= 0x1p-112f; });
            };
            if ((flagA & 0x0F) == LBM_FLAG_EQUILIBRIUM) eq(fa, tA, gx);
            if ((flagB & 0x0F) == LBM_FLAG_EQUILIBRIUM) eq(fb, tA + 1u, gx + 1);
        }
    }

    // ---- collide each cell
    float* bcA = a.bc + (tA + (uint64_t)T * K * tile);
    S* po = fout + own;
    if constexpr (!GENERAL) {
        if constexpr (FAST) {
            collide_fast<L, COLL, LES, SCALED>(fa, a, bcA, T, 0);
            collide_fast<L, COLL, LES, SCALED>(fb, a, bcA + 1, T, 0);
        } else {
            collide<L, COLL, LES>(fa, a.tau, a, bcA, T, 0);
            collide<L, COLL, LES>(fb, a.tau, a, bcA + 1, T, 0);
        }
        static_for<0, Q>([&](auto qc) { W::st(po + (int32_t)(T * qc.value), fa[qc.value], fb[qc.value]); });
        return;
    }
    if (actA) {
        if constexpr (FAST) collide_fast<L, COLL, LES, SCALED>(fa, a, bcA, T, flagA);
        else collide<L, COLL, LES>(fa, a.tau, a, bcA, T, flagA);
    }
    if (actB) {
        if constexpr (FAST) collide_fast<L, COLL, LES, SCALED>(fb, a, bcA + 1, T, flagB);
        else collide<L, COLL, LES>(fb, a.tau, a, bcA + 1, T, flagB);
    }

    // ---- store: one word per direction, or the active cell's half
    if (actA && actB) {
        static_for<0, Q>([&](auto qc) { W::st(po + (int32_t)(T * qc.value), fa[qc.value], fb[qc.value]); });
    } else if (actA) {
        static_for<0, Q>([&](auto qc) { st(po + (int32_t)(T * qc.value), fa[qc.value]); });
    } else {
        static_for<0, Q>([&](auto qc) { st(po + 1 + (int32_t)(T * qc.value), fb[qc.value]); });
    }
}

template <class L, bool F16C, int COLL, int LES, bool FAST>
__device__ __forceinline__ void pair_step(const StepArgs& a, const uint32_t tile, const uint32_t t) {
    const uint32_t byz = a.lay.d_ntx.div(tile);
    const uint32_t bx = tile - byz * (uint32_t)a.lay.ntx;
    const uint32_t bz = a.lay.d_nty.div(byz);
    const uint32_t by = byz - bz * (uint32_t)a.lay.nty;
    // ---- the warp's two boxes (cells 64w .. 64w + 63) all plain FLUID with FLUID neighbours?
    const uint32_t mask = (uint32_t)__ldg(a.tile_near + tile);
    if (__all_sync(0xffffffffu, ((mask >> ((t >> 5) * 2u)) & 3u) == 0u))
        pair_cells<L, F16C, COLL, LES, FAST, false>(a, tile, t, mask, bx, by, bz);
    else
        pair_cells<L, F16C, COLL, LES, FAST, true>(a, tile, t, mask, bx, by, bz);
}

// Resident CTAs (of 128 threads) per SM the pair kernels are built for: the populations of two
// cells stay in registers across both collisions, so the budget is wider than the per-cell
// kernel's.  Float16C in the fast arithmetic 8 (64 registers: 63.7 GLUPs on the 256^3 Float16C
// cavity against 60.0 at 9, 61.2 at 7 and 58.0 at 6), float32 8 (64 registers, a few spilled
// bytes in the wall warps' form only: 43.05 GLUPs on the float32 cavity against 42.46 at 7), the
// exact Float16C build 7 (72 registers; at 64 it spills), TRT 6 (80), KBC and D3Q27 4 (128).
#ifndef LBM_PAIR_MIN_BLOCKS_F16C_FAST
#define LBM_PAIR_MIN_BLOCKS_F16C_FAST 8
#endif
#ifndef LBM_PAIR_MIN_BLOCKS_F16C
#define LBM_PAIR_MIN_BLOCKS_F16C 7
#endif
#ifndef LBM_PAIR_MIN_BLOCKS
#define LBM_PAIR_MIN_BLOCKS 8
#endif
#ifndef LBM_PAIR_MIN_BLOCKS_HEAVY
#define LBM_PAIR_MIN_BLOCKS_HEAVY 4
#endif
template <class L, bool F16C, int COLL, bool FAST>
constexpr int pair_min_blocks() {
    return (COLL == LBM_KBC || L::Q == 27) ? LBM_PAIR_MIN_BLOCKS_HEAVY
           : COLL == LBM_TRT               ? 6
           : (F16C && FAST)                ? LBM_PAIR_MIN_BLOCKS_F16C_FAST
           : F16C                          ? LBM_PAIR_MIN_BLOCKS_F16C
                                           : LBM_PAIR_MIN_BLOCKS;
}

template <class L, bool F16C, int COLL, int LES, bool FAST>
__global__ void __launch_bounds__(kPairThreads, (pair_min_blocks<L, F16C, COLL, FAST>())) step_kernel_pair(const StepArgs a) {
    static_assert(LES != kLesLearned, "the learned closure runs in step_kernel_learned");
    pdl_enter();
    pair_step<L, F16C, COLL, LES, FAST>(a, blockIdx.x, threadIdx.x);
}

template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_pair(const StepArgs& a, int, cudaStream_t s) {
    static_assert(METHOD == LBM_DOUBLE_BUFFER, "the cell-pair kernel is double-buffer only");
    return launch_pdl(step_kernel_pair<L, F16C, COLL, LES, false>, a.lay.ncells / kTileCells, kPairThreads, s, a);
}
template <class L, int METHOD, bool F16C, int COLL, int LES>
cudaError_t launch_step_pair_fast(const StepArgs& a, int, cudaStream_t s) {
    static_assert(METHOD == LBM_DOUBLE_BUFFER, "the cell-pair kernel is double-buffer only");
    return launch_pdl(step_kernel_pair<L, F16C, COLL, LES, true>, a.lay.ncells / kTileCells, kPairThreads, s, a);
}

}  // namespace lbm
