// Host side of the staged kernel (lbm_stage.cuh): the list of bulk copies that stages one tile.
#include <cuda_runtime.h>

#include <vector>

#include "lbm_stage.cuh"

namespace lbm {

namespace {

template <class L>
std::vector<StageSeg> segments(int tx, int ty, int tz, int esz) {
    std::vector<StageSeg> out;  // in elements until the end
    auto add = [&](uint32_t src, uint32_t dst, uint32_t len, uint32_t nbr) {
        if (!out.empty()) {
            StageSeg& b = out.back();
            if (b.nbr == nbr && b.src + b.bytes == src && b.dst + b.bytes == dst) {
                b.bytes += len;
                return;
            }
        }
        out.push_back(StageSeg{src, dst, len, nbr});
    };
    const int T = (int)kTileCells;
    for (int q = 0; q < L::Q; ++q) {
        const int cx = L::c(q, 0), cy = L::c(q, 1), cz = L::c(q, 2);
        const uint32_t region = stage_off<L>(q);
        for (int part = 0; part < (cx == 0 ? 1 : 2); ++part) {
            const int dxt = part == 0 ? 0 : -cx;  // the tile column the rows come from
            const uint32_t base = region + (uint32_t)(part * T);
            for (int lz = 0; lz < tz; ++lz) {
                const int sz = lz - cz, dzt = sz < 0 ? -1 : (sz >= tz ? 1 : 0), szl = sz - dzt * tz;
                for (int ly = 0; ly < ty; ++ly) {
                    const int sy = ly - cy, dyt = sy < 0 ? -1 : (sy >= ty ? 1 : 0), syl = sy - dyt * ty;
                    const uint32_t src = (uint32_t)(q * T + tx * (syl + ty * szl));
                    const uint32_t dst = base + (uint32_t)(tx * (ly + ty * lz));
                    add(src, dst, (uint32_t)tx, (uint32_t)((dxt + 1) + 3 * (dyt + 1) + 9 * (dzt + 1)));
                }
            }
        }
    }
    for (StageSeg& s : out) {
        s.dst *= (uint32_t)esz;
        s.bytes *= (uint32_t)esz;
    }
    return out;
}

}  // namespace

// The copy segments of the stage of one tile (tx x ty x tz = 256, populations of esz bytes), or an
// empty list when its rows are not multiples of 16 bytes.  *stage_bytes: the bytes they move, the
// size of one stage buffer.
__attribute__((visibility("hidden"))) std::vector<StageSeg> build_stage_segments(int lattice, int tx, int ty, int tz,
                                                                                 int esz, uint32_t* stage_bytes) {
    *stage_bytes = 0;
    if ((tx * esz) % 16 != 0 || tx * ty * tz != (int)kTileCells) return {};
    std::vector<StageSeg> s;
    uint32_t total = 0;
    switch (lattice) {
        case LBM_D2Q9: s = segments<D2Q9>(tx, ty, tz, esz); total = stage_off<D2Q9>(D2Q9::Q); break;
        case LBM_D3Q19: s = segments<D3Q19>(tx, ty, tz, esz); total = stage_off<D3Q19>(D3Q19::Q); break;
        default: s = segments<D3Q27>(tx, ty, tz, esz); total = stage_off<D3Q27>(D3Q27::Q); break;
    }
    *stage_bytes = total * (uint32_t)esz;
    return s;
}

}  // namespace lbm

extern "C" {
// Test hook (no counterpart in the reference): the stage segments of a tile shape, as
// (src element, dst byte, bytes, neighbour code) quadruples.  Returns their count (at most
// max_segs are written) and the bytes of one stage in *stage_bytes; 0 when the shape cannot be
// staged.
__attribute__((visibility("default"))) int32_t lbm_stage_segments(int32_t lattice, int32_t tx, int32_t ty, int32_t tz,
                                                                   int32_t esz, uint32_t* out, int32_t max_segs,
                                                                   uint32_t* stage_bytes) {
    uint32_t sb = 0;
    const std::vector<lbm::StageSeg> s = lbm::build_stage_segments(lattice, tx, ty, tz, esz, &sb);
    if (stage_bytes) *stage_bytes = sb;
    for (int32_t i = 0; i < (int32_t)s.size() && i < max_segs && out; ++i) {
        out[4 * i] = s[i].src;
        out[4 * i + 1] = s[i].dst;
        out[4 * i + 2] = s[i].bytes;
        out[4 * i + 3] = s[i].nbr;
    }
    return (int32_t)s.size();
}
}
