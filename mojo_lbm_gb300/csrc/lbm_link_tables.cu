// Tables of the interpolated bounce-back fused into the step (lbm_set_links, lbm_batch_set_link_mode):
// the caller's links (fluid cell, direction into the wall, wall distance) regrouped per cell.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <string>
#include <vector>

#include "lbm_link_tables.h"

namespace lbm {

__attribute__((visibility("hidden"))) std::string build_link_tables(
    int64_t ncells_total, int Q, int64_t n, const int32_t* dom, const uint64_t* cell0, const uint64_t* ncells,
    int32_t ndom, const int32_t* ids, const int32_t* dirs, const float* dists, LinkTables& out) {
    std::vector<uint64_t> cell(n);
    for (int64_t t = 0; t < n; ++t) {
        const int32_t d = dom ? dom[t] : 0;
        if (d < 0 || d >= ndom) return "link " + std::to_string(t) + ": domain index out of range";
        const uint64_t nc = ncells ? ncells[d] : (uint64_t)ncells_total;
        if (ids[t] < 0 || (uint64_t)ids[t] >= nc) return "link " + std::to_string(t) + ": fluid id out of range";
        if (dirs[t] < 1 || dirs[t] >= Q) return "link " + std::to_string(t) + ": direction must be in [1, Q)";
        if (!(dists[t] == dists[t])) return "link " + std::to_string(t) + ": wall distance is NaN";
        cell[t] = (cell0 ? cell0[d] : 0) + (uint64_t)ids[t];
    }
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), (int64_t)0);
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return cell[a] != cell[b] ? cell[a] < cell[b] : dirs[a] < dirs[b];
    });
    out.table.assign((size_t)ncells_total, make_uint2(0u, 0u));
    out.dist.resize(n);
    out.id.resize(n);
    for (int64_t k = 0; k < n; ++k) {
        const int64_t t = order[k];
        uint2& e = out.table[cell[t]];
        const uint32_t bit = 1u << dirs[t];
        if (e.x & bit) return "link " + std::to_string(t) + ": a second link with the same cell and direction";
        if (e.x == 0u) e.y = (uint32_t)k;
        e.x |= bit;
        out.dist[k] = dists[t];
        out.id[k] = (int32_t)t;
    }
    return "";
}

}  // namespace lbm
