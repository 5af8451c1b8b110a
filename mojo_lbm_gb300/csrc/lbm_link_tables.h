// Host-side tables of the interpolated bounce-back fused into the step (lbm_link_tables.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace lbm {

// Per-cell table and CSR arrays of a set of links.  table[c] = (bit i for each link (c, i),
// index of the cell's first link in dist / id), links ordered by cell, then direction; id[k] is
// the link's index in the caller's arrays.
struct LinkTables {
    std::vector<uint2> table;
    std::vector<float> dist;
    std::vector<int32_t> id;
};

// Builds the tables from host copies of the caller's arrays.  Cell c of link t is
// cell0[dom[t]] + ids[t] (dom and cell0 may be null: one domain at 0), valid when
// 0 <= ids[t] < ncells[dom[t]] (ncells null: ncells_total).  Returns an error message, or "" on
// success.
std::string build_link_tables(int64_t ncells_total, int Q, int64_t n, const int32_t* dom, const uint64_t* cell0,
                              const uint64_t* ncells, int32_t ndom, const int32_t* ids, const int32_t* dirs,
                              const float* dists, LinkTables& out);

}  // namespace lbm
