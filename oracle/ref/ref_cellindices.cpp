// TEST INFRASTRUCTURE: runs the reference's cellindices kernel
// (rtpslib/system/common/cl_src/cellindices.cl:12-107) with the host steps of
// CellIndices::execute (rtpslib/system/common/CellIndices.cpp:42-99).
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_ci {
#include "cl_common/cellindices.cl"
}
#include <vector>

extern "C" int ref_cellindices(int n, const uint32_t* keys, const uint32_t* idx, uint32_t* start, uint32_t* end,
                               const void* gp) {
    auto* g = (rk_ci::GridParams*)gp;
    const int nb = g->nb_cells;
    for (int k = 0; k <= nb; ++k) start[k] = 0xffffffffu;  // CellIndices.cpp:58-62
    const size_t local = 64, global = round_up(n, local);
    // The sort buffers hold max_num entries filled with INT_MAX beyond num
    // (System.cpp:274-278); work-items past num read that padding.
    std::vector<uint32_t> k2(global + 1, 0x7fffffffu), i2(global + 1, 0x7fffffffu);
    for (int i = 0; i < n; ++i) { k2[i] = keys[i]; i2[i] = idx[i]; }
    std::vector<uint32_t> shared(local + 1);
    clshim::launch_groups(global, local, [&] {
        rk_ci::cellindices(n, k2.data(), i2.data(), start, end, g, shared.data());
    });
    return (int)start[nb];  // CellIndices.cpp:95-99
}
