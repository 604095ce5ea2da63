// TEST INFRASTRUCTURE: runs the reference's hash kernel
// (rtpslib/system/common/cl_src/hash.cl:50-157) on the host.  The kernel
// source is compiled from the reference tree by build_ref.py.
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_hash {
#include "cl_common/hash.cl"
}
#include <vector>

extern "C" void ref_hash(int n, const float* pos_u, const void* gp, uint32_t* keys, uint32_t* idx) {
    // Hash::execute: global = num rounded up to the local size 128 (Hash.cpp:72-75)
    std::vector<float4> clf(n > 0 ? n : 1);
    std::vector<int4> cli(n > 0 ? n : 1);
    auto* g = (rk_hash::GridParams*)gp;
    clshim::launch_flat(round_up(n, 128), 128, [&] {
        rk_hash::hash(n, (float4*)pos_u, keys, idx, g, clf.data(), cli.data());
    });
}
