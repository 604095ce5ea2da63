// TEST INFRASTRUCTURE: runs the reference's permute kernel
// (rtpslib/system/common/cl_src/permute.cl:10-46).
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_perm {
#include "cl_common/permute.cl"
}
#include <vector>

extern "C" void ref_permute(int n, const uint32_t* idx, const float* pos_u, const float* vel_u,
                            const float* veleval_u, float* pos_s, float* vel_s, float* veleval_s) {
    std::vector<float4> col_u(n > 0 ? n : 1), col_s(n > 0 ? n : 1);
    std::vector<float> m_u(n > 0 ? n : 1), m_s(n > 0 ? n : 1);
    std::vector<uint32_t> o_u(n > 0 ? n : 1), o_s(n > 0 ? n : 1);
    // Permute::execute: local size 64 (Permute.cpp:93-99)
    clshim::launch_flat(round_up(n, 64), 64, [&] {
        rk_perm::permute(n, (float4*)pos_u, (float4*)pos_s, (float4*)vel_u, (float4*)vel_s, (float4*)veleval_u,
                         (float4*)veleval_s, col_u.data(), col_s.data(), m_u.data(), m_s.data(), o_u.data(),
                         o_s.data(), (uint32_t*)idx);
    });
}
