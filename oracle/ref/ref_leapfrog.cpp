// TEST INFRASTRUCTURE: runs the reference's leapfrog kernel
// (rtpslib/system/sph/cl_src/leapfrog.cl:30-121).
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_lf {
#include "cl_sph/leapfrog.cl"
}
#include <vector>

extern "C" void ref_leapfrog(int n, float* pos_u, const float* pos_s, float* vel_u, const float* vel_s,
                             float* veleval_u, const float* force, const float* xsph, const uint32_t* idx,
                             const void* sphp, float dt) {
    rk_lf::SPHParams sp = *(const rk_lf::SPHParams*)sphp;
    sp.num = n;
    std::vector<float4> col_u(n > 0 ? n : 1), col_s(n > 0 ? n : 1);
    // LeapFrog::execute: local size 128 (sph/LeapFrog.cpp:79-80)
    clshim::launch_flat(round_up(n, 128), 128, [&] {
        rk_lf::leapfrog((float4*)pos_u, (float4*)pos_s, (float4*)vel_u, (float4*)vel_s, (float4*)veleval_u,
                        (float4*)force, (float4*)xsph, col_u.data(), col_s.data(), (int*)idx, &sp, dt);
    });
}
