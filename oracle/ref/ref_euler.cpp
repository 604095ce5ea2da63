// TEST INFRASTRUCTURE: runs the reference's SPH Euler integrator
// (rtpslib/system/sph/cl_src/euler.cl:33-78), the integrator SPH::integrate
// selects with integrator=euler (SPH.cpp:392-411).
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_eu {
#include "cl_sph/euler.cl"
}

extern "C" void ref_euler(int n, float* pos_u, const float* pos_s, float* vel_u, const float* vel_s,
                          const float* force, const uint32_t* idx, const void* sphp, float dt) {
    rk_eu::SPHParams sp = *(const rk_eu::SPHParams*)sphp;
    sp.num = n;
    clshim::launch_flat(round_up(n, 128), 128, [&] {
        rk_eu::euler((float4*)pos_u, (float4*)pos_s, (float4*)vel_u, (float4*)vel_s, (float4*)force, (int*)idx, &sp,
                     dt);
    });
}
