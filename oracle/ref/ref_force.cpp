// TEST INFRASTRUCTURE: runs the reference's force_update kernel
// (rtpslib/system/sph/cl_src/force.cl:148-186, ForNeighbor :43-140).
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_force {
#include "cl_sph/force.cl"
}
#include <vector>

extern "C" void ref_force(int n, const float* pos_s, const float* density, const float* veleval_s, float* force,
                          float* xsph, const uint32_t* start, const uint32_t* end, const void* gps,
                          const void* sphp) {
    rk_force::SPHParams sp = *(const rk_force::SPHParams*)sphp;
    sp.num = n;
    std::vector<float4> clf(round_up(n, 64) + 1);
    std::vector<int4> cli(round_up(n, 64) + 1);
    // Force::execute: local size 64 (sph/Force.cpp:82-85)
    clshim::launch_flat(round_up(n, 64), 64, [&] {
        rk_force::force_update((float4*)pos_s, (float*)density, (float4*)veleval_s, (float4*)force, (float4*)xsph,
                               (int*)start, (int*)end, (rk_force::GridParams*)gps, &sp, clf.data(), cli.data());
    });
}
