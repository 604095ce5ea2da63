// TEST INFRASTRUCTURE: runs the reference's density_update kernel
// (rtpslib/system/sph/cl_src/density.cl:86-126 with cl_sph_neighbors.h and
// cl_sph_kernels.h).
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_dens {
#include "cl_sph/density.cl"
}
#include <vector>

extern "C" void ref_density(int n, const float* pos_s, float* density, const uint32_t* start, const uint32_t* end,
                            const void* gps, const void* sphp) {
    rk_dens::SPHParams sp = *(const rk_dens::SPHParams*)sphp;
    sp.num = n;  // updateParams uploads num_particles (SPHSettings.cpp:191)
    std::vector<float4> clf(round_up(n, 64) + 1);
    std::vector<int4> cli(round_up(n, 64) + 1);
    // Density::execute: local size 64 (sph/Density.cpp:80-83)
    clshim::launch_flat(round_up(n, 64), 64, [&] {
        rk_dens::density_update((float4*)pos_s, density, (int*)start, (int*)end, (rk_dens::GridParams*)gps, &sp,
                                clf.data(), cli.data());
    });
}
