// TEST INFRASTRUCTURE: runs the reference's point-source gravity kernel
// (rtpslib/system/common/cl_src/gravity.cl:9-35) as Gravity::execute does
// (common/Gravity.cpp:43-75): accel (the sorted force) += the sources' pull
// on the sorted positions.
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_grav {
#include "cl_common/gravity.cl"
}

extern "C" void ref_gravity(int n, int nsrc, const float* points, const float* masses, const float* alphas,
                            const float* pos_s, float* force, float scale) {
    // Kernel::execute with the default local size (Gravity.cpp:68)
    clshim::launch_flat(round_up(n, 128), 128, [&] {
        rk_grav::gravity(n, nsrc, (float4*)points, (float*)masses, (float*)alphas, (float4*)pos_s, (float4*)force,
                         scale);
    });
}
