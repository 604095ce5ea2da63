// TEST INFRASTRUCTURE: runs the reference's collision_wall kernel
// (rtpslib/system/sph/cl_src/collision_wall.cl:31-118).
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_cw {
#include "cl_sph/collision_wall.cl"
}
#include <cstring>
#include <vector>

extern "C" void ref_collision_wall(int n, const float* pos_s, const float* vel_s, float* force, const void* gps,
                                   const void* sphp) {
    rk_cw::SPHParams sp = *(const rk_cw::SPHParams*)sphp;
    sp.num = n;
    // The kernel's bound test is `i > num`, so item num also runs; the
    // reference's buffers hold max_num entries.  Give it one spare element.
    const size_t g = round_up(n + 1, 128);
    std::vector<float4> p(g), v(g), f(g);
    std::memcpy(p.data(), pos_s, 16 * (size_t)n);
    std::memcpy(v.data(), vel_s, 16 * (size_t)n);
    std::memcpy(f.data(), force, 16 * (size_t)n);
    // CollisionWall::execute: local size 128 (sph/Collision_wall.cpp:61-62)
    clshim::launch_flat(round_up(n, 128), 128, [&] {
        rk_cw::collision_wall(p.data(), v.data(), f.data(), (rk_cw::GridParams*)gps, &sp);
    });
    std::memcpy(force, f.data(), 16 * (size_t)n);
}
