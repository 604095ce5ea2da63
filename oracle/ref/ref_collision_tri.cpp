// TEST INFRASTRUCTURE: runs the reference's triangle-collision kernel
// (rtpslib/system/sph/cl_src/collision_tri.cl:436-520) as
// CollisionTriangle::execute does (sph/Collision_triangle.cpp:91-116): local
// size 32, 220 triangles of local memory.  Work-groups share local memory
// and barriers, so they run as fibers (launch_groups).  The kernel reads one
// slot past the particle count for the padding work-items and writes force
// for i == num (its `if (i > num) return`); the driver pads its copies so
// that both stay inside them.
#include "clshim.hpp"
#include "ref_api.h"
namespace rk_tri {
#include "cl_sph/collision_tri.cl"
}
#include <vector>

extern "C" void ref_collision_triangles(int n, const float* pos_s, const float* vel_s, float* force,
                                        const float* tris, int ntri, const void* params, float dt) {
    rk_tri::SPHParams sp = *(const rk_tri::SPHParams*)params;
    sp.num = n;
    const size_t global = round_up((size_t)(n > 0 ? n : 1), 32);
    std::vector<float4> p_buf(global + 1), v_buf(global + 1), f_buf(global + 1), dbg_f(global + 1);
    std::vector<int4> dbg_i(global + 1);
    std::memset(p_buf.data(), 0, p_buf.size() * 16);
    std::memset(v_buf.data(), 0, v_buf.size() * 16);
    std::memset(f_buf.data(), 0, f_buf.size() * 16);
    std::memcpy(p_buf.data(), pos_s, 16 * (size_t)n);
    std::memcpy(v_buf.data(), vel_s, 16 * (size_t)n);
    std::memcpy(f_buf.data(), force, 16 * (size_t)n);
    std::vector<rk_tri::Triangle> tri((size_t)(ntri > 0 ? ntri : 1));
    std::memcpy(tri.data(), tris, 64 * (size_t)ntri);
    static rk_tri::Triangle local_tris[220];
    clshim::launch_groups(global, 32, [&] {
        rk_tri::collision_triangle(p_buf.data(), v_buf.data(), f_buf.data(), tri.data(), ntri, dt, &sp, local_tris,
                                   dbg_f.data(), dbg_i.data());
    });
    std::memcpy(force, f_buf.data(), 16 * (size_t)n);
}
