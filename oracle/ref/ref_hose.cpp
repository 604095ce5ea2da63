// TEST INFRASTRUCTURE: the reference's Hose (rtpslib/system/common/Hose.cpp)
// with addDiscRandom (rtpslib/domain/IV.cpp:313-367), built from the
// reference tree unchanged.  Hose.h includes the OpenCL runtime headers (and
// util.h, which includes them again), which do not compile without an OpenCL
// SDK; Hose uses nothing from them, so their include guards are defined
// first and the includes expand to nothing.
#define RTPS_UTIL_H_INCLUDED
#define RTPS_CL_H_INCLUDED
#define RTPS_BUFFER_H_INCLUDED
#define RTPS_KERNEL_H_INCLUDED
#define _TIME_EB_H_
#include "system/common/Hose.cpp"

#include <cstdlib>
#include <vector>

#include "ref_api.h"

namespace {
rtps::float4 f4(const float* v) { return rtps::float4(v[0], v[1], v[2], v[3]); }
}  // namespace

extern "C" {
void* ref_hose_create(float dt, int total_n, const float* center, const float* velocity, float radius,
                      float spacing) {
    return new rtps::Hose(dt, total_n, f4(center), f4(velocity), radius, spacing, rtps::float4(1, 0, 0, 1));
}
// One Hose::spray; returns the particle count, writes at most cap of them and
// the velocity they are pushed with (Hose::getVelocity).
int ref_hose_spray(void* h, float* out, int cap, float* velocity) {
    rtps::Hose* hose = (rtps::Hose*)h;
    std::vector<rtps::float4> p = hose->spray();
    const int k = (int)p.size();
    for (int i = 0; i < k && i < cap; ++i) {
        out[4 * i] = p[i].x;
        out[4 * i + 1] = p[i].y;
        out[4 * i + 2] = p[i].z;
        out[4 * i + 3] = p[i].w;
    }
    const rtps::float4 v = hose->getVelocity();
    velocity[0] = v.x;
    velocity[1] = v.y;
    velocity[2] = v.z;
    velocity[3] = v.w;
    return k;
}
void ref_hose_update(void* h, const float* center, const float* velocity, float radius, float spacing) {
    ((rtps::Hose*)h)->update(f4(center), f4(velocity), radius, spacing, rtps::float4(1, 0, 0, 1));
}
void ref_hose_refill(void* h, int n) { ((rtps::Hose*)h)->refill(n); }
void ref_hose_destroy(void* h) { delete (rtps::Hose*)h; }
void ref_srand(unsigned seed) { std::srand(seed); }
}
