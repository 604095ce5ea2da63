// TEST INFRASTRUCTURE: runs the reference's marching cubes
// (rtpslib/system/common/cl_src/classifycubes.cl, constructhp.cl,
// traversehp.cl: the histopyramid marching cubes of G. Smistad) as
// MarchingCubes::execute does (common/MarchingCubes.cpp:166-370): classify
// the (res-1)^3 cubes into the RGBA base level (triangle count, case index,
// corner value), sum 2x2 blocks level by level, read the total from the 2x2
// top level, and let `total` work-items walk the pyramid down to their
// triangle.  The traversal kernel is compiled once per pyramid depth
// (-DLEVELS, MarchingCubes.cpp:80-89); here each depth is its own namespace.
// Images are zero-initialised as MarchingCubes::initializeData makes them.
#include <cmath>
#include <vector>

#include "clshim.hpp"
#include "ref_api.h"

namespace rk_classify {
#include "cl_common/classifycubes.cl"
}
#undef _INDEXMAP_H_
namespace rk_construct {
#include "cl_common/constructhp.cl"
}
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 1
namespace rk_tr1 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 2
namespace rk_tr2 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 3
namespace rk_tr3 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 4
namespace rk_tr4 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 5
namespace rk_tr5 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 6
namespace rk_tr6 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 7
namespace rk_tr7 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 8
namespace rk_tr8 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS
#undef _INDEXMAP_H_
#undef _TRAVERSEHP_CL_
#define LEVELS 9
namespace rk_tr9 {
#include "cl_common/traversehp.cl"
}
#undef LEVELS

extern "C" int ref_marching_cubes(int res, const float* field, float isolevel, float* tris, float* normals,
                                  int cap_tri, float* base_level) {
    if (res < 2) res = 2;
    const unsigned slices = (unsigned)ref_colorfield_slices(res);
    const int tex = res * (int)slices;
    const int levels = (int)std::ceil(std::log((float)tex) / std::log(2.0f));
    // the colour field as ColorField leaves it: a one-channel tiled image
    std::vector<float4> cf((size_t)tex * tex, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int r = 0; r < res; ++r)
        for (int t = 0; t < res; ++t)
            for (int s = 0; s < res; ++s) {
                const int px = (r % (int)slices) * res + s, py = (r / (int)slices) * res + t;
                if (px < tex && py < tex)
                    cf[(size_t)py * tex + px] =
                        make_float4(field[(size_t)s + (size_t)t * res + (size_t)r * res * res], 0.f, 0.f, 1.f);
            }
    image2d_t cfi{cf.data(), tex, tex, 1};
    std::vector<std::vector<float4>> store((size_t)levels);
    std::vector<image2d_t> hp((size_t)levels);
    int lr = tex;
    for (int i = 0; i < levels; ++i) {
        if (i > 0) lr /= 2;
        store[i].assign((size_t)lr * lr, make_float4(0.f, 0.f, 0.f, 0.f));
        hp[i] = image2d_t{store[i].data(), lr, lr, i == 0 ? 4 : 1};
    }
    clshim::launch_flat3((size_t)res - 1, (size_t)res - 1, (size_t)res - 1,
                         [&] { rk_classify::classifyCubes2D(hp[0], cfi, (unsigned)res, slices, isolevel); });
    lr = tex;
    for (int i = 1; i < levels; ++i) {
        lr /= 2;
        clshim::launch_flat3((size_t)lr, (size_t)lr, 1, [&] { rk_construct::constructHPLevel2D(hp[i], hp[i - 1]); });
    }
    if (base_level)
        for (size_t k = 0; k < store[0].size(); ++k) {
            base_level[4 * k] = store[0][k].x;
            base_level[4 * k + 1] = store[0][k].y;
            base_level[4 * k + 2] = store[0][k].z;
            base_level[4 * k + 3] = store[0][k].w;
        }
    // the 2x2 read of the top level; a smaller top level makes the read fail
    // and leaves the totals at zero
    float totals[4] = {0.f, 0.f, 0.f, 0.f};
    const image2d_t& top = hp[levels - 1];
    if (top.w >= 2 && top.h >= 2)
        for (int k = 0; k < 4; ++k) totals[k] = top.data[(size_t)(k / 2) * top.w + (k % 2)].x;
    const unsigned total = (unsigned)(totals[0] + totals[1] + totals[2] + totals[3]);
    if (total == 0) return 0;
    std::vector<float> tv((size_t)total * 9), nv((size_t)total * 9);
    switch (levels - 1) {
        case 1:
            clshim::launch_flat(total, 1, [&] {
                rk_tr1::traverseHP2D(hp[0], hp[1], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        case 2:
            clshim::launch_flat(total, 1, [&] {
                rk_tr2::traverseHP2D(hp[0], hp[1], hp[2], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        case 3:
            clshim::launch_flat(total, 1, [&] {
                rk_tr3::traverseHP2D(hp[0], hp[1], hp[2], hp[3], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        case 4:
            clshim::launch_flat(total, 1, [&] {
                rk_tr4::traverseHP2D(hp[0], hp[1], hp[2], hp[3], hp[4], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        case 5:
            clshim::launch_flat(total, 1, [&] {
                rk_tr5::traverseHP2D(hp[0], hp[1], hp[2], hp[3], hp[4], hp[5], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        case 6:
            clshim::launch_flat(total, 1, [&] {
                rk_tr6::traverseHP2D(hp[0], hp[1], hp[2], hp[3], hp[4], hp[5], hp[6], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        case 7:
            clshim::launch_flat(total, 1, [&] {
                rk_tr7::traverseHP2D(hp[0], hp[1], hp[2], hp[3], hp[4], hp[5], hp[6], hp[7], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        case 8:
            clshim::launch_flat(total, 1, [&] {
                rk_tr8::traverseHP2D(hp[0], hp[1], hp[2], hp[3], hp[4], hp[5], hp[6], hp[7], hp[8], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        case 9:
            clshim::launch_flat(total, 1, [&] {
                rk_tr9::traverseHP2D(hp[0], hp[1], hp[2], hp[3], hp[4], hp[5], hp[6], hp[7], hp[8], hp[9], tv.data(), nv.data(), (unsigned)res, slices, isolevel, (int)total);
            });
            break;
        default:
            return -1;
    }
    const size_t k = (size_t)(total < (unsigned)cap_tri ? total : (unsigned)cap_tri) * 9;
    for (size_t i = 0; i < k; ++i) {
        tris[i] = tv[i];
        normals[i] = nv[i];
    }
    return (int)total;
}
