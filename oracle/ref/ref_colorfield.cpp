// TEST INFRASTRUCTURE: runs the reference's colour-field kernel
// (rtpslib/system/sph/cl_src/colorfield.cl, colorfield_update) as
// ColorField::execute does (sph/ColorField.cpp:84-121): an NDRange of
// res x res x res sample points writing a one-channel image of
// texRes2D x texRes2D texels, z slices tiled `slices` to a row
// (ColorField::initializeData, ColorField.cpp:66-81).  The driver returns the
// image and the res^3 field read back out of it in (s + t res + r res^2)
// order.
#include <cmath>
#include <vector>

#include "clshim.hpp"
#include "ref_api.h"
namespace rk_cf {
#include "cl_sph/colorfield.cl"
}

// ColorField::initializeData's tiling (ColorField.cpp:68-69), with its
// float functions: slices = 2^ceil(log(ceil(sqrt(res)) / log 2)).
extern "C" int ref_colorfield_slices(int res) {
    return (int)(1u << static_cast<unsigned int>(std::ceil(std::log(std::ceil(std::sqrt((float)res)) / std::log(2.0f)))));
}

extern "C" int ref_colorfield(int res, int n, const float* pos_s, const float* density, const unsigned* cell_start,
                              const unsigned* cell_end, const void* grid_scaled, const void* sphp, float* field,
                              float* image) {
    if (res < 2) res = 2;
    const unsigned slices = (unsigned)ref_colorfield_slices(res);
    const int tex = res * (int)slices;
    std::vector<float4> img((size_t)tex * tex, make_float4(0.f, 0.f, 0.f, 0.f));
    image2d_t im{img.data(), tex, tex, 1};
    rk_cf::SPHParams sp = *(const rk_cf::SPHParams*)sphp;
    sp.num = n;
    rk_cf::GridParams gp = *(const rk_cf::GridParams*)grid_scaled;
    clshim::launch_flat3((size_t)res, (size_t)res, (size_t)res, [&] {
        rk_cf::colorfield_update((unsigned)res, slices, (float4*)pos_s, (float*)density, im, (int*)cell_start,
                                 (int*)cell_end, &gp, &sp, nullptr, nullptr);  // debug buffers: not written
    });
    for (int r = 0; r < res; ++r)
        for (int t = 0; t < res; ++t)
            for (int s = 0; s < res; ++s) {
                const int px = (r % (int)slices) * res + s, py = (r / (int)slices) * res + t;
                field[(size_t)s + (size_t)t * res + (size_t)r * res * res] =
                    (px < tex && py < tex) ? img[(size_t)py * tex + px].x : 0.f;
            }
    if (image)
        for (size_t k = 0; k < img.size(); ++k) image[k] = img[k].x;
    return tex;
}
