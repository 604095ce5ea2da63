// TEST INFRASTRUCTURE: the reference's SPH::calculate and SPH::updateParams
// (rtpslib/system/SPHSettings.cpp, compiled unchanged from a scratch copy
// whose SPH.h is sph_settings_shim.h) over its own RTPSSettings
// (rtpslib/RTPSSettings.cpp, unchanged), driven as SPH::SPH drives them
// (rtpslib/system/SPH.cpp:50-66; System::System, System.cpp:54-62): a
// settings map in; the parameter block, the grids of System::setupDomain and
// SPH::spacing out.
#define RTPS_UTIL_H_INCLUDED  // util.h includes the OpenCL headers
#include <iostream>

#include "debug.h"
#include "RTPSSettings.cpp"
#include "SPHSettings.cpp"

#include <cstring>
#include <string>

#include "ref_api.h"

extern "C" int ref_params_from_settings(int count, const char* const* keys, const char* const* values, void* sphp,
                                        void* grid, void* grid_scaled, float* spacing) {
    rtps::RTPSSettings S;
    for (int k = 0; k < count; ++k) S.SetSetting(std::string(keys[k]), std::string(values[k]));
    rtps::SPH sys;
    sys.settings = &S;
    sys.max_num = S.GetSettingAs<unsigned int>("max_num_particles");
    const rtps::float4 lo = S.GetSettingAs<rtps::float4>("domain_min");
    const rtps::float4 hi = S.GetSettingAs<rtps::float4>("domain_max");
    sys.grid = rtps::Domain(lo, hi);
    sys.calculate();
    sys.updateParams();
    const float bmin[4] = {lo.x, lo.y, lo.z, lo.w}, bmax[4] = {hi.x, hi.y, hi.z, hi.w};
    ref_setup_domain(bmin, bmax, sys.sphp.smoothing_distance / sys.sphp.simulation_scale, sys.sphp.simulation_scale,
                     grid, grid_scaled);
    static_assert(sizeof(rtps::SPHParams) >= 116, "SPHParams layout");
    std::memcpy(sphp, &sys.sphp, sizeof(rtps::SPHParams));
    *spacing = S.GetSettingAs<float>("spacing");
    return (int)sizeof(rtps::SPHParams);
}
