// sph_params.cpp — host-side parameter derivation of the SPH system, no device
// work.
//   sph_setup_domain        Domain::calculateCells (rtpslib/domain/Domain.cpp:38-81)
//                           + System::setupDomain (rtpslib/system/System.cpp:294-329)
//   sph_settings_round      RTPSSettings::SetSetting / GetSettingAs round trip
//                           (rtpslib/RTPSSettings.h:65-85)
//   sph_kernel_coefficients SPH::calculate (rtpslib/system/SPHSettings.cpp:104-119)
//   sph_dambreak_params     the dam-break parameter block of the benchmark scenes
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/rtps_sph.h"

namespace {

sph_float4 f4(float x, float y, float z, float w) {
    sph_float4 r;
    r.x = x; r.y = y; r.z = z; r.w = w;
    return r;
}

// structs.h:523-538: float4 * float multiplies each lane; float4 / float
// multiplies by the float reciprocal.
sph_float4 f4_mul(const sph_float4& a, float s) { return f4(s * a.x, s * a.y, s * a.z, s * a.w); }
sph_float4 f4_div(const sph_float4& a, float s) {
    const float d = 1.f / s;
    return f4(d * a.x, d * a.y, d * a.z, d * a.w);
}

bool finite4(const sph_float4& v) {
    return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z) && std::isfinite(v.w);
}

}  // namespace

extern "C" {

int sph_setup_domain(const sph_float4* bnd_min, const sph_float4* bnd_max, float cell_size, float sim_scale,
                     GridParams* grid, GridParams* grid_scaled) {
    if (!bnd_min || !bnd_max || !grid) return SPH_EINVAL;
    if (!(cell_size > 0.f) || !std::isfinite(cell_size) || !(sim_scale > 0.f) || !std::isfinite(sim_scale))
        return SPH_EINVAL;
    if (!finite4(*bnd_min) || !finite4(*bnd_max)) return SPH_EINVAL;
    // Domain::calculateCells: the pad 2*cell is formed in double and stored
    // in float lanes (w lane 0).
    const double s2 = 2. * cell_size;
    const sph_float4 pad = f4((float)s2, (float)s2, (float)s2, 0.f);
    const sph_float4 mn = f4(bnd_min->x - pad.x, bnd_min->y - pad.y, bnd_min->z - pad.z, bnd_min->w - pad.w);
    const sph_float4 mx = f4(pad.x + bnd_max->x, pad.y + bnd_max->y, pad.z + bnd_max->z, pad.w + bnd_max->w);
    sph_float4 size = f4(mx.x - mn.x, mx.y - mn.y, mx.z - mn.z, 0.f);
    const sph_float4 res = f4(std::ceil(size.x / cell_size), std::ceil(size.y / cell_size),
                              std::ceil(size.z / cell_size), 0.f);
    size = f4(res.x * cell_size, res.y * cell_size, res.z * cell_size, 0.f);
    const sph_float4 delta = f4(res.x / size.x, res.y / size.y, res.z / size.z, 0.f);
    GridParams g;
    std::memset(&g, 0, sizeof(g));
    g.grid_min = mn;
    g.grid_max = f4(size.x + mn.x, size.y + mn.y, size.z + mn.z, size.w + mn.w);
    g.bnd_min = *bnd_min;
    g.bnd_max = *bnd_max;
    g.grid_res = res;
    g.grid_size = size;
    g.grid_delta = delta;
    const float cells = res.x * res.y * res.z;
    if (!(cells >= 1.f) || cells > 2147483647.f) return SPH_EINVAL;
    g.nb_cells = (int)cells;
    *grid = g;
    if (grid_scaled) {
        GridParams s = g;
        s.grid_min = f4_mul(g.grid_min, sim_scale);
        s.grid_max = f4_mul(g.grid_max, sim_scale);
        s.bnd_min = f4_mul(g.bnd_min, sim_scale);
        s.bnd_max = f4_mul(g.bnd_max, sim_scale);
        s.grid_size = f4_mul(g.grid_size, sim_scale);
        s.grid_delta = f4_div(g.grid_delta, sim_scale);
        *grid_scaled = s;
    }
    return SPH_OK;
}

float sph_settings_round(float value) {
    // ostringstream << float at the default precision 6 is "%g" with 6
    // significant digits; istringstream >> float parses it back.
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.6g", (double)value);
    return std::strtof(buf, nullptr);
}

static float settings_round_double(double value) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.6g", value);
    return std::strtof(buf, nullptr);
}

int sph_kernel_coefficients(float h, SPHParams* sp) {
    if (!sp || !(h > 0.f) || !std::isfinite(h)) return SPH_EINVAL;
    const float pi = (float)M_PI;
    const float h9 = std::pow(h, 9.f);
    const float h6 = std::pow(h, 6.f);
    const float h3 = std::pow(h, 3.f);
    // Float expressions (SPHSettings.cpp:111-115) and double ones (:116-119,
    // unsuffixed literals), each stored through the settings strings.
    sp->wpoly6_coef = sph_settings_round(315.f / 64.0f / pi / h9);
    sp->wpoly6_d_coef = sph_settings_round(-945.f / (32.0f * pi * h9));
    sp->wpoly6_dd_coef = sph_settings_round(-945.f / (32.0f * pi * h9));
    sp->wspiky_coef = sph_settings_round(15.f / pi / h6);
    sp->wspiky_d_coef = sph_settings_round(-45.f / (pi * h6));
    sp->wspiky_dd_coef = settings_round_double(15. / (2. * pi * h3));
    sp->wvisc_coef = settings_round_double(15. / (2. * pi * h3));
    sp->wvisc_d_coef = settings_round_double(15. / (2. * pi * h3));
    sp->wvisc_dd_coef = settings_round_double(45. / (pi * h6));
    return SPH_OK;
}

int sph_dambreak_params(int num, float spacing, float viscosity, SPHParams* sp, GridParams* grid,
                        GridParams* grid_scaled) {
    if (!sp || !grid || num <= 0 || !(spacing > 0.f) || !std::isfinite(spacing) || !(viscosity >= 0.f))
        return SPH_EINVAL;
    SPHParams p;
    std::memset(&p, 0, sizeof(p));
    const float s = sph_settings_round(spacing);
    const float rho0 = 1000.f;
    p.rest_density = rho0;
    p.rest_distance = s;
    p.smoothing_distance = sph_settings_round(2.f * s);
    p.mass = sph_settings_round(rho0 * s * s * s);
    p.simulation_scale = 1.f;
    p.boundary_stiffness = 20000.f;
    p.boundary_dampening = 256.f;
    p.boundary_distance = sph_settings_round(.5f * s);
    p.K = 15.f;
    p.viscosity = sph_settings_round(viscosity);
    p.velocity_limit = 600.f;
    p.xsph_factor = 0.15f;
    p.friction_coef = 0.f;
    p.restitution_coef = 0.f;
    p.shear = 0.f;
    p.attraction = 0.f;
    p.spring = 0.f;
    p.EPSILON = sph_settings_round(1e-6f);
    int rc = sph_kernel_coefficients(p.smoothing_distance, &p);
    if (rc) return rc;
    p.num = 0;
    p.max_num = num;
    p.gravity = f4(0.f, 0.f, -9.8f, 0.f);
    const sph_float4 lo = f4(0.f, 0.f, 0.f, 0.f), hi = f4(1.f, 1.f, 1.f, 0.f);
    rc = sph_setup_domain(&lo, &hi, p.smoothing_distance / p.simulation_scale, p.simulation_scale, grid, grid_scaled);
    if (rc) return rc;
    *sp = p;
    return SPH_OK;
}

}  // extern "C"
