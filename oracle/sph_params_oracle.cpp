// sph_params_oracle.cpp — TEST INFRASTRUCTURE, not part of the product.
//
// The parameter block of the dam-break benchmark scenes, derived on the host
// the way the reference derives it, for the checkers that must not load the
// product library (the CPU reference arm of bench.py):
//   * every value that passes through the settings map is written with
//     `ostringstream << value` (6 significant digits, float or double as the
//     expression's type) and read back with `istringstream >> float`
//     (rtpslib/RTPSSettings.h:65-85, SetSetting / GetSettingAs);
//   * kernel coefficients: SPH::calculate (rtpslib/system/SPHSettings.cpp:
//     104-119), float expressions for wpoly6/wspiky, double ones (unsuffixed
//     literals) for wspiky_dd/wvisc/wvisc_d/wvisc_dd; epsilon 1E-6 (:140);
//   * grid: Domain::calculateCells (rtpslib/domain/Domain.cpp:38-81), the
//     2*cell pad formed in double; the scaled copy of System::setupDomain
//     (rtpslib/system/System.cpp:318-325): lanes times sim_scale, delta times
//     the float reciprocal of sim_scale (structs.h float4 operators).
// The benchmark scenes override mass, rest distance and h (h = 2 s,
// m = 1000 s^3, simulation_scale = 1), as their configuration states.
#include <cmath>
#include <cstring>
#include <sstream>
#include <string>

#include "../include/rtps_sph.h"

namespace {

template <class T>
float through_settings(T value) {
    std::ostringstream os;
    os << value;
    std::istringstream is(os.str());
    float out = 0.f;
    is >> out;
    return out;
}

sph_float4 v4(float x, float y, float z, float w) {
    sph_float4 r;
    r.x = x;
    r.y = y;
    r.z = z;
    r.w = w;
    return r;
}

void calculate_cells(const sph_float4& bmin, const sph_float4& bmax, float cell, GridParams& g) {
    const double pad = 2. * cell;  // Domain.cpp:40
    const float p = (float)pad;
    const sph_float4 lo = v4(bmin.x - p, bmin.y - p, bmin.z - p, bmin.w - 0.f);
    const sph_float4 hi = v4(bmax.x + p, bmax.y + p, bmax.z + p, bmax.w + 0.f);
    sph_float4 size = v4(hi.x - lo.x, hi.y - lo.y, hi.z - lo.z, 0.f);
    const sph_float4 res = v4(std::ceil(size.x / cell), std::ceil(size.y / cell), std::ceil(size.z / cell), 0.f);
    size = v4(res.x * cell, res.y * cell, res.z * cell, 0.f);
    std::memset(&g, 0, sizeof(g));
    g.grid_size = size;
    g.grid_min = lo;
    g.grid_max = v4(lo.x + size.x, lo.y + size.y, lo.z + size.z, lo.w + size.w);
    g.bnd_min = bmin;
    g.bnd_max = bmax;
    g.grid_res = res;
    g.grid_delta = v4(res.x / size.x, res.y / size.y, res.z / size.z, 0.f);
    g.nb_cells = (int)(res.x * res.y * res.z);
}

sph_float4 scale4(const sph_float4& a, float s) { return v4(a.x * s, a.y * s, a.z * s, a.w * s); }

}  // namespace

extern "C" {

// spacing: the lattice spacing s of the scene; viscosity as given (it goes
// through the settings map too).  Returns 0, or -1 on an invalid argument.
int oracle_dambreak_params(int num, float spacing, float viscosity, SPHParams* sp, GridParams* grid,
                           GridParams* grid_scaled) {
    if (!sp || !grid || num <= 0 || !(spacing > 0.f) || !(viscosity >= 0.f)) return -1;
    SPHParams p;
    std::memset(&p, 0, sizeof(p));
    const float s = through_settings(spacing);
    p.rest_density = 1000.f;
    p.rest_distance = s;
    p.smoothing_distance = through_settings(2.f * s);
    p.mass = through_settings(1000.f * s * s * s);
    p.simulation_scale = 1.f;
    p.boundary_stiffness = 20000.f;
    p.boundary_dampening = 256.f;
    p.boundary_distance = through_settings(.5f * s);  // SPHSettings.cpp:89
    p.K = 15.f;
    p.viscosity = through_settings(viscosity);
    p.velocity_limit = 600.f;
    p.xsph_factor = 0.15f;
    p.EPSILON = through_settings(1E-6);  // a double literal, SPHSettings.cpp:140
    const float h = p.smoothing_distance;
    const float pi = (float)M_PI;
    const float h9 = std::pow(h, 9.f), h6 = std::pow(h, 6.f), h3 = std::pow(h, 3.f);
    p.wpoly6_coef = through_settings(315.f / 64.0f / pi / h9);
    p.wpoly6_d_coef = through_settings(-945.f / (32.0f * pi * h9));
    p.wpoly6_dd_coef = through_settings(-945.f / (32.0f * pi * h9));
    p.wspiky_coef = through_settings(15.f / pi / h6);
    p.wspiky_d_coef = through_settings(-45.f / (pi * h6));
    p.wspiky_dd_coef = through_settings(15. / (2. * pi * h3));
    p.wvisc_coef = through_settings(15. / (2. * pi * h3));
    p.wvisc_d_coef = through_settings(15. / (2. * pi * h3));
    p.wvisc_dd_coef = through_settings(45. / (pi * h6));
    p.num = 0;
    p.max_num = num;
    p.gravity = v4(0.f, 0.f, -9.8f, 0.f);
    GridParams g;
    calculate_cells(v4(0.f, 0.f, 0.f, 0.f), v4(1.f, 1.f, 1.f, 0.f), h / p.simulation_scale, g);
    *grid = g;
    if (grid_scaled) {
        const float sc = p.simulation_scale, inv = 1.f / sc;
        GridParams gs = g;
        gs.grid_min = scale4(g.grid_min, sc);
        gs.grid_max = scale4(g.grid_max, sc);
        gs.bnd_min = scale4(g.bnd_min, sc);
        gs.bnd_max = scale4(g.bnd_max, sc);
        gs.grid_size = scale4(g.grid_size, sc);
        gs.grid_delta = scale4(g.grid_delta, inv);
        *grid_scaled = gs;
    }
    *sp = p;
    return 0;
}

}  // extern "C"

extern "C" {

// A float written to the settings map and read back (RTPSSettings.h:65-85):
// what SPH::getSpacing returns for spacing = rest_distance / simulation_scale
// (SPHSettings.cpp:94-96, SPH.cpp:66).
float oracle_settings_round(float value) { return through_settings(value); }

}  // extern "C"
