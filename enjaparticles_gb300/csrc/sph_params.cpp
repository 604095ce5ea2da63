// sph_params.cpp — host-side parameter derivation of the SPH system, no device
// work.
//   sph_setup_domain        Domain::calculateCells (rtpslib/domain/Domain.cpp:38-81)
//                           + System::setupDomain (rtpslib/system/System.cpp:294-329)
//   sph_settings_round      RTPSSettings::SetSetting / GetSettingAs round trip
//                           (rtpslib/RTPSSettings.h:65-85)
//   sph_kernel_coefficients SPH::calculate (rtpslib/system/SPHSettings.cpp:104-119)
//   sph_dambreak_params     the dam-break parameter block of the benchmark scenes
//   sph_params_from_settings the parameter block and grids an RTPSSettings
//                           map gives an SPH system (SPH::SPH, SPH.cpp:50-58)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

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

namespace {

// The settings store of the reference (rtpslib/RTPSSettings.h:43-106): every
// value is a string; SetSetting writes `ostringstream << value` (6
// significant digits for float and double), GetSettingAs reads it back with
// `istringstream >> T`, a missing key reading as "0".
class SettingsMap {
public:
    void set(const std::string& k, const std::string& v) { m_[k] = v; }
    void set_float(const std::string& k, float v) { m_[k] = fmt(v); }
    void set_double(const std::string& k, double v) { m_[k] = fmt(v); }
    const char* raw(const std::string& k) const {
        auto it = m_.find(k);
        return it == m_.end() ? "0" : it->second.c_str();
    }
    float f(const std::string& k) const { return std::strtof(raw(k), nullptr); }
    long long i(const std::string& k) const { return std::strtoll(raw(k), nullptr, 10); }
    // float4 reads four whitespace-separated floats (structs.h:549-553);
    // components that are not there read as 0
    sph_float4 f4v(const std::string& k) const {
        float v[4] = {0.f, 0.f, 0.f, 0.f};
        const char* p = raw(k);
        for (int c = 0; c < 4; ++c) {
            char* end = nullptr;
            const float x = std::strtof(p, &end);
            if (end == p) break;
            v[c] = x;
            p = end;
        }
        return f4(v[0], v[1], v[2], v[3]);
    }

private:
    static std::string fmt(double v) {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%.6g", v);
        return buf;
    }
    std::map<std::string, std::string> m_;
};

}  // namespace

extern "C" {

int sph_params_from_settings(int count, const char* const* keys, const char* const* values, SPHParams* sp,
                             GridParams* grid, GridParams* grid_scaled, float* spacing) {
    if (count < 0 || (count > 0 && (!keys || !values)) || !sp || !grid) return SPH_EINVAL;
    SettingsMap S;
    for (int k = 0; k < count; ++k) {
        if (!keys[k] || !values[k]) return SPH_EINVAL;
        S.set(keys[k], values[k]);  // a later entry of a key replaces an earlier one
    }
    // SPH::calculate (SPHSettings.cpp:30-144).  Its file sees std:: through a
    // using-directive, so log and pow are the float overloads.
    const float rho0 = S.f("rest_density");
    const long long max_ll = S.i("max_num_particles");
    if (!(rho0 > 0.f) || max_ll < 2 || max_ll > 0x7fffffffLL) return SPH_EINVAL;
    const unsigned max_num = (unsigned)max_ll;
    const int log2n = (int)(std::log((float)max_num) / std::log(2.0f));
    const float mass = (float)(0.0256 / log2n);
    const float VP = mass / rho0;
    const float rest_distance = (float)(.87 * std::pow(mass / rho0, 1.f / 3.f));
    const float smoothing_distance = 2.0f * rest_distance;
    // the domain of System::System (System.cpp:62): the boundary box
    const sph_float4 dmin = S.f4v("domain_min"), dmax = S.f4v("domain_max");
    const float domain_vol = ((dmax.x - dmin.x) * (dmax.y - dmin.y) * (dmax.z - dmin.z)) / 2;
    if (!(domain_vol > 0.f) || !std::isfinite(domain_vol)) return SPH_EINVAL;
    const float simulation_scale = std::pow(.5f * VP * (float)max_num / domain_vol, 1.f / 3.f);
    S.set_float("mass", mass);
    S.set_float("rest_distance", rest_distance);
    S.set_float("smoothing_distance", smoothing_distance);
    S.set_float("simulation_scale", simulation_scale);
    S.set_float("boundary_distance", .5f * rest_distance);
    S.set_float("spacing", rest_distance / simulation_scale);
    {
        // the kernel coefficients from the unrounded smoothing distance
        if (!(smoothing_distance > 0.f) || !std::isfinite(smoothing_distance)) return SPH_EINVAL;
        const float pi = (float)M_PI;
        const float h9 = std::pow(smoothing_distance, 9.f), h6 = std::pow(smoothing_distance, 6.f),
                    h3 = std::pow(smoothing_distance, 3.f);
        S.set_float("wpoly6", 315.f / 64.0f / pi / h9);
        S.set_float("wpoly6_d", -945.f / (32.0f * pi * h9));
        S.set_float("wpoly6_dd", -945.f / (32.0f * pi * h9));
        S.set_float("wspiky", 15.f / pi / h6);
        S.set_float("wspiky_d", -45.f / (pi * h6));
        S.set_double("wspiky_dd", 15. / (2. * pi * h3));
        S.set_double("wvisc", 15. / (2. * pi * h3));
        S.set_double("wvisc_d", 15. / (2. * pi * h3));
        S.set_double("wvisc_dd", 45. / (pi * h6));
    }
    S.set_double("epsilon", 1E-6);
    S.set("num_particles", "0");
    // SPH::updateParams (SPHSettings.cpp:150-199)
    SPHParams p;
    std::memset(&p, 0, sizeof(p));
    p.rest_density = S.f("rest_density");
    p.mass = S.f("mass");
    p.rest_distance = S.f("rest_distance");
    p.smoothing_distance = S.f("smoothing_distance");
    p.simulation_scale = S.f("simulation_scale");
    p.boundary_stiffness = S.f("boundary_stiffness");
    p.boundary_dampening = S.f("boundary_dampening");
    p.boundary_distance = S.f("boundary_distance");
    p.K = S.f("gas_constant");
    p.viscosity = S.f("viscosity");
    p.velocity_limit = S.f("velocity_limit");
    p.xsph_factor = S.f("xsph_factor");
    p.gravity = S.f4v("gravity");
    p.friction_coef = S.f("friction_kinetic");
    p.restitution_coef = S.f("restitution");
    p.shear = S.f("shear");
    p.attraction = S.f("attraction");
    p.spring = S.f("spring");
    p.EPSILON = S.f("epsilon");
    p.wpoly6_coef = S.f("wpoly6");
    p.wpoly6_d_coef = S.f("wpoly6_d");
    p.wpoly6_dd_coef = S.f("wpoly6_dd");
    p.wspiky_coef = S.f("wspiky");
    p.wspiky_d_coef = S.f("wspiky_d");
    p.wspiky_dd_coef = S.f("wspiky_dd");
    p.wvisc_coef = S.f("wvisc");
    p.wvisc_d_coef = S.f("wvisc_d");
    p.wvisc_dd_coef = S.f("wvisc_dd");
    p.num = (int)S.i("num_particles");
    p.max_num = (int)S.i("max_num_particles");
    // System::setupDomain(h / scale, scale) (SPH.cpp:58, System.cpp:294-329)
    const int rc = sph_setup_domain(&dmin, &dmax, p.smoothing_distance / p.simulation_scale, p.simulation_scale,
                                    grid, grid_scaled);
    if (rc) return rc;
    *sp = p;
    if (spacing) *spacing = S.f("spacing");  // SPH::spacing (SPH.cpp:66)
    return SPH_OK;
}

}  // extern "C"
