// rtps_sph.hpp — header-only C++ class with the method names of the
// reference's rtps::System / rtps::SPH (rtpslib/system/System.h:61-186,
// rtpslib/system/SPH.h:56-155), forwarding to the C ABI of rtps_sph.h.
//
// A frame loop written against the reference (acquireGLBuffers -> update ->
// interact -> integrate -> postProcess -> releaseGLBuffers, as in
// test/glwidget.cpp:876-916) runs unchanged against this class.  Rendering
// is not part of the library: the GL buffer calls are no-ops and the particle
// arrays are device buffers (devicePointer) or host copies (getPositions).
// Errors, which the reference prints and ignores, throw rtps::SPHError.
#ifndef RTPS_SPH_HPP
#define RTPS_SPH_HPP

#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "rtps_sph.h"

namespace rtps {

typedef sph_float4 float4;

inline float4 make_float4(float x, float y, float z, float w) {
    float4 v;
    v.x = x;
    v.y = y;
    v.z = z;
    v.w = w;
    return v;
}

// rtps::Triangle (rtpslib/structs.h:586-590): three vertices and a normal.
struct Triangle {
    float4 verts[3];
    float4 normal;
};
static_assert(sizeof(Triangle) == 64, "Triangle must be 16 floats");

class SPHError : public std::runtime_error {
public:
    SPHError(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

// addRect (rtpslib/domain/IV.cpp:165-202): lattice points of spacing
// `spacing` from min to max, z outermost, at most num of them.
inline std::vector<float4> addRect(int num, float4 min, float4 max, float spacing, float scale) {
    const float xmin = min.x / scale, xmax = max.x / scale;
    const float ymin = min.y / scale, ymax = max.y / scale;
    const float zmin = min.z / scale, zmax = max.z / scale;
    std::vector<float4> rvec(num > 0 ? num : 0);
    int i = 0;
    for (float z = zmin; z <= zmax; z += spacing)
        for (float y = ymin; y <= ymax; y += spacing)
            for (float x = xmin; x <= xmax; x += spacing) {
                if (i >= num) break;
                rvec[i] = make_float4(x, y, z, 1.0f);
                ++i;
            }
    rvec.resize(i);
    return rvec;
}

// The reference's settings store (rtpslib/RTPSSettings.h:43-106): every
// value is a string, SetSetting writes `ostringstream << value`, GetSettingAs
// reads it with `istringstream >> T`, and a missing key reads as the default
// ("0").  A float4 is written and read as its four lanes, space separated.
class RTPSSettings {
public:
    template <class T>
    void SetSetting(const std::string& key, const T& value) {
        std::ostringstream os;
        os << value;
        settings_[key] = os.str();
        changed_ = true;
    }
    void SetSetting(const std::string& key, const float4& v) {
        std::ostringstream os;
        os << v.x << " " << v.y << " " << v.z << " " << v.w;
        settings_[key] = os.str();
        changed_ = true;
    }
    template <class T>
    T GetSettingAs(const std::string& key, const std::string& defaultval = "0") const {
        auto it = settings_.find(key);
        std::istringstream is(it == settings_.end() ? defaultval : it->second);
        T v{};
        is >> v;
        return v;
    }
    bool Exists(const std::string& key) const { return settings_.count(key) != 0; }
    bool hasChanged() const { return changed_; }
    void updated() { changed_ = false; }
    const std::map<std::string, std::string>& entries() const { return settings_; }

private:
    std::map<std::string, std::string> settings_;
    bool changed_ = false;
};
template <>
inline float4 RTPSSettings::GetSettingAs<float4>(const std::string& key, const std::string& defaultval) const {
    auto it = settings_.find(key);
    std::istringstream is(it == settings_.end() ? defaultval : it->second);
    float4 v = make_float4(0, 0, 0, 0);
    is >> v.x >> v.y >> v.z >> v.w;
    return v;
}

class SPH {
public:
    // The reference builds its parameters from a settings map
    // (SPH::calculate, SPHSettings.cpp:30-144) and its grid with
    // System::setupDomain; here both come in as the C structs.
    SPH(const SPHParams& sphp, const GridParams& grid, int max_num, const GridParams* grid_scaled = nullptr,
        float time_step = 0.001f)
        : dt_(time_step) {
        check(sph_create(&sphp, &grid, grid_scaled, max_num, &ctx_), nullptr);
        max_num_ = max_num;
    }
    // SPH::SPH(RTPSSettings*, CL*) (SPH.cpp:50-98), as
    // RTPS::generateSystemInstance builds it for system "sph": the
    // parameters of SPH::calculate / updateParams and the grid of
    // System::setupDomain from the settings (sph_params_from_settings), the
    // integrator of the "integrator" setting and the "time_step" setting's dt.
    explicit SPH(const RTPSSettings* settings) {
        std::vector<const char*> keys, values;
        for (const auto& kv : settings->entries()) {
            keys.push_back(kv.first.c_str());
            values.push_back(kv.second.c_str());
        }
        SPHParams sphp;
        GridParams grid, grid_scaled;
        float spacing = 0.f;
        check(sph_params_from_settings((int)keys.size(), keys.data(), values.data(), &sphp, &grid, &grid_scaled,
                                       &spacing),
              nullptr);
        check(sph_create(&sphp, &grid, &grid_scaled, sphp.max_num, &ctx_), nullptr);
        max_num_ = sphp.max_num;
        spacing_ = spacing;
        dt_ = settings->GetSettingAs<float>("time_step");
        const std::string integ = settings->GetSettingAs<std::string>("integrator", "");
        if (integ == "euler") check(sph_set_integrator(ctx_, SPH_INTEGRATOR_EULER));
        // point sources (System::System, System.cpp:260-272): the settings
        // gravity_sources (x y z w per source), gravity_mass, gravity_alphas
        if (settings->Exists("gravity_sources")) {
            const std::vector<float> p = floats(settings->entries().at("gravity_sources"));
            const std::vector<float> m =
                settings->Exists("gravity_mass") ? floats(settings->entries().at("gravity_mass")) : std::vector<float>();
            const std::vector<float> a = settings->Exists("gravity_alphas")
                                             ? floats(settings->entries().at("gravity_alphas"))
                                             : std::vector<float>();
            const int ns = (int)(p.size() / 4);
            if (ns > 0) {
                std::vector<float4> pts(ns);
                for (int k = 0; k < ns; ++k) pts[k] = make_float4(p[4 * k], p[4 * k + 1], p[4 * k + 2], p[4 * k + 3]);
                std::vector<float> mass(ns, 0.f), alpha(ns, 0.f);
                for (int k = 0; k < ns && k < (int)m.size(); ++k) mass[k] = m[k];
                for (int k = 0; k < ns && k < (int)a.size(); ++k) alpha[k] = a[k];
                check(sph_set_gravity_sources(ctx_, ns, pts.data(), mass.data(), alpha.data()));
            }
        }
    }
    ~SPH() {
        if (ctx_) sph_destroy(ctx_);
    }
    SPH(const SPH&) = delete;
    SPH& operator=(const SPH&) = delete;
    SPH(SPH&& o) noexcept
        : ctx_(o.ctx_),
          max_num_(o.max_num_),
          dt_(o.dt_),
          spacing_(o.spacing_),
          color_field_(o.color_field_),
          color_field_res_(o.color_field_res_) {
        o.ctx_ = nullptr;
    }

    // --- System virtual API (System.h:64-75) ---
    void update() { check(sph_update(ctx_)); }           // hash .. density, force, walls, mesh (SPH::updateGPU)
    void interact() {}                                    // no coupled systems
    void integrate() { check(sph_integrate(ctx_, dt_)); } // leapfrog (SPH::integrate)
    // SPH::postProcess (SPH.cpp:338-386) with the settings use_color_field /
    // color_field_res set by useColorField: the colour field and its mesh,
    // kept on the device (getMesh gives views of them).
    void postProcess() {
        if (color_field_) check(sph_post_process(ctx_, color_field_res_, nullptr));
    }
    void useColorField(bool on, int res = 2) {
        color_field_ = on;
        color_field_res_ = res;
    }
    // Device views of the last mesh: ntri triangles, 9 floats each.
    int getMesh(const float** vertices, const float** normals) {
        int ntri = 0;
        check(sph_get_surface(ctx_, nullptr, vertices, normals, nullptr, &ntri));
        return ntri;
    }
    // update + integrate fused, nsteps times, replayed from a CUDA graph
    void step(int nsteps = 1) { check(sph_step(ctx_, dt_, nsteps)); }

    // Headless: there are no GL buffers to acquire or release.
    void acquireGLBuffers() {}
    void releaseGLBuffers() {}

    // --- particles (System.h:80-90, 120-160; SPH.h:81-84) ---
    int getNum() {
        int n = 0;
        check(sph_get_num(ctx_, &n));
        return n;
    }
    void setNum(int nn) { check(sph_set_num(ctx_, nn)); }
    int getMaxNum() const { return max_num_; }
    // SPH::getSpacing (SPH.cpp:66): the "spacing" setting, written by
    // SPH::calculate as rest_distance / simulation_scale (SPHSettings.cpp:
    // 94-96) and read back through the settings map (6 significant digits).
    float getSpacing() {
        if (spacing_ > 0.f) return spacing_;  // built from settings: SPH::calculate's own value
        SPHParams p = params();
        return sph_settings_round(p.rest_distance / p.simulation_scale);
    }
    // System::addBox (System.cpp:331-338): addRect at the SPH spacing, zero
    // velocity.  color and mass are accepted for interface parity and unused.
    int addBox(int nn, float4 min, float4 max, bool scaled, float4 color = make_float4(1, 0, 0, 1),
               float mass = 0.0f) {
        (void)scaled;
        (void)color;
        (void)mass;
        std::vector<float4> rect = addRect(nn, min, max, getSpacing(), 1.0f);
        pushParticles(rect, make_float4(0, 0, 0, 0));
        return (int)rect.size();
    }
    void pushParticles(const std::vector<float4>& pos, float4 velo, float4 color = make_float4(1, 0, 0, 1),
                       float mass = 0.0f) {
        pushParticles(pos, std::vector<float4>(pos.size(), velo), color, mass);
    }
    // SPH::pushParticles (SPH.cpp:560-602): appends after the current
    // particles; exceeding max_num throws (the reference prints and returns).
    void pushParticles(const std::vector<float4>& pos, const std::vector<float4>& vel,
                       float4 color = make_float4(1, 0, 0, 1), float mass = 0.0f) {
        (void)color;
        (void)mass;
        if (pos.size() != vel.size()) throw SPHError(SPH_EINVAL, "pushParticles: pos and vel sizes differ");
        check(sph_push_particles(ctx_, pos.data(), vel.data(), (int)pos.size()));
    }
    // SPH::loadTriangles (sph/Collision_triangle.cpp:44-82): the mesh that
    // SPH::collision tests after the walls; an empty vector unloads it.
    void loadTriangles(std::vector<Triangle>& triangles) {
        check(sph_load_triangles(ctx_, triangles.empty() ? nullptr : &triangles[0].verts[0],
                                 (int)triangles.size()));
    }
    // SPH::addHose / updateHose / refillHose (SPH.cpp:523-545): radius in
    // particle spacings; update() sprays the hoses first.  color and mass are
    // accepted for interface parity and unused.
    int addHose(int total_n, float4 center, float4 velocity, float radius, float4 color = make_float4(1, 0, 0, 1),
                float mass = 0.0f) {
        (void)color;
        (void)mass;
        int index = -1;
        check(sph_add_hose(ctx_, total_n, center, velocity, radius, dt_, &index));
        return index;
    }
    void updateHose(int index, float4 center, float4 velocity, float radius,
                    float4 color = make_float4(1, 0, 0, 1)) {
        (void)color;
        check(sph_update_hose(ctx_, index, center, velocity, radius));
    }
    void refillHose(int index, int refill) { check(sph_refill_hose(ctx_, index, refill)); }
    void sprayHoses() { check(sph_spray_hoses(ctx_, nullptr)); }
    std::vector<float4> getDeletedPos() { return deleted(true); }
    std::vector<float4> getDeletedVel() { return deleted(false); }

    // Host copies of the state (original particle order).
    std::vector<float4> getPositions() { return download(SPH_FIELD_POS_U); }
    std::vector<float4> getVelocities() { return download(SPH_FIELD_VEL_U); }
    std::vector<float4> getVelEval() { return download(SPH_FIELD_VELEVAL_U); }
    // Device view of a field (what the reference's Buffer<T> objects held).
    void* devicePointer(int field) {
        void* p = nullptr;
        check(sph_get_device_ptr(ctx_, field, &p));
        return p;
    }

    // --- parameters ---
    SPHParams params() {
        SPHParams p;
        check(sph_get_params(ctx_, &p, nullptr, nullptr));
        return p;
    }
    void updateParams(const SPHParams& p) { check(sph_set_params(ctx_, &p)); }
    void setTimeStep(float dt) { dt_ = dt; }
    float getTimeStep() const { return dt_; }
    void sync() { check(sph_sync(ctx_)); }
    void printTimers() {}
    sph_ctx* handle() { return ctx_; }

private:
    void check(int rc, sph_ctx* c) {
        if (rc == SPH_OK) return;
        char buf[512];
        sph_last_error(c, buf, (int)sizeof(buf));
        throw SPHError(rc, buf);
    }
    void check(int rc) { check(rc, ctx_); }
    std::vector<float4> download(int field) {
        std::vector<float4> out((size_t)getNum());
        if (!out.empty()) check(sph_download(ctx_, field, out.data(), (int)out.size()));
        return out;
    }
    std::vector<float4> deleted(bool pos) {
        int count = 0;
        check(sph_get_deleted(ctx_, nullptr, nullptr, 0, &count));
        std::vector<float4> out((size_t)count);
        if (count > 0)
            check(sph_get_deleted(ctx_, pos ? out.data() : nullptr, pos ? nullptr : out.data(), count, &count));
        return out;
    }

    sph_ctx* ctx_ = nullptr;
    // the whitespace-separated floats of a setting (structs.h:594-603)
    static std::vector<float> floats(const std::string& text) {
        std::istringstream is(text);
        std::vector<float> v;
        float x;
        while (is >> x) v.push_back(x);
        return v;
    }

    int max_num_ = 0;
    float dt_ = 0.001f;
    float spacing_ = 0.f;  // the "spacing" setting when built from settings
    bool color_field_ = false;
    int color_field_res_ = 2;
};

}  // namespace rtps

#endif  // RTPS_SPH_HPP
