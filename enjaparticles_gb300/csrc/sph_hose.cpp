// sph_hose.cpp — hoses: a disc of new particles pushed into the system every
// few steps.  The reference's Hose (rtpslib/system/common/Hose.cpp:30-130)
// with addDiscRandom (rtpslib/domain/IV.cpp:313-367), on the host.
//
// Every operation keeps the reference's types and order: the float and
// double mix of the random perturbations, the loop variables perturbed in
// place, the unit vectors of calc_vectors (including its replacement of a
// zero y or z velocity by 1e-7, which also changes the velocity the
// particles are pushed with).  The random numbers are the C library's rand(),
// as in the reference: seed it with srand() for reproducible runs.  This file
// is compiled without floating-point contraction, so the results are the
// same on every host.
#include <cmath>
#include <cstdlib>
#include <vector>

#include "rtps_sph.h"

struct sph_hose {
    float dt = 0.f;
    int total_n = 0;  // particles the hose was filled with
    int n_count = 0;  // particles left
    sph_float4 center{}, velocity{};
    sph_float4 u{}, w{};  // unit vectors spanning the disc
    float radius = 0.f, spacing = 0.f;
    int em = 0;        // sprays between emissions
    int em_count = 0;  // sprays since the last emission
    std::vector<sph_float4> last;
};

namespace {

sph_float4 f4(float x, float y, float z, float w) {
    sph_float4 v;
    v.x = x;
    v.y = y;
    v.z = z;
    v.w = w;
    return v;
}

float magnitude3(const sph_float4& a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// normalize (structs.cpp:53-57): x, y, z divided by the length, w kept.
sph_float4 normalize3(const sph_float4& a) {
    const float mag = magnitude3(a);
    return f4(a.x / mag, a.y / mag, a.z / mag, a.w);
}

// Hose::calc_vectors (Hose.cpp:65-90): two unit vectors orthogonal to the
// velocity.
void calc_vectors(sph_hose* h) {
    sph_float4& v = h->velocity;
    if (v.y == 0.) v.y = (float).0000001;
    if (v.z == 0.) v.z = (float).0000001;
    const float b = 1.f;
    const float a = b * v.x / v.y;
    const float c = -b * (v.x * v.x + v.y * v.y) / (v.y * v.z);
    h->u = normalize3(f4(1.f, -(v.x / v.y), 0.f, 1.f));
    h->w = normalize3(f4(a, b, c, 1.f));
}

// Hose::calc_em (Hose.cpp:92-106): emit every 1 + spacing/dt/|v|/10 sprays.
void calc_em(sph_hose* h) {
    const float magv = magnitude3(h->velocity);
    h->em = (int)(1 + h->spacing / h->dt / magv / 10);
}

// A random number in [-amp, amp] as the reference draws it: the int from
// rand() times a float, then in double, rounded to float at the end.
float perturbation(float amp) {
    const float r = (float)std::rand() * amp;
    return (float)((double)r * 2. / RAND_MAX - (double)amp);
}

// addDiscRandom (IV.cpp:313-367): up to num points of a jittered grid of the
// given spacing over the square [-radius, radius]^2 in the (u, w) plane around
// center, each moved along v by a random multiple in [-10, 10], kept when
// inside the disc of the given radius.
std::vector<sph_float4> add_disc_random(int num, sph_float4 center, sph_float4 v, sph_float4 u, sph_float4 w,
                                        float radius, float spacing) {
    const float pert = .05f * spacing;
    const float vpert = 10.f;
    const float mr = -radius;
    const sph_float4 umin = f4(mr * u.x, mr * u.y, mr * u.z, mr * u.w);
    const sph_float4 wmin = f4(mr * w.x, mr * w.y, mr * w.z, mr * w.w);
    std::vector<sph_float4> out;
    int i = 0;
    const float r2 = radius * radius;
    for (float du = 0.; du < 2. * radius; du += spacing) {
        for (float dw = 0.; dw < 2. * radius; dw += spacing) {
            if (i >= num) break;
            const float rrv = perturbation(vpert);
            const float rru = perturbation(pert);
            const float rrw = perturbation(pert);
            du += rru;
            dw += rrw;
            // center + umin + u*du + wmin + w*dw + rrv*v, left to right
            sph_float4 p;
            p.x = center.x + umin.x;
            p.y = center.y + umin.y;
            p.z = center.z + umin.z;
            p.x = p.x + du * u.x;
            p.y = p.y + du * u.y;
            p.z = p.z + du * u.z;
            p.x = p.x + wmin.x;
            p.y = p.y + wmin.y;
            p.z = p.z + wmin.z;
            p.x = p.x + dw * w.x;
            p.y = p.y + dw * w.y;
            p.z = p.z + dw * w.z;
            p.x = p.x + rrv * v.x;
            p.y = p.y + rrv * v.y;
            p.z = p.z + rrv * v.z;
            p.w = 1.0f;
            const float dx = p.x - center.x, dy = p.y - center.y, dz = p.z - center.z;
            const float d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < r2) {
                out.push_back(p);
                ++i;
            }
        }
    }
    return out;
}

bool finite4(const sph_float4& v) {
    return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z) && std::isfinite(v.w);
}

}  // namespace

extern "C" {

int sph_hose_create(float dt, int total_n, sph_float4 center, sph_float4 velocity, float radius, float spacing,
                    sph_hose** out) {
    if (!out) return SPH_EINVAL;
    *out = nullptr;
    if (!(dt > 0.f) || !std::isfinite(dt) || total_n < 0 || !(spacing > 0.f) || !std::isfinite(spacing) ||
        !(radius >= 0.f) || !std::isfinite(radius) || !finite4(center) || !finite4(velocity))
        return SPH_EINVAL;
    sph_hose* h = new sph_hose();
    h->dt = dt;
    h->total_n = total_n;
    h->n_count = total_n;
    h->center = center;
    h->velocity = velocity;
    h->radius = radius;
    h->spacing = spacing;
    calc_vectors(h);
    *out = h;
    return SPH_OK;
}

int sph_hose_update(sph_hose* h, sph_float4 center, sph_float4 velocity, float radius, float spacing) {
    if (!h || !(spacing > 0.f) || !std::isfinite(spacing) || !(radius >= 0.f) || !std::isfinite(radius) ||
        !finite4(center) || !finite4(velocity))
        return SPH_EINVAL;
    h->center = center;
    h->velocity = velocity;
    h->radius = radius;
    h->spacing = spacing;
    calc_vectors(h);
    return SPH_OK;
}

int sph_hose_refill(sph_hose* h, int n) {
    if (!h || n < 0) return SPH_EINVAL;
    h->total_n = n;
    h->n_count = n;
    return SPH_OK;
}

int sph_hose_spray(sph_hose* h, int* count) {
    if (!h) return SPH_EINVAL;
    h->last.clear();
    h->em_count++;
    calc_em(h);
    if (h->em_count >= h->em && h->n_count > 0) {
        const sph_float4 v = f4(h->dt * h->velocity.x, h->dt * h->velocity.y, h->dt * h->velocity.z,
                                h->dt * h->velocity.w);
        h->last = add_disc_random(h->n_count, h->center, v, h->u, h->w, h->radius, h->spacing);
        h->n_count -= (int)h->last.size();
        h->em_count = 0;
    }
    if (count) *count = (int)h->last.size();
    return SPH_OK;
}

int sph_hose_particles(const sph_hose* h, sph_float4* pos, int cap, sph_float4* velocity) {
    if (!h || cap < 0 || (cap > 0 && !pos)) return SPH_EINVAL;
    const int k = (int)h->last.size() < cap ? (int)h->last.size() : cap;
    for (int i = 0; i < k; ++i) pos[i] = h->last[i];
    if (velocity) *velocity = h->velocity;
    return SPH_OK;
}

int sph_hose_remaining(const sph_hose* h, int* n) {
    if (!h || !n) return SPH_EINVAL;
    *n = h->n_count;
    return SPH_OK;
}

void sph_hose_destroy(sph_hose* h) { delete h; }

}  // extern "C"
