// sph_oracle.cpp — TEST INFRASTRUCTURE, not part of the product.
//
// C entry points (for ctypes) over the restatement in sph_oracle.hpp, plus a
// whole-system stepper that follows SPH::updateGPU (rtpslib/system/SPH.cpp:
// 149-300, with SPH::collision :303-336 enabled after gravity) and
// SPH::integrate (SPH.cpp:389-441).  Per-particle stages run under OpenMP;
// the stable sort is a parallel LSD radix sort checked against std::stable_sort
// by the tests.
#include "sph_oracle.hpp"

#include <algorithm>
#include <cstdio>
#include <numeric>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace sph_oracle {

static int omp_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Stable LSD radix sort of (key, value) pairs, 11-bit digits, per-thread
// histograms over contiguous chunks so that equal keys keep their order.
void stable_sort_pairs(int n, uint32_t* keys, uint32_t* vals) {
    if (n <= 1) return;
    uint32_t kmax = 0;
    for (int i = 0; i < n; ++i) kmax = std::max(kmax, keys[i]);
    int bits = 0;
    while (bits < 32 && (kmax >> bits) != 0) ++bits;
    if (bits == 0) return;
    const int D = 11, R = 1 << D;
    const int passes = (bits + D - 1) / D;
    std::vector<uint32_t> k2(n), v2(n);
    uint32_t *ks = keys, *vs = vals, *kd = k2.data(), *vd = v2.data();
    const int T = std::max(1, std::min(omp_threads(), n / 65536 + 1));
    std::vector<size_t> hist((size_t)T * R);
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = pass * D;
        std::fill(hist.begin(), hist.end(), 0);
#pragma omp parallel num_threads(T)
        {
#ifdef _OPENMP
            const int t = omp_get_thread_num();
#else
            const int t = 0;
#endif
            const size_t lo = (size_t)n * t / T, hi = (size_t)n * (t + 1) / T;
            size_t* h = &hist[(size_t)t * R];
            for (size_t i = lo; i < hi; ++i) h[(ks[i] >> shift) & (R - 1)]++;
#pragma omp barrier
#pragma omp single
            {
                size_t run = 0;
                for (int d = 0; d < R; ++d)
                    for (int tt = 0; tt < T; ++tt) {
                        size_t c = hist[(size_t)tt * R + d];
                        hist[(size_t)tt * R + d] = run;
                        run += c;
                    }
            }
            for (size_t i = lo; i < hi; ++i) {
                size_t o = h[(ks[i] >> shift) & (R - 1)]++;
                kd[o] = ks[i];
                vd[o] = vs[i];
            }
        }
        std::swap(ks, kd);
        std::swap(vs, vd);
    }
    if (ks != keys) {
        std::memcpy(keys, ks, sizeof(uint32_t) * (size_t)n);
        std::memcpy(vals, vs, sizeof(uint32_t) * (size_t)n);
    }
}

int cellindices(int n, const uint32_t* keys, uint32_t* start, uint32_t* end, int nb_cells) {
    const uint32_t ncells = (uint32_t)nb_cells;
#pragma omp parallel for schedule(static)
    for (long k = 0; k <= (long)nb_cells; ++k) start[k] = kEmpty;
    // Each boundary i (key change) writes start[key[i]] and end[key[i-1]];
    // those targets are distinct across i, so the loop is race-free.
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const uint32_t hcur = keys[i];
        if (hcur > ncells) continue;
        if (i == 0) {
            start[hcur] = 0;
        } else {
            uint32_t prev = keys[i - 1] < ncells ? keys[i - 1] : ncells;
            if (prev != hcur) {
                start[hcur] = (uint32_t)i;
                end[prev] = (uint32_t)i;
            }
        }
        if (i == n - 1) end[hcur] = (uint32_t)n;
    }
    return (int)start[nb_cells];
}

}  // namespace sph_oracle

using namespace sph_oracle;

// ---------------------------------------------------------------------------
// Whole-system state, the reference's buffer set (System.h:199-223, SPH.h:99-106)
// in host memory.
struct OracleSim {
    SPHParams sp;
    GridParams gp, gps;
    int max_num = 0, num = 0;
    int use_f64 = 0;
    std::vector<float> pos_u, vel_u, veleval_u, pos_s, vel_s, veleval_s, force_s, xsph_s, density_s;
    std::vector<uint32_t> keys, idx, start, end, nbr;
    std::vector<float> deleted_pos, deleted_vel;
    int last_nc = -1;
    // point sources (System.cpp:260-272) and the integrator (SPH.cpp:392-436)
    std::vector<float> grav_points, grav_masses, grav_alphas;
    int integrator = 0;  // 0 leapfrog, 1 euler
    std::vector<float> triangles;  // 16 floats per triangle (CollisionTriangle::loadTriangles)
};

template <class T>
static void run_density(OracleSim& s) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s.num; ++i)
        density_one<T>(i, s.pos_s.data(), s.start.data(), s.end.data(), s.gps, s.sp, s.density_s.data(),
                       s.nbr.data());
}
template <class T>
static void run_force(OracleSim& s) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s.num; ++i)
        force_one<T>(i, s.pos_s.data(), s.density_s.data(), s.veleval_s.data(), s.start.data(), s.end.data(),
                     s.gps, s.sp, s.force_s.data(), s.xsph_s.data());
}
template <class T>
static void run_collision(OracleSim& s) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.num; ++i) collision_one<T>(i, s.pos_s.data(), s.vel_s.data(), s.force_s.data(), s.gps, s.sp);
}
template <class T>
static void run_leapfrog(OracleSim& s, float dt) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.num; ++i)
        leapfrog_one<T>(i, s.pos_s.data(), s.vel_s.data(), s.force_s.data(), s.xsph_s.data(), s.idx.data(), s.sp, dt,
                        s.pos_u.data(), s.vel_u.data(), s.veleval_u.data());
}

template <class T>
static void run_gravity(OracleSim& s) {
    const int nsrc = (int)s.grav_masses.size();
    if (nsrc == 0) return;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.num; ++i)
        gravity_one<T>(i, nsrc, s.grav_points.data(), s.grav_masses.data(), s.grav_alphas.data(), s.pos_s.data(),
                       s.force_s.data(), s.sp.simulation_scale);
}
template <class T>
static void run_triangles(OracleSim& s) {
    const int ntri = (int)(s.triangles.size() / 16);
    if (ntri == 0) return;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s.num; ++i)
        collision_tri_one<T>(i, s.pos_s.data(), s.vel_s.data(), s.force_s.data(), s.triangles.data(), ntri, s.sp);
}
template <class T>
static void run_euler(OracleSim& s, float dt) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.num; ++i)
        euler_one<T>(i, s.pos_s.data(), s.vel_s.data(), s.force_s.data(), s.idx.data(), s.sp, dt, s.pos_u.data(),
                     s.vel_u.data());
}

static void run_hash_and_sort(OracleSim& s) {
    // hash.cl: unscaled grid.  Hashing is integer work on float positions; the
    // FP64 instantiation hashes the same float positions.
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.num; ++i) hash_one<float>(s.pos_u.data(), s.gp, i, s.keys.data(), s.idx.data());
    stable_sort_pairs(s.num, s.keys.data(), s.idx.data());
}

static void run_permute(OracleSim& s) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.num; ++i) {
        const size_t o = (size_t)s.idx[i] * 4, d = (size_t)i * 4;
        std::memcpy(&s.pos_s[d], &s.pos_u[o], 16);
        std::memcpy(&s.vel_s[d], &s.vel_u[o], 16);
        std::memcpy(&s.veleval_s[d], &s.veleval_u[o], 16);
    }
}

// SPH::updateGPU (SPH.cpp:149-300) + collision (:303-336).
static void sim_update(OracleSim& s) {
    run_hash_and_sort(s);
    int nc = cellindices(s.num, s.keys.data(), s.start.data(), s.end.data(), s.gp.nb_cells);
    s.last_nc = nc;
    run_permute(s);
    if (nc <= s.num && nc >= 0) {
        // Out-of-grid deletion (SPH.cpp:220-250): keep the first nc sorted
        // particles, copy sorted -> unsorted (call_prep(2), :445-457), re-hash
        // and re-sort; cell ranges and permuted arrays are not recomputed.
        const int n = s.num;
        s.deleted_pos.assign(s.pos_s.begin() + 4 * (size_t)nc, s.pos_s.begin() + 4 * (size_t)n);
        s.deleted_vel.assign(s.vel_s.begin() + 4 * (size_t)nc, s.vel_s.begin() + 4 * (size_t)n);
        s.num = nc;
        std::memcpy(s.pos_u.data(), s.pos_s.data(), 16 * (size_t)nc);
        std::memcpy(s.vel_u.data(), s.vel_s.data(), 16 * (size_t)nc);
        std::memcpy(s.veleval_u.data(), s.veleval_s.data(), 16 * (size_t)nc);
        run_hash_and_sort(s);
    }
    if (s.use_f64) {
        run_density<double>(s);
        run_force<double>(s);
        run_gravity<double>(s);
        run_collision<double>(s);
        run_triangles<double>(s);
    } else {
        run_density<float>(s);
        run_force<float>(s);
        run_gravity<float>(s);
        run_collision<float>(s);
        run_triangles<float>(s);
    }
}

// SPH::integrate (SPH.cpp:389-441): euler or leapfrog.
static void sim_integrate(OracleSim& s, float dt) {
    if (s.integrator == 1) {
        if (s.use_f64)
            run_euler<double>(s, dt);
        else
            run_euler<float>(s, dt);
    } else if (s.use_f64) {
        run_leapfrog<double>(s, dt);
    } else {
        run_leapfrog<float>(s, dt);
    }
}

extern "C" {

const char* oracle_info(void) {
#ifdef _OPENMP
    static std::string info = "sph_oracle openmp threads=" + std::to_string(omp_get_max_threads());
#else
    static std::string info = "sph_oracle serial";
#endif
    return info.c_str();
}

int oracle_threads(void) { return omp_threads(); }
void oracle_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

// --- individual stages on caller arrays (float32 data, float4 = 4 floats) ---
void oracle_hash(int n, const float* pos_u, const GridParams* gp, uint32_t* keys, uint32_t* idx) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) hash_one<float>(pos_u, *gp, i, keys, idx);
}
void oracle_sort(int n, uint32_t* keys, uint32_t* idx) { stable_sort_pairs(n, keys, idx); }
void oracle_sort_std(int n, uint32_t* keys, uint32_t* idx) {
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    std::vector<uint32_t> k(n), v(n);
    for (int i = 0; i < n; ++i) {
        k[i] = keys[order[i]];
        v[i] = idx[order[i]];
    }
    std::memcpy(keys, k.data(), 4 * (size_t)n);
    std::memcpy(idx, v.data(), 4 * (size_t)n);
}
int oracle_cellindices(int n, const uint32_t* keys, uint32_t* start, uint32_t* end, int nb_cells) {
    return cellindices(n, keys, start, end, nb_cells);
}
void oracle_permute(int n, const uint32_t* idx, const float* pos_u, const float* vel_u, const float* veleval_u,
                    float* pos_s, float* vel_s, float* veleval_s) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const size_t o = (size_t)idx[i] * 4, d = (size_t)i * 4;
        std::memcpy(pos_s + d, pos_u + o, 16);
        std::memcpy(vel_s + d, vel_u + o, 16);
        std::memcpy(veleval_s + d, veleval_u + o, 16);
    }
}
void oracle_density(int f64, int n, const float* pos_s, const uint32_t* start, const uint32_t* end,
                    const GridParams* gps, const SPHParams* sp, float* density, uint32_t* nbr) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        if (f64)
            density_one<double>(i, pos_s, start, end, *gps, *sp, density, nbr);
        else
            density_one<float>(i, pos_s, start, end, *gps, *sp, density, nbr);
    }
}
void oracle_force(int f64, int n, const float* pos_s, const float* density, const float* veleval_s,
                  const uint32_t* start, const uint32_t* end, const GridParams* gps, const SPHParams* sp,
                  float* force, float* xsph) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        if (f64)
            force_one<double>(i, pos_s, density, veleval_s, start, end, *gps, *sp, force, xsph);
        else
            force_one<float>(i, pos_s, density, veleval_s, start, end, *gps, *sp, force, xsph);
    }
}
void oracle_collision(int f64, int n, const float* pos_s, const float* vel_s, float* force, const GridParams* gps,
                      const SPHParams* sp) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (f64)
            collision_one<double>(i, pos_s, vel_s, force, *gps, *sp);
        else
            collision_one<float>(i, pos_s, vel_s, force, *gps, *sp);
    }
}
void oracle_leapfrog(int f64, int n, const float* pos_s, const float* vel_s, const float* force, const float* xsph,
                     const uint32_t* idx, const SPHParams* sp, float dt, float* pos_u, float* vel_u,
                     float* veleval_u) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (f64)
            leapfrog_one<double>(i, pos_s, vel_s, force, xsph, idx, *sp, dt, pos_u, vel_u, veleval_u);
        else
            leapfrog_one<float>(i, pos_s, vel_s, force, xsph, idx, *sp, dt, pos_u, vel_u, veleval_u);
    }
}

void oracle_gravity(int f64, int n, int nsrc, const float* points, const float* masses, const float* alphas,
                    const float* pos_s, float* force, float scale) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (f64)
            gravity_one<double>(i, nsrc, points, masses, alphas, pos_s, force, scale);
        else
            gravity_one<float>(i, nsrc, points, masses, alphas, pos_s, force, scale);
    }
}
void oracle_collision_triangles(int f64, int n, const float* pos_s, const float* vel_s, float* force,
                                const float* tris, int ntri, const SPHParams* sp) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        if (f64)
            collision_tri_one<double>(i, pos_s, vel_s, force, tris, ntri, *sp);
        else
            collision_tri_one<float>(i, pos_s, vel_s, force, tris, ntri, *sp);
    }
}
void oracle_colorfield(int f64, int res, const float* pos_s, const float* density, const uint32_t* start,
                       const uint32_t* end, const GridParams* gps, const SPHParams* sp, float* field) {
    const long total = (long)res * res * res;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < total; ++k) {
        const int s = (int)(k % res), t = (int)((k / res) % res), r = (int)(k / ((long)res * res));
        field[k] = f64 ? colorfield_one<double>(s, t, r, res, pos_s, density, start, end, *gps, *sp)
                       : colorfield_one<float>(s, t, r, res, pos_s, density, start, end, *gps, *sp);
    }
}
void oracle_euler(int f64, int n, const float* pos_s, const float* vel_s, const float* force, const uint32_t* idx,
                  const SPHParams* sp, float dt, float* pos_u, float* vel_u) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (f64)
            euler_one<double>(i, pos_s, vel_s, force, idx, *sp, dt, pos_u, vel_u);
        else
            euler_one<float>(i, pos_s, vel_s, force, idx, *sp, dt, pos_u, vel_u);
    }
}

// --- whole system ----------------------------------------------------------
void* oracle_sim_create(const SPHParams* sp, const GridParams* gp, const GridParams* gps, int max_num, int f64) {
    OracleSim* s = new OracleSim();
    s->sp = *sp;
    s->gp = *gp;
    s->gps = *gps;
    s->max_num = max_num;
    s->use_f64 = f64;
    const size_t m4 = 4 * (size_t)max_num;
    for (auto* v : {&s->pos_u, &s->vel_u, &s->veleval_u, &s->pos_s, &s->vel_s, &s->veleval_s, &s->force_s,
                    &s->xsph_s})
        v->assign(m4, 0.f);
    s->density_s.assign(max_num, 0.f);
    s->keys.assign(max_num, 0x7fffffffu);  // prepareSorted fills INT_MAX (System.cpp:274-278)
    s->idx.assign(max_num, 0x7fffffffu);
    s->nbr.assign(max_num, 0u);
    s->start.assign((size_t)gp->nb_cells + 1, 666u);  // SPH::prepareSorted fills 666 (SPH.cpp:508-512)
    s->end.assign((size_t)gp->nb_cells + 1, 666u);
    return s;
}
void oracle_sim_destroy(void* h) { delete (OracleSim*)h; }
void oracle_sim_set_params(void* h, const SPHParams* sp) { ((OracleSim*)h)->sp = *sp; }
int oracle_sim_upload(void* h, const float* pos, const float* vel, const float* veleval, int n) {
    OracleSim* s = (OracleSim*)h;
    if (n < 0 || n > s->max_num) return -1;
    std::memcpy(s->pos_u.data(), pos, 16 * (size_t)n);
    std::memcpy(s->vel_u.data(), vel, 16 * (size_t)n);
    if (veleval)
        std::memcpy(s->veleval_u.data(), veleval, 16 * (size_t)n);
    else
        std::fill(s->veleval_u.begin(), s->veleval_u.begin() + 4 * (size_t)n, 0.f);
    s->num = n;
    return 0;
}
// SPH::pushParticles (SPH.cpp:560-602): pos and vel appended after the
// current particles, veleval left as it is; a push past max_num is dropped
// (returns -1).
int oracle_sim_push(void* h, const float* pos, const float* vel, int n) {
    OracleSim* s = (OracleSim*)h;
    if (n < 0 || s->num + n > s->max_num) return -1;
    std::memcpy(s->pos_u.data() + 4 * (size_t)s->num, pos, 16 * (size_t)n);
    std::memcpy(s->vel_u.data() + 4 * (size_t)s->num, vel, 16 * (size_t)n);
    s->num += n;
    return 0;
}
void oracle_sim_update(void* h) { sim_update(*(OracleSim*)h); }
void oracle_sim_integrate(void* h, float dt) { sim_integrate(*(OracleSim*)h, dt); }
void oracle_sim_step(void* h, float dt, int nsteps) {
    OracleSim* s = (OracleSim*)h;
    for (int k = 0; k < nsteps; ++k) {
        sim_update(*s);
        sim_integrate(*s, dt);
    }
}
void oracle_sim_set_gravity(void* h, int nsrc, const float* points, const float* masses, const float* alphas) {
    OracleSim* s = (OracleSim*)h;
    s->grav_points.assign(points, points + 4 * (size_t)(nsrc > 0 ? nsrc : 0));
    s->grav_masses.assign(masses, masses + (nsrc > 0 ? nsrc : 0));
    s->grav_alphas.assign(alphas, alphas + (nsrc > 0 ? nsrc : 0));
}
void oracle_sim_set_integrator(void* h, int integrator) { ((OracleSim*)h)->integrator = integrator; }
void oracle_sim_set_triangles(void* h, const float* tris, int ntri) {
    ((OracleSim*)h)->triangles.assign(tris, tris + 16 * (size_t)(ntri > 0 ? ntri : 0));
}
int oracle_sim_num(void* h) { return ((OracleSim*)h)->num; }
int oracle_sim_last_nc(void* h) { return ((OracleSim*)h)->last_nc; }
// field ids follow enum sph_field of include/rtps_sph.h
int oracle_sim_get(void* h, int field, void* out, int n) {
    OracleSim* s = (OracleSim*)h;
    const void* src = nullptr;
    size_t esz = 16;
    switch (field) {
        case SPH_FIELD_POS_U: src = s->pos_u.data(); break;
        case SPH_FIELD_VEL_U: src = s->vel_u.data(); break;
        case SPH_FIELD_VELEVAL_U: src = s->veleval_u.data(); break;
        case SPH_FIELD_POS_S: src = s->pos_s.data(); break;
        case SPH_FIELD_VEL_S: src = s->vel_s.data(); break;
        case SPH_FIELD_VELEVAL_S: src = s->veleval_s.data(); break;
        case SPH_FIELD_DENSITY_S: src = s->density_s.data(); esz = 4; break;
        case SPH_FIELD_FORCE_S: src = s->force_s.data(); break;
        case SPH_FIELD_XSPH_S: src = s->xsph_s.data(); break;
        case SPH_FIELD_SORT_HASHES: src = s->keys.data(); esz = 4; break;
        case SPH_FIELD_SORT_INDICES: src = s->idx.data(); esz = 4; break;
        case SPH_FIELD_CELL_START: src = s->start.data(); esz = 4; break;
        case SPH_FIELD_CELL_END: src = s->end.data(); esz = 4; break;
        case SPH_FIELD_NEIGHBOR_COUNT: src = s->nbr.data(); esz = 4; break;
        default: return -1;
    }
    std::memcpy(out, src, esz * (size_t)n);
    return 0;
}
int oracle_sim_deleted(void* h, float* pos, float* vel, int cap) {
    OracleSim* s = (OracleSim*)h;
    int nd = (int)(s->deleted_pos.size() / 4);
    int k = std::min(nd, cap);
    if (pos) std::memcpy(pos, s->deleted_pos.data(), 16 * (size_t)k);
    if (vel) std::memcpy(vel, s->deleted_vel.data(), 16 * (size_t)k);
    return nd;
}

}  // extern "C"
