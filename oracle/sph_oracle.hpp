// sph_oracle.hpp — TEST INFRASTRUCTURE, not part of the product.
//
// CPU restatement of the RTPS / EnjaParticles SPH step (the reference's OpenCL
// kernels), used only as the checker by tests/, by __graft_entry__.smoke() and
// by bench.py's CPU-baseline leg.  Nothing in enjaparticles_gb300/ links or
// calls it.
//
// Every function names the reference file:line it restates.  Arithmetic is
// written operation by operation in the reference's order and compiled with
// -ffp-contract=off, so that the FP32 instantiation gives the same bits as
// the reference kernels compiled for a CPU (see ref/ and tests/golden/):
//   * length(r) = sqrt(((x*x + y*y) + z*z) + w*w), dot likewise;
//   * double literals keep double semantics, as a C/C++ compile of the kernel
//     source gives them: 1.0/density is a double division, and
//     `2.0 * mass * wpoly6` is evaluated in double and rounded once to float
//     when it meets a float4;
//   * float -> int conversion truncates toward zero and saturates, NaN -> 0.
// The FP64 instantiation (T = double) runs every operation in double; it is
// the finite-difference reference for gradients.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/rtps_sph.h"

namespace sph_oracle {

static const uint32_t kEmpty = 0xffffffffu;

template <class T>
struct V4 {
    T x, y, z, w;
};

template <class T>
inline V4<T> load4(const float* p) {
    return V4<T>{(T)p[0], (T)p[1], (T)p[2], (T)p[3]};
}
template <class T>
inline void store4(float* p, const V4<T>& v) {
    p[0] = (float)v.x; p[1] = (float)v.y; p[2] = (float)v.z; p[3] = (float)v.w;
}
template <class T> inline V4<T> add(V4<T> a, V4<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
template <class T> inline V4<T> sub(V4<T> a, V4<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
template <class T> inline V4<T> mul(V4<T> a, T s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
template <class T> inline V4<T> smul(T s, V4<T> a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }
template <class T> inline V4<T> divs(V4<T> a, T s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }
template <class T> inline T dot4(V4<T> a, V4<T> b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
template <class T> inline T length4(V4<T> a) { return std::sqrt(dot4(a, a)); }

// A scalar computed in double by the reference source (a double literal in
// the expression) that then multiplies a float4: rounded once to T.
template <class T> inline T from_double(double v) { return (T)v; }

// (int)x of the kernels: truncation toward zero, saturating, NaN -> 0 (the
// CUDA cvt.rzi.s32 semantics; OpenCL leaves out-of-range values undefined).
template <class T>
inline int32_t trunc_sat(T v) {
    if (v != v) return 0;
    if (v >= (T)2147483648.0) return INT32_MAX;
    if (v < (T)-2147483648.0) return INT32_MIN;
    return (int32_t)v;
}

struct Cell { int32_t x, y, z; };

// calcGridCell (system/common/cl_src/cl_hash.h:33-54): per axis
// (int)((p - grid_min) * grid_delta), evaluated in T.
template <class T>
inline Cell calc_grid_cell(const V4<T>& p, const GridParams& gp) {
    T px = (p.x - (T)gp.grid_min.x) * (T)gp.grid_delta.x;
    T py = (p.y - (T)gp.grid_min.y) * (T)gp.grid_delta.y;
    T pz = (p.z - (T)gp.grid_min.z) * (T)gp.grid_delta.z;
    return Cell{trunc_sat(px), trunc_sat(py), trunc_sat(pz)};
}

// calcGridHash (cl_hash.h:57-114, wrapEdges=false): the key
// (gz*res.y + gy)*res.x + gx is evaluated in float (grid_res is float4),
// then converted to int.
inline int32_t calc_grid_hash(int32_t gx, int32_t gy, int32_t gz, const GridParams& gp) {
    float a = (float)gz * gp.grid_res.y;
    float b = a + (float)gy;
    float c = b * gp.grid_res.x;
    float d = c + (float)gx;
    return trunc_sat(d);
}

// ---------------------------------------------------------------------------
// hash (system/common/cl_src/hash.cl:50-157; Hash.cpp:42-75).  Unscaled grid.
template <class T>
inline void hash_one(const float* pos_u, const GridParams& gp, int i, uint32_t* keys, uint32_t* idx) {
    V4<T> p = load4<T>(pos_u + 4 * (size_t)i);
    Cell c = calc_grid_cell(p, gp);
    int32_t h = calc_grid_hash(c.x, c.y, c.z, gp);
    h = h > gp.nb_cells ? gp.nb_cells : h;
    h = h < 0 ? gp.nb_cells : h;
    keys[i] = (uint32_t)h;
    idx[i] = (uint32_t)i;
}

// Stable key/value sort: ascending keys, equal keys in ascending original
// index.  This is the canonical order that the reference's (unstable)
// bitonic sort (common/BitonicSort.cpp:62-171) is compared in.
void stable_sort_pairs(int n, uint32_t* keys, uint32_t* vals);

// cellindices (system/common/cl_src/cellindices.cl:12-107;
// CellIndices.cpp:42-99).  start[0..C] is reset to 0xffffffff (the host upload
// of CellIndices.cpp:58-62), end[] keeps stale entries.  Returns start[C] as
// int (-1 when no particle is outside the grid).
int cellindices(int n, const uint32_t* keys, uint32_t* start, uint32_t* end, int nb_cells);

// Neighbour walk (sph/cl_src/cl_sph_neighbors.h:49-140): cells z, y, x in
// [cell-1, cell+1], each cell's particles j in [start, end) ascending.  Cells
// whose hash (as uint) is >= nb_cells are skipped; no per-axis clamping (x-1
// of the first column is the previous row's last cell, as in the reference).
template <class T, class F>
inline void for_each_candidate(const V4<T>& pi, const GridParams& gps, const uint32_t* start,
                               const uint32_t* end, F&& f) {
    Cell c = calc_grid_cell(pi, gps);
    for (int z = c.z - 1; z <= c.z + 1; ++z)
        for (int y = c.y - 1; y <= c.y + 1; ++y)
            for (int x = c.x - 1; x <= c.x + 1; ++x) {
                uint32_t h = (uint32_t)calc_grid_hash(x, y, z, gps);
                if (h >= (uint32_t)gps.nb_cells) continue;
                uint32_t s = start[h];
                if (s == kEmpty) continue;
                uint32_t e = end[h];
                for (uint32_t j = s; j < e; ++j) f(j);
            }
}

// density_update (sph/cl_src/density.cl:44-126; Wpoly6 cl_sph_kernels.h:29-45).
// Scaled grid.  Self term included.  nbr (optional) counts accepted j.
template <class T>
inline void density_one(int i, const float* pos_s, const uint32_t* start, const uint32_t* end,
                        const GridParams& gps, const SPHParams& sp, float* density, uint32_t* nbr) {
    const T sc = (T)sp.simulation_scale, h = (T)sp.smoothing_distance;
    V4<T> pi = mul(load4<T>(pos_s + 4 * (size_t)i), sc);
    T acc = 0;
    uint32_t cnt = 0;
    for_each_candidate(pi, gps, start, end, [&](uint32_t j) {
        V4<T> pj = mul(load4<T>(pos_s + 4 * (size_t)j), sc);
        V4<T> r = sub(pi, pj);
        r.w = 0;
        T rlen = length4(r);
        if (rlen <= h) {
            T r2 = r.x * r.x + r.y * r.y + r.z * r.z;
            T hr2 = h * h - r2;
            acc += hr2 * hr2 * hr2;
            ++cnt;
        }
    });
    density[i] = (float)(((T)sp.wpoly6_coef * (T)sp.mass) * acc);
    if (nbr) nbr[i] = cnt;
}

// force_update (sph/cl_src/force.cl:43-186; Wspiky_dr cl_sph_kernels.h:81-97,
// Wvisc_lapl :118-127).  Scaled grid, veleval velocities.
template <class T>
inline void force_one(int i, const float* pos_s, const float* density, const float* veleval_s,
                      const uint32_t* start, const uint32_t* end, const GridParams& gps,
                      const SPHParams& sp, float* force, float* xsph) {
    const T sc = (T)sp.simulation_scale, h = (T)sp.smoothing_distance;
    const T eps = (T)sp.EPSILON, K = (T)sp.K, rho0 = (T)sp.rest_density;
    V4<T> pi = mul(load4<T>(pos_s + 4 * (size_t)i), sc);
    const T di = (T)density[i];
    V4<T> F{0, 0, 0, 0}, V{0, 0, 0, 0}, X{0, 0, 0, 0};
    for_each_candidate(pi, gps, start, end, [&](uint32_t j) {
        V4<T> pj = mul(load4<T>(pos_s + 4 * (size_t)j), sc);
        V4<T> r = sub(pi, pj);
        r.w = 0;
        T rlen = length4(r);
        if (!(rlen <= h)) return;
        const T iej = ((uint32_t)i != j) ? (T)1 : (T)0;
        rlen = (rlen < eps) ? eps : rlen;             // max(rlen, EPSILON)
        T hr = h - rlen;
        T dWijdr = hr * hr / rlen;                     // Wspiky_dr
        const T dj = (T)density[j];
        const T idj = (T)(1.0 / (double)dj);           // float idj = 1.0/dj
        T Pi = K * (di - rho0);
        T Pj = K * (dj - rho0);
        T kern = dWijdr * (Pi + Pj) * idj;
        V4<T> veli = load4<T>(veleval_s + 4 * (size_t)i);
        V4<T> velj = load4<T>(veleval_s + 4 * (size_t)j);
        T lapl = h - rlen;                             // Wvisc_lapl
        V4<T> dv = sub(velj, veli);
        V4<T> visc = mul(mul(dv, lapl), idj);
        V = add(V, mul(visc, iej));
        T r2 = r.x * r.x + r.y * r.y + r.z * r.z;      // Wpoly6
        T hr2 = h * h - r2;
        T w6 = hr2 * hr2 * hr2;
        V4<T> xs = divs(smul(w6, dv), di + dj);
        X = add(X, mul(xs, iej));
        X.w = 0;
        F = add(F, mul(mul(r, kern), iej));
        F.w = 0;
    });
    // force = (mass * (1.0/density)) * ((-0.5*wspiky_d*F) + (viscosity*wvisc_dd*V))
    const T a = from_double<T>((double)sp.mass * (1.0 / (double)density[i]));
    const T b = from_double<T>(-0.5 * (double)sp.wspiky_d_coef);
    const T s = (T)sp.viscosity * (T)sp.wvisc_dd_coef;
    V4<T> f = smul(a, add(smul(b, F), smul(s, V)));
    // xsph = 2.0 * mass * wpoly6 * X
    const T d = from_double<T>(2.0 * (double)sp.mass * (double)sp.wpoly6_coef);
    V4<T> x = smul(d, X);
    store4(force + 4 * (size_t)i, f);
    store4(xsph + 4 * (size_t)i, x);
}

// calculateRepulsionForce / calculateFrictionForce
// (sph/cl_src/cl_sph_collision.h:31-73); kinetic and static friction are the
// constants 0 of collision_wall.cl:61-62.
template <class T>
inline V4<T> repulsion(V4<T> n, V4<T> v, T k, T c, T dist) {
    v.w = 0;
    V4<T> rf = smul(k * dist - c * dot4(n, v), n);
    rf.w = 0;
    return rf;
}
template <class T>
inline V4<T> friction(V4<T> v, V4<T> f, V4<T> n) {
    const T kinetic = 0, static_limit = 0;
    f.w = 0;
    v.w = 0;
    V4<T> vn = mul(v, dot4(n, v));
    V4<T> vt = sub(v, vn);
    V4<T> neg{-vt.x, -vt.y, -vt.z, -vt.w};
    if ((vt.x + vt.y + vt.z) / (T)3 > static_limit) return neg;
    return smul(kinetic, neg);
}

// collision_wall (sph/cl_src/collision_wall.cl:31-118).  Scaled grid bounds,
// bound distance rest_distance*0.5, sorted velocity vel_s.
template <class T>
inline void collision_one(int i, const float* pos_s, const float* vel_s, float* force,
                          const GridParams& gps, const SPHParams& sp) {
    const T bound = (T)sp.rest_distance * (T)0.5;
    const T eps = (T)sp.EPSILON, k = (T)sp.boundary_stiffness, c = (T)sp.boundary_dampening;
    V4<T> p = mul(load4<T>(pos_s + 4 * (size_t)i), (T)sp.simulation_scale);
    V4<T> v = load4<T>(vel_s + 4 * (size_t)i);
    V4<T> f = load4<T>(force + 4 * (size_t)i);
    V4<T> rf{0, 0, 0, 0}, ff{0, 0, 0, 0};
    auto wall = [&](T diff, V4<T> n) {
        if (diff > eps) {
            rf = add(rf, repulsion(n, v, k, c, diff));
            ff = add(ff, friction(v, f, n));
        }
    };
    wall(bound - (p.z - (T)gps.bnd_min.z), V4<T>{0, 0, 1, 0});
    wall(bound - ((T)gps.bnd_max.z - p.z), V4<T>{0, 0, -1, 0});
    wall(bound - (p.y - (T)gps.bnd_min.y), V4<T>{0, 1, 0, 0});
    wall(bound - ((T)gps.bnd_max.y - p.y), V4<T>{0, -1, 0, 0});
    wall(bound - (p.x - (T)gps.bnd_min.x), V4<T>{1, 0, 0, 0});
    wall(bound - ((T)gps.bnd_max.x - p.x), V4<T>{-1, 0, 0, 0});
    store4(force + 4 * (size_t)i, add(f, add(rf, ff)));
}

// leapfrog (sph/cl_src/leapfrog.cl:30-121): gravity, acceleration clamp by
// velocity_limit, XSPH, scatter to original order.
template <class T>
inline void leapfrog_one(int i, const float* pos_s, const float* vel_s, const float* force,
                         const float* xsph, const uint32_t* idx, const SPHParams& sp, float dt_f,
                         float* pos_u, float* vel_u, float* veleval_u) {
    const T sc = (T)sp.simulation_scale, dt = (T)dt_f, lim = (T)sp.velocity_limit;
    V4<T> p = mul(load4<T>(pos_s + 4 * (size_t)i), sc);
    V4<T> v = load4<T>(vel_s + 4 * (size_t)i);
    V4<T> f = load4<T>(force + 4 * (size_t)i);
    V4<T> g{(T)sp.gravity.x, (T)sp.gravity.y, (T)sp.gravity.z, (T)sp.gravity.w};
    f = add(f, g);
    f.w = 0;
    T speed = length4(f);
    if (speed > lim) f = mul(f, lim / speed);
    V4<T> vnext = add(v, smul(dt, f));
    vnext = add(vnext, smul((T)sp.xsph_factor, load4<T>(xsph + 4 * (size_t)i)));
    V4<T> veval = smul((T)0.5, add(v, vnext));
    p = add(p, smul(dt, vnext));
    p.w = 1;
    const uint32_t o = idx[i];
    p.x = p.x / sc;
    p.y = p.y / sc;
    p.z = p.z / sc;
    store4(vel_u + 4 * (size_t)o, vnext);
    store4(veleval_u + 4 * (size_t)o, veval);
    store4(pos_u + 4 * (size_t)o, V4<T>{p.x, p.y, p.z, (T)1});
}

// Point-source gravity, gravity (system/common/cl_src/gravity.cl:9-35) as
// SPH::updateGPU calls it after force (SPH.cpp:289-296): for each source s,
// vect = scale * (point_s - pos_s[i]) with w = 0, accel += mag * direction,
// direction = fast_normalize(vect) = vect * (1 / sqrt(dot(vect, vect))) (the
// precision of fast_normalize is the implementation's; this is the choice of
// the host build of the reference kernels too), mag = alpha_s * mass_s divided
// by dist2, or by -(0.5 scale)^2 inside that radius.
template <class T>
inline void gravity_one(int i, int nsrc, const float* points, const float* masses, const float* alphas,
                        const float* pos_s, float* accel, float scale_f) {
    const T scale = (T)scale_f;
    const V4<T> p = load4<T>(pos_s + 4 * (size_t)i);
    V4<T> a = load4<T>(accel + 4 * (size_t)i);
    for (int s = 0; s < nsrc; ++s) {
        V4<T> vect = smul(scale, sub(load4<T>(points + 4 * (size_t)s), p));
        vect.w = 0;
        const V4<T> direction = mul(vect, (T)1 / std::sqrt(dot4(vect, vect)));
        const T dist2 = dot4(vect, vect);
        T mag = (T)alphas[s] * (T)masses[s];
        T cutoff = (T)0.5f * scale;
        cutoff *= cutoff;
        if (dist2 < cutoff)
            mag /= -cutoff;
        else
            mag /= dist2;
        a = add(a, smul(mag, direction));
    }
    store4(accel + 4 * (size_t)i, a);
}

// SPH Euler integrator, euler (sph/cl_src/euler.cl:33-78), the integrator of
// SPH::integrate when the settings say "euler" (SPH.cpp:392-411).  Its
// gravity is the constant -9.8 in z and its acceleration limit the constant
// 600 (not SPHParams.gravity / velocity_limit); it writes pos_u and vel_u and
// leaves veleval_u alone; no XSPH.
template <class T>
inline void euler_one(int i, const float* pos_s, const float* vel_s, const float* force, const uint32_t* idx,
                      const SPHParams& sp, float dt_f, float* pos_u, float* vel_u) {
    const T sc = (T)sp.simulation_scale, dt = (T)dt_f;
    V4<T> p = mul(load4<T>(pos_s + 4 * (size_t)i), sc);
    V4<T> v = load4<T>(vel_s + 4 * (size_t)i);
    V4<T> f = load4<T>(force + 4 * (size_t)i);
    f.z += (T)-9.8f;
    const T speed = std::sqrt(f.x * f.x + f.y * f.y + f.z * f.z);
    if (speed > (T)600.0f) f = mul(f, (T)600.0f / speed);
    v = add(v, smul(dt, f));
    p = add(p, smul(dt, v));
    const uint32_t o = idx[i];
    store4(vel_u + 4 * (size_t)o, v);
    store4(pos_u + 4 * (size_t)o, V4<T>{p.x / sc, p.y / sc, p.z / sc, (T)1});
}

// Triangle-mesh collision, collision_triangle (sph/cl_src/collision_tri.cl:
// 436-520 with collisions_triangle :274-374 and intersect_triangle_segment
// :203-247), run by SPH::collision after the walls (SPH.cpp:303-336).
// Triangles: 16 floats each (three vertices and a normal, rtpslib/structs.h:
// 586-590); the normal is not read: the kernel recomputes it from the
// scaled vertices.  Per particle, triangles in groups of 220 (the kernel's
// shared-memory chunk): f sums the contributions of a group, then rf += f.
// A triangle contributes when the segment pos -+ boundary_distance * v/|v|
// crosses it (Ericson's segment test) at a point tp with
// d = boundary_distance - |pos - tp| > 1e-6: f += n_hat (k d - c n_hat.v)
// (repulsion) and then the zero-coefficient "friction" (as the walls).
// f.w counts the triangles, so force.w grows by the triangle count.  A zero
// velocity gives NaNs, and no contribution.
template <class T>
inline V4<T> cross3(V4<T> a, V4<T> b) {
    return V4<T>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, (T)0};
}
template <class T>
inline V4<T> v3normalize(V4<T> a) {
    const T mag = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return V4<T>{a.x / mag, a.y / mag, a.z / mag, (T)0};
}
template <class T>
inline T tri_segment_distance(V4<T> pos, V4<T> vel, V4<T> a, V4<T> b, V4<T> c, V4<T> n, T dist) {
    const V4<T> ab = sub(b, a), ac = sub(c, a);
    const V4<T> vn = v3normalize(vel);
    const V4<T> p = sub(pos, mul(vn, dist));
    const V4<T> q = add(pos, mul(vn, dist));
    const V4<T> qp = sub(p, q);
    const T d = dot4(qp, n);
    if (d <= (T)0) return (T)2 * dist;
    const V4<T> ap = sub(p, a);
    T t = dot4(ap, n);
    if (t < (T)0 || t > d) return (T)2 * dist;
    const V4<T> e = cross3(qp, ap);
    T v = dot4(ac, e);
    if (v < (T)0 || v > d) return (T)2 * dist;
    T w = -dot4(ab, e);
    if (w < (T)0 || v + w > d) return (T)2 * dist;
    const T ood = (T)1 / d;
    t *= ood;
    v *= ood;
    w *= ood;
    const T u = (T)1 - v - w;
    const V4<T> tp = add(add(smul(u, a), smul(v, b)), smul(w, c));
    const V4<T> r = sub(pos, tp);
    return std::sqrt(r.x * r.x + r.y * r.y + r.z * r.z);
}
template <class T>
inline void collision_tri_one(int i, const float* pos_s, const float* vel_s, float* force, const float* tris,
                              int ntri, const SPHParams& sp) {
    const T scale = (T)sp.simulation_scale, bound = (T)sp.boundary_distance;
    const T k = (T)sp.boundary_stiffness, c = (T)sp.boundary_dampening, eps = (T)1e-6f;
    const V4<T> pos = mul(load4<T>(pos_s + 4 * (size_t)i), scale);
    const V4<T> vel = load4<T>(vel_s + 4 * (size_t)i);
    const V4<T> f0 = load4<T>(force + 4 * (size_t)i);
    V4<T> rf{0, 0, 0, 0};
    for (int first = 0; first < ntri; first += 220) {
        const int last = first + 220 < ntri ? first + 220 : ntri;
        V4<T> f{0, 0, 0, 0};
        for (int j = first; j < last; ++j) {
            const float* tj = tris + 16 * (size_t)j;
            const V4<T> a = mul(load4<T>(tj), scale), b = mul(load4<T>(tj + 4), scale),
                        cc = mul(load4<T>(tj + 8), scale);
            const V4<T> n = cross3(sub(b, a), sub(cc, a));
            const V4<T> nhat = v3normalize(n);
            const T dd = bound - tri_segment_distance(pos, vel, a, b, cc, n, bound);
            if (dd > eps) {
                f = add(f, repulsion(nhat, vel, k, c, dd));
                f = add(f, friction(vel, f0, nhat));
            }
            f.w += (T)1;
        }
        rf = add(rf, f);
    }
    store4(force + 4 * (size_t)i, add(f0, rf));
}

// Colour field, colorfield_update (sph/cl_src/colorfield.cl:66-103; Wspiky
// cl_sph_kernels.h:71-78), as ColorField::execute runs it over res^3 sample
// points (sph/ColorField.cpp:84-121) with the scaled grid.  Sample (s, t, r)
// sits at (s, t, r) / (res - 1) of the way from bnd_min to bnd_max; its value
// is mass * sum over the particles within h (27-cell walk, as density) of
// Wspiky(max(|r|, EPSILON)) / rho_j.  The kernel forms 1/rho_j and the product
// in double (1.0 is a double literal) and rounds the product to float.
template <class T>
inline T wspiky(T rlen, T h) {
    const T h6 = h * h * h * h * h * h;
    const T alpha = (T)15.f / (T)3.14159265358979323846f / h6;
    const T hr2 = h - rlen;
    return alpha * hr2 * hr2 * hr2;
}
template <class T>
inline float colorfield_one(int s, int t, int r, int res, const float* pos_s, const float* density,
                            const uint32_t* start, const uint32_t* end, const GridParams& gps, const SPHParams& sp) {
    const float tmp = 1.0f / (float)(unsigned)(res - 1);
    const float fx = (float)(unsigned)s * tmp, fy = (float)(unsigned)t * tmp, fz = (float)(unsigned)r * tmp;
    V4<T> p{(T)fx * ((T)gps.bnd_max.x - (T)gps.bnd_min.x) + (T)gps.bnd_min.x,
            (T)fy * ((T)gps.bnd_max.y - (T)gps.bnd_min.y) + (T)gps.bnd_min.y,
            (T)fz * ((T)gps.bnd_max.z - (T)gps.bnd_min.z) + (T)gps.bnd_min.z, (T)1};
    const T sc = (T)sp.simulation_scale, h = (T)sp.smoothing_distance, eps = (T)sp.EPSILON;
    T acc = 0;
    for_each_candidate(p, gps, start, end, [&](uint32_t j) {
        V4<T> pj = mul(load4<T>(pos_s + 4 * (size_t)j), sc);
        V4<T> d = sub(p, pj);
        d.w = 0;
        T rlen = length4(d);
        if (rlen <= h) {
            rlen = rlen < eps ? eps : rlen;
            const T kern = (T)((double)wspiky(rlen, h) * (1.0 / (double)density[j]));
            acc += kern;
        }
    });
    return (float)(acc * (T)sp.mass);
}

}  // namespace sph_oracle
