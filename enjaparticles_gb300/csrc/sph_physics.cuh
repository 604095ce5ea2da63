// sph_physics.cuh — per-particle physics shared by the staged kernels and the
// fused force+collision+leapfrog kernel.  Every operation is written with an
// explicitly rounded intrinsic, in the reference's order, so the staged and
// fused paths give the same bits and both match the FP32 oracle.
#pragma once

#include "sph_device.cuh"

namespace sphk {

__device__ __forceinline__ float4 v4add(float4 a, float4 b) {
    return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ float4 v4sub(float4 a, float4 b) {
    return make_float4(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __fsub_rn(a.w, b.w));
}
__device__ __forceinline__ float4 v4scale(float4 a, float s) {
    return make_float4(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s));
}
__device__ __forceinline__ float v4dot(float4 a, float4 b) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z)),
                     __fmul_rn(a.w, b.w));
}

// One wall of collision_wall.cl:31-118: calculateRepulsionForce and
// calculateFrictionForce (cl_sph_collision.h:31-73), friction coefficients 0.
__device__ __forceinline__ void wall_term(float diff, float4 n, float4 v, const StepParams& P, float4& rf,
                                          float4& ff) {
    if (!(diff > P.eps)) return;
    float4 vv = v;
    vv.w = 0.f;
    const float s = __fsub_rn(__fmul_rn(P.kwall, diff), __fmul_rn(P.cwall, v4dot(n, vv)));
    float4 rep = v4scale(n, s);
    rep.w = 0.f;
    rf = v4add(rf, rep);
    const float4 vn = v4scale(vv, v4dot(n, vv));
    const float4 vt = v4sub(vv, vn);
    const float4 neg = make_float4(-vt.x, -vt.y, -vt.z, -vt.w);
    const float mean = __fdiv_rn(__fadd_rn(__fadd_rn(vt.x, vt.y), vt.z), 3.0f);
    ff = v4add(ff, mean > 0.f ? neg : v4scale(neg, 0.f));
}

// force += r_f + f_f for the six walls in the reference's order (Z, Y, X).
// p is the scaled position pos_s*simulation_scale, v the sorted velocity.
__device__ __forceinline__ float4 collide_walls(float4 p, float4 v, float4 f, const StepParams& P) {
    float4 rf = make_float4(0.f, 0.f, 0.f, 0.f), ff = rf;
    wall_term(__fsub_rn(P.bound, __fsub_rn(p.z, P.gs_bnd_min.z)), make_float4(0.f, 0.f, 1.f, 0.f), v, P, rf, ff);
    wall_term(__fsub_rn(P.bound, __fsub_rn(P.gs_bnd_max.z, p.z)), make_float4(0.f, 0.f, -1.f, 0.f), v, P, rf, ff);
    wall_term(__fsub_rn(P.bound, __fsub_rn(p.y, P.gs_bnd_min.y)), make_float4(0.f, 1.f, 0.f, 0.f), v, P, rf, ff);
    wall_term(__fsub_rn(P.bound, __fsub_rn(P.gs_bnd_max.y, p.y)), make_float4(0.f, -1.f, 0.f, 0.f), v, P, rf, ff);
    wall_term(__fsub_rn(P.bound, __fsub_rn(p.x, P.gs_bnd_min.x)), make_float4(1.f, 0.f, 0.f, 0.f), v, P, rf, ff);
    wall_term(__fsub_rn(P.bound, __fsub_rn(P.gs_bnd_max.x, p.x)), make_float4(-1.f, 0.f, 0.f, 0.f), v, P, rf, ff);
    return v4add(f, v4add(rf, ff));
}

// leapfrog.cl:30-121 for one particle: p is pos_s*simulation_scale.
__device__ __forceinline__ void leapfrog_core(float4 p, float4 v, float4 f, float4 xs, float dt, const StepParams& P,
                                              float4& pos_out, float4& vel_out, float4& veleval_out) {
    f = v4add(f, P.gravity);
    f.w = 0.f;
    const float speed = __fsqrt_rn(v4dot(f, f));
    if (speed > P.vlimit) f = v4scale(f, __fdiv_rn(P.vlimit, speed));
    float4 vnext = v4add(v, make_float4(__fmul_rn(dt, f.x), __fmul_rn(dt, f.y), __fmul_rn(dt, f.z), __fmul_rn(dt, f.w)));
    vnext = v4add(vnext, make_float4(__fmul_rn(P.xsph_factor, xs.x), __fmul_rn(P.xsph_factor, xs.y),
                                     __fmul_rn(P.xsph_factor, xs.z), __fmul_rn(P.xsph_factor, xs.w)));
    const float4 vs = v4add(v, vnext);
    veleval_out = make_float4(__fmul_rn(0.5f, vs.x), __fmul_rn(0.5f, vs.y), __fmul_rn(0.5f, vs.z), __fmul_rn(0.5f, vs.w));
    p = v4add(p, make_float4(__fmul_rn(dt, vnext.x), __fmul_rn(dt, vnext.y), __fmul_rn(dt, vnext.z),
                             __fmul_rn(dt, vnext.w)));
    if (!P.unit_scale) {
        p.x = __fdiv_rn(p.x, P.sc);
        p.y = __fdiv_rn(p.y, P.sc);
        p.z = __fdiv_rn(p.z, P.sc);
    }
    pos_out = make_float4(p.x, p.y, p.z, 1.0f);
    vel_out = vnext;
}

// Point-source gravity (system/common/cl_src/gravity.cl:9-35), added to the
// force f of the particle at unscaled sorted position pos, as
// SPH::updateGPU does after force (SPH.cpp:289-296): per source,
// vect = sc * (point - pos) (w = 0), direction = vect / |vect|,
// f += (alpha * mass / d) * direction with d = |vect|^2, or
// d = -(0.5 sc)^2 inside that radius (the pull turns into a push).  The
// normalisation is OpenCL's fast_normalize, whose precision the
// implementation chooses: exact arithmetic takes vect * (1 / sqrt(|vect|^2))
// with both operations correctly rounded, fast arithmetic an rsqrt.
template <bool Exact>
__device__ __forceinline__ float4 gravity_add(float4 f, float4 pos, const StepParams& P) {
    const float cut0 = __fmul_rn(0.5f, P.sc);
    const float cut = __fmul_rn(cut0, cut0);
    for (int s = 0; s < P.n_grav; ++s) {
        float4 vect = v4scale(v4sub(__ldg(P.grav_pos + s), pos), P.sc);
        vect.w = 0.f;
        const float d2 = v4dot(vect, vect);
        const float inv = Exact ? __fdiv_rn(1.f, __fsqrt_rn(d2)) : rsqrtf(d2);
        const float4 dir = v4scale(vect, inv);
        float mag = __fmul_rn(__ldg(P.grav_alpha + s), __ldg(P.grav_mass + s));
        mag = d2 < cut ? __fdiv_rn(mag, -cut) : __fdiv_rn(mag, d2);
        f = v4add(f, v4scale(dir, mag));
    }
    return f;
}

// The SPH Euler integrator (sph/cl_src/euler.cl:33-78) for one particle: p is
// pos_s*simulation_scale.  Its gravity is the constant -9.8 in z and its
// acceleration limit the constant 600 (SPHParams.gravity / velocity_limit are
// not used); it gives position and velocity (veleval is left as it was).
__device__ __forceinline__ void euler_core(float4 p, float4 v, float4 f, float dt, const StepParams& P,
                                           float4& pos_out, float4& vel_out) {
    f.z = __fadd_rn(f.z, -9.8f);
    const float speed =
        __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(f.x, f.x), __fmul_rn(f.y, f.y)), __fmul_rn(f.z, f.z)));
    if (speed > 600.0f) f = v4scale(f, __fdiv_rn(600.0f, speed));
    v = v4add(v, v4scale(f, dt));
    p = v4add(p, v4scale(v, dt));
    if (!P.unit_scale) {
        p.x = __fdiv_rn(p.x, P.sc);
        p.y = __fdiv_rn(p.y, P.sc);
        p.z = __fdiv_rn(p.z, P.sc);
    }
    pos_out = make_float4(p.x, p.y, p.z, 1.0f);
    vel_out = v;
}

__device__ __forceinline__ float4 scaled(float4 p, const StepParams& P) {
    return P.unit_scale ? p : v4scale(p, P.sc);
}

// Effective particle count after the step's cell ranges: an out-of-grid
// deletion (SPH.cpp:220-250) keeps the first out_start sorted particles.
__device__ __forceinline__ int effective_num(const int* info, int& n_old, int& out) {
    n_old = info[kNum];
    out = info[kOutStart];
    return out >= 0 ? (out < n_old ? out : n_old) : n_old;
}

}  // namespace sphk
