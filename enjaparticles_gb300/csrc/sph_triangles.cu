// sph_triangles.cu — triangle-mesh collision: CollisionTriangle::execute
// (rtpslib/system/sph/Collision_triangle.cpp:84-116) running collision_triangle
// (sph/cl_src/collision_tri.cl:436-520, with collisions_triangle :274-374 and
// intersect_triangle_segment :203-247) after the walls (SPH.cpp:303-336).
//
// The reference walks every triangle for every particle, 220 triangles of
// local memory at a time.  Here a prep kernel computes, once per launch, each
// triangle's scaled vertices, its normal and unit normal, and its bounding
// box widened by the boundary distance plus a rounding margin.  A block of
// 256 sorted (so spatially close) particles then tests only the triangles
// whose widened box meets the box of its particles, and each particle only
// those whose widened box holds it.  A triangle outside the widened box
// cannot contribute: the contact point lies in the triangle (to rounding) and
// within the boundary distance of the particle.  A triangle that does not
// contribute adds nothing but 1 to force.w, so skipping it changes no bit.
//
// The arithmetic is the reference's, operation for operation, in explicitly
// rounded intrinsics, in every arithmetic mode: the contact test is a chain
// of branches on signs and thresholds, where a fused or approximate operation
// would move particles across them.  The grouping of the sums is kept: f
// collects the contributions of the triangles [220k, 220k + 220) in order and
// rf += f once per group; force += rf, rf.w being the triangle count.
//
// The w lanes of the vertices are not read.  In the reference they enter the
// dot products only multiplied by the zero w of a cross product, which for
// finite vertices adds a signed zero and changes no comparison and no result
// bit that is kept; the loader rejects non-finite vertices.
#include "sph_physics.cuh"

namespace sphk {

namespace {

constexpr int kTriThreads = 256;
constexpr int kTriChunk = 220;  // triangles per local-memory chunk of the reference

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// geo[4j..4j+3] = (a, n.x), (b, n.y), (c, n.z), (n_hat, 0) with a, b, c the
// scaled vertices, n = (b - a) x (c - a) and n_hat = n / |n| (cross_product,
// v3normalize: collision_tri.cl:44-58); box[2j], box[2j+1] the widened
// bounding box.
__global__ void __launch_bounds__(256) k_tri_prep(const float4* __restrict__ tris, int ntri, float4* __restrict__ geo,
                                                  float4* __restrict__ box, const StepParams P) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ntri) return;
    const float sc = P.sc;
    const float4 va = __ldg(tris + 4 * (size_t)j), vb = __ldg(tris + 4 * (size_t)j + 1),
                 vc = __ldg(tris + 4 * (size_t)j + 2);
    const float ax = __fmul_rn(va.x, sc), ay = __fmul_rn(va.y, sc), az = __fmul_rn(va.z, sc);
    const float bx = __fmul_rn(vb.x, sc), by = __fmul_rn(vb.y, sc), bz = __fmul_rn(vb.z, sc);
    const float cx = __fmul_rn(vc.x, sc), cy = __fmul_rn(vc.y, sc), cz = __fmul_rn(vc.z, sc);
    const float abx = __fsub_rn(bx, ax), aby = __fsub_rn(by, ay), abz = __fsub_rn(bz, az);
    const float acx = __fsub_rn(cx, ax), acy = __fsub_rn(cy, ay), acz = __fsub_rn(cz, az);
    const float nx = __fsub_rn(__fmul_rn(aby, acz), __fmul_rn(abz, acy));
    const float ny = __fsub_rn(__fmul_rn(abz, acx), __fmul_rn(abx, acz));
    const float nz = __fsub_rn(__fmul_rn(abx, acy), __fmul_rn(aby, acx));
    const float mag = __fsqrt_rn(dot3(nx, ny, nz, nx, ny, nz));
    geo[4 * (size_t)j] = make_float4(ax, ay, az, nx);
    geo[4 * (size_t)j + 1] = make_float4(bx, by, bz, ny);
    geo[4 * (size_t)j + 2] = make_float4(cx, cy, cz, nz);
    geo[4 * (size_t)j + 3] = make_float4(__fdiv_rn(nx, mag), __fdiv_rn(ny, mag), __fdiv_rn(nz, mag), 0.f);
    // widened box: boundary distance plus 1e-4 (bound + max |coordinate|),
    // far above the few-ulp error of the contact point and the distance
    float m = fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fabsf(az));
    m = fmaxf(m, fmaxf(fmaxf(fabsf(bx), fabsf(by)), fabsf(bz)));
    m = fmaxf(m, fmaxf(fmaxf(fabsf(cx), fabsf(cy)), fabsf(cz)));
    const float bound = fabsf(P.tri_bound);
    const float w = bound + 1e-4f * (bound + m);
    box[2 * (size_t)j] = make_float4(fminf(fminf(ax, bx), cx) - w, fminf(fminf(ay, by), cy) - w,
                                     fminf(fminf(az, bz), cz) - w, 0.f);
    box[2 * (size_t)j + 1] = make_float4(fmaxf(fmaxf(ax, bx), cx) + w, fmaxf(fmaxf(ay, by), cy) + w,
                                         fmaxf(fmaxf(az, bz), cz) + w, 0.f);
}

// tile[2t], tile[2t+1]: the union of the widened boxes of triangles
// [256t, 256t + 256), so that a block can pass over a whole tile.
__global__ void __launch_bounds__(256) k_tri_tiles(const float4* __restrict__ box, int ntri,
                                                   float4* __restrict__ tile) {
    __shared__ float s[6][8];
    const int j = blockIdx.x * 256 + threadIdx.x;
    float r[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    if (j < ntri) {
        const float4 lo = box[2 * (size_t)j], hi = box[2 * (size_t)j + 1];
        r[0] = lo.x; r[1] = lo.y; r[2] = lo.z; r[3] = hi.x; r[4] = hi.y; r[5] = hi.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) r[k] = fminf(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
#pragma unroll
        for (int k = 3; k < 6; ++k) r[k] = fmaxf(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
    }
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) s[k][threadIdx.x >> 5] = r[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w)
#pragma unroll
            for (int k = 0; k < 6; ++k) s[k][0] = k < 3 ? fminf(s[k][0], s[k][w]) : fmaxf(s[k][0], s[k][w]);
        tile[2 * (size_t)blockIdx.x] = make_float4(s[0][0], s[1][0], s[2][0], 0.f);
        tile[2 * (size_t)blockIdx.x + 1] = make_float4(s[3][0], s[4][0], s[5][0], 0.f);
    }
}

// Per-particle part of intersect_triangle_segment: the segment
// p = pos - v_hat d .. q = pos + v_hat d of half-length d = boundary
// distance along the velocity (collision_tri.cl:218-221).
struct Segment {
    float px, py, pz, qpx, qpy, qpz;
};

__device__ __forceinline__ Segment make_segment(float4 pos, float4 vel, float dist) {
    const float mag = __fsqrt_rn(dot3(vel.x, vel.y, vel.z, vel.x, vel.y, vel.z));
    const float vx = __fdiv_rn(vel.x, mag), vy = __fdiv_rn(vel.y, mag), vz = __fdiv_rn(vel.z, mag);
    Segment s;
    s.px = __fsub_rn(pos.x, __fmul_rn(vx, dist));
    s.py = __fsub_rn(pos.y, __fmul_rn(vy, dist));
    s.pz = __fsub_rn(pos.z, __fmul_rn(vz, dist));
    const float qx = __fadd_rn(pos.x, __fmul_rn(vx, dist));
    const float qy = __fadd_rn(pos.y, __fmul_rn(vy, dist));
    const float qz = __fadd_rn(pos.z, __fmul_rn(vz, dist));
    s.qpx = __fsub_rn(s.px, qx);
    s.qpy = __fsub_rn(s.py, qy);
    s.qpz = __fsub_rn(s.pz, qz);
    return s;
}

// The rest of intersect_triangle_segment (Ericson's segment-triangle test,
// :222-246) and the contact condition of collisions_triangle (:320-328):
// returns bound - |pos - tp| when it exceeds 1e-6, else 0.
__device__ __forceinline__ float contact_depth(float4 pos, const Segment& s, float4 g0, float4 g1, float4 g2,
                                               float bound) {
    const float nx = g0.w, ny = g1.w, nz = g2.w;
    const float d = dot3(s.qpx, s.qpy, s.qpz, nx, ny, nz);
    if (d <= 0.f) return 0.f;
    const float apx = __fsub_rn(s.px, g0.x), apy = __fsub_rn(s.py, g0.y), apz = __fsub_rn(s.pz, g0.z);
    const float t = dot3(apx, apy, apz, nx, ny, nz);
    if (t < 0.f || t > d) return 0.f;
    const float ex = __fsub_rn(__fmul_rn(s.qpy, apz), __fmul_rn(s.qpz, apy));
    const float ey = __fsub_rn(__fmul_rn(s.qpz, apx), __fmul_rn(s.qpx, apz));
    const float ez = __fsub_rn(__fmul_rn(s.qpx, apy), __fmul_rn(s.qpy, apx));
    const float acx = __fsub_rn(g2.x, g0.x), acy = __fsub_rn(g2.y, g0.y), acz = __fsub_rn(g2.z, g0.z);
    float v = dot3(acx, acy, acz, ex, ey, ez);
    if (v < 0.f || v > d) return 0.f;
    const float abx = __fsub_rn(g1.x, g0.x), aby = __fsub_rn(g1.y, g0.y), abz = __fsub_rn(g1.z, g0.z);
    float w = -dot3(abx, aby, abz, ex, ey, ez);
    if (w < 0.f || __fadd_rn(v, w) > d) return 0.f;
    const float ood = __fdiv_rn(1.0f, d);
    v = __fmul_rn(v, ood);
    w = __fmul_rn(w, ood);
    const float u = __fsub_rn(__fsub_rn(1.0f, v), w);
    const float tx = __fadd_rn(__fadd_rn(__fmul_rn(u, g0.x), __fmul_rn(v, g1.x)), __fmul_rn(w, g2.x));
    const float ty = __fadd_rn(__fadd_rn(__fmul_rn(u, g0.y), __fmul_rn(v, g1.y)), __fmul_rn(w, g2.y));
    const float tz = __fadd_rn(__fadd_rn(__fmul_rn(u, g0.z), __fmul_rn(v, g1.z)), __fmul_rn(w, g2.z));
    const float rx = __fsub_rn(pos.x, tx), ry = __fsub_rn(pos.y, ty), rz = __fsub_rn(pos.z, tz);
    const float dd = __fsub_rn(bound, __fsqrt_rn(dot3(rx, ry, rz, rx, ry, rz)));
    return dd > 1e-6f ? dd : 0.f;
}

// calculateRepulsionForce then calculateFrictionForce with zero coefficients
// (cl_sph_collision.h:31-73), added to f in that order (collision_tri.cl:
// 326-328).
__device__ __forceinline__ void add_contact(float4& f, float4 vel, float4 g3, float dd, const StepParams& P) {
    const float4 vv = make_float4(vel.x, vel.y, vel.z, 0.f);
    const float4 nh = make_float4(g3.x, g3.y, g3.z, 0.f);
    const float dn = v4dot(nh, vv);
    const float s = __fsub_rn(__fmul_rn(P.kwall, dd), __fmul_rn(P.cwall, dn));
    f.x = __fadd_rn(f.x, __fmul_rn(nh.x, s));
    f.y = __fadd_rn(f.y, __fmul_rn(nh.y, s));
    f.z = __fadd_rn(f.z, __fmul_rn(nh.z, s));
    const float4 vt = v4sub(vv, v4scale(vv, dn));
    const float mean = __fdiv_rn(__fadd_rn(__fadd_rn(vt.x, vt.y), vt.z), 3.0f);
    const float4 neg = make_float4(-vt.x, -vt.y, -vt.z, -vt.w);
    const float4 fr = mean > 0.f ? neg : v4scale(neg, 0.f);
    f.x = __fadd_rn(f.x, fr.x);
    f.y = __fadd_rn(f.y, fr.y);
    f.z = __fadd_rn(f.z, fr.z);
}

__device__ __forceinline__ bool box_holds(float4 lo, float4 hi, float4 p) {
    return p.x >= lo.x && p.x <= hi.x && p.y >= lo.y && p.y <= hi.y && p.z >= lo.z && p.z <= hi.z;
}

// The rest of the step after the force pass, when the kernel ends it (Step):
// sorted xsph and sort_indices in, the integrated state out.  After an
// out-of-grid deletion the kept particles are re-indexed in sorted order
// (sort_indices becomes the identity), as in the fused force pass.
struct TriStepTail {
    const float4* xsph_s;
    uint32_t* idx;
    float4* pos_u;
    float4* vel_u;
    float4* veleval_u;
    float dt;
};

// Step = false: the stage (force_s holds the force after the walls; it gets
// the triangle contacts added).  Step = true: the end of the step with a
// mesh: per particle, the force pass's output plus the point sources and the
// walls (gravity.cl, collision_wall.cl), the triangle contacts, then the
// integrator (leapfrog.cl or euler.cl) scattered to the unsorted state: the
// same operations as those staged kernels, in one pass over the particles.
template <bool Step, bool Exact>
__global__ void __launch_bounds__(kTriThreads) k_triangles(const float4* __restrict__ pos_s,
                                                           const float4* __restrict__ vel_s,
                                                           float4* __restrict__ force_s, const int* __restrict__ info,
                                                           const float4* __restrict__ geo,
                                                           const float4* __restrict__ box,
                                                           const float4* __restrict__ tile_box, const StepParams P,
                                                           const TriStepTail S) {
    __shared__ int s_cand[kTriThreads];
    __shared__ int s_wcnt[kTriThreads / 32];
    __shared__ float s_red[6][kTriThreads / 32];
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    if ((int)(blockIdx.x * kTriThreads) >= n) return;  // uniform over the block
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int i = blockIdx.x * kTriThreads + tid;
    const bool valid = i < n;
    const int ntri = P.n_tri;
    const float bound = P.tri_bound;
    float4 pos = make_float4(0.f, 0.f, 0.f, 0.f), vel = pos, f0 = pos;
    if (valid) {
        const float4 raw = __ldg(pos_s + i);
        pos = scaled(raw, P);
        vel = __ldg(vel_s + i);
        f0 = force_s[i];
        if (Step) {
            if (P.n_grav > 0) f0 = gravity_add<Exact>(f0, raw, P);
            f0 = collide_walls(pos, vel, f0, P);
        }
    }
    // box of the block's particles (NaN coordinates drop out of fminf/fmaxf;
    // such a particle never makes contact)
    float r[6] = {valid ? pos.x : INFINITY, valid ? pos.y : INFINITY, valid ? pos.z : INFINITY,
                  valid ? pos.x : -INFINITY, valid ? pos.y : -INFINITY, valid ? pos.z : -INFINITY};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) r[k] = fminf(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
#pragma unroll
        for (int k = 3; k < 6; ++k) r[k] = fmaxf(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
    }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) s_red[k][warp] = r[k];
    __syncthreads();
    float4 blo = make_float4(INFINITY, INFINITY, INFINITY, 0.f), bhi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
#pragma unroll
    for (int w = 0; w < kTriThreads / 32; ++w) {
        blo.x = fminf(blo.x, s_red[0][w]);
        blo.y = fminf(blo.y, s_red[1][w]);
        blo.z = fminf(blo.z, s_red[2][w]);
        bhi.x = fmaxf(bhi.x, s_red[3][w]);
        bhi.y = fmaxf(bhi.y, s_red[4][w]);
        bhi.z = fmaxf(bhi.z, s_red[5][w]);
    }
    const Segment seg = make_segment(pos, vel, bound);
    float4 f = make_float4(0.f, 0.f, 0.f, 0.f), rf = f;
    int chunk = 0;
    for (int t0 = 0; t0 < ntri; t0 += kTriThreads) {
        {  // a tile whose union box misses the block's box has no candidate
            const float4 lo = __ldg(tile_box + 2 * (size_t)(t0 / kTriThreads));
            const float4 hi = __ldg(tile_box + 2 * (size_t)(t0 / kTriThreads) + 1);
            if (!(lo.x <= bhi.x && hi.x >= blo.x && lo.y <= bhi.y && hi.y >= blo.y && lo.z <= bhi.z &&
                  hi.z >= blo.z))
                continue;  // the same for every thread of the block
        }
        // candidates of this tile, in triangle order
        const int j = t0 + tid;
        bool cand = false;
        if (j < ntri) {
            const float4 lo = __ldg(box + 2 * (size_t)j), hi = __ldg(box + 2 * (size_t)j + 1);
            cand = lo.x <= bhi.x && hi.x >= blo.x && lo.y <= bhi.y && hi.y >= blo.y && lo.z <= bhi.z &&
                   hi.z >= blo.z;
        }
        const unsigned m = __ballot_sync(0xffffffffu, cand);
        if (lane == 0) s_wcnt[warp] = __popc(m);
        __syncthreads();
        int off = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kTriThreads / 32; ++w) {
            const int c = s_wcnt[w];
            off += w < warp ? c : 0;
            total += c;
        }
        if (cand) s_cand[off + __popc(m & ((1u << lane) - 1u))] = j;
        __syncthreads();
        for (int k = 0; k < total; ++k) {
            const int jj = s_cand[k];
            const int ck = jj / kTriChunk;
            if (ck != chunk) {  // same for every thread of the block
                rf = v4add(rf, f);
                f = make_float4(0.f, 0.f, 0.f, 0.f);
                chunk = ck;
            }
            if (!valid || !box_holds(__ldg(box + 2 * (size_t)jj), __ldg(box + 2 * (size_t)jj + 1), pos)) continue;
            const float4 g0 = __ldg(geo + 4 * (size_t)jj), g1 = __ldg(geo + 4 * (size_t)jj + 1),
                         g2 = __ldg(geo + 4 * (size_t)jj + 2);
            const float dd = contact_depth(pos, seg, g0, g1, g2, bound);
            if (dd > 0.f) add_contact(f, vel, __ldg(geo + 4 * (size_t)jj + 3), dd, P);
        }
        __syncthreads();  // s_cand and s_wcnt are rewritten by the next tile
    }
    rf = v4add(rf, f);
    if (!valid) return;
    // rf.w: each group adds its triangle count, an exact integer sum
    const float4 ff = make_float4(__fadd_rn(f0.x, rf.x), __fadd_rn(f0.y, rf.y), __fadd_rn(f0.z, rf.z),
                                  __fadd_rn(f0.w, (float)ntri));
    if (!Step) {
        force_s[i] = ff;
        return;
    }
    uint32_t o;
    if (out >= 0) {
        o = (uint32_t)i;
        S.idx[i] = o;
    } else {
        o = S.idx[i];
    }
    if (!in_bounds(o, P.chk_cap, P.chk_err)) return;
    float4 po, vo, eo;
    if (P.integrator == kIntegratorEuler) {
        euler_core(pos, vel, ff, S.dt, P, po, vo);
        S.vel_u[o] = vo;
        S.pos_u[o] = po;
        return;
    }
    leapfrog_core(pos, vel, ff, __ldg(S.xsph_s + i), S.dt, P, po, vo, eo);
    S.vel_u[o] = vo;
    S.veleval_u[o] = eo;
    S.pos_u[o] = po;
}

}  // namespace

void launch_triangles(const float4* pos_s, const float4* vel_s, float4* force_s, const int* info, const StepParams& p,
                      int grid_items, cudaStream_t st) {
    if (p.n_tri <= 0) return;
    k_tri_prep<<<(p.n_tri + 255) / 256, 256, 0, st>>>(p.tri_raw, p.n_tri, p.tri_geo, p.tri_box, p);
    k_tri_tiles<<<(p.n_tri + 255) / 256, 256, 0, st>>>(p.tri_box, p.n_tri, p.tri_tile);
    int blocks = (grid_items + kTriThreads - 1) / kTriThreads;
    if (blocks < 1) blocks = 1;
    k_triangles<false, false><<<blocks, kTriThreads, 0, st>>>(pos_s, vel_s, force_s, info, p.tri_geo, p.tri_box,
                                                              p.tri_tile, p, TriStepTail{});
}

void launch_triangles_step(const float4* pos_s, const float4* vel_s, const float4* force_s, const float4* xsph_s,
                           uint32_t* idx, float4* pos_u, float4* vel_u, float4* veleval_u, const int* info,
                           const StepParams& p, float dt, int grid_items, cudaStream_t st) {
    if (p.n_tri <= 0) return;
    k_tri_prep<<<(p.n_tri + 255) / 256, 256, 0, st>>>(p.tri_raw, p.n_tri, p.tri_geo, p.tri_box, p);
    k_tri_tiles<<<(p.n_tri + 255) / 256, 256, 0, st>>>(p.tri_box, p.n_tri, p.tri_tile);
    int blocks = (grid_items + kTriThreads - 1) / kTriThreads;
    if (blocks < 1) blocks = 1;
    const TriStepTail S{xsph_s, idx, pos_u, vel_u, veleval_u, dt};
    float4* f = const_cast<float4*>(force_s);  // only read when Step
    if (p.exact)
        k_triangles<true, true><<<blocks, kTriThreads, 0, st>>>(pos_s, vel_s, f, info, p.tri_geo, p.tri_box,
                                                                p.tri_tile, p, S);
    else
        k_triangles<true, false><<<blocks, kTriThreads, 0, st>>>(pos_s, vel_s, f, info, p.tri_geo, p.tri_box,
                                                                 p.tri_tile, p, S);
}

}  // namespace sphk
