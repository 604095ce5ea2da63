// sph_adjoint.cu — the differentiable rollout: reverse-mode gradients of a
// loss of the final particle state with respect to the initial state and the
// viscosity coefficient, through hand-written adjoints of the step's density,
// force, wall collision and leapfrog stages.
//
// Forward step (one fused step, sorted index i, o = sort_indices[i]; the
// reference formulas of density.cl:44-126, force.cl:43-186,
// collision_wall.cl:31-118 and leapfrog.cl:30-121):
//   rho_i = Dc * sum_{j in N(i) + i} w(q_ij),   w(q) = (h^2 - q)^3, q = |p_i - p_j|^2
//   F_i = sum_j d_ij phi(q) (P_i + P_j) / rho_j,   phi = (h - r)^2 / r,  P = K (rho - rho0)
//   V_i = sum_j (e_j - e_i) (h - r) / rho_j
//   X_i = sum_j w(q) (e_j - e_i) / (rho_i + rho_j)
//   f_i = (m / rho_i) (cb F_i + mu cv V_i) + walls(p_i, v_i),   xs_i = cd X_i
//   g = clamp(f_i + gravity),  vn = v_i + dt g + xf xs_i,  e' = (v_i + vn) / 2,  p' = p_i + dt vn
// with p the scaled position, e the veleval velocity, mu the viscosity.
// Sorting and hashing are piecewise constant and are not differentiated:
// each reverse step reuses the forward step's permutation, cell ranges,
// neighbour bitmask and per-particle records.
//
// Reverse step, three kernels:
//   A  per particle: leapfrog, acceleration clamp and walls; gives the
//      adjoint of the step's input velocity, a_i = (m / rho_i) * fbar_i (the
//      force adjoint seen by the pair sums), the XSPH sum adjoint and the
//      density adjoint of the m / rho_i factor.
//   B  neighbour gather: pressure, viscosity and XSPH pair terms.  Each
//      thread accumulates both its own (i-side) terms and the terms its
//      neighbours' sums contribute to it (j-side), so nothing is scattered:
//      no atomics.  Gives the veleval adjoint, the complete density adjoint
//      and the viscosity gradient.
//   C  neighbour gather: the density sum's position terms, with both
//      particles' density adjoints; completes the position adjoint.
//
// Memory: the state (pos, vel, veleval) is checkpointed every K steps during
// the recorded forward run.  The backward pass recomputes one segment of K
// steps at a time from its checkpoint with the unchanged forward kernels,
// which write their per-step records straight into a K-slot tape, then
// reverses the segment.  Tape per step: sort_indices, cell start/end, the
// (position, rho) and (veleval, 1/rho) records, the neighbour bitmask, the
// pre-wall force and the input velocity: 132 B per particle + 8 B per cell.
// The whole backward pass is one CUDA graph.
//
// Batches (sph_batch_adjoint_*) run the same kernels over every scene of a
// batch at once: the scene of a sorted particle comes from its tape key, the
// viscosity gradient is accumulated per scene.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "sph_batch.cuh"
#include "sph_ctx.cuh"
#include "sph_walk.cuh"

using sphk::StepParams;

namespace {

constexpr int kAdjThreads = 128;

struct TapeStep {
    const uint32_t* idx;
    const uint32_t* keys;  // sort keys (batches: the scene of each sorted particle)
    const uint32_t* cs;
    const uint32_t* ce;
    const float4* rec_pd;  // (scaled position, rho)
    const float4* rec_vi;  // (veleval, 1/rho)
    const uint32_t* mask;
    const float4* fsph;    // SPH force before the walls
    const float4* vin;     // velocity the step integrated
};

__device__ __forceinline__ float3 xyz(const float4& v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// ---------------------------------------------------------------------------
// A: leapfrog, clamp and walls, per sorted particle.
//
// Walls: for an active wall with normal n (diff > EPSILON) the repulsion
// n (k diff - c n.v) has d/dp = -k n n^T and d/dv = -c n n^T; the "friction"
// -v_t = -v + v (n.v), taken when mean(v_t) > 0, has d/dv = (n.v - 1) I + v n^T.
// The branch tests repeat the forward arithmetic operation by operation.
__device__ __forceinline__ void wall_adjoint(float diff, float4 n, float4 v, float3 fb, const StepParams& P,
                                             float3& pb, float3& vb) {
    if (!(diff > P.eps)) return;
    const float3 nn = xyz(n);
    const float nf = dot(nn, fb);
    pb = pb - (P.kwall * nf) * nn;
    vb = vb - (P.cwall * nf) * nn;
    float4 vv = v;
    vv.w = 0.f;
    const float s = sphk::v4dot(n, vv);
    const float4 vt = sphk::v4sub(vv, sphk::v4scale(vv, s));
    const float mean = __fdiv_rn(__fadd_rn(__fadd_rn(vt.x, vt.y), vt.z), 3.0f);
    if (mean > 0.f) vb = vb + (s - 1.f) * fb + dot(xyz(vv), fb) * nn;
}

template <class Scenes>
__global__ void __launch_bounds__(256) k_adj_integrate(int n, const Scenes R, float dt, TapeStep T,
                                                       const float4* __restrict__ xb_out,
                                                       const float4* __restrict__ vb_out,
                                                       const float4* __restrict__ eb_out, float4* __restrict__ vb_in,
                                                       float4* __restrict__ adj_a, float4* __restrict__ adj_x,
                                                       float4* __restrict__ pbar) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const StepParams& P = R.params(i);
    const uint32_t o = __ldg(T.idx + i);
    const float isc = P.unit_scale ? 1.f : 1.f / P.sc;
    const float3 pbn = isc * xyz(__ldg(xb_out + o));  // adjoint of p' = p + dt vn
    const float3 vbo = xyz(__ldg(vb_out + o));
    const float3 ebo = xyz(__ldg(eb_out + o));
    const float3 vnb = vbo + dt * pbn + 0.5f * ebo;  // adjoint of vn
    float3 pb = pbn;
    float3 vb = 0.5f * ebo + vnb;
    float3 gb = dt * vnb;
    const float4 pd = __ldg(T.rec_pd + i);
    const float4 p4 = make_float4(pd.x, pd.y, pd.z, pd.w);
    const float4 v = __ldg(T.vin + i);
    const float4 fs = __ldg(T.fsph + i);
    // the forward's total force, bit for bit, for the clamp test
    float4 g = sphk::collide_walls(p4, v, fs, P);
    g = sphk::v4add(g, P.gravity);
    g.w = 0.f;
    const float speed = __fsqrt_rn(sphk::v4dot(g, g));
    if (speed > P.vlimit) {
        // g' = L g / |g|:  dg'/dg = (L / |g|) (I - u u^T), u = g / |g|
        const float3 u = (1.f / speed) * xyz(g);
        gb = (P.vlimit / speed) * (gb - dot(u, gb) * u);
    }
    const float3 fb = gb;
    wall_adjoint(__fsub_rn(P.bound, __fsub_rn(p4.z, P.gs_bnd_min.z)), make_float4(0.f, 0.f, 1.f, 0.f), v, fb, P, pb,
                 vb);
    wall_adjoint(__fsub_rn(P.bound, __fsub_rn(P.gs_bnd_max.z, p4.z)), make_float4(0.f, 0.f, -1.f, 0.f), v, fb, P, pb,
                 vb);
    wall_adjoint(__fsub_rn(P.bound, __fsub_rn(p4.y, P.gs_bnd_min.y)), make_float4(0.f, 1.f, 0.f, 0.f), v, fb, P, pb,
                 vb);
    wall_adjoint(__fsub_rn(P.bound, __fsub_rn(P.gs_bnd_max.y, p4.y)), make_float4(0.f, -1.f, 0.f, 0.f), v, fb, P, pb,
                 vb);
    wall_adjoint(__fsub_rn(P.bound, __fsub_rn(p4.x, P.gs_bnd_min.x)), make_float4(1.f, 0.f, 0.f, 0.f), v, fb, P, pb,
                 vb);
    wall_adjoint(__fsub_rn(P.bound, __fsub_rn(P.gs_bnd_max.x, p4.x)), make_float4(-1.f, 0.f, 0.f, 0.f), v, fb, P, pb,
                 vb);
    const float rho = pd.w;
    const float A = P.mass * __ldg(T.rec_vi + i).w;
    // f_sph = A * (...):  rho enters through A = m / rho
    const float rhob_a = -dot(fb, xyz(fs)) / rho;
    const float3 a = A * fb;
    const float3 xb = (P.coef_d * P.xsph_factor) * vnb;
    adj_a[i] = make_float4(a.x, a.y, a.z, rhob_a);
    adj_x[i] = make_float4(xb.x, xb.y, xb.z, 0.f);
    pbar[i] = make_float4(pb.x, pb.y, pb.z, 0.f);
    vb_in[o] = make_float4(vb.x, vb.y, vb.z, 0.f);
}

// ---------------------------------------------------------------------------
// Neighbours of sorted particle i as the forward density pass recorded them:
// the bitmask over the first kMaskBits candidates in walk order, the rest
// tested again.  When every lane's candidates fit the bitmask each lane runs
// through its own set bits; otherwise lanes advance in lock step, one
// neighbour each per iteration, with a vote per iteration; fn(j) runs for
// each j != i, in walk order either way.
// Particles outside the integer-hash range walk the 27 cells directly.
template <class Fn>
__device__ __forceinline__ void for_each_neighbour(const StepParams& P, const uint32_t* cs, const uint32_t* ce,
                                                   const TapeStep& T, size_t mstride, int i, const float4& pi,
                                                   unsigned wmask, uint32_t (*s_rs)[kAdjThreads],
                                                   uint32_t (*s_off)[kAdjThreads], Fn&& fn) {
    const int t = threadIdx.x;
    const float rc2 = P.rcut2;
    int nrows = 0;
    uint32_t M = 0;
    const int3 c = sphk::grid_cell(pi.x, pi.y, pi.z, P.gs_min, P.gs_delta);
    if (sphk::cell_fast(P, c)) {
        sphk::walk_rows_fast_batched(P, cs, ce, c, [&](uint32_t rs, uint32_t re) {
            s_rs[nrows][t] = rs - M;  // sorted index minus walk position over the run
            s_off[nrows][t] = M;
            M += re - rs;
            ++nrows;
        });
    } else {
        sphk::walk_rows_slow(P, cs, ce, c, [&](uint32_t rs, uint32_t re) {
            for (uint32_t j = rs; j < re; ++j) {
                const float4 pj = __ldg(T.rec_pd + j);
                const float r2 = sphk::dist2_exact(__fsub_rn(pi.x, pj.x), __fsub_rn(pi.y, pj.y), __fsub_rn(pi.z, pj.z));
                if (r2 <= rc2 && j != (uint32_t)i) fn(j);
            }
        });
    }
    s_off[nrows][t] = M;
    const uint32_t* mrow = T.mask + i;
    const uint32_t mbits = M < (uint32_t)sphk::kMaskBits ? M : (uint32_t)sphk::kMaskBits;
    // wb: walk position of the current word's bit 0; mnext: the word after it
    uint32_t wb = 0, m = (mbits > 0) ? __ldg(mrow) : 0u;
    const uint32_t* mnext = mrow + mstride;
    // the next mask word, in flight while this one's neighbours are processed
    uint32_t m_next = (mbits > 32u) ? __ldg(mrow + mstride) : 0u;
    uint32_t q = (uint32_t)sphk::kMaskBits;
    int r = 0;
    uint32_t next_off = s_off[1][t], delta = s_rs[0][t];  // row r's end and index offset
    if (!__any_sync(wmask, M > (uint32_t)sphk::kMaskBits)) {
        // Every lane's candidates fit the bitmask: each lane runs through its
        // own set bits, with no vote per neighbour.
        for (;;) {
            while (m == 0 && wb + 32u < mbits) {
                wb += 32u;
                m = m_next;
                mnext += mstride;
                m_next = (wb + 32u < mbits) ? __ldg(mnext) : 0u;
            }
            if (m == 0) return;
            const uint32_t p = wb + (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
            while (p >= next_off) {
                ++r;
                next_off = s_off[r + 1][t];
                delta = s_rs[r][t];
            }
            fn(p + delta);
        }
    }
    for (;;) {
        bool have = false;
        uint32_t p = 0;
        while (m == 0 && wb + 32u < mbits) {
            wb += 32u;
            m = m_next;
            mnext += mstride;
            m_next = (wb + 32u < mbits) ? __ldg(mnext) : 0u;
        }
        if (m != 0) {
            p = wb + (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
            have = true;
        } else {
            while (q < M) {
                const uint32_t pp = q++;
                while (pp >= next_off) {
                    ++r;
                    next_off = s_off[r + 1][t];
                    delta = s_rs[r][t];
                }
                const uint32_t j = pp + delta;
                const float4 pj = __ldg(T.rec_pd + j);
                const float r2 = sphk::dist2_exact(__fsub_rn(pi.x, pj.x), __fsub_rn(pi.y, pj.y), __fsub_rn(pi.z, pj.z));
                if (r2 <= rc2 && j != (uint32_t)i) {
                    p = pp;
                    have = true;
                    break;
                }
            }
        }
        if (!__any_sync(wmask, have)) break;
        if (have) {
            while (p >= next_off) {
                ++r;
                next_off = s_off[r + 1][t];
                delta = s_rs[r][t];
            }
            fn(p + delta);
        }
    }
}

// acc[scene] += v over the warp: one atomic per warp when all its lanes
// belong to one scene, one per lane otherwise (warps at scene boundaries).
// Every lane of the warp calls it; lanes without a value pass scene ~0u.
// The warp sum is formed in double, so that the result does not depend on
// how a scene's particles fall onto warps beyond double rounding.
__device__ __forceinline__ void warp_add_double(double* acc, uint32_t scene, float v) {
    const unsigned peers = __match_any_sync(0xffffffffu, scene);
    if (peers == 0xffffffffu) {
        double d = (double)v;
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) d += __shfl_xor_sync(0xffffffffu, d, s);
        if ((threadIdx.x & 31) == 0 && d != 0.0 && scene != ~0u) atomicAdd(acc + scene, d);
    } else if (scene != ~0u && v != 0.f) {
        atomicAdd(acc + scene, (double)v);
    }
}

// ---------------------------------------------------------------------------
// B: pressure, viscosity and XSPH pair terms.  Thread k, neighbour j,
// d = p_k - p_j, r = max(|d|, EPSILON):
//   d phi / d d = psi d,   psi = -(h - r)(h + r) / r^3   (0 when clamped)
//   d r / d d   = d / r                                  (0 when clamped)
//   d w / d d   = -6 (h^2 - q)^2 d
// i-side: the derivatives of k's own sums F_k, V_k, X_k (adjoints cb a_k,
// mu cv a_k, xbar_k) with respect to p_k, e_k and rho_k; j-side: those of
// j's sums with respect to the same variables of k.
template <class Scenes>
__global__ void __launch_bounds__(kAdjThreads) k_adj_force(int n, const Scenes R, TapeStep T, size_t mstride,
                                                           const float4* __restrict__ adj_a,
                                                           const float4* __restrict__ adj_x,
                                                           float4* __restrict__ pbar, float* __restrict__ rhob_out,
                                                           float4* __restrict__ eb_in, double* __restrict__ visc_acc) {
    __shared__ uint32_t s_rs[9][kAdjThreads];
    __shared__ uint32_t s_off[10][kAdjThreads];
    const int k = blockIdx.x * kAdjThreads + threadIdx.x;
    const bool live = k < n;
    const unsigned wmask = __ballot_sync(0xffffffffu, live);
    float visc_part = 0.f;
    uint32_t scene = ~0u;
    if (live) {
        const StepParams& P = R.params(k);
        scene = R.scene(k);
        const uint32_t* cell_s = T.cs + R.cell_base(k);
        const uint32_t* cell_e = T.ce + R.cell_base(k);
        const float4 pk = __ldg(T.rec_pd + k);
        const float4 vk = __ldg(T.rec_vi + k);
        const float4 ak4 = __ldg(adj_a + k);
        const float3 ak = xyz(ak4), xk = xyz(__ldg(adj_x + k)), ek = xyz(vk);
        const float dk = pk.w, idk = vk.w;
        const float Pk = P.K * (dk - P.rho0);
        const float cb = P.coef_b, cs = P.coef_s;
        float3 pb = make_float3(0.f, 0.f, 0.f), eb = pb, Vs = pb;
        float rhob = 0.f;
        for_each_neighbour(P, cell_s, cell_e, T, mstride, k, pk, wmask, s_rs, s_off, [&](uint32_t j) {
            const float4 pj = __ldg(T.rec_pd + j);
            const float4 vj = __ldg(T.rec_vi + j);
            const float3 aj = xyz(__ldg(adj_a + j)), xj = xyz(__ldg(adj_x + j));
            const float3 d = make_float3(pk.x - pj.x, pk.y - pj.y, pk.z - pj.z);
            const float q = dot(d, d);
            const float rt = sqrtf(q);
            const bool clamped = !(rt >= P.eps);
            const float rr = clamped ? P.eps : rt;
            const float ir = 1.f / rr;
            const float hr = P.h - rr;
            const float hq = P.h2 - q;
            const float w = hq * hq * hq;
            const float wd = -6.f * hq * hq;
            const float phi = hr * hr * ir;
            const float psi = clamped ? 0.f : -hr * (P.h + rr) * ir * ir * ir;
            const float gr = clamped ? 0.f : ir;
            const float dj = pj.w, idj = vj.w;
            const float Pj = P.K * (dj - P.rho0);
            const float isum = 1.f / (dk + dj);
            const float3 de = xyz(vj) - ek;
            const float skj = (Pk + Pj) * idj, sjk = (Pj + Pk) * idk;
            const float cFk = cb * dot(ak, d), cFj = cb * dot(aj, d);
            const float cVk = cs * dot(ak, de), cVj = cs * dot(aj, de);
            const float cXk = dot(xk, de), cXj = dot(xj, de);
            // positions
            const float sd = psi * (skj * cFk - sjk * cFj) + gr * (cVj * idk - cVk * idj) + wd * isum * (cXk - cXj);
            pb = pb + sd * d + (phi * cb) * (skj * ak - sjk * aj);
            // veleval
            eb = eb + (hr * idk * cs) * aj - (hr * idj * cs) * ak + (w * isum) * (xj - xk);
            // density
            rhob += P.K * phi * idj * cFk + phi * cFj * idk * ((Pj + Pk) * idk - P.K) + hr * cVj * idk * idk +
                    w * isum * isum * (cXj - cXk);
            Vs = Vs + (hr * idj) * de;
        });
        const float4 p0 = pbar[k];
        pbar[k] = make_float4(p0.x + pb.x, p0.y + pb.y, p0.z + pb.z, 0.f);
        rhob_out[k] = ak4.w + rhob;
        eb_in[__ldg(T.idx + k)] = make_float4(eb.x, eb.y, eb.z, 0.f);
        visc_part = P.wvisc_dd * dot(ak, Vs);
    }
    warp_add_double(visc_acc, scene, visc_part);
}

// ---------------------------------------------------------------------------
// C: density position terms.  rho_k and rho_j both hold w(|p_k - p_j|^2):
// pbar_k += Dc * (-6 (h^2 - q)^2) * (rhobar_k + rhobar_j) * d.
template <class Scenes>
__global__ void __launch_bounds__(kAdjThreads) k_adj_density(int n, const Scenes R, TapeStep T, size_t mstride,
                                                             const float* __restrict__ rhob,
                                                             const float4* __restrict__ pbar,
                                                             float4* __restrict__ xb_in) {
    __shared__ uint32_t s_rs[9][kAdjThreads];
    __shared__ uint32_t s_off[10][kAdjThreads];
    const int k = blockIdx.x * kAdjThreads + threadIdx.x;
    const bool live = k < n;
    const unsigned wmask = __ballot_sync(0xffffffffu, live);
    if (!live) return;
    const StepParams& P = R.params(k);
    const uint32_t* cs = T.cs + R.cell_base(k);
    const uint32_t* ce = T.ce + R.cell_base(k);
    const float4 pk = __ldg(T.rec_pd + k);
    const float rk = __ldg(rhob + k);
    float3 pb = make_float3(0.f, 0.f, 0.f);
    for_each_neighbour(P, cs, ce, T, mstride, k, pk, wmask, s_rs, s_off, [&](uint32_t j) {
        const float4 pj = __ldg(T.rec_pd + j);
        const float3 d = make_float3(pk.x - pj.x, pk.y - pj.y, pk.z - pj.z);
        const float hq = P.h2 - dot(d, d);
        pb = pb + (-6.f * hq * hq * (rk + __ldg(rhob + j))) * d;
    });
    const float4 p0 = pbar[k];
    const float s = P.unit_scale ? 1.f : P.sc;
    const float3 x = s * (xyz(p0) + P.dens_coef * pb);
    xb_in[__ldg(T.idx + k)] = make_float4(x.x, x.y, x.z, 0.f);
}

// ---------------------------------------------------------------------------
// Distance loss of positions against targets, per scene, summed in FP64:
//   L_s = (w/N_s) sum_{i in s} rho(|x_i - x*_i|)
// with rho(d) = d^2 (mean squared distance, delta = 0) or the Huber function
// rho(d) = d^2 for d <= delta, 2 delta d - delta^2 beyond, delta = huber * h_s
// (h_s the scene's smoothing distance).  The gradient goes to grad; slots past
// a scene's particle count get a zero gradient.
__global__ void __launch_bounds__(256) k_loss_mse(const float4* __restrict__ pos, const float4* __restrict__ target,
                                                  float4* __restrict__ grad, int nslots,
                                                  const uint16_t* __restrict__ scene_of,
                                                  const uint32_t* __restrict__ slot_off,
                                                  const int* __restrict__ num, int n_single, float weight,
                                                  const StepParams* __restrict__ table, float huber,
                                                  double* __restrict__ loss) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t scene = ~0u;
    float v = 0.f;
    if (t < nslots) {
        const uint32_t s = scene_of ? scene_of[t] : 0u;
        const int cnt = scene_of ? num[s] : n_single;
        const bool valid = scene_of ? (int)(t - slot_off[s]) < cnt : t < n_single;
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid) {
            const float4 x = __ldg(pos + t), y = __ldg(target + t);
            const float dx = x.x - y.x, dy = x.y - y.y, dz = x.z - y.z;
            const float inv = weight / (float)cnt;
            const double d2 = (double)dx * dx + (double)dy * dy + (double)dz * dz;
            const float delta = huber > 0.f ? huber * table[s].h : 0.f;
            float gs = 2.f * inv;  // d rho / d x = gs * (x - x*)
            double r = d2;
            if (delta > 0.f && d2 > (double)delta * delta) {
                const double d = sqrt(d2);
                r = 2.0 * delta * d - (double)delta * delta;
                gs = (float)(2.0 * delta / d) * inv;
            }
            g = make_float4(gs * dx, gs * dy, gs * dz, 0.f);
            scene = s;
            // the per-particle term rounded once; the sum is in double
            v = (float)(r * (double)weight / (double)cnt);
        }
        grad[t] = g;
    }
    warp_add_double(loss, scene, v);
}

// x += seed (the loss gradient at an intermediate time), xyz lanes.
__global__ void __launch_bounds__(256) k_add_seed(float4* __restrict__ x, const float4* __restrict__ seed, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = x[i], b = __ldg(seed + i);
    x[i] = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, 0.f);
}

}  // namespace

// ---------------------------------------------------------------------------
// Recorded rollout and adjoint buffers of a context or a batch.
struct AdjState {
    int recorded = 0;
    int nsteps = 0, K = 0, n = 0, exact = 0;
    float dt = 0.f;
    unsigned params_version = 0;
    // slot capacity, cell-array stride (the cell entries rounded up to 4
    // words so that every slot's cell arrays start 16-byte aligned for the
    // 128-bit accesses of the sort's scan), state elements checkpointed
    size_t N = 0, C1 = 0, state_elems = 0;
    int nscenes = 1;
    bool tape_keys = false;
    int cap_K = 0, cap_ckpt = 0;
    float4* ckpt = nullptr;  // [cap_ckpt][3][N]: pos, vel, veleval at steps 0, K, 2K, ..., then the final state
    float4* seeds = nullptr; // [cap_seeds][N]: position-loss gradients at the checkpoint times
    int cap_seeds = 0;
    uint32_t *t_idx = nullptr, *t_keys = nullptr, *t_cs = nullptr, *t_ce = nullptr, *t_mask = nullptr;
    float4 *t_pd = nullptr, *t_vi = nullptr, *t_f = nullptr, *t_v = nullptr;
    float4* xb[2] = {nullptr, nullptr};
    float4* vb[2] = {nullptr, nullptr};
    float4* eb[2] = {nullptr, nullptr};
    float4 *adj_a = nullptr, *adj_x = nullptr, *pbar = nullptr;
    float* rhob = nullptr;
    double* visc_acc = nullptr;   // [nscenes]
    double* host_visc = nullptr;  // [nscenes], pinned
    cudaGraphExec_t graph = nullptr;
    int g_nsteps = -1, g_K = -1, g_n = -1, g_exact = -1;
    float g_dt = 0.f;
    unsigned g_version = 0;
    cudaStream_t g_stream = nullptr;
    int g_seeded = -1;
};
struct sph_adjoint : AdjState {};
struct sph_batch_adjoint : AdjState {};

namespace {

void free_tape(AdjState* a) {
    void* ptrs[] = {a->t_idx, a->t_keys, a->t_cs, a->t_ce, a->t_pd, a->t_vi, a->t_mask, a->t_f, a->t_v};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    a->t_idx = a->t_keys = a->t_cs = a->t_ce = a->t_mask = nullptr;
    a->t_pd = a->t_vi = a->t_f = a->t_v = nullptr;
    a->cap_K = 0;
}

void drop_graph(AdjState* a) {
    if (a->graph) cudaGraphExecDestroy(a->graph);
    a->graph = nullptr;
}

void free_state(AdjState* a) {
    drop_graph(a);
    free_tape(a);
    void* ptrs[] = {a->ckpt, a->xb[0], a->xb[1], a->vb[0], a->vb[1], a->eb[0], a->eb[1], a->adj_a, a->adj_x,
                    a->pbar, a->rhob, a->visc_acc, a->seeds};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (a->host_visc) cudaFreeHost(a->host_visc);
}

// Allocation of the adjoint buffers (once), the checkpoints (nckpt slots)
// and the tape (K slots); returns a cudaError_t.
cudaError_t ensure_buffers(AdjState* a, int K, int nckpt) {
    const size_t N = a->N, C1 = a->C1;
    cudaError_t e = cudaSuccess;
#define AL(ptr, bytes) \
    if (e == cudaSuccess) e = cudaMalloc((void**)&(ptr), (bytes))
    if (!a->xb[0]) {
        for (int s = 0; s < 2; ++s) {
            AL(a->xb[s], N * 16);
            AL(a->vb[s], N * 16);
            AL(a->eb[s], N * 16);
        }
        AL(a->adj_a, N * 16);
        AL(a->adj_x, N * 16);
        AL(a->pbar, N * 16);
        AL(a->rhob, N * 4);
        AL(a->visc_acc, sizeof(double) * a->nscenes);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&a->host_visc, sizeof(double) * a->nscenes);
        for (int s = 0; s < 2 && e == cudaSuccess; ++s) {
            e = cudaMemset(a->xb[s], 0, N * 16);
            if (e == cudaSuccess) e = cudaMemset(a->vb[s], 0, N * 16);
            if (e == cudaSuccess) e = cudaMemset(a->eb[s], 0, N * 16);
        }
        if (e != cudaSuccess) return e;
    }
    if (nckpt > a->cap_ckpt) {
        drop_graph(a);
        if (a->ckpt) cudaFree(a->ckpt);
        a->ckpt = nullptr;
        a->cap_ckpt = 0;
        AL(a->ckpt, (size_t)nckpt * 3 * N * 16);
        if (e != cudaSuccess) return e;
        a->cap_ckpt = nckpt;
    }
    if (K > a->cap_K) {
        drop_graph(a);
        free_tape(a);
        const size_t k = (size_t)K;
        AL(a->t_idx, k * N * 4);
        if (a->tape_keys) AL(a->t_keys, k * N * 4);
        AL(a->t_cs, k * C1 * 4);
        AL(a->t_ce, k * C1 * 4);
        AL(a->t_pd, k * N * 16);
        AL(a->t_vi, k * N * 16);
        AL(a->t_mask, k * N * 4 * sphk::kMaskWords);
        AL(a->t_f, k * N * 16);
        AL(a->t_v, k * N * 16);
        if (e != cudaSuccess) {
            free_tape(a);
            return e;
        }
        a->cap_K = K;
    }
#undef AL
    return cudaSuccess;
}

TapeStep tape_step(const AdjState* a, int slot) {
    const size_t N = a->N, C1 = a->C1, s = (size_t)slot;
    TapeStep T;
    T.idx = a->t_idx + s * N;
    T.keys = a->t_keys ? a->t_keys + s * N : nullptr;
    T.cs = a->t_cs + s * C1;
    T.ce = a->t_ce + s * C1;
    T.rec_pd = a->t_pd + s * N;
    T.rec_vi = a->t_vi + s * N;
    T.mask = a->t_mask + s * N * sphk::kMaskWords;
    T.fsph = a->t_f + s * N;
    T.vin = a->t_v + s * N;
    return T;
}

float4* ckpt_slot(const AdjState* a, int slot, int field) {
    return a->ckpt + ((size_t)slot * 3 + field) * a->N;
}

// Checkpoint `slot` <-> the state arrays (pos, vel, veleval).
cudaError_t copy_state(const AdjState* a, float4* const st[3], int slot, bool save, cudaStream_t stream) {
    const size_t b = a->state_elems * 16;
    for (int f = 0; f < 3; ++f) {
        float4* ck = ckpt_slot(a, slot, f);
        const cudaError_t e =
            cudaMemcpyAsync(save ? ck : st[f], save ? st[f] : ck, b, cudaMemcpyDeviceToDevice, stream);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <class Scenes>
void launch_reverse(const AdjState* a, const Scenes& R, const TapeStep& T, int src, cudaStream_t st) {
    const int n = a->n, dst = 1 - src;
    const size_t mstride = a->N;
    const int b256 = (n + 255) / 256, b128 = (n + kAdjThreads - 1) / kAdjThreads;
    k_adj_integrate<Scenes><<<b256, 256, 0, st>>>(n, R, a->dt, T, a->xb[src], a->vb[src], a->eb[src], a->vb[dst],
                                                  a->adj_a, a->adj_x, a->pbar);
    k_adj_force<Scenes><<<b128, kAdjThreads, 0, st>>>(n, R, T, mstride, a->adj_a, a->adj_x, a->pbar, a->rhob,
                                                      a->eb[dst], a->visc_acc);
    k_adj_density<Scenes><<<b128, kAdjThreads, 0, st>>>(n, R, T, mstride, a->rhob, a->pbar, a->xb[dst]);
}

// --- contexts ----------------------------------------------------------------
float4* const* ctx_state(sph_ctx* c, float4* st[3]) {
    st[0] = c->pos_u;
    st[1] = c->vel_u;
    st[2] = c->veleval_u;
    return st;
}

// One forward step whose records land in tape slot `slot`: the context's
// record buffers are pointed at the slot for the enqueue and restored after.
int ctx_taped_step(sph_ctx* c, int slot) {
    const TapeStep T = tape_step(c->adj, slot);
    float4 *rec_pd = c->rec_pd, *rec_vi = c->rec_vi;
    uint32_t *mask = c->mask, *cs = c->cell_start, *ce = c->cell_end, *idx_a = c->idx_a;
    c->rec_pd = const_cast<float4*>(T.rec_pd);
    c->rec_vi = const_cast<float4*>(T.rec_vi);
    c->mask = const_cast<uint32_t*>(T.mask);
    c->cell_start = const_cast<uint32_t*>(T.cs);
    c->cell_end = const_cast<uint32_t*>(T.ce);
    c->idx_a = const_cast<uint32_t*>(T.idx);
    c->keep_f = const_cast<float4*>(T.fsph);
    c->keep_v = const_cast<float4*>(T.vin);
    const int rc = enqueue_fused_step(c, c->adj->dt);
    c->rec_pd = rec_pd;
    c->rec_vi = rec_vi;
    c->mask = mask;
    c->cell_start = cs;
    c->cell_end = ce;
    c->idx_a = idx_a;
    c->keys_cur = c->keys_a;
    c->idx_cur = idx_a;
    c->keep_f = nullptr;
    c->keep_v = nullptr;
    return rc;
}

// --- batches -----------------------------------------------------------------
float4* const* batch_state(sph_batch* b, float4* st[3]) {
    st[0] = b->pos_u;
    st[1] = b->vel_u;
    st[2] = b->veleval_u;
    return st;
}

int batch_taped_step(sph_batch* b, int slot, float dt) {
    const TapeStep T = tape_step(b->adj, slot);
    float4 *rec_pd = b->rec_pd, *rec_vi = b->rec_vi;
    uint32_t *mask = b->mask, *cs = b->cell_start, *ce = b->cell_end, *idx_a = b->idx_a, *keys_a = b->keys_a;
    b->rec_pd = const_cast<float4*>(T.rec_pd);
    b->rec_vi = const_cast<float4*>(T.rec_vi);
    b->mask = const_cast<uint32_t*>(T.mask);
    b->cell_start = const_cast<uint32_t*>(T.cs);
    b->cell_end = const_cast<uint32_t*>(T.ce);
    b->idx_a = const_cast<uint32_t*>(T.idx);
    b->keys_a = const_cast<uint32_t*>(T.keys);
    b->keep_f = const_cast<float4*>(T.fsph);
    b->keep_v = const_cast<float4*>(T.vin);
    const int rc = batch_enqueue_step(b, dt);
    b->rec_pd = rec_pd;
    b->rec_vi = rec_vi;
    b->mask = mask;
    b->cell_start = cs;
    b->cell_end = ce;
    b->idx_a = idx_a;
    b->keys_a = keys_a;
    b->keep_f = nullptr;
    b->keep_v = nullptr;
    return rc;
}

// The whole backward pass: for each segment, last first, restore its
// checkpoint, recompute it into the tape, reverse it; then restore the final
// state.  Starts from the adjoints in buffers 0; ends in buffers nsteps % 2.
// Returns SPH_OK or the error of the first failing enqueue (set on the owner).
template <class Owner, class TapedStep, class Reverse>
int enqueue_backward(Owner* o, AdjState* a, float4* const st[3], cudaStream_t stream, bool seeded, TapedStep&& taped,
                     Reverse&& reverse, int (*fail)(Owner*, const char*, cudaError_t)) {
    const int T = a->nsteps, K = a->K;
    const int nseg = (T + K - 1) / K;
    int src = 0, rc;
    cudaError_t e;
    for (int s = nseg - 1; s >= 0; --s) {
        const int t0 = s * K, t1 = (t0 + K < T) ? t0 + K : T;
        if ((e = copy_state(a, st, s, false, stream)) != cudaSuccess) return fail(o, "checkpoint restore", e);
        for (int t = t0; t < t1; ++t)
            if ((rc = taped(t - t0))) return rc;
        for (int t = t1 - 1; t >= t0; --t) {
            reverse(tape_step(a, t - t0), src);
            src = 1 - src;
        }
        if (seeded) {
            // the loss gradient with respect to the positions at time t0
            const int n = (int)a->state_elems;
            k_add_seed<<<(n + 255) / 256, 256, 0, stream>>>(a->xb[src], a->seeds + (size_t)s * a->N, n);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(o, "reverse kernels", e);
    }
    if ((e = copy_state(a, st, nseg, false, stream)) != cudaSuccess) return fail(o, "state restore", e);
    return SPH_OK;
}

int ctx_fail(sph_ctx* c, const char* what, cudaError_t e) {
    return set_err(c, SPH_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}
int batch_fail(sph_batch* b, const char* what, cudaError_t e) {
    return berr(b, SPH_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

bool graph_stale(const AdjState* a, cudaStream_t stream, int seeded) {
    return !a->graph || a->g_nsteps != a->nsteps || a->g_K != a->K || a->g_n != a->n || a->g_exact != a->exact ||
           a->g_dt != a->dt || a->g_version != a->params_version || a->g_stream != stream || a->g_seeded != seeded;
}

void graph_key(AdjState* a, cudaStream_t stream, int seeded) {
    a->g_nsteps = a->nsteps;
    a->g_K = a->K;
    a->g_n = a->n;
    a->g_exact = a->exact;
    a->g_dt = a->dt;
    a->g_version = a->params_version;
    a->g_stream = stream;
    a->g_seeded = seeded;
}

// Loads the final-state adjoints (NULL: zero) into buffers 0 and clears the
// viscosity accumulators.
cudaError_t load_seeds(AdjState* a, const sph_float4* dpos, const sph_float4* dvel, const sph_float4* dveleval,
                       cudaStream_t st) {
    const size_t b = a->state_elems * 16;
    const sph_float4* src[3] = {dpos, dvel, dveleval};
    float4* dst[3] = {a->xb[0], a->vb[0], a->eb[0]};
    for (int f = 0; f < 3; ++f) {
        const cudaError_t e = src[f] ? cudaMemcpyAsync(dst[f], src[f], b, cudaMemcpyDeviceToDevice, st)
                                     : cudaMemsetAsync(dst[f], 0, b, st);
        if (e != cudaSuccess) return e;
    }
    return cudaMemsetAsync(a->visc_acc, 0, sizeof(double) * a->nscenes, st);
}

cudaError_t store_results(AdjState* a, sph_float4* dpos0, sph_float4* dvel0, sph_float4* dveleval0,
                          cudaStream_t st) {
    const size_t b = a->state_elems * 16;
    const int fin = a->nsteps & 1;
    sph_float4* dst[3] = {dpos0, dvel0, dveleval0};
    const float4* src[3] = {a->xb[fin], a->vb[fin], a->eb[fin]};
    for (int f = 0; f < 3; ++f) {
        if (!dst[f]) continue;
        const cudaError_t e = cudaMemcpyAsync(dst[f], src[f], b, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
    }
    return cudaMemcpyAsync(a->host_visc, a->visc_acc, sizeof(double) * a->nscenes, cudaMemcpyDeviceToHost, st);
}

int ctx_adj_check(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->adj || !c->adj->recorded)
        return set_err(c, SPH_ESTATE, "no recorded rollout: call sph_adjoint_record first");
    if (c->adj->params_version != c->params_version || c->adj->exact != c->exact)
        return set_err(c, SPH_ESTATE, "parameters changed since the rollout was recorded");
    return SPH_OK;
}

int batch_adj_check(sph_batch* b) {
    if (!b) return SPH_EINVAL;
    cudaSetDevice(b->device);
    if (!b->adj || !b->adj->recorded)
        return berr(b, SPH_ESTATE, "no recorded rollout: call sph_batch_adjoint_record first");
    if (b->adj->params_version != b->params_version || b->adj->exact != b->exact ||
        b->adj->n != b->nvalid)
        return berr(b, SPH_ESTATE, "parameters or particles changed since the rollout was recorded");
    return SPH_OK;
}

// The neighbour-pass counters into b->host_info, after sph_batch_sync has
// checked the sort's device error word.
int batch_read_info(sph_batch* b) {
    const int rc = sph_batch_sync(b);
    if (rc) return rc;
    BCK(b, cudaMemcpyAsync(b->host_info, b->info_nb, sizeof(int) * sphk::kInfoSlots, cudaMemcpyDeviceToHost,
                           b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    return SPH_OK;
}

}  // namespace

void sph_adjoint_release(sph_ctx* c) {
    if (!c || !c->adj) return;
    free_state(c->adj);
    delete c->adj;
    c->adj = nullptr;
}

void sph_batch_adjoint_release(sph_batch* b) {
    if (!b || !b->adj) return;
    free_state(b->adj);
    delete b->adj;
    b->adj = nullptr;
}

extern "C" {

int sph_adjoint_record(sph_ctx* c, float dt, int nsteps, int K) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (nsteps <= 0 || K <= 0 || !std::isfinite(dt))
        return set_err(c, SPH_EINVAL, "sph_adjoint_record: bad arguments (nsteps=%d, K=%d)", nsteps, K);
    if (!c->adj) {
        c->adj = new sph_adjoint();
        c->adj->N = (size_t)c->max_num;
        c->adj->C1 = ((size_t)c->gp.nb_cells + 1 + 3) & ~(size_t)3;
    }
    sph_adjoint* a = c->adj;
    a->recorded = 0;
    if (c->n_grav > 0 || c->n_tri > 0 || !c->hoses.empty() || c->integrator != sphk::kIntegratorLeapfrog)
        return set_err(c, SPH_ESTATE,
                       "the differentiable rollout covers the leapfrog step without point gravity sources, a "
                       "triangle mesh or hoses");
    if ((rc = read_info(c))) return rc;
    if (c->host_info[sphk::kOutStart] >= 0)
        return set_err(c, SPH_ESTATE, "an out-of-grid deletion is pending; step once before recording");
    const int n = c->host_info[sphk::kNum];
    if (n <= 0) return set_err(c, SPH_ESTATE, "no particles to record");
    if (K > nsteps) K = nsteps;
    const int nseg = (nsteps + K - 1) / K;
    const cudaError_t e = ensure_buffers(a, K, nseg + 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(c, SPH_ENOMEM, "adjoint buffers (K=%d, %d checkpoints): %s", K, nseg + 1,
                       cudaGetErrorString(e));
    }
    a->n = n;
    a->state_elems = (size_t)n;
    a->dt = dt;
    a->nsteps = nsteps;
    a->K = K;
    a->exact = c->exact;
    a->params_version = c->params_version;
    float4* st[3];
    ctx_state(c, st);
    for (int s = 0; s < nseg; ++s) {
        CK(c, copy_state(a, st, s, true, c->stream));
        const int steps = (s + 1) * K <= nsteps ? K : nsteps - s * K;
        if ((rc = sph_step(c, dt, steps))) return rc;
    }
    CK(c, copy_state(a, st, nseg, true, c->stream));
    if ((rc = read_info(c))) return rc;
    const int out = c->host_info[sphk::kOutStart], now = c->host_info[sphk::kNum];
    if (now != n || out >= 0)
        return set_err(c, SPH_EOOB, "particles left the grid during the rollout; its gradient is not defined");
    a->recorded = 1;
    return SPH_OK;
}

int sph_adjoint_backward(sph_ctx* c, const sph_float4* dL_dpos, const sph_float4* dL_dvel,
                         const sph_float4* dL_dveleval, sph_float4* dL_dpos0, sph_float4* dL_dvel0,
                         sph_float4* dL_dveleval0, double* dL_dvisc) {
    int rc = ctx_adj_check(c);
    if (rc) return rc;
    sph_adjoint* a = c->adj;
    CK(c, load_seeds(a, dL_dpos, dL_dvel, dL_dveleval, c->stream));
    if (graph_stale(a, c->stream, 0)) {
        drop_graph(a);
        float4* st[3];
        ctx_state(c, st);
        cudaGraph_t g = nullptr;
        CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const sphk::OneScene R{c->P};
        rc = enqueue_backward(
            c, a, st, c->stream, false, [&](int slot) { return ctx_taped_step(c, slot); },
            [&](const TapeStep& T, int src) { launch_reverse(a, R, T, src, c->stream); }, ctx_fail);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return set_err(c, SPH_ECUDA, "backward graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&a->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            a->graph = nullptr;
            return set_err(c, SPH_ECUDA, "backward graph instantiate: %s", cudaGetErrorString(e));
        }
        graph_key(a, c->stream, 0);
    }
    CK(c, cudaGraphLaunch(a->graph, c->stream));
    CK(c, store_results(a, dL_dpos0, dL_dvel0, dL_dveleval0, c->stream));
    if ((rc = read_info(c))) return rc;
    if (dL_dvisc) *dL_dvisc = a->host_visc[0];
    return SPH_OK;
}

int sph_adjoint_rollout(sph_ctx* c, int nsteps, int K, const sph_float4* dL_dpos_final, sph_float4* dL_dvel0,
                        float* dL_dvisc) {
    int rc = ctx_adj_check(c);
    if (rc) return rc;
    const int k_eff = K > c->adj->nsteps ? c->adj->nsteps : K;
    if (nsteps != c->adj->nsteps || k_eff != c->adj->K)
        return set_err(c, SPH_EINVAL, "sph_adjoint_rollout: (nsteps=%d, K=%d) differ from the recorded (%d, %d)",
                       nsteps, K, c->adj->nsteps, c->adj->K);
    double v = 0.0;
    rc = sph_adjoint_backward(c, dL_dpos_final, nullptr, nullptr, nullptr, dL_dvel0, nullptr, &v);
    if (rc == SPH_OK && dL_dvisc) *dL_dvisc = (float)v;
    return rc;
}

int sph_adjoint_rewind(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->adj || !c->adj->recorded) return set_err(c, SPH_ESTATE, "no recorded rollout to rewind");
    float4* st[3];
    CK(c, copy_state(c->adj, ctx_state(c, st), 0, false, c->stream));
    return read_info(c);
}

int sph_loss_mse(sph_ctx* c, const sph_float4* target, sph_float4* dL_dpos, double* loss) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!target || !dL_dpos) return set_err(c, SPH_EINVAL, "sph_loss_mse: null array");
    if (!c->adj) {
        c->adj = new sph_adjoint();
        c->adj->N = (size_t)c->max_num;
        c->adj->C1 = ((size_t)c->gp.nb_cells + 1 + 3) & ~(size_t)3;
    }
    const cudaError_t e = ensure_buffers(c->adj, 0, 0);
    if (e != cudaSuccess) return set_err(c, SPH_ENOMEM, "sph_loss_mse: %s", cudaGetErrorString(e));
    if ((rc = read_info(c))) return rc;
    const int n = c->host_info[sphk::kNum];
    CK(c, cudaMemsetAsync(c->adj->visc_acc, 0, sizeof(double), c->stream));
    const int blocks = (n + 255) / 256;
    if (n > 0)
        k_loss_mse<<<blocks, 256, 0, c->stream>>>(c->pos_u, reinterpret_cast<const float4*>(target),
                                                  reinterpret_cast<float4*>(dL_dpos), n, nullptr, nullptr, nullptr, n,
                                                  1.f, nullptr, 0.f, c->adj->visc_acc);
    CK_LAUNCH(c);
    CK(c, cudaMemcpyAsync(c->adj->host_visc, c->adj->visc_acc, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if ((rc = read_info(c))) return rc;
    if (loss) *loss = c->adj->host_visc[0];
    return SPH_OK;
}

// --- batches -----------------------------------------------------------------
int sph_batch_adjoint_record(sph_batch* b, float dt, int nsteps, int K) {
    if (!b || nsteps <= 0 || K <= 0 || !std::isfinite(dt))
        return berr(b, SPH_EINVAL, "sph_batch_adjoint_record: bad arguments (nsteps=%d, K=%d)", nsteps, K);
    cudaSetDevice(b->device);
    {
        const int rc = batch_refresh_num(b);  // counts after earlier deletions
        if (rc) return rc;
    }
    if (!b->adj) {
        b->adj = new sph_batch_adjoint();
        b->adj->N = (size_t)b->nslots;
        b->adj->C1 = ((size_t)b->ncells_total + 3) & ~(size_t)3;
        b->adj->nscenes = b->nscenes;
        b->adj->tape_keys = true;
        b->adj->state_elems = (size_t)b->nslots;
    }
    sph_batch_adjoint* a = b->adj;
    a->recorded = 0;
    if (b->nvalid <= 0) return berr(b, SPH_ESTATE, "no particles to record");
    if (K > nsteps) K = nsteps;
    const int nseg = (nsteps + K - 1) / K;
    const cudaError_t e = ensure_buffers(a, K, nseg + 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return berr(b, SPH_ENOMEM, "adjoint buffers (K=%d, %d checkpoints): %s", K, nseg + 1, cudaGetErrorString(e));
    }
    a->n = b->nvalid;
    a->dt = dt;
    a->nsteps = nsteps;
    a->K = K;
    a->exact = b->exact;
    a->params_version = b->params_version;
    BCK(b, cudaMemsetAsync(b->info_nb + kBatchFrozenTotal, 0, sizeof(int), b->stream));
    float4* st[3];
    batch_state(b, st);
    int rc;
    for (int s = 0; s < nseg; ++s) {
        BCK(b, copy_state(a, st, s, true, b->stream));
        const int steps = (s + 1) * K <= nsteps ? K : nsteps - s * K;
        if ((rc = sph_batch_step(b, dt, steps))) return rc;
    }
    BCK(b, copy_state(a, st, nseg, true, b->stream));
    if ((rc = batch_read_info(b))) return rc;
    if (b->host_info[kBatchFrozenTotal] != 0)
        return berr(b, SPH_EOOB, "particles left their scene's grid during the rollout; its gradient is not defined");
    a->recorded = 1;
    return SPH_OK;
}

namespace {

int batch_backward(sph_batch* b, bool seeded, const sph_float4* dL_dpos, const sph_float4* dL_dvel,
                   const sph_float4* dL_dveleval, sph_float4* dL_dpos0, sph_float4* dL_dvel0, sph_float4* dL_dveleval0,
                   double* dL_dvisc) {
    sph_batch_adjoint* a = b->adj;
    int rc;
    BCK(b, load_seeds(a, dL_dpos, dL_dvel, dL_dveleval, b->stream));
    if (graph_stale(a, b->stream, seeded)) {
        drop_graph(a);
        float4* st[3];
        batch_state(b, st);
        cudaGraph_t g = nullptr;
        BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const float dt = a->dt;
        rc = enqueue_backward(
            b, a, st, b->stream, seeded, [&](int slot) { return batch_taped_step(b, slot, dt); },
            [&](const TapeStep& T, int src) {
                const sphk::ManyScenes R{b->d_table, b->d_cbase, T.keys, b->cell_bits};
                launch_reverse(a, R, T, src, b->stream);
            },
            batch_fail);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return berr(b, SPH_ECUDA, "backward graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&a->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            a->graph = nullptr;
            return berr(b, SPH_ECUDA, "backward graph instantiate: %s", cudaGetErrorString(e));
        }
        graph_key(a, b->stream, seeded);
    }
    BCK(b, cudaGraphLaunch(a->graph, b->stream));
    BCK(b, store_results(a, dL_dpos0, dL_dvel0, dL_dveleval0, b->stream));
    if ((rc = sph_batch_sync(b))) return rc;
    if (dL_dvisc)
        for (int s = 0; s < b->nscenes; ++s) dL_dvisc[s] = a->host_visc[s];
    return SPH_OK;
}

int nseg_of(const AdjState* a) { return (a->nsteps + a->K - 1) / a->K; }

}  // namespace

int sph_batch_adjoint_backward(sph_batch* b, const sph_float4* dL_dpos, const sph_float4* dL_dvel,
                               const sph_float4* dL_dveleval, sph_float4* dL_dpos0, sph_float4* dL_dvel0,
                               sph_float4* dL_dveleval0, double* dL_dvisc) {
    int rc = batch_adj_check(b);
    if (rc) return rc;
    return batch_backward(b, false, dL_dpos, dL_dvel, dL_dveleval, dL_dpos0, dL_dvel0, dL_dveleval0, dL_dvisc);
}

int sph_batch_trajectory(sph_batch* b, sph_float4* pos_traj) {
    int rc = batch_adj_check(b);
    if (rc) return rc;
    if (!pos_traj) return berr(b, SPH_EINVAL, "sph_batch_trajectory: null array");
    sph_batch_adjoint* a = b->adj;
    const int nseg = nseg_of(a);
    for (int c = 0; c <= nseg; ++c)
        BCK(b, cudaMemcpyAsync(pos_traj + (size_t)c * a->N, ckpt_slot(a, c, 0), a->N * 16, cudaMemcpyDeviceToDevice,
                               b->stream));
    return sph_batch_sync(b);
}

int sph_batch_loss_traj(sph_batch* b, const sph_float4* targets, sph_float4* dL_dpos_traj, float huber,
                        double* loss) {
    int rc = batch_adj_check(b);
    if (rc) return rc;
    if (!targets || !dL_dpos_traj || !(huber >= 0.f)) return berr(b, SPH_EINVAL, "sph_batch_loss_traj: bad arguments");
    sph_batch_adjoint* a = b->adj;
    const int nseg = nseg_of(a);
    const size_t N = a->N;
    BCK(b, cudaMemsetAsync(a->visc_acc, 0, sizeof(double) * b->nscenes, b->stream));
    BCK(b, cudaMemsetAsync(dL_dpos_traj, 0, N * 16, b->stream));  // time 0: the given initial positions
    const float w = 1.f / (float)nseg;
    const int blocks = (b->nslots + 255) / 256;
    for (int c = 1; c <= nseg; ++c)
        k_loss_mse<<<blocks, 256, 0, b->stream>>>(ckpt_slot(a, c, 0), reinterpret_cast<const float4*>(targets) + c * N,
                                                  reinterpret_cast<float4*>(dL_dpos_traj) + c * N, b->nslots,
                                                  b->scene_of, b->d_slot_off, b->d_num, 0, w, b->d_table, huber,
                                                  a->visc_acc);
    BCK(b, cudaGetLastError());
    BCK(b, cudaMemcpyAsync(a->host_visc, a->visc_acc, sizeof(double) * b->nscenes, cudaMemcpyDeviceToHost,
                           b->stream));
    if ((rc = sph_batch_sync(b))) return rc;
    if (loss)
        for (int s = 0; s < b->nscenes; ++s) loss[s] = a->host_visc[s];
    return SPH_OK;
}

int sph_batch_adjoint_backward_traj(sph_batch* b, const sph_float4* dL_dpos_traj, sph_float4* dL_dpos0,
                                    sph_float4* dL_dvel0, sph_float4* dL_dveleval0, double* dL_dvisc) {
    int rc = batch_adj_check(b);
    if (rc) return rc;
    if (!dL_dpos_traj) return berr(b, SPH_EINVAL, "sph_batch_adjoint_backward_traj: null array");
    sph_batch_adjoint* a = b->adj;
    const int nseg = nseg_of(a);
    if (nseg + 1 > a->cap_seeds) {
        if (a->seeds) cudaFree(a->seeds);
        a->seeds = nullptr;
        a->cap_seeds = 0;
        drop_graph(a);
        BCK(b, cudaMalloc((void**)&a->seeds, (size_t)(nseg + 1) * a->N * 16));
        a->cap_seeds = nseg + 1;
    }
    BCK(b, cudaMemcpyAsync(a->seeds, dL_dpos_traj, (size_t)(nseg + 1) * a->N * 16, cudaMemcpyDeviceToDevice,
                           b->stream));
    return batch_backward(b, true, dL_dpos_traj + (size_t)nseg * a->N, nullptr, nullptr, dL_dpos0, dL_dvel0,
                          dL_dveleval0, dL_dvisc);
}

int sph_batch_adjoint_rewind(sph_batch* b) {
    if (!b) return SPH_EINVAL;
    cudaSetDevice(b->device);
    if (!b->adj || !b->adj->recorded) return berr(b, SPH_ESTATE, "no recorded rollout to rewind");
    float4* st[3];
    BCK(b, copy_state(b->adj, batch_state(b, st), 0, false, b->stream));
    return sph_batch_sync(b);
}

int sph_batch_loss_mse(sph_batch* b, const sph_float4* target, sph_float4* dL_dpos, double* loss) {
    if (!b || !target || !dL_dpos) return berr(b, SPH_EINVAL, "sph_batch_loss_mse: null argument");
    cudaSetDevice(b->device);
    if (!b->adj) {
        b->adj = new sph_batch_adjoint();
        b->adj->N = (size_t)b->nslots;
        b->adj->C1 = ((size_t)b->ncells_total + 3) & ~(size_t)3;
        b->adj->nscenes = b->nscenes;
        b->adj->tape_keys = true;
        b->adj->state_elems = (size_t)b->nslots;
    }
    sph_batch_adjoint* a = b->adj;
    const cudaError_t e = ensure_buffers(a, 0, 0);
    if (e != cudaSuccess) return berr(b, SPH_ENOMEM, "sph_batch_loss_mse: %s", cudaGetErrorString(e));
    BCK(b, cudaMemsetAsync(a->visc_acc, 0, sizeof(double) * b->nscenes, b->stream));
    const int blocks = (b->nslots + 255) / 256;
    k_loss_mse<<<blocks, 256, 0, b->stream>>>(b->pos_u, reinterpret_cast<const float4*>(target),
                                              reinterpret_cast<float4*>(dL_dpos), b->nslots, b->scene_of,
                                              b->d_slot_off, b->d_num, 0, 1.f, nullptr, 0.f, a->visc_acc);
    BCK(b, cudaGetLastError());
    BCK(b, cudaMemcpyAsync(a->host_visc, a->visc_acc, sizeof(double) * b->nscenes, cudaMemcpyDeviceToHost,
                           b->stream));
    const int rc = sph_batch_sync(b);
    if (rc) return rc;
    if (loss)
        for (int s = 0; s < b->nscenes; ++s) loss[s] = a->host_visc[s];
    return SPH_OK;
}

}  // extern "C"
