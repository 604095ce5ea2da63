// sph_neighbors.cu — the two neighbour passes (density, force), with the wall
// collision and leapfrog integration fused into the force pass.
//
//   density: rtpslib/system/sph/cl_src/density.cl:44-126 (poly6,
//            cl_sph_kernels.h:29-45; neighbour walk cl_sph_neighbors.h:49-140)
//   force:   rtpslib/system/sph/cl_src/force.cl:43-186 (spiky gradient
//            cl_sph_kernels.h:81-97, viscosity Laplacian :118-127, XSPH)
//
// Neighbour walk.  The reference visits 27 cells (z, y, x in [c-1, c+1]) and
// each cell's sorted range.  Keys of the three cells x-1, x, x+1 of one row
// are consecutive integers, so their particles are one contiguous run of the
// sorted arrays: the walk here is 9 row runs, visited in the reference's
// order.  Integer row hashing equals the reference's float hash formula
// whenever every intermediate value is an integer below 2^24 in magnitude
// (checked on the host: int_hash_ok); otherwise each of the 27 cells is hashed
// with the float formula.
//
// Cutoff.  |r| <= h with |r| = sqrtf(r2) is the same test as r2 <= rcut2,
// rcut2 being the largest float whose correctly rounded square root is <= h
// (sqrt is monotonic); r2 is formed without contraction, so neighbour sets are
// identical to the oracle's.
//
// Density keeps the reference's summation order and rounding: it equals the
// FP32 oracle bit for bit.  While it tests the candidates it also records,
// per particle, which of its first kMaskBits candidates (in walk order) are
// neighbours (self excluded) as a bitmask, and (rho, 1/rho, K(rho-rho0)).
// Force does not test those candidates again: it decodes the bitmask into a
// per-thread list in shared memory (candidates past kMaskBits are tested
// directly) and runs the heavy arithmetic over the list with all lanes busy;
// the list keeps the walk order.
// Exact=true evaluates force with the oracle's exact operations (IEEE
// divisions, no contraction: bitwise equal); Exact=false uses FMA and
// reciprocals (within the FP32 tolerance of the tests).
#include <climits>

#include "sph_physics.cuh"

namespace sphk {

// Integer row hashing applies: every intermediate of the float hash formula is
// an integer below 2^24 for cells within one cell of the grid.
__device__ __forceinline__ bool cell_fast(const StepParams& P, const int3& c) {
    return P.int_hash_ok && c.x >= -1 && c.x <= P.res_x && c.y >= -1 && c.y <= P.res_y && c.z >= -1 &&
           c.z <= P.res_z;
}

// The 9 row runs of cell c (at most 9 calls of f(rs, re), in walk order).
template <class F>
__device__ __forceinline__ void walk_rows_fast(const StepParams& P, const uint32_t* __restrict__ cs,
                                               const uint32_t* __restrict__ ce, const int3& c, F&& f) {
    const uint32_t C = (uint32_t)P.nb_cells;
#pragma unroll 1
    for (int dz = -1; dz <= 1; ++dz) {
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            const int base = ((c.z + dz) * P.res_y + (c.y + dy)) * P.res_x + c.x;
            uint32_t rs = kEmpty, last = 0;
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                const uint32_t h = (uint32_t)(base + dx);
                if (h < C) {
                    const uint32_t s = __ldg(cs + h);
                    if (s != kEmpty) {
                        if (rs == kEmpty) rs = s;
                        last = h;
                    }
                }
            }
            if (rs != kEmpty) f(rs, __ldg(ce + last));
        }
    }
}

// The 27 cells one by one with the reference's float hash (up to 27 calls).
template <class F>
__device__ __forceinline__ void walk_rows_slow(const StepParams& P, const uint32_t* __restrict__ cs,
                                               const uint32_t* __restrict__ ce, const int3& c, F&& f) {
    const uint32_t C = (uint32_t)P.nb_cells;
#pragma unroll 1
    for (int z = c.z - 1; z <= c.z + 1; ++z)
#pragma unroll 1
        for (int y = c.y - 1; y <= c.y + 1; ++y)
#pragma unroll 1
            for (int x = c.x - 1; x <= c.x + 1; ++x) {
                const uint32_t h = (uint32_t)grid_hash_f(x, y, z, P.gs_res);
                if (h >= C) continue;
                const uint32_t s = __ldg(cs + h);
                if (s != kEmpty) f(s, __ldg(ce + h));
            }
}

// Visit the sorted-index runs of the 27 neighbour cells of scaled position
// (px,py,pz), in the reference's order; f(rs, re) gets each non-empty run.
template <class F>
__device__ __forceinline__ void walk_rows(const StepParams& P, const uint32_t* __restrict__ cs,
                                          const uint32_t* __restrict__ ce, float px, float py, float pz, F&& f) {
    const int3 c = grid_cell(px, py, pz, P.gs_min, P.gs_delta);
    if (cell_fast(P, c))
        walk_rows_fast(P, cs, ce, c, f);
    else
        walk_rows_slow(P, cs, ce, c, f);
}

// ---------------------------------------------------------------------------
// Density.  One thread per sorted particle.  When called from the fused step
// it also does the out-of-grid deletion bookkeeping (vel_s != nullptr).
template <bool Unit>
__global__ void __launch_bounds__(256) k_density(const float4* __restrict__ pos_s, const float4* __restrict__ veleval_s,
                                                 float* __restrict__ density, float4* __restrict__ rec_pd,
                                                 float4* __restrict__ rec_vi, uint32_t* __restrict__ nbr,
                                                 uint32_t* __restrict__ mask, const size_t mstride,
                                                 const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
                                                 int* __restrict__ info, const uint32_t* __restrict__ idx,
                                                 const float4* __restrict__ vel_u, float4* __restrict__ vel_s,
                                                 float4* __restrict__ del_pos, float4* __restrict__ del_vel,
                                                 const StepParams P) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (vel_s != nullptr && out >= 0 && i < n_old) {
        // SPH.cpp:220-250: the kept particles' velocities in sorted order
        // (call_prep copies vel_s to vel_u), the removed ones saved.
        const float4 v = __ldg(vel_u + __ldg(idx + i));
        if (i < n) {
            vel_s[i] = v;
        } else {
            del_pos[i - n] = __ldg(pos_s + i);
            del_vel[i - n] = v;
            if (i == n) info[kDeleted] = n_old - n;
        }
    }
    if (i >= n) return;
    float4 pi = __ldg(pos_s + i);
    if (!Unit) pi = v4scale(pi, P.sc);
    const float rc2 = P.rcut2, h2 = P.h2;
    float acc = 0.f;
    uint32_t cnt = 0, cur = 0, bit = 1, word = 0;
    uint32_t* mrow = mask + i;
    walk_rows(P, cs, ce, pi.x, pi.y, pi.z, [&](uint32_t rs, uint32_t re) {
        for (uint32_t j = rs; j < re; ++j) {
            float4 pj = __ldg(pos_s + j);
            if (!Unit) pj = v4scale(pj, P.sc);
            const float r2 = dist2_exact(__fsub_rn(pi.x, pj.x), __fsub_rn(pi.y, pj.y), __fsub_rn(pi.z, pj.z));
            if (r2 <= rc2) {
                const float hr2 = __fsub_rn(h2, r2);
                acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(hr2, hr2), hr2));
                ++cnt;
                if (j != (uint32_t)i) cur |= bit;
            }
            bit <<= 1;
            if (bit == 0) {
                if (word < kMaskWords) mrow[word * mstride] = cur;
                ++word;
                cur = 0;
                bit = 1;
            }
        }
    });
    if (bit != 1 && word < kMaskWords) mrow[word * mstride] = cur;
    const float rho = __fmul_rn(P.dens_coef, acc);
    density[i] = rho;
    // Neighbour records for the force pass: 32 bytes per particle.
    const float4 ve = __ldg(veleval_s + i);
    rec_pd[i] = make_float4(pi.x, pi.y, pi.z, rho);
    rec_vi[i] = make_float4(ve.x, ve.y, ve.z, __frcp_rn(rho));
    if (nbr) nbr[i] = cnt;
}

void launch_density(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd, float4* rec_vi,
                    uint32_t* nbr, uint32_t* mask, size_t mask_stride, const uint32_t* cell_start,
                    const uint32_t* cell_end, const int* info, const uint32_t* idx, const float4* vel_u,
                    float4* vel_s, float4* del_pos, float4* del_vel, const StepParams& p, int grid_items,
                    cudaStream_t st) {
    const int threads = 256;
    int blocks = (grid_items + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    if (p.unit_scale)
        k_density<true><<<blocks, threads, 0, st>>>(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride,
                                                    cell_start, cell_end, (int*)info, idx, vel_u, vel_s, del_pos,
                                                    del_vel, p);
    else
        k_density<false><<<blocks, threads, 0, st>>>(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask,
                                                     mask_stride, cell_start, cell_end, (int*)info, idx, vel_u,
                                                     vel_s, del_pos, del_vel, p);
}

// ---------------------------------------------------------------------------
// Force (+ collision + leapfrog when Fused).
//
// One thread per sorted particle.  The thread first lays out its 9 row runs
// (sorted-index start and walk-order offset of each) in shared memory, then
// walks its neighbours with a cursor over the density pass's bitmask
// (candidates past kMaskBits are tested).  The warp advances all cursors in
// lock step, one neighbour per lane per iteration, and runs the pair
// arithmetic for every lane in the same iteration, until no lane has a
// neighbour left: lanes never serialise on each other's neighbour lists.
// Neighbour data is the 32-byte record (x, y, z, rho), (veleval.xyz, 1/rho)
// written by the density pass, read through L1.
constexpr int kForceThreads = 128;

struct ForceSums {
    float fx = 0.f, fy = 0.f, fz = 0.f, vx = 0.f, vy = 0.f, vz = 0.f, xx = 0.f, xy = 0.f, xz = 0.f;
};

// One accepted neighbour j of i (force.cl:43-140 with iej = 1): pd = (scaled
// position, rho_j), vj = (veleval_j, 1/rho_j).
template <bool Exact>
__device__ __forceinline__ void force_pair(ForceSums& a, const float4& pi, const float4& vi, float di, float Pi,
                                           const float4& pd, const float4& vj, const StepParams& P) {
    const float dx = __fsub_rn(pi.x, pd.x), dy = __fsub_rn(pi.y, pd.y), dz = __fsub_rn(pi.z, pd.z);
    const float r2 = dist2_exact(dx, dy, dz);
    const float dj = pd.w, idj = vj.w;
    const float Pj = __fmul_rn(P.K, __fsub_rn(dj, P.rho0));
    const float dvx = __fsub_rn(vj.x, vi.x), dvy = __fsub_rn(vj.y, vi.y), dvz = __fsub_rn(vj.z, vi.z);
    const float hr2 = __fsub_rn(P.h2, r2);
    const float w6 = __fmul_rn(__fmul_rn(hr2, hr2), hr2);
    const float dsum = __fadd_rn(di, dj);
    if (Exact) {
        float rlen = __fsqrt_rn(r2);
        rlen = rlen < P.eps ? P.eps : rlen;
        const float hr = __fsub_rn(P.h, rlen);
        const float dWdr = __fdiv_rn(__fmul_rn(hr, hr), rlen);
        const float kern = __fmul_rn(__fmul_rn(dWdr, __fadd_rn(Pi, Pj)), idj);
        a.vx = __fadd_rn(a.vx, __fmul_rn(__fmul_rn(dvx, hr), idj));
        a.vy = __fadd_rn(a.vy, __fmul_rn(__fmul_rn(dvy, hr), idj));
        a.vz = __fadd_rn(a.vz, __fmul_rn(__fmul_rn(dvz, hr), idj));
        a.xx = __fadd_rn(a.xx, __fdiv_rn(__fmul_rn(w6, dvx), dsum));
        a.xy = __fadd_rn(a.xy, __fdiv_rn(__fmul_rn(w6, dvy), dsum));
        a.xz = __fadd_rn(a.xz, __fdiv_rn(__fmul_rn(w6, dvz), dsum));
        a.fx = __fadd_rn(a.fx, __fmul_rn(dx, kern));
        a.fy = __fadd_rn(a.fy, __fmul_rn(dy, kern));
        a.fz = __fadd_rn(a.fz, __fmul_rn(dz, kern));
    } else {
        // r2 == 0 (coincident particles) gives NaN here and is caught by the
        // same clamp as rlen < EPSILON.
        const float inv_r = rsqrtf(r2);
        float rlen = r2 * inv_r;
        float irl = inv_r;
        if (!(rlen >= P.eps)) {
            rlen = P.eps;
            irl = __frcp_rn(P.eps);
        }
        const float hr = P.h - rlen;
        const float kern = hr * hr * irl * ((Pi + Pj) * idj);
        const float vh = hr * idj;
        a.vx = fmaf(dvx, vh, a.vx);
        a.vy = fmaf(dvy, vh, a.vy);
        a.vz = fmaf(dvz, vh, a.vz);
        const float wx = w6 * __frcp_rn(dsum);
        a.xx = fmaf(wx, dvx, a.xx);
        a.xy = fmaf(wx, dvy, a.xy);
        a.xz = fmaf(wx, dvz, a.xz);
        a.fx = fmaf(dx, kern, a.fx);
        a.fy = fmaf(dy, kern, a.fy);
        a.fz = fmaf(dz, kern, a.fz);
    }
}

template <bool Fused, bool Exact, bool Unit>
__global__ void __launch_bounds__(kForceThreads) k_force(
    const float4* __restrict__ pos_s, const float4* __restrict__ rec_pd, const float4* __restrict__ rec_vi,
    const uint32_t* __restrict__ mask, const size_t mstride, const uint32_t* __restrict__ cs,
    const uint32_t* __restrict__ ce, const int* __restrict__ info, float4* __restrict__ force_s,
    float4* __restrict__ xsph_s, uint32_t* __restrict__ idx, const float4* __restrict__ vel_s,
    float4* __restrict__ pos_u, float4* __restrict__ vel_u, float4* __restrict__ veleval_u, const StepParams P,
    const float dt) {
    // Row table of each thread: sorted index of the run's first candidate and
    // walk-order offset of it; rows without candidates are left out.
    __shared__ uint32_t s_rs[9][kForceThreads];
    __shared__ uint32_t s_off[10][kForceThreads];
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int t = threadIdx.x;
    const int i = blockIdx.x * kForceThreads + t;
    const unsigned wmask = __ballot_sync(0xffffffffu, i < n);
    if (i >= n) return;

    const float4 pi = __ldg(rec_pd + i);  // scaled position, rho_i
    const float4 vi = __ldg(rec_vi + i);  // veleval_i, 1/rho_i
    const float di = pi.w;
    const float Pi = __fmul_rn(P.K, __fsub_rn(di, P.rho0));
    const float rc2 = P.rcut2;

    ForceSums a;
    int nrows = 0;
    uint32_t M = 0;
    const int3 c = grid_cell(pi.x, pi.y, pi.z, P.gs_min, P.gs_delta);
    if (cell_fast(P, c)) {
        walk_rows_fast(P, cs, ce, c, [&](uint32_t rs, uint32_t re) {  // at most 9 runs
            s_rs[nrows][t] = rs;
            s_off[nrows][t] = M;
            M += re - rs;
            ++nrows;
        });
    } else {
        // Cells beyond the integer-hash range (particles far outside the
        // walls): the 27 cells tested one by one, pairs accumulated at once.
        walk_rows_slow(P, cs, ce, c, [&](uint32_t rs, uint32_t re) {
            for (uint32_t j = rs; j < re; ++j) {
                const float4 pj = __ldg(rec_pd + j);
                const float r2 = dist2_exact(__fsub_rn(pi.x, pj.x), __fsub_rn(pi.y, pj.y), __fsub_rn(pi.z, pj.z));
                if (r2 <= rc2 && j != (uint32_t)i) force_pair<Exact>(a, pi, vi, di, Pi, pj, __ldg(rec_vi + j), P);
            }
        });
    }
    s_off[nrows][t] = M;

    // Cursor: bit position p of the last neighbour taken, row r containing it.
    const uint32_t* mrow = mask + i;
    const uint32_t mbits = M < (uint32_t)kMaskBits ? M : (uint32_t)kMaskBits;
    uint32_t w = 0, m = (mbits > 0) ? __ldg(mrow) : 0u;
    uint32_t q = (uint32_t)kMaskBits;  // next candidate past the bitmask to test
    int r = 0;
    for (;;) {
        // next neighbour of this lane, as its walk-order position p
        bool have = false;
        uint32_t p = 0;
        while (m == 0 && (w + 1) * 32u < mbits) {
            ++w;
            m = __ldg(mrow + (size_t)w * mstride);
        }
        if (m != 0) {
            p = w * 32u + (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
            have = true;
        } else {
            while (q < M) {
                const uint32_t pp = q++;
                while (pp >= s_off[r + 1][t]) ++r;
                const uint32_t j = s_rs[r][t] + (pp - s_off[r][t]);
                const float4 pj = __ldg(rec_pd + j);
                const float r2 = dist2_exact(__fsub_rn(pi.x, pj.x), __fsub_rn(pi.y, pj.y), __fsub_rn(pi.z, pj.z));
                // The self term is multiplied by iej = 0 in the reference
                // (force.cl:67,113,131,137): it adds a signed zero, so it is skipped.
                if (r2 <= rc2 && j != (uint32_t)i) {
                    p = pp;
                    have = true;
                    break;
                }
            }
        }
        if (!__any_sync(wmask, have)) break;
        if (have) {
            while (p >= s_off[r + 1][t]) ++r;
            const uint32_t j = s_rs[r][t] + (p - s_off[r][t]);
            force_pair<Exact>(a, pi, vi, di, Pi, __ldg(rec_pd + j), __ldg(rec_vi + j), P);
        }
    }

    // force.cl:180-185: force = (mass/di)*(-0.5*wspiky_d*F + visc*wvisc_dd*V),
    // xsph = 2*mass*wpoly6*X; the w lanes are zero.
    float A;
    if (Exact)
        A = (float)((double)P.mass * (1.0 / (double)di));
    else
        A = P.mass * vi.w;
    float4 f, xs;
    f.x = __fmul_rn(A, __fadd_rn(__fmul_rn(P.coef_b, a.fx), __fmul_rn(P.coef_s, a.vx)));
    f.y = __fmul_rn(A, __fadd_rn(__fmul_rn(P.coef_b, a.fy), __fmul_rn(P.coef_s, a.vy)));
    f.z = __fmul_rn(A, __fadd_rn(__fmul_rn(P.coef_b, a.fz), __fmul_rn(P.coef_s, a.vz)));
    f.w = 0.f;
    xs = make_float4(__fmul_rn(P.coef_d, a.xx), __fmul_rn(P.coef_d, a.xy), __fmul_rn(P.coef_d, a.xz), 0.f);
    if (!Fused) {
        force_s[i] = f;
        xsph_s[i] = xs;
        return;
    }
    // Fused collision_wall + leapfrog for particle i.  After an out-of-grid
    // deletion the kept particles are re-indexed in sorted order
    // (sort_indices becomes the identity; their velocities are in vel_s).
    uint32_t orig;
    float4 v;
    if (out >= 0) {
        orig = (uint32_t)i;
        v = vel_s[i];
        idx[i] = (uint32_t)i;
    } else {
        orig = __ldg(idx + i);
        v = vel_u[orig];
    }
    const float4 pp = __ldg(pos_s + i);
    const float4 psc = Unit ? pp : v4scale(pp, P.sc);
    f = collide_walls(psc, v, f, P);
    float4 po, vo, eo;
    leapfrog_core(psc, v, f, xs, dt, P, po, vo, eo);
    vel_u[orig] = vo;
    veleval_u[orig] = eo;
    pos_u[orig] = po;
}

void launch_force(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                  size_t mask_stride, const uint32_t* cell_start, const uint32_t* cell_end, const int* info,
                  int* /*tile_ctr*/, int /*nsm*/, float4* force_s, float4* xsph_s, uint32_t* idx,
                  const float4* vel_s, float4* pos_u, float4* vel_u, float4* veleval_u, const StepParams& p,
                  float dt, int fused, int exact, int grid_items, cudaStream_t st) {
    int blocks = (grid_items + kForceThreads - 1) / kForceThreads;
    if (blocks < 1) blocks = 1;
#define SPH_FORCE_LAUNCH(F, E, U)                                                                            \
    k_force<F, E, U><<<blocks, kForceThreads, 0, st>>>(pos_s, rec_pd, rec_vi, mask, mask_stride, cell_start, \
                                                       cell_end, info, force_s, xsph_s, idx, vel_s, pos_u,   \
                                                       vel_u, veleval_u, p, dt)
    const bool u = p.unit_scale != 0;
    if (fused) {
        if (exact) {
            if (u) SPH_FORCE_LAUNCH(true, true, true); else SPH_FORCE_LAUNCH(true, true, false);
        } else {
            if (u) SPH_FORCE_LAUNCH(true, false, true); else SPH_FORCE_LAUNCH(true, false, false);
        }
    } else {
        if (exact) {
            if (u) SPH_FORCE_LAUNCH(false, true, true); else SPH_FORCE_LAUNCH(false, true, false);
        } else {
            if (u) SPH_FORCE_LAUNCH(false, false, true); else SPH_FORCE_LAUNCH(false, false, false);
        }
    }
#undef SPH_FORCE_LAUNCH
}

}  // namespace sphk
