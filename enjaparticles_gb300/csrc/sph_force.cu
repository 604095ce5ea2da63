// sph_force.cu — force pass (rtpslib/system/sph/cl_src/force.cl:43-186:
// spiky gradient cl_sph_kernels.h:81-97, viscosity Laplacian :118-127,
// XSPH), with the wall collision and leapfrog integration of the step fused in.
// Compiled with FMA contraction allowed: the default (fast) arithmetic uses
// it; the exact variant spells every operation with a rounding intrinsic.
#include <type_traits>

#include "sph_queue.cuh"
#include "sph_walk.cuh"

namespace sphk {

// ---------------------------------------------------------------------------
// Force (+ collision + leapfrog when Fused).
//
// One thread per sorted particle.  The thread first lays out its 9 row runs
// in shared memory (walk-order end of each, and sorted index minus walk
// position over it), from cell range loads issued together, then walks its
// neighbours with a cursor over the density pass's bitmask (candidates past
// kMaskBits are tested), the next mask word already in flight.  The warp
// advances all cursors in lock step, one neighbour per lane per iteration,
// and runs the pair arithmetic for every lane in the same iteration, until no
// lane has a neighbour left: lanes never serialise on each other's neighbour
// lists.  Neighbour data is the 32-byte record (x, y, z, rho),
// (veleval.xyz, 1/rho) written by the density pass and the velocity pass,
// read through L1.
// Threads per block: 64, 128 (the default) or 256, a launch shape the
// autotuner picks; every shape gives the same results bit for bit.
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
        // 1/|r| and 1/(rho_i + rho_j) by the approximate reciprocal (square
        // root) instructions with denormals flushed (a few ulp, inside the
        // default mode's tolerance).  r2 == 0 (coincident particles) gives
        // NaN in rlen and is caught by the same clamp as rlen < EPSILON.
        float inv_r;
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(inv_r) : "f"(r2));
        float rlen = r2 * inv_r;
        float irl = inv_r;
        if (!(rlen >= P.eps)) {
            rlen = P.eps;
            irl = P.inv_eps;
        }
        const float hr = P.h - rlen;
        const float kern = hr * hr * irl * ((Pi + Pj) * idj);
        const float vh = hr * idj;
        a.vx = fmaf(dvx, vh, a.vx);
        a.vy = fmaf(dvy, vh, a.vy);
        a.vz = fmaf(dvz, vh, a.vz);
        // the XSPH weight is a smoothing term, far inside the tolerance
        float rd;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rd) : "f"(dsum));
        const float wx = w6 * rd;
        a.xx = fmaf(wx, dvx, a.xx);
        a.xy = fmaf(wx, dvy, a.xy);
        a.xz = fmaf(wx, dvz, a.xz);
        a.fx = fmaf(dx, kern, a.fx);
        a.fy = fmaf(dy, kern, a.fy);
        a.fz = fmaf(dz, kern, a.fz);
    }
}

// The arrays of the force pass (force_s, xsph_s: the staged pass's outputs;
// the rest of the second half: the fused integration's).
struct ForceArgs {
    const float4* pos_s;
    const float4* rec_pd;
    const float4* rec_vi;
    const uint32_t* mask;
    size_t mstride;
    const uint32_t* nbr;
    const uint32_t* cs0;
    const uint32_t* ce0;
    float4* force_s;
    float4* xsph_s;
    uint32_t* idx;
    const float4* vel_s;
    float4* pos_u;
    float4* vel_u;
    float4* veleval_u;
    float4* keep_f;
    float4* keep_v;
    float dt;
    // the counting sort's prefix of the cell counts (launch_cell_scan), for
    // the row runs of one system; null: the runs from cs0 / ce0
    const uint32_t* pre;
};

// Sorted particle i (in_range: i below the step's particle count) with the
// thread's column of the row table: per run, the walk-order position just
// past its last candidate and the sorted index minus walk-order position
// over the run (j = p + delta, modulo 2^32), one 8-byte entry; rows without
// candidates are left out.  Every
// lane of the warp calls it (the neighbour loop is warp-wide).
template <int T, bool Fused, bool Exact, bool Unit, class Scenes>
__device__ __forceinline__ void force_one(const int i, const bool in_range, const int out, const ForceArgs& G,
                                          const Scenes& R, uint2 (*s_row)[T]) {
    const float4* __restrict__ pos_s = G.pos_s;
    const float4* __restrict__ rec_pd = G.rec_pd;
    const float4* __restrict__ rec_vi = G.rec_vi;
    const uint32_t* __restrict__ mask = G.mask;
    const size_t mstride = G.mstride;
    const uint32_t* __restrict__ nbr = G.nbr;
    const uint32_t* __restrict__ cs0 = G.cs0;
    const uint32_t* __restrict__ ce0 = G.ce0;
    float4* __restrict__ force_s = G.force_s;
    float4* __restrict__ xsph_s = G.xsph_s;
    uint32_t* __restrict__ idx = G.idx;
    const float4* __restrict__ vel_s = G.vel_s;
    float4* __restrict__ pos_u = G.pos_u;
    float4* __restrict__ vel_u = G.vel_u;
    float4* __restrict__ veleval_u = G.veleval_u;
    float4* __restrict__ keep_f = G.keep_f;
    float4* __restrict__ keep_v = G.keep_v;
    const float dt = G.dt;
    const int t = threadIdx.x;
    const bool live = in_range && !R.frozen(i);
    if constexpr (Scenes::kBatch) {
        // A batch particle outside its scene's grid: removed from the scene
        // (SPH.cpp:220-250), stored after the scene's kept particles (in
        // sorted order, as a lone system's deleted list); the first one sets
        // the scene's new count.  The scene's kept particles read their
        // velocities from vel_s and are re-indexed below, so no slot written
        // here is read by this pass.
        if (Fused && in_range && !live) {
            const uint32_t sc = R.scene(i), os = R.out_start(sc), kept = os - __ldg(R.seg + sc);
            const uint32_t j = (uint32_t)i - os, dst = __ldg(R.slot_off + sc) + kept + j;
            const StepParams& Q = R.params(i);
            if (in_bounds(dst, Q.chk_cap, Q.chk_err)) {
                pos_u[dst] = __ldg(pos_s + i);
                vel_u[dst] = __ldg(R.vel_s + i);
            }
            if (j == 0) {
                R.del[sc] = R.num[sc] - (int)kept;
                R.num[sc] = (int)kept;
            }
        }
    }
    const unsigned wmask = __ballot_sync(0xffffffffu, live);
    if (!live) return;
    const StepParams& P = R.params(i);
    const uint32_t* cs = cs0 + R.cell_base(i);
    const uint32_t* ce = ce0 + R.cell_base(i);

    const float4 pi = __ldg(rec_pd + i);  // scaled position, rho_i
    const float4 vi = __ldg(rec_vi + i);  // veleval_i, 1/rho_i
    const float di = pi.w;
    const float Pi = __fmul_rn(P.K, __fsub_rn(di, P.rho0));
    const float rc2 = P.rcut2;

    ForceSums a;
    int nrows = 0;
    uint32_t M = 0;
    const int3 c = grid_cell(pi.x, pi.y, pi.z, P.gs_min, P.gs_delta);
    auto add_row = [&](uint32_t rs, uint32_t re) {  // at most 9 runs
        s_row[nrows][t] = make_uint2(M + (re - rs), rs - M);
        M += re - rs;
        ++nrows;
    };
    if (cell_fast(P, c)) {
        if (G.pre != nullptr)
            walk_rows_prefix(P, G.pre + R.cell_base(i), c, add_row);
        else
            walk_rows_fast_batched(P, cs, ce, c, add_row);
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

    // Cursor: bit position p of the last neighbour taken, row r containing it.
    const uint32_t* mrow = mask + i;
    const uint32_t mbits = M < (uint32_t)kMaskBits ? M : (uint32_t)kMaskBits;
    // wb: walk position of the current word's bit 0; mnext: the word after it
    uint32_t wb = 0, m = (mbits > 0) ? __ldg(mrow) : 0u;
    const uint32_t* mnext = mrow + mstride;
    // the next mask word, in flight while this one's neighbours are processed
    uint32_t m_next = (mbits > 32u) ? __ldg(mrow + mstride) : 0u;
    int r = 0;
    const uint2* srow = &s_row[0][t];  // the cursor's row entry (one system)
    // One scene: row r's end and index offset in registers, reloaded when the
    // cursor changes row.  Batches read them from shared memory: with the
    // scene lookups the registers would spill (measured slower).
    constexpr bool kRegCursor = !Scenes::kBatch;
    uint32_t next_off = 0, delta = 0;
    if constexpr (kRegCursor) {
        const uint2 e = s_row[0][t];
        next_off = e.x;
        delta = e.y;
    }
    // sorted index of the candidate at walk position p, advancing row r
    auto index_of = [&](uint32_t p) -> uint32_t {
        if constexpr (kRegCursor) {
            while (p >= next_off) {
                srow += T;  // the next row's entry of this thread's column
                const uint2 e = *srow;
                next_off = e.x;
                delta = e.y;
            }
            return p + delta;
        } else {
            uint2 e = s_row[r][t];
            while (p >= e.x) e = s_row[++r][t];
            return p + e.y;
        }
    };
    // the lane's next neighbour from the bitmask (one is left)
    auto next_bit = [&]() -> uint32_t {
        while (m == 0) {
            wb += 32u;
            m = m_next;
            mnext += mstride;
            m_next = (wb + 32u < mbits) ? __ldg(mnext) : 0u;
        }
        const uint32_t p = wb + (uint32_t)(__ffs(m) - 1);
        m &= m - 1u;
        return p;
    };
    if (!__any_sync(wmask, M > (uint32_t)kMaskBits)) {
        // Every lane's candidates fit the bitmask: the density pass counted
        // the lane's neighbours (itself included), so each lane loops over
        // its own count, taking its next set bit each time (the warp runs
        // while any lane has one left).
        const uint32_t cnt = M > 0 ? __ldg(nbr + i) - 1u : 0u;
        auto visit = [&]() {
            const uint32_t p = next_bit();
            if (!in_bounds(p, M, P.chk_err)) return;  // a mask bit past the walk's candidates
            const uint32_t j = index_of(p);
            if (in_bounds(j, P.chk_cap, P.chk_err))
                force_pair<Exact>(a, pi, vi, di, Pi, __ldg(rec_pd + j), __ldg(rec_vi + j), P);
        };
        if constexpr (!Exact && !Scenes::kBatch) {
            // two neighbours per loop trip (measured 1 % faster; the exact and
            // batched variants would spill)
#pragma unroll 2
            for (uint32_t k = 0; k < cnt; ++k) visit();
        } else {
            for (uint32_t k = 0; k < cnt; ++k) visit();
        }
    } else {
        // Some lane has candidates past the bitmask (crowded cells): the
        // general loop, which also tests those.
        uint32_t q = (uint32_t)kMaskBits;  // next candidate past the bitmask to test
        for (;;) {
            // next neighbour of this lane, as its walk-order position p
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
                    const uint32_t j = index_of(pp);
                    if (!in_bounds(j, P.chk_cap, P.chk_err)) continue;
                    const float4 pj = __ldg(rec_pd + j);
                    const float r2 =
                        dist2_exact(__fsub_rn(pi.x, pj.x), __fsub_rn(pi.y, pj.y), __fsub_rn(pi.z, pj.z));
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
            if (have && in_bounds(p, M, P.chk_err)) {
                const uint32_t j = index_of(p);
                if (in_bounds(j, P.chk_cap, P.chk_err))
                    force_pair<Exact>(a, pi, vi, di, Pi, __ldg(rec_pd + j), __ldg(rec_vi + j), P);
            }
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
    bool reindex = out >= 0;
    if constexpr (Scenes::kBatch) {
        // a scene that deletes keeps its particles in sorted order
        const uint32_t sc = R.scene(i);
        if (R.out_start(sc) != kEmpty) {
            orig = __ldg(R.slot_off + sc) + ((uint32_t)i - __ldg(R.seg + sc));
            v = __ldg(R.vel_s + i);
            idx[i] = orig;
            reindex = true;
        }
    }
    if (!reindex) {
        orig = __ldg(idx + i);
        if (!in_bounds(orig, P.chk_cap, P.chk_err)) return;
        v = vel_u[orig];
    } else if (out >= 0) {
        orig = (uint32_t)i;
        v = vel_s[i];
        idx[i] = (uint32_t)i;
    }
    if (keep_f != nullptr) {
        keep_f[i] = f;
        keep_v[i] = v;
    }
    if (!in_bounds(orig, P.chk_cap, P.chk_err)) return;
    const float4 pp = __ldg(pos_s + i);
    // point sources after force (SPH.cpp:289-296), then the walls
    if (P.n_grav > 0) f = gravity_add<Exact>(f, pp, P);
    const float4 psc = Unit ? pp : v4scale(pp, P.sc);
    f = collide_walls(psc, v, f, P);
    float4 po, vo, eo;
    if (P.integrator == kIntegratorEuler) {
        euler_core(psc, v, f, dt, P, po, vo);
        vel_u[orig] = vo;
        pos_u[orig] = po;
        return;
    }
    leapfrog_core(psc, v, f, xs, dt, P, po, vo, eo);
    vel_u[orig] = vo;
    veleval_u[orig] = eo;
    pos_u[orig] = po;
}

// Minimum resident blocks per SM the force kernel is compiled for, in
// threads per SM over T (each measured against the unbounded build):
//   one system, default arithmetic: 1280 (10 blocks of 128, 48 registers,
//     no spills), 3 % faster;
//   one system, exact arithmetic: 1152 (9 blocks of 128, 56 registers, no
//     spills; unbounded it took 56 with 24 B of spills), 2 % faster;
//   a batch, default arithmetic: 1152 (56 registers and a few bytes of
//     spills against 64 unbounded), the batch step 2 % faster;
//   a batch, exact arithmetic: unbounded.
template <int T, bool Exact, class Scenes>
constexpr int force_min_blocks() {
    return !Scenes::kBatch ? (Exact ? 1152 / T : 1280 / T) : (Exact ? 0 : 1152 / T);
}

template <int T, bool Fused, bool Exact, bool Unit, class Scenes>
__global__ void __launch_bounds__(T, (force_min_blocks<T, Exact, Scenes>()))
    k_force(const ForceArgs A, const int* __restrict__ info, const Scenes R) {
    __shared__ uint2 s_row[9][T];
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * T + threadIdx.x;
    force_one<T, Fused, Exact, Unit>(i, i < n, out, A, R, s_row);
}

template <int T, class Scenes>
void launch_force_tt(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                     size_t mask_stride, const uint32_t* nbr, const uint32_t* cell_start, const uint32_t* cell_end,
                     const int* info, float4* force_s, float4* xsph_s, uint32_t* idx, const float4* vel_s,
                     float4* pos_u, float4* vel_u, float4* veleval_u, float4* keep_f, float4* keep_v, const Scenes& R,
                     bool unit, float dt, int fused, int exact, int grid_items, cudaStream_t st,
                     const uint32_t* cell_pre) {
    int blocks = (grid_items + T - 1) / T;
    if (blocks < 1) blocks = 1;
    const ForceArgs A{pos_s, rec_pd,  rec_vi, mask,      mask_stride, nbr,    cell_start, cell_end, force_s,
                      xsph_s, idx, vel_s, pos_u, vel_u, veleval_u, keep_f, keep_v, dt, cell_pre};
#define SPH_FORCE_LAUNCH(F, E, U) k_force<T, F, E, U, Scenes><<<blocks, T, 0, st>>>(A, info, R)
    if (fused) {
        if (exact) {
            if (unit) SPH_FORCE_LAUNCH(true, true, true); else SPH_FORCE_LAUNCH(true, true, false);
        } else {
            if (unit) SPH_FORCE_LAUNCH(true, false, true); else SPH_FORCE_LAUNCH(true, false, false);
        }
    } else if constexpr (T == kForceThreads) {
        if (exact) {
            if (unit) SPH_FORCE_LAUNCH(false, true, true); else SPH_FORCE_LAUNCH(false, true, false);
        } else {
            if (unit) SPH_FORCE_LAUNCH(false, false, true); else SPH_FORCE_LAUNCH(false, false, false);
        }
    }
#undef SPH_FORCE_LAUNCH
}

template <class Scenes>
void launch_force_t(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                    size_t mask_stride, const uint32_t* nbr, const uint32_t* cell_start, const uint32_t* cell_end,
                    const int* info, float4* force_s, float4* xsph_s, uint32_t* idx, const float4* vel_s,
                    float4* pos_u, float4* vel_u, float4* veleval_u, float4* keep_f, float4* keep_v, const Scenes& R,
                    bool unit, float dt, int fused, int exact, int grid_items, int threads, cudaStream_t st,
                    const uint32_t* cell_pre = nullptr) {
    // the staged (unfused) pass keeps the default shape
    if (fused && threads == 64)
        launch_force_tt<64>(pos_s, rec_pd, rec_vi, mask, mask_stride, nbr, cell_start, cell_end, info, force_s,
                            xsph_s, idx, vel_s, pos_u, vel_u, veleval_u, keep_f, keep_v, R, unit, dt, fused, exact,
                            grid_items, st, cell_pre);
    else if (fused && threads == 256)
        launch_force_tt<256>(pos_s, rec_pd, rec_vi, mask, mask_stride, nbr, cell_start, cell_end, info, force_s,
                             xsph_s, idx, vel_s, pos_u, vel_u, veleval_u, keep_f, keep_v, R, unit, dt, fused, exact,
                             grid_items, st, cell_pre);
    else
        launch_force_tt<kForceThreads>(pos_s, rec_pd, rec_vi, mask, mask_stride, nbr, cell_start, cell_end, info,
                                       force_s, xsph_s, idx, vel_s, pos_u, vel_u, veleval_u, keep_f, keep_v, R, unit,
                                       dt, fused, exact, grid_items, st, cell_pre);
}

// The batch's fused force pass under the queue scheduler (sph_queue.cuh).
template <int T, bool Exact, bool Unit>
__global__ void __launch_bounds__(T) k_force_queue(const ForceArgs A, const BatchQueue Q) {
    __shared__ QueueShared<T> S;
    __shared__ uint2 s_row[9][T];
    if (!queue_start<T>(Q, S)) return;
    while (queue_next<T>(Q, S)) {
        const TileScene R = queue_scene<T>(Q, S);
        const int i = (int)(S.first + threadIdx.x);
        force_one<T, true, Exact, Unit>(i, threadIdx.x < S.count, -1, A, R, s_row);
    }
}

template <int T, bool Exact, bool Unit>
void force_queue_launch(const ForceArgs& A, const BatchQueue& Q, cudaStream_t st) {
    static std::atomic<int> grid[kQueueMaxDevices];
    k_force_queue<T, Exact, Unit><<<queue_grid(k_force_queue<T, Exact, Unit>, T, grid), T, 0, st>>>(A, Q);
}

template <int T>
void force_queue_t(const ForceArgs& A, const BatchQueue& Q, bool unit, bool exact, cudaStream_t st) {
    if (exact)
        unit ? force_queue_launch<T, true, true>(A, Q, st) : force_queue_launch<T, true, false>(A, Q, st);
    else
        unit ? force_queue_launch<T, false, true>(A, Q, st) : force_queue_launch<T, false, false>(A, Q, st);
}

void launch_force_queue(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                        size_t mask_stride, const uint32_t* nbr, const uint32_t* cell_start,
                        const uint32_t* cell_end, uint32_t* idx, float4* pos_u, float4* vel_u, float4* veleval_u,
                        float4* keep_f, float4* keep_v, const BatchQueue& Q, bool unit, float dt, int exact,
                        int threads, cudaStream_t st) {
    const ForceArgs A{pos_s, rec_pd,  rec_vi, mask,      mask_stride, nbr,    cell_start, cell_end, nullptr,
                      nullptr, idx,   nullptr, pos_u,    vel_u,       veleval_u, keep_f, keep_v,     dt};
    if (threads == 64)
        force_queue_t<64>(A, Q, unit, exact != 0, st);
    else if (threads == 256)
        force_queue_t<256>(A, Q, unit, exact != 0, st);
    else
        force_queue_t<kForceThreads>(A, Q, unit, exact != 0, st);
}

void launch_force(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                  size_t mask_stride, const uint32_t* nbr, const uint32_t* cell_start, const uint32_t* cell_end, const int* info,
                  float4* force_s, float4* xsph_s, uint32_t* idx, const float4* vel_s, float4* pos_u, float4* vel_u,
                  float4* veleval_u, float4* keep_f, float4* keep_v, const StepParams& p, float dt, int fused,
                  int exact, int grid_items, int threads, cudaStream_t st, const uint32_t* cell_pre) {
    launch_force_t(pos_s, rec_pd, rec_vi, mask, mask_stride, nbr, cell_start, cell_end, info, force_s, xsph_s, idx, vel_s,
                   pos_u, vel_u, veleval_u, keep_f, keep_v, OneScene{p}, p.unit_scale != 0, dt, fused, exact,
                   grid_items, threads, st, cell_pre);
}

void launch_force_batch(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                        size_t mask_stride, const uint32_t* nbr, const uint32_t* cell_start, const uint32_t* cell_end, const int* info,
                        uint32_t* idx, float4* pos_u, float4* vel_u, float4* veleval_u, float4* keep_f,
                        float4* keep_v, const ManyScenes& scenes, bool unit, float dt, int exact, int grid_items,
                        int threads, cudaStream_t st, const uint32_t* cell_pre) {
    launch_force_t(pos_s, rec_pd, rec_vi, mask, mask_stride, nbr, cell_start, cell_end, info, nullptr, nullptr, idx,
                   nullptr, pos_u, vel_u, veleval_u, keep_f, keep_v, scenes, unit, dt, 1, exact, grid_items, threads,
                   st, cell_pre);
}

}  // namespace sphk
