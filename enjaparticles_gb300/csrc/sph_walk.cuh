// sph_walk.cuh — the neighbour walk shared by the density and force passes
// (rtpslib/system/sph/cl_src/cl_sph_neighbors.h:49-140).
//
// The reference visits 27 cells (z, y, x in [c-1, c+1]) and each cell's
// sorted range.  Keys of the three cells x-1, x, x+1 of one row are
// consecutive integers, so their particles are one contiguous run of the
// sorted arrays: the walk here is 9 row runs, visited in the reference's
// order.  Integer row hashing equals the reference's float hash formula
// whenever every intermediate value is an integer below 2^24 in magnitude
// (checked on the host: int_hash_ok); otherwise each of the 27 cells is
// hashed with the float formula.
//
// Cutoff.  |r| <= h with |r| = sqrtf(r2) is the same test as r2 <= rcut2,
// rcut2 being the largest float whose correctly rounded square root is <= h
// (sqrt is monotonic); r2 is formed without contraction, so neighbour sets
// are identical to the oracle's.
#pragma once

#include <climits>

#include "sph_physics.cuh"

namespace sphk {

// A run [rs, re) of sorted indices: non-empty and inside the particle arrays
// (bounds-checked builds; always true otherwise).
__device__ __forceinline__ bool run_ok(const StepParams& P, uint32_t rs, uint32_t re) {
    return in_bounds(rs, re, P.chk_err) && in_bounds(re - 1u, P.chk_cap, P.chk_err);
}

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
            if (rs != kEmpty) {
                const uint32_t re = __ldg(ce + last);
                if (run_ok(P, rs, re)) f(rs, re);
            }
        }
    }
}

// The same 9 row runs as walk_rows_fast, in the same order, with every
// cell_start load of the 27 cells issued before any is used and the 9
// cell_end loads issued together after them: two memory round trips instead
// of two per row, for callers that do little per run (the force pass only
// records the runs).
template <class F>
__device__ __forceinline__ void walk_rows_fast_batched(const StepParams& P, const uint32_t* __restrict__ cs,
                                                       const uint32_t* __restrict__ ce, const int3& c, F&& f) {
    const uint32_t C = (uint32_t)P.nb_cells;
    uint32_t s[27];
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const int base = ((c.z + r / 3 - 1) * P.res_y + (c.y + r % 3 - 1)) * P.res_x + c.x;
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
            const uint32_t h = (uint32_t)(base + dx - 1);
            s[3 * r + dx] = h < C ? __ldg(cs + h) : kEmpty;
        }
    }
    uint32_t rs[9], re[9];
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const int base = ((c.z + r / 3 - 1) * P.res_y + (c.y + r % 3 - 1)) * P.res_x + c.x;
        rs[r] = kEmpty;
        uint32_t last = 0;
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
            if (s[3 * r + dx] != kEmpty) {
                if (rs[r] == kEmpty) rs[r] = s[3 * r + dx];
                last = (uint32_t)(base + dx - 1);
            }
        }
        re[r] = rs[r] != kEmpty ? __ldg(ce + last) : 0u;
    }
#pragma unroll
    for (int r = 0; r < 9; ++r)
        if (rs[r] != kEmpty && run_ok(P, rs[r], re[r])) f(rs[r], re[r]);
}

// The same 9 row runs from the exclusive prefix of the cell counts (pre[k]:
// sorted particles with a key below k, k = 0..C): the row's cells lo..hi
// (base - 1 .. base + 1 within the grid) hold sorted particles
// pre[lo] .. pre[hi + 1] - 1, empty cells included, so each run is two loads.
template <class F>
__device__ __forceinline__ void walk_rows_prefix(const StepParams& P, const uint32_t* __restrict__ pre, const int3& c,
                                                 F&& f) {
    const int C = P.nb_cells;
    uint32_t rs[9], re[9];
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const int base = ((c.z + r / 3 - 1) * P.res_y + (c.y + r % 3 - 1)) * P.res_x + c.x;
        const int lo = base - 1 < 0 ? 0 : base - 1;
        const int hi = base + 1 > C - 1 ? C - 1 : base + 1;
        rs[r] = lo <= hi ? __ldg(pre + lo) : 0u;
        re[r] = lo <= hi ? __ldg(pre + hi + 1) : 0u;
    }
#pragma unroll
    for (int r = 0; r < 9; ++r)
        if (rs[r] < re[r] && run_ok(P, rs[r], re[r])) f(rs[r], re[r]);
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
                if (s != kEmpty) {
                    const uint32_t e = __ldg(ce + h);
                    if (run_ok(P, s, e)) f(s, e);
                }
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

}  // namespace sphk
