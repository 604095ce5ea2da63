// sph_density.cu — density pass (rtpslib/system/sph/cl_src/density.cl:44-126,
// poly6 cl_sph_kernels.h:29-45).
//
// In exact mode density keeps the reference's summation order and rounding:
// it equals the FP32 oracle bit for bit.  Every multiply and add is a
// separately rounded scalar operation.  The default mode keeps the order but
// forms r^2 and the poly6 sum with fused multiply-adds, two instructions fewer
// per candidate in a loop that is instruction-issue bound; a neighbour on the
// cutoff may fall either side there, where its poly6 weight is ~0.  (Packed two-lane FP32 arithmetic was tried and rejected:
// with this compiler a packed multiply followed by a packed add does not give
// the separately rounded result, even with contraction disabled, which would
// change |r|^2 and with it the neighbour sets.)
//
// nbr gets every particle's neighbour count (itself included): the force
// pass's loop length.  The fused step's out-of-grid bookkeeping is its own
// kernel (sph_integrate.cu), so this pass reads no velocity.  veleval_s is optional too: without it the
// pass writes only the 1/rho lane of rec_vi, and the fused step's velocity
// kernel fills the veleval lanes beside it.
//
// While it tests the candidates the pass also records, per particle, which of
// its first kMaskBits candidates (in walk order) are neighbours (self
// excluded) as a bitmask, and the 32-byte record (position, rho),
// (veleval, 1/rho) the force pass reads for every neighbour.
#include <type_traits>

#include "sph_queue.cuh"
#include "sph_walk.cuh"

namespace sphk {

// The arrays of the density pass (pxy / pz: the default arithmetic's pairs).
struct DensityArgs {
    const float4* pos_s;
    const float4* pxy;
    const float2* pz;
    const float4* veleval_s;
    float* density;
    float4* rec_pd;
    float4* rec_vi;
    uint32_t* nbr;
    uint32_t* mask;
    size_t mstride;
    const uint32_t* cs0;
    const uint32_t* ce0;
    // sorted cell keys (the counting sort's), for the cell-pair pass; null
    // where the pass is not used
    const uint32_t* keys;
    // the counting sort's prefix of the cell counts (launch_cell_scan), for
    // the cell-pair pass's row runs; null: the runs from cs0 / ce0
    const uint32_t* pre;
};

// Sorted particle i, scalar candidates (every operation rounded on its own
// in exact arithmetic).
template <bool Exact, bool Unit, class Scenes>
__device__ __forceinline__ void density_one(const int i, const DensityArgs& A, const Scenes& R) {
    const float4* __restrict__ pos_s = A.pos_s;
    const float4* __restrict__ veleval_s = A.veleval_s;
    float* __restrict__ density = A.density;
    float4* __restrict__ rec_pd = A.rec_pd;
    float4* __restrict__ rec_vi = A.rec_vi;
    uint32_t* __restrict__ nbr = A.nbr;
    uint32_t* __restrict__ mask = A.mask;
    const size_t mstride = A.mstride;
    const uint32_t* __restrict__ cs0 = A.cs0;
    const uint32_t* __restrict__ ce0 = A.ce0;
    const StepParams& P = R.params(i);
    const uint32_t* cs = cs0 + R.cell_base(i);
    const uint32_t* ce = ce0 + R.cell_base(i);
    float4 pi = __ldg(pos_s + i);
    if (!Unit) pi = v4scale(pi, P.sc);
    if (R.frozen(i)) {
        density[i] = 0.f;
        rec_pd[i] = make_float4(pi.x, pi.y, pi.z, 0.f);
        if (veleval_s != nullptr)
            rec_vi[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        else
            reinterpret_cast<float*>(rec_vi + i)[3] = 0.f;
        nbr[i] = 0;
        return;
    }
    const float rc2 = P.rcut2, h2 = P.h2;
    float acc = 0.f;
    uint32_t cnt = 0;
    // bitmask: `cur` collects the bits of word p >> 5, p the walk position;
    // candidates are taken in chunks that end at a word boundary
    uint32_t cur = 0, p = 0;
    uint32_t* mrow = mask + i;
    // walk position of i itself (its bit is cleared when its word is stored,
    // instead of testing j != i for every candidate)
    uint32_t pself = 0xffffffffu;
    auto run = [&](uint32_t rs, uint32_t re) {
        if ((uint32_t)i - rs < re - rs) pself = p + ((uint32_t)i - rs);
        uint32_t j = rs;
        while (j < re) {
            const uint32_t b0 = p & 31u;
            uint32_t k = 32u - b0;
            if (k > re - j) k = re - j;
            const uint32_t jend = j + k;
            uint32_t bit = 1u << b0;
#pragma unroll 4
            for (; j < jend; ++j, bit <<= 1) {
                float4 q = __ldg(pos_s + j);
                if (!Unit) q = v4scale(q, P.sc);
                const float dx = __fsub_rn(pi.x, q.x), dy = __fsub_rn(pi.y, q.y), dz = __fsub_rn(pi.z, q.z);
                const float r2 = Exact ? dist2_exact(dx, dy, dz) : __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
                if (r2 <= rc2) {
                    const float hr2 = __fsub_rn(h2, r2);
                    acc = Exact ? __fadd_rn(acc, __fmul_rn(__fmul_rn(hr2, hr2), hr2))
                                : __fmaf_rn(__fmul_rn(hr2, hr2), hr2, acc);
                    ++cnt;
                    cur |= bit;
                }
            }
            p += k;
            if ((p & 31u) == 0) {
                const uint32_t w = (p >> 5) - 1;
                if (w == (pself >> 5)) cur &= ~(1u << (pself & 31u));
                if (w < (uint32_t)kMaskWords) mrow[(size_t)w * mstride] = cur;
                cur = 0;
            }
        }
    };
    const int3 c = grid_cell(pi.x, pi.y, pi.z, P.gs_min, P.gs_delta);
    if (cell_fast(P, c)) {
        if (A.pre != nullptr)
            walk_rows_prefix(P, A.pre + R.cell_base(i), c, run);
        else
            walk_rows_fast(P, cs, ce, c, run);
    } else {
        walk_rows_slow(P, cs, ce, c, run);
    }
    if ((p & 31u) != 0 && (p >> 5) < (uint32_t)kMaskWords) {
        if ((p >> 5) == (pself >> 5)) cur &= ~(1u << (pself & 31u));
        mrow[(size_t)(p >> 5) * mstride] = cur;
    }
    const float rho = __fmul_rn(P.dens_coef, acc);
    density[i] = rho;
    rec_pd[i] = make_float4(pi.x, pi.y, pi.z, rho);
    if (veleval_s != nullptr) {
        const float4 ve = __ldg(veleval_s + i);
        rec_vi[i] = make_float4(ve.x, ve.y, ve.z, __frcp_rn(rho));
    } else {
        reinterpret_cast<float*>(rec_vi + i)[3] = __frcp_rn(rho);
    }
    nbr[i] = cnt;
}

template <int T, bool Exact, bool Unit, class Scenes>
__global__ void __launch_bounds__(T) k_density(const DensityArgs A, const int* __restrict__ info, const Scenes R) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) density_one<Exact, Unit>(i, A, R);
}

// ---------------------------------------------------------------------------
// Default arithmetic, unit simulation scale: the same walk, candidates taken
// two at a time with Blackwell's two-lane FP32 instructions.  The sorted
// positions are also kept as pairs, pxy[k] = (x, x', y, y') and
// pz[k] = (z, z') of sorted particles 2k and 2k+1, so that the x, y and z of
// two candidates are one register pair each; one packed instruction forms
// both candidates' dx (dy, dz), r^2 takes three, the clamped weight
// (h^2 - r^2)^3 and its sum two more.  A run [rs, re) of sorted indices is
// walked as the pairs that hold it; the first and the last pair may hold one
// element outside the run, which takes no part (neither in the sum nor in
// the mask).  The density is the sum of the two lanes' partial sums: the
// summation order differs from the reference's, within the default mode's
// tolerance.  The neighbour bitmask is the one the scalar pass writes (bit b:
// the b-th candidate in walk order), built per segment of up to 16 pairs and
// appended to the word stream.
constexpr int kPairSegment = 16;  // pairs per mask segment (32 bits)

template <class Scenes>
__device__ __forceinline__ void density_pairs_one(const int i, const DensityArgs& A, const Scenes& R) {
    const float4* __restrict__ pos_s = A.pos_s;
    const float4* __restrict__ pxy = A.pxy;
    const float2* __restrict__ pz = A.pz;
    const float4* __restrict__ veleval_s = A.veleval_s;
    float* __restrict__ density = A.density;
    float4* __restrict__ rec_pd = A.rec_pd;
    float4* __restrict__ rec_vi = A.rec_vi;
    uint32_t* __restrict__ nbr = A.nbr;
    uint32_t* __restrict__ mask = A.mask;
    const size_t mstride = A.mstride;
    const uint32_t* __restrict__ cs0 = A.cs0;
    const uint32_t* __restrict__ ce0 = A.ce0;
    const StepParams& P = R.params(i);
    const uint32_t* cs = cs0 + R.cell_base(i);
    const uint32_t* ce = ce0 + R.cell_base(i);
    const float4 pi = __ldg(pos_s + i);
    if (R.frozen(i)) {
        density[i] = 0.f;
        rec_pd[i] = make_float4(pi.x, pi.y, pi.z, 0.f);
        if (veleval_s != nullptr)
            rec_vi[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        else
            reinterpret_cast<float*>(rec_vi + i)[3] = 0.f;
        nbr[i] = 0;
        return;
    }
    const float rc2 = P.rcut2;
    const float2 px = make_float2(pi.x, pi.x), py = make_float2(pi.y, pi.y), pzz = make_float2(pi.z, pi.z);
    const float2 h2 = make_float2(P.h2, P.h2), neg1 = make_float2(-1.f, -1.f);
    float2 acc = make_float2(0.f, 0.f);
    uint32_t cnt = 0;
    // word stream of the bitmask: `cur` holds `fill` bits of word `wo`
    uint32_t cur = 0, fill = 0, wo = 0;
    uint32_t* mrow = mask + i;
    auto append = [&](uint32_t v, uint32_t len) {  // len in [0, 32], v has no bits at or above len
        cur |= v << fill;
        if (fill + len >= 32u) {
            if (wo < (uint32_t)kMaskWords) mrow[(size_t)wo * mstride] = cur;
            ++wo;
            cur = fill ? (v >> (32u - fill)) : 0u;
            fill = fill + len - 32u;
        } else {
            fill += len;
        }
    };
    auto pair_of = [&](uint32_t k, bool v0, bool v1, uint32_t& seg, uint32_t bit) {
        const float4 xy = __ldg(pxy + k);
        const float2 zz = __ldg(pz + k);
        const float2 dx = __ffma2_rn(make_float2(xy.x, xy.y), neg1, px);
        const float2 dy = __ffma2_rn(make_float2(xy.z, xy.w), neg1, py);
        const float2 dz = __ffma2_rn(zz, neg1, pzz);
        const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
        float2 hr = __ffma2_rn(r2, neg1, h2);
        const bool n0 = v0 && r2.x <= rc2, n1 = v1 && r2.y <= rc2;
        hr.x = n0 ? hr.x : 0.f;
        hr.y = n1 ? hr.y : 0.f;
        acc = __ffma2_rn(__fmul2_rn(hr, hr), hr, acc);
        if (n0) seg |= bit;
        if (n1) seg |= bit << 1;
    };
    auto run = [&](uint32_t rs, uint32_t re) {
        const uint32_t kend = (re + 1u) >> 1;
        for (uint32_t ks = rs >> 1; ks < kend; ks += kPairSegment) {
            const uint32_t ke = ks + kPairSegment < kend ? ks + kPairSegment : kend;
            uint32_t seg = 0;
            uint32_t k = ks;
            // the run's first pair (its element 2k may precede rs)
            if (2u * k < rs) {
                pair_of(k, false, 2u * k + 1u < re, seg, 1u);
                ++k;
            }
            // inner pairs: both elements in the run
            const uint32_t kin = (2u * ke <= re) ? ke : ke - 1u;
#pragma unroll 2
            for (; k < kin; ++k) pair_of(k, true, true, seg, 1u << (2u * (k - ks)));
            // the run's last pair (its element 2k+1 may be re)
            if (k < ke) pair_of(k, true, 2u * k + 1u < re, seg, 1u << (2u * (k - ks)));
            cnt += (uint32_t)__popc(seg);
            const uint32_t e0 = 2u * ks;
            if ((uint32_t)i - e0 < 32u) seg &= ~(1u << ((uint32_t)i - e0));  // not itself
            const uint32_t lo = rs > e0 ? rs - e0 : 0u;
            const uint32_t hi = (re < 2u * ke ? re : 2u * ke) - e0;
            append(seg >> lo, hi - lo);
        }
    };
    const int3 c = grid_cell(pi.x, pi.y, pi.z, P.gs_min, P.gs_delta);
    if (cell_fast(P, c))
        walk_rows_fast(P, cs, ce, c, run);
    else
        walk_rows_slow(P, cs, ce, c, run);
    if (fill != 0 && wo < (uint32_t)kMaskWords) mrow[(size_t)wo * mstride] = cur;
    const float rho = P.dens_coef * (acc.x + acc.y);
    density[i] = rho;
    rec_pd[i] = make_float4(pi.x, pi.y, pi.z, rho);
    if (veleval_s != nullptr) {
        const float4 ve = __ldg(veleval_s + i);
        rec_vi[i] = make_float4(ve.x, ve.y, ve.z, __frcp_rn(rho));
    } else {
        reinterpret_cast<float*>(rec_vi + i)[3] = __frcp_rn(rho);
    }
    nbr[i] = cnt;
}

// One system: compiled for 1536 resident threads per SM (6 blocks of 256),
// 39 registers without spills instead of 48 (5 blocks): 1 % faster.  A
// batch's variant (scene lookups) stays unbounded (0).
template <int T, class Scenes>
__global__ void __launch_bounds__(T, (Scenes::kBatch ? 0 : 1536 / T))
    k_density_pairs(const DensityArgs A, const int* __restrict__ info, const Scenes R) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) density_pairs_one(i, A, R);
}

// ---------------------------------------------------------------------------
// Two particles of one cell per thread (default arithmetic, unit scale, one
// system, the step's counting sort).  Particles of one cell walk the same
// 9 row runs, so a thread that takes two of them loads each candidate pair
// once and runs the pair arithmetic for both: the loads, the loop and the
// row lookups, most of the pass's instructions, are paid once for two
// particles.  Each block takes T consecutive sorted particles and pairs them
// within their cells (the part of a cell inside the block's range: the
// particles at even rank from its first one, each with the next one when it
// lies in the same cell), compacts the pairs and the lone particles into its
// first threads, and every such thread runs the same walk, the second
// particle of a lone one switched off.  Each particle keeps its own sums,
// count and mask stream and meets its candidates in its own walk order with
// the pair alignment of density_pairs_one, so its results are those of
// density_pairs_one bit for bit.
struct CellPairLane {
    float2 px, py, pz;  // the particle's coordinates in both lanes
    float2 acc;         // poly6 sums of the even and the odd candidates
    uint32_t cnt;       // neighbours, itself included
    uint32_t cur;       // the mask word being filled (the item's stream position below)
    uint32_t self;      // its sorted index
};

// The two particles' mask word streams advance together (both walk the same
// candidates): `fill` bits of word `wo` are in each lane's `cur`.  Appends
// len bits of each (va, vb) and stores the words that fill up.
__device__ __forceinline__ void cellpair_append2(CellPairLane& La, CellPairLane& Lb, uint32_t& fill, uint32_t& wo,
                                                 uint32_t* __restrict__ mrow_a, uint32_t* __restrict__ mrow_b,
                                                 size_t mstride, uint32_t va, uint32_t vb, uint32_t len,
                                                 bool store_b) {
    La.cur |= va << fill;
    Lb.cur |= vb << fill;
    if (fill + len >= 32u) {
        if (wo < (uint32_t)kMaskWords) {
            mrow_a[(size_t)wo * mstride] = La.cur;
            if (store_b) mrow_b[(size_t)wo * mstride] = Lb.cur;
        }
        ++wo;
        La.cur = fill ? (va >> (32u - fill)) : 0u;
        Lb.cur = fill ? (vb >> (32u - fill)) : 0u;
        fill = fill + len - 32u;
    } else {
        fill += len;
    }
}

// One candidate pair (xy = (x, x', y, y'), zz = (z, z')) for one particle:
// the neighbour bits of both elements into seg, the weights into L.acc.
__device__ __forceinline__ void cellpair_pair(CellPairLane& L, const float4& xy, const float2& zz, bool v0, bool v1,
                                              float rc2, float2 h2, uint32_t& seg, uint32_t bit) {
    const float2 neg1 = make_float2(-1.f, -1.f);
    const float2 dx = __ffma2_rn(make_float2(xy.x, xy.y), neg1, L.px);
    const float2 dy = __ffma2_rn(make_float2(xy.z, xy.w), neg1, L.py);
    const float2 dz = __ffma2_rn(zz, neg1, L.pz);
    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
    float2 hr = __ffma2_rn(r2, neg1, h2);
    const bool n0 = v0 && r2.x <= rc2, n1 = v1 && r2.y <= rc2;
    hr.x = n0 ? hr.x : 0.f;
    hr.y = n1 ? hr.y : 0.f;
    L.acc = __ffma2_rn(__fmul2_rn(hr, hr), hr, L.acc);
    if (n0) seg |= bit;
    if (n1) seg |= bit << 1;
}

__device__ __forceinline__ void cellpair_finish(const CellPairLane& L, uint32_t fill, uint32_t wo, const float4& p,
                                                const DensityArgs& A, const StepParams& P,
                                                uint32_t* __restrict__ mrow) {
    const uint32_t i = L.self;
    if (fill != 0 && wo < (uint32_t)kMaskWords) mrow[(size_t)wo * A.mstride] = L.cur;
    const float rho = P.dens_coef * (L.acc.x + L.acc.y);
    A.density[i] = rho;
    A.rec_pd[i] = make_float4(p.x, p.y, p.z, rho);
    if (A.veleval_s != nullptr) {
        const float4 ve = __ldg(A.veleval_s + i);
        A.rec_vi[i] = make_float4(ve.x, ve.y, ve.z, __frcp_rn(rho));
    } else {
        reinterpret_cast<float*>(A.rec_vi + i)[3] = __frcp_rn(rho);
    }
    A.nbr[i] = L.cnt;
}

// Sorted particles a and, when has_b, a + 1 of the same cell (of one scene).
template <class Scenes>
__device__ __forceinline__ void density_cellpair(const uint32_t a, const bool has_b, const DensityArgs& A,
                                                 const Scenes& R) {
    const StepParams& P = R.params((int)a);
    const float4 pa = __ldg(A.pos_s + a);
    const int3 c = grid_cell(pa.x, pa.y, pa.z, P.gs_min, P.gs_delta);
    if (R.frozen((int)a) || !cell_fast(P, c)) {
        density_pairs_one((int)a, A, R);
        if (has_b) density_pairs_one((int)a + 1, A, R);
        return;
    }
    const float4 pb = has_b ? __ldg(A.pos_s + a + 1) : pa;
    const uint32_t* __restrict__ cs = A.cs0 + R.cell_base((int)a);
    const uint32_t* __restrict__ ce = A.ce0 + R.cell_base((int)a);
    const uint32_t* __restrict__ pre = A.pre != nullptr ? A.pre + R.cell_base((int)a) : nullptr;
    const float4* __restrict__ pxy = A.pxy;
    const float2* __restrict__ pz = A.pz;
    const uint32_t C = (uint32_t)P.nb_cells;
    const float rc2 = P.rcut2;
    const float2 h2 = make_float2(P.h2, P.h2);
    CellPairLane La, Lb;
    La.px = make_float2(pa.x, pa.x), La.py = make_float2(pa.y, pa.y), La.pz = make_float2(pa.z, pa.z);
    Lb.px = make_float2(pb.x, pb.x), Lb.py = make_float2(pb.y, pb.y), Lb.pz = make_float2(pb.z, pb.z);
    La.acc = Lb.acc = make_float2(0.f, 0.f);
    La.cnt = Lb.cnt = 0;
    La.cur = Lb.cur = 0;
    uint32_t fill = 0, wo = 0;  // the mask word streams' position
    La.self = a;
    Lb.self = a + 1u;
    uint32_t* mrow_a = A.mask + a;
    uint32_t* mrow_b = mrow_a + 1;
    const size_t ms = A.mstride;
#pragma unroll 1
    for (int dz = -1; dz <= 1; ++dz) {
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            const int base = ((c.z + dz) * P.res_y + (c.y + dy)) * P.res_x + c.x;
            uint32_t rs, re;
            if (pre != nullptr) {
                // the row's cells base-1 .. base+1 within the grid: two loads
                const int lo = base - 1 < 0 ? 0 : base - 1;
                const int hi = base + 1 > (int)C - 1 ? (int)C - 1 : base + 1;
                if (lo > hi) continue;
                rs = __ldg(pre + lo);
                re = __ldg(pre + hi + 1);
                if (rs >= re) continue;
            } else {
                uint32_t last = 0;
                rs = kEmpty;
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx) {
                    const uint32_t h = (uint32_t)(base + dx);
                    if (h < C) {
                        const uint32_t s0 = __ldg(cs + h);
                        if (s0 != kEmpty) {
                            if (rs == kEmpty) rs = s0;
                            last = h;
                        }
                    }
                }
                if (rs == kEmpty) continue;
                re = __ldg(ce + last);
            }
            if (!run_ok(P, rs, re)) continue;  // bounds-checked builds
            const uint32_t kend = (re + 1u) >> 1;
            for (uint32_t ks = rs >> 1; ks < kend; ks += kPairSegment) {
                const uint32_t ke = ks + kPairSegment < kend ? ks + kPairSegment : kend;
                uint32_t sa = 0, sb = 0;
                uint32_t k = ks;
                if (2u * k < rs) {  // the run's first pair (its element 2k precedes rs)
                    const float4 xy = __ldg(pxy + k);
                    const float2 zz = __ldg(pz + k);
                    const bool v1 = 2u * k + 1u < re;
                    cellpair_pair(La, xy, zz, false, v1, rc2, h2, sa, 1u);
                    cellpair_pair(Lb, xy, zz, false, v1, rc2, h2, sb, 1u);
                    ++k;
                }
                const uint32_t kin = (2u * ke <= re) ? ke : ke - 1u;
                uint32_t bit = 1u << (2u * (k - ks));  // bit of pair k's first element in sa / sb
#pragma unroll 2
                for (; k < kin; ++k, bit <<= 2) {
                    const float4 xy = __ldg(pxy + k);
                    const float2 zz = __ldg(pz + k);
                    cellpair_pair(La, xy, zz, true, true, rc2, h2, sa, bit);
                    cellpair_pair(Lb, xy, zz, true, true, rc2, h2, sb, bit);
                }
                if (k < ke) {  // the run's last pair (its element 2k+1 may be re)
                    const float4 xy = __ldg(pxy + k);
                    const float2 zz = __ldg(pz + k);
                    const bool v1 = 2u * k + 1u < re;
                    cellpair_pair(La, xy, zz, true, v1, rc2, h2, sa, bit);
                    cellpair_pair(Lb, xy, zz, true, v1, rc2, h2, sb, bit);
                }
                const uint32_t e0 = 2u * ks;
                const uint32_t lo = rs > e0 ? rs - e0 : 0u;
                const uint32_t hi = (re < 2u * ke ? re : 2u * ke) - e0;
                La.cnt += (uint32_t)__popc(sa);
                Lb.cnt += (uint32_t)__popc(sb);
                if (a - e0 < 32u) sa &= ~(1u << (a - e0));
                if (a + 1u - e0 < 32u) sb &= ~(1u << (a + 1u - e0));
                cellpair_append2(La, Lb, fill, wo, mrow_a, mrow_b, ms, sa >> lo, sb >> lo, hi - lo, has_b);
            }
        }
    }
    cellpair_finish(La, fill, wo, pa, A, P, mrow_a);
    if (has_b) cellpair_finish(Lb, fill, wo, pb, A, P, mrow_b);
}

// Particles per block of the cell-pair pass: about two per thread, less the
// lone particles a block's range holds at 8 to 12 particles per cell, so that
// the items (pairs and lone particles) about fill the block's threads.
template <int T>
constexpr int cellpair_chunk() {
    return T * 7 / 4;
}

// Block b takes sorted particles [bC, bC + C): the particle at an even rank
// of its cell's part in that range starts an item (with the next particle
// when it is in the same cell and the range); the items are compacted in
// order and the block's threads take them in turn.
// Index into the cell arrays of sorted key `key` (a batch: the scene's
// segment of them).
__device__ __forceinline__ uint32_t key_cell(const OneScene&, uint32_t key) { return key; }
__device__ __forceinline__ uint32_t key_cell(const ManyScenes& R, uint32_t key) {
    return __ldg(R.cbase + (key >> R.cell_bits)) + (key & ((1u << R.cell_bits) - 1u));
}

template <int T, class Scenes>
__global__ void __launch_bounds__(T, 1024 / T) k_density_cellpairs(const DensityArgs A, const int* __restrict__ info,
                                                         const Scenes R) {
    constexpr int Cp = cellpair_chunk<T>();
    __shared__ uint32_t s_item[Cp];
    __shared__ uint32_t s_warp[2][T / 32];
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int base = blockIdx.x * Cp;
    if (base >= n) return;  // the whole block
    const int end = base + Cp < n ? base + Cp : n;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // item flags of the block's particles base + tid and base + T + tid
    bool start[2], has_b[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int p = base + h * T + (int)threadIdx.x;
        start[h] = has_b[h] = false;
        if (p < end) {
            const uint32_t key = __ldg(A.keys + p);
            const uint32_t cs = __ldg(A.cs0 + key_cell(R, key));
            const uint32_t first = cs > (uint32_t)base ? cs : (uint32_t)base;  // the cell's first particle in range
            start[h] = (((uint32_t)p - first) & 1u) == 0u;
            has_b[h] = start[h] && p + 1 < end && __ldg(A.keys + p + 1) == key;
        }
    }
    unsigned bal[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        bal[h] = __ballot_sync(0xffffffffu, start[h]);
        if (lane == 0) s_warp[h][warp] = (uint32_t)__popc(bal[h]);
    }
    __syncthreads();
    uint32_t before0 = 0, total0 = 0, before1 = 0, total1 = 0;
#pragma unroll
    for (int w = 0; w < T / 32; ++w) {
        const uint32_t c0 = s_warp[0][w], c1 = s_warp[1][w];
        before0 += (unsigned)w < warp ? c0 : 0u;
        before1 += (unsigned)w < warp ? c1 : 0u;
        total0 += c0;
        total1 += c1;
    }
    const uint32_t below = (1u << lane) - 1u;
    if (start[0])
        s_item[before0 + (uint32_t)__popc(bal[0] & below)] =
            (uint32_t)(base + (int)threadIdx.x) | (has_b[0] ? 0x80000000u : 0u);
    if (start[1])
        s_item[total0 + before1 + (uint32_t)__popc(bal[1] & below)] =
            (uint32_t)(base + T + (int)threadIdx.x) | (has_b[1] ? 0x80000000u : 0u);
    __syncthreads();
    const uint32_t total = total0 + total1;
    for (uint32_t t = threadIdx.x; t < total; t += T) {
        const uint32_t it = s_item[t];
        density_cellpair(it & 0x7fffffffu, (it >> 31) != 0u, A, R);
    }
}

// Sorted positions as pairs (see k_density_pairs), for the passes whose
// permute does not write them.
__global__ void k_pack_pairs(const float4* __restrict__ pos_s, float4* __restrict__ pxy, float2* __restrict__ pz,
                             const int* __restrict__ info) {
    const int n = info[kNum];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (2 * k >= n) return;
    const float4 a = __ldg(pos_s + 2 * k);
    const float4 b = 2 * k + 1 < n ? __ldg(pos_s + 2 * k + 1) : make_float4(kFarAway, kFarAway, kFarAway, 1.f);
    pxy[k] = make_float4(a.x, b.x, a.y, b.y);
    pz[k] = make_float2(a.z, b.z);
}

template <int T, class Scenes>
void launch_density_tt(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd, float4* rec_vi,
                       uint32_t* nbr, uint32_t* mask, size_t mask_stride, const uint32_t* cell_start,
                       const uint32_t* cell_end, const int* info, const Scenes& R, bool unit, bool exact,
                       int grid_items, float4* pxy, float2* pz, bool pack, cudaStream_t st,
                       const uint32_t* keys, const uint32_t* cell_pre = nullptr) {
    int blocks = (grid_items + T - 1) / T;
    if (blocks < 1) blocks = 1;
    const DensityArgs A{pos_s, pxy, pz, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start,
                        cell_end, keys, cell_pre};
    if (pxy != nullptr && pz != nullptr && unit && !exact) {
        if (pack) {
            const int pb = ((grid_items + 1) / 2 + 255) / 256;
            k_pack_pairs<<<pb < 1 ? 1 : pb, 256, 0, st>>>(pos_s, pxy, pz, info);
        }
        if (A.keys != nullptr) {
            const int cp_blocks = (grid_items + cellpair_chunk<T>() - 1) / cellpair_chunk<T>();
            k_density_cellpairs<T, Scenes><<<cp_blocks < 1 ? 1 : cp_blocks, T, 0, st>>>(A, info, R);
            return;
        }
        k_density_pairs<T, Scenes><<<blocks, T, 0, st>>>(A, info, R);
        return;
    }
#define SPH_DENSITY_LAUNCH(E, U) k_density<T, E, U, Scenes><<<blocks, T, 0, st>>>(A, info, R)
    if (exact) {
        if (unit) SPH_DENSITY_LAUNCH(true, true); else SPH_DENSITY_LAUNCH(true, false);
    } else {
        if (unit) SPH_DENSITY_LAUNCH(false, true); else SPH_DENSITY_LAUNCH(false, false);
    }
#undef SPH_DENSITY_LAUNCH
}

// The density pass with `threads` threads per block (128, 256 or 512: the
// same results bit for bit, a launch shape the autotuner picks).
template <class Scenes>
void launch_density_t(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd, float4* rec_vi,
                      uint32_t* nbr, uint32_t* mask, size_t mask_stride, const uint32_t* cell_start,
                      const uint32_t* cell_end, const int* info, const Scenes& R, bool unit, bool exact,
                      int grid_items, float4* pxy, float2* pz, bool pack, int threads, cudaStream_t st,
                      const uint32_t* keys = nullptr, const uint32_t* cell_pre = nullptr) {
    switch (threads) {
        case 128:
            launch_density_tt<128>(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start,
                                   cell_end, info, R, unit, exact, grid_items, pxy, pz, pack, st, keys, cell_pre);
            break;
        case 512:
            launch_density_tt<512>(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start,
                                   cell_end, info, R, unit, exact, grid_items, pxy, pz, pack, st, keys, cell_pre);
            break;
        default:
            launch_density_tt<256>(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start,
                                   cell_end, info, R, unit, exact, grid_items, pxy, pz, pack, st, keys, cell_pre);
    }
}

// The batch's density pass under the queue scheduler (sph_queue.cuh): the
// same per-particle work as k_density_pairs / k_density, scene by scene.
template <int T, bool Pairs, bool Exact, bool Unit>
__global__ void __launch_bounds__(T) k_density_queue(const DensityArgs A, const BatchQueue Q) {
    __shared__ QueueShared<T> S;
    if (!queue_start<T>(Q, S)) return;
    while (queue_next<T>(Q, S)) {
        const TileScene R = queue_scene<T>(Q, S);
        if (threadIdx.x < S.count) {
            const int i = (int)(S.first + threadIdx.x);
            if constexpr (Pairs)
                density_pairs_one(i, A, R);
            else
                density_one<Exact, Unit>(i, A, R);
        }
    }
}

template <int T, bool Pairs, bool Exact, bool Unit>
void density_queue_launch(const DensityArgs& A, const BatchQueue& Q, cudaStream_t st) {
    static std::atomic<int> grid[kQueueMaxDevices];
    k_density_queue<T, Pairs, Exact, Unit>
        <<<queue_grid(k_density_queue<T, Pairs, Exact, Unit>, T, grid), T, 0, st>>>(A, Q);
}

template <int T>
void density_queue_t(const DensityArgs& A, const BatchQueue& Q, bool unit, bool exact, cudaStream_t st) {
    if (unit && !exact && A.pxy != nullptr)
        density_queue_launch<T, true, false, true>(A, Q, st);
    else if (exact)
        unit ? density_queue_launch<T, false, true, true>(A, Q, st) : density_queue_launch<T, false, true, false>(A, Q, st);
    else
        unit ? density_queue_launch<T, false, false, true>(A, Q, st)
             : density_queue_launch<T, false, false, false>(A, Q, st);
}

void launch_density_queue(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd,
                          float4* rec_vi, uint32_t* nbr, uint32_t* mask, size_t mask_stride,
                          const uint32_t* cell_start, const uint32_t* cell_end, float4* pxy, float2* pz,
                          const BatchQueue& Q, bool unit, int exact, int threads, cudaStream_t st) {
    const DensityArgs A{pos_s, pxy, pz, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start,
                        cell_end};
    if (threads == 128)
        density_queue_t<128>(A, Q, unit, exact != 0, st);
    else if (threads == 512)
        density_queue_t<512>(A, Q, unit, exact != 0, st);
    else
        density_queue_t<256>(A, Q, unit, exact != 0, st);
}

void launch_density(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd, float4* rec_vi,
                    uint32_t* nbr, uint32_t* mask, size_t mask_stride, const uint32_t* cell_start,
                    const uint32_t* cell_end, const int* info, const StepParams& p, int grid_items, float4* pxy,
                    float2* pz, bool pack, int threads, cudaStream_t st, const uint32_t* keys,
                    const uint32_t* cell_pre) {
    launch_density_t(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start, cell_end, info,
                     OneScene{p}, p.unit_scale != 0, p.exact != 0, grid_items, pxy, pz, pack, threads, st, keys,
                     cell_pre);
}

void launch_density_batch(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd,
                          float4* rec_vi, uint32_t* nbr, uint32_t* mask, size_t mask_stride,
                          const uint32_t* cell_start, const uint32_t* cell_end, const int* info,
                          const ManyScenes& scenes, bool unit, int exact, int grid_items, float4* pxy, float2* pz,
                          bool pack, int threads, cudaStream_t st, const uint32_t* cell_pre) {
    // the batch's sort leaves every particle's (scene, cell) key in scenes.keys
    launch_density_t(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start, cell_end, info,
                     scenes, unit, exact != 0, grid_items, pxy, pz, pack, threads, st, scenes.keys, cell_pre);
}

}  // namespace sphk
