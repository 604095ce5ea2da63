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
// nbr (neighbour counts) is optional: the fused step leaves it out.  The
// fused step's out-of-grid bookkeeping is its own kernel (sph_integrate.cu),
// so this pass reads no velocity.  veleval_s is optional too: without it the
// pass writes only the 1/rho lane of rec_vi, and the fused step's velocity
// kernel fills the veleval lanes beside it.
//
// While it tests the candidates the pass also records, per particle, which of
// its first kMaskBits candidates (in walk order) are neighbours (self
// excluded) as a bitmask, and the 32-byte record (position, rho),
// (veleval, 1/rho) the force pass reads for every neighbour.
#include "sph_walk.cuh"

namespace sphk {

template <bool Exact, bool Unit, bool WantCount, class Scenes>
__global__ void __launch_bounds__(256) k_density(const float4* __restrict__ pos_s, const float4* __restrict__ veleval_s,
                                                 float* __restrict__ density, float4* __restrict__ rec_pd,
                                                 float4* __restrict__ rec_vi, uint32_t* __restrict__ nbr,
                                                 uint32_t* __restrict__ mask, const size_t mstride,
                                                 const uint32_t* __restrict__ cs0, const uint32_t* __restrict__ ce0,
                                                 const int* __restrict__ info, const Scenes R) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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
        if (WantCount) nbr[i] = 0;
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
                    if (WantCount) ++cnt;
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
    if (cell_fast(P, c))
        walk_rows_fast(P, cs, ce, c, run);
    else
        walk_rows_slow(P, cs, ce, c, run);
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
    if (WantCount) nbr[i] = cnt;
}

template <class Scenes>
void launch_density_t(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd, float4* rec_vi,
                      uint32_t* nbr, uint32_t* mask, size_t mask_stride, const uint32_t* cell_start,
                      const uint32_t* cell_end, const int* info, const Scenes& R, bool unit, bool exact,
                      int grid_items, cudaStream_t st) {
    const int threads = 256;
    int blocks = (grid_items + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
#define SPH_DENSITY_LAUNCH(E, U, W)                                                                               \
    k_density<E, U, W, Scenes><<<blocks, threads, 0, st>>>(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, \
                                                           mask_stride, cell_start, cell_end, info, R)
#define SPH_DENSITY_LAUNCH_E(E)                                                                \
    if (unit) {                                                                                \
        if (nbr) SPH_DENSITY_LAUNCH(E, true, true); else SPH_DENSITY_LAUNCH(E, true, false);   \
    } else {                                                                                   \
        if (nbr) SPH_DENSITY_LAUNCH(E, false, true); else SPH_DENSITY_LAUNCH(E, false, false); \
    }
    if (exact) {
        SPH_DENSITY_LAUNCH_E(true)
    } else {
        SPH_DENSITY_LAUNCH_E(false)
    }
#undef SPH_DENSITY_LAUNCH_E
#undef SPH_DENSITY_LAUNCH
}

void launch_density(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd, float4* rec_vi,
                    uint32_t* nbr, uint32_t* mask, size_t mask_stride, const uint32_t* cell_start,
                    const uint32_t* cell_end, const int* info, const StepParams& p, int grid_items, cudaStream_t st) {
    launch_density_t(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start, cell_end, info,
                     OneScene{p}, p.unit_scale != 0, p.exact != 0, grid_items, st);
}

void launch_density_batch(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd,
                          float4* rec_vi, uint32_t* nbr, uint32_t* mask, size_t mask_stride,
                          const uint32_t* cell_start, const uint32_t* cell_end, const int* info,
                          const ManyScenes& scenes, bool unit, int exact, int grid_items, cudaStream_t st) {
    launch_density_t(pos_s, veleval_s, density, rec_pd, rec_vi, nbr, mask, mask_stride, cell_start, cell_end, info,
                     scenes, unit, exact != 0, grid_items, st);
}

}  // namespace sphk
