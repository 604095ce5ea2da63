// sph_surface.cu — the post-process of SPH::postProcess (SPH.cpp:338-386),
// headless: the colour field (sph/cl_src/colorfield.cl, ColorField.cpp) and
// its marching-cubes surface (common/MarchingCubes.cpp with
// common/cl_src/classifycubes.cl, constructhp.cl, traversehp.cl) as device
// buffers.
//
// Colour field.  One thread per sample point of a res^3 lattice spanning the
// scaled grid's bounds; the 27-cell walk of the density pass; per particle
// within h, Wspiky(max(|r|, EPSILON)) / rho_j, the reciprocal and product in
// double as the reference's double literal makes them; times mass.  In exact
// mode every operation is the reference's, explicitly rounded: the field
// equals the oracle's bit for bit; the default mode forms the product in
// float.  It is stored linearly (s + t res + r res^2) where the
// reference tiles z slices into a 2-D image; the reference's tiling holds
// all slices only up to res = 64.
//
// Marching cubes.  The reference builds a histopyramid over its 2-D image
// and lets one work-item per triangle walk down it.  Here three kernels do
// the same job with a scan: classify every cube and sum the triangle counts
// per block; scan the block sums; classify again, scan within the block and
// write each cube's triangles at its offset.  The cubes are taken in the
// order the reference's pyramid walk emits them (Morton order over its
// slice-tiled image), so the triangle list lines up with the reference's
// cube by cube.
// What the reference computes per triangle vertex is kept exactly:
//   - the case index from the 8 corners (value > isolevel) in the
//     reference's corner order (classifycubes.cl);
//   - each vertex interpolated along the cube's local edge in the
//     direction of the reference's edge list (offsets3 of traversehp.cl: four
//     edges run against the axes, so a shared edge can round differently in
//     neighbouring cubes, as in the reference);
//   - the values interpolated are the pyramid base level's corner values,
//     which the reference writes only for corners of cubes (coordinates below
//     res - 1): corners on the last layer read 0 there, as in the reference;
//   - the normal: central differences of those values, a neighbour outside
//     the lattice replaced by the point itself (map3Dto2DClamp), mixed along
//     the edge and normalised as v * (1 / sqrt(v.v));
//   - positions scaled to the reference's render box: p / (res - 1) * 10.
//   - the triangles of each case, in order: the reference's case table
//     (traversehp.cl:74), carried in sph_mc_table.inc; it decides which
//     diagonal splits a quad or pentagon, so the triangle list equals the
//     reference's triangle for triangle.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "sph_ctx.cuh"
#include "sph_walk.cuh"

namespace {

constexpr int kMcMaxTriEdges = 18;  // up to 6 triangles per case
// Corner k of the case index: bit k (classifycubes.cl:38-47 with cubeOffsets
// of indexmap.h:28-37).
constexpr int kMcCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
// Local edges as (point0 corner, point1 corner): the reference's edge list
// and interpolation direction (traversehp.cl:35-72).
constexpr int kMcEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

struct McTable {
    signed char tri[256][kMcMaxTriEdges];
    unsigned char count[256];
    int max_count;
};

#include "sph_mc_table.inc"

// The case table unpacked: the triangles of case cs as edge numbers, the
// triangle count, the largest count.
const McTable& mc_table() {
    static McTable T = [] {
        McTable t;
        std::memset(t.tri, -1, sizeof(t.tri));
        std::memset(t.count, 0, sizeof(t.count));
        t.max_count = 0;
        for (int cs = 0; cs < 256; ++cs) {
            const unsigned long long w = kMcCasePacked[cs];
            const int nt = (int)((w >> 60) & 7u);
            for (int e = 0; e < 3 * nt; ++e) t.tri[cs][e] = (signed char)((w >> (4 * e)) & 15u);
            t.count[cs] = (unsigned char)nt;
            t.max_count = std::max(t.max_count, nt);
        }
        return t;
    }();
    return T;
}

}  // namespace

namespace sphk {
namespace {

constexpr int kSurfThreads = 256;
__constant__ int kMcCornerDev[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1},
                                       {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
__constant__ int kMcEdgeDev[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                      {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

__device__ __forceinline__ float wspiky_f(float alpha, float h, float rlen) {
    const float hr = __fsub_rn(h, rlen);
    return __fmul_rn(__fmul_rn(__fmul_rn(alpha, hr), hr), hr);
}

// 1/rho_j in double, once per particle: the value the reference's
// (1.0 / density[j]) forms for every pair.
__global__ void __launch_bounds__(kSurfThreads) k_inv_density(const float* __restrict__ density, int n,
                                                              double* __restrict__ inv) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) inv[j] = __ddiv_rn(1.0, (double)__ldg(density + j));
}

// Work split: warps take 32 consecutive samples (one row piece, so their
// neighbour runs mostly coincide), but chunk c goes to warp (c * stride) mod
// chunks with stride coprime to the chunk count, so that every block mixes
// chunks from the whole lattice: samples inside the fluid, which carry all
// the work, would otherwise sit in a few blocks.
//
// The cutoff |r| <= h is tested as r^2 <= rcut2 (the same test, as in the
// density pass); the square root is taken for neighbours only.  Exact: the
// reference's double product W * (1/rho_j), rounded to float, with 1/rho_j
// from k_inv_density (the double pipe bounds this mode).  Default: the
// product in float with the float 1/rho_j the density pass stored in
// rec_vi.w, within a few ulps of the exact term.
template <bool Exact>
__global__ void __launch_bounds__(kSurfThreads) k_colorfield(float* __restrict__ field, int res,
                                                             unsigned long long chunks, unsigned long long stride,
                                                             const float4* __restrict__ pos_s,
                                                             const double* __restrict__ inv_rho,
                                                             const float4* __restrict__ rec_vi,
                                                             const uint32_t* __restrict__ cs,
                                                             const uint32_t* __restrict__ ce, const StepParams P) {
    const long long total = (long long)res * res * res;
    const unsigned long long gw = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw >= chunks) return;
    const long long k = (long long)(((gw * stride) % chunks) * 32ull + (threadIdx.x & 31));
    if (k >= total) return;
    const int s = (int)(k % res), t = (int)((k / res) % res), r = (int)(k / ((long long)res * res));
    const float tmp = __fdiv_rn(1.0f, (float)(unsigned)(res - 1));
    const float px =
        __fadd_rn(__fmul_rn(__fmul_rn((float)(unsigned)s, tmp), __fsub_rn(P.gs_bnd_max.x, P.gs_bnd_min.x)), P.gs_bnd_min.x);
    const float py =
        __fadd_rn(__fmul_rn(__fmul_rn((float)(unsigned)t, tmp), __fsub_rn(P.gs_bnd_max.y, P.gs_bnd_min.y)), P.gs_bnd_min.y);
    const float pz =
        __fadd_rn(__fmul_rn(__fmul_rn((float)(unsigned)r, tmp), __fsub_rn(P.gs_bnd_max.z, P.gs_bnd_min.z)), P.gs_bnd_min.z);
    const float h = P.h, eps = P.eps;
    const float h6 = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(h, h), h), h), h), h);
    const float alpha = __fdiv_rn(__fdiv_rn(15.f, 3.14159265358979323846f), h6);
    float acc = 0.f;
    walk_rows(P, cs, ce, px, py, pz, [&](uint32_t rs, uint32_t re) {
        for (uint32_t j = rs; j < re; ++j) {
            float4 q = __ldg(pos_s + j);
            if (!P.unit_scale) q = v4scale(q, P.sc);
            const float r2 = dist2_exact(__fsub_rn(px, q.x), __fsub_rn(py, q.y), __fsub_rn(pz, q.z));
            if (r2 <= P.rcut2) {
                float rlen = __fsqrt_rn(r2);
                rlen = rlen < eps ? eps : rlen;
                const float w = wspiky_f(alpha, h, rlen);
                if (Exact)
                    acc = __fadd_rn(acc, __double2float_rn(__dmul_rn((double)w, __ldg(inv_rho + j))));
                else
                    acc = __fadd_rn(acc, __fmul_rn(w, __ldg(&rec_vi[j].w)));
            }
        }
    });
    field[k] = __fmul_rn(acc, P.mass);
}

struct McDev {
    const signed char* tri;      // [256][kMcMaxTriEdges]
    const unsigned char* count;  // [256]
};

__device__ __forceinline__ int mc_case(const float* __restrict__ f, int res, int x, int y, int z, float iso) {
    const size_t sx = 1, sy = (size_t)res, sz = (size_t)res * res;
    const size_t b = (size_t)x + (size_t)y * sy + (size_t)z * sz;
    return (int)(__ldg(f + b) > iso) | ((int)(__ldg(f + b + sx) > iso) << 1) |
           ((int)(__ldg(f + b + sx + sz) > iso) << 2) | ((int)(__ldg(f + b + sz) > iso) << 3) |
           ((int)(__ldg(f + b + sy) > iso) << 4) | ((int)(__ldg(f + b + sx + sy) > iso) << 5) |
           ((int)(__ldg(f + b + sx + sy + sz) > iso) << 6) | ((int)(__ldg(f + b + sy + sz) > iso) << 7);
}

// Block-wide exclusive scan of v (kSurfThreads threads); *sum gets the total.
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* sh, unsigned* sum) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    unsigned off = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kSurfThreads / 32; ++w) {
        const unsigned c = sh[w];
        off += w < warp ? c : 0u;
        tot += c;
    }
    __syncthreads();
    *sum = tot;
    return off + x - v;
}

// Cube order.  The reference lays z slices side by side in a 2-D image
// (slices to a row) and its pyramid walk visits the image's texels in Morton
// order (x in the low bit).  Texel k of that order here: the cube whose
// corner 0 sits in it, if any.
__device__ __forceinline__ unsigned compact_bits(unsigned v) {
    v &= 0x55555555u;
    v = (v | (v >> 1)) & 0x33333333u;
    v = (v | (v >> 2)) & 0x0f0f0f0fu;
    v = (v | (v >> 4)) & 0x00ff00ffu;
    v = (v | (v >> 8)) & 0x0000ffffu;
    return v;
}
__device__ __forceinline__ bool mc_cube_of(unsigned k, int res, int slices, int& x, int& y, int& z) {
    const unsigned tx = compact_bits(k), ty = compact_bits(k >> 1);
    const unsigned tex = (unsigned)res * (unsigned)slices;
    if (tx >= tex || ty >= tex) return false;
    x = (int)(tx % res);
    y = (int)(ty % res);
    z = (int)((ty / res) * slices + tx / res);
    return x < res - 1 && y < res - 1 && z < res - 1;
}

__global__ void __launch_bounds__(kSurfThreads) k_mc_count(const float* __restrict__ f, int res, int slices,
                                                           unsigned items, float iso, McDev T,
                                                           unsigned* __restrict__ block_sum) {
    __shared__ unsigned sh[kSurfThreads / 32];
    const unsigned k = blockIdx.x * kSurfThreads + threadIdx.x;
    unsigned cnt = 0;
    int x, y, z;
    if (k < items && mc_cube_of(k, res, slices, x, y, z)) cnt = __ldg(T.count + mc_case(f, res, x, y, z, iso));
    unsigned tot;
    block_exclusive_scan(cnt, sh, &tot);
    if (threadIdx.x == 0) block_sum[blockIdx.x] = tot;
}

// Exclusive scan of the block sums in one block; off[nb] = the total.
__global__ void __launch_bounds__(1024) k_mc_scan(const unsigned* __restrict__ block_sum, int nb,
                                                  unsigned* __restrict__ off) {
    __shared__ unsigned sh[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const unsigned v = i < nb ? block_sum[i] : 0u;
        unsigned x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sh[warp] = x;
        __syncthreads();
        unsigned woff = 0, tot = 0;
        for (int w = 0; w < 32; ++w) {
            const unsigned c = sh[w];
            woff += w < warp ? c : 0u;
            tot += c;
        }
        if (i < nb) off[i] = carry + woff + x - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) off[nb] = carry;
}

// The pyramid base level's corner value (traversehp.cl reads hp0.z): the
// field where classifycubes.cl wrote it (cube corners), 0 on the last layer.
__device__ __forceinline__ float mc_base(const float* __restrict__ f, int res, int x, int y, int z) {
    if (x >= res - 1 || y >= res - 1 || z >= res - 1) return 0.f;
    return __ldg(f + (size_t)x + (size_t)y * res + (size_t)z * res * res);
}

// map3Dto2DClamp + read: the neighbour at p + d along one axis, or p itself
// when the neighbour leaves the lattice.
__device__ __forceinline__ float mc_base_nb(const float* __restrict__ f, int res, int x, int y, int z, int ax, int d) {
    int q[3] = {x, y, z};
    q[ax] += d;
    if (q[ax] < 0 || q[ax] > res - 1) q[ax] -= d;
    return mc_base(f, res, q[0], q[1], q[2]);
}

__device__ __forceinline__ float3 mc_grad(const float* __restrict__ f, int res, int x, int y, int z) {
    float3 g;
    g.x = __fadd_rn(-mc_base_nb(f, res, x, y, z, 0, 1), mc_base_nb(f, res, x, y, z, 0, -1));
    g.y = __fadd_rn(-mc_base_nb(f, res, x, y, z, 1, 1), mc_base_nb(f, res, x, y, z, 1, -1));
    g.z = __fadd_rn(-mc_base_nb(f, res, x, y, z, 2, 1), mc_base_nb(f, res, x, y, z, 2, -1));
    return g;
}

__global__ void __launch_bounds__(kSurfThreads) k_mc_emit(const float* __restrict__ f, int res, int slices,
                                                          unsigned items, float iso, McDev T,
                                                          const unsigned* __restrict__ off, float* __restrict__ vtx,
                                                          float* __restrict__ nrm, unsigned cap_tri) {
    __shared__ unsigned sh[kSurfThreads / 32];
    const unsigned k = blockIdx.x * kSurfThreads + threadIdx.x;
    int x = 0, y = 0, z = 0, cs = 0;
    unsigned cnt = 0;
    if (k < items && mc_cube_of(k, res, slices, x, y, z)) {
        cs = mc_case(f, res, x, y, z, iso);
        cnt = __ldg(T.count + cs);
    }
    unsigned tot;
    const unsigned base = __ldg(off + blockIdx.x) + block_exclusive_scan(cnt, sh, &tot);
    if (cnt == 0 || base + cnt > cap_tri) return;
    const float rm1 = (float)(unsigned)(res - 1);
    for (unsigned t = 0; t < cnt; ++t) {
        for (int v = 0; v < 3; ++v) {
            const int e = __ldg(T.tri + cs * kMcMaxTriEdges + 3 * t + v);
            const int* c0 = kMcCornerDev[kMcEdgeDev[e][0]];
            const int* c1 = kMcCornerDev[kMcEdgeDev[e][1]];
            const int x0 = x + c0[0], y0 = y + c0[1], z0 = z + c0[2];
            const int x1 = x + c1[0], y1 = y + c1[1], z1 = z + c1[2];
            const float v0 = mc_base(f, res, x0, y0, z0);
            const float diff = __fdiv_rn(__fsub_rn(iso, v0), __fsub_rn(mc_base(f, res, x1, y1, z1), v0));
            const size_t o = ((size_t)(base + t) * 3 + v) * 3;
            const float p0[3] = {(float)x0, (float)y0, (float)z0}, p1[3] = {(float)x1, (float)y1, (float)z1};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float mx = __fadd_rn(p0[a], __fmul_rn(__fsub_rn(p1[a], p0[a]), diff));
                vtx[o + a] = __fmul_rn(__fdiv_rn(mx, rm1), 10.0f);
            }
            const float3 g0 = mc_grad(f, res, x0, y0, z0), g1 = mc_grad(f, res, x1, y1, z1);
            const float nx = __fadd_rn(g0.x, __fmul_rn(__fsub_rn(g1.x, g0.x), diff));
            const float ny = __fadd_rn(g0.y, __fmul_rn(__fsub_rn(g1.y, g0.y), diff));
            const float nz = __fadd_rn(g0.z, __fmul_rn(__fsub_rn(g1.z, g0.z), diff));
            const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dist2_exact(nx, ny, nz)));
            nrm[o] = __fmul_rn(nx, inv);
            nrm[o + 1] = __fmul_rn(ny, inv);
            nrm[o + 2] = __fmul_rn(nz, inv);
        }
    }
}

}  // namespace
}  // namespace sphk

// --- host side -----------------------------------------------------------------
namespace {

constexpr int kMaxSurfaceRes = 512;

template <class T>
int grow(sph_ctx* c, T*& p, size_t& cap, size_t n) {
    if (n <= cap && p) return SPH_OK;
    CK(c, cudaStreamSynchronize(c->stream));
    if (p) CK(c, cudaFree(p));
    p = nullptr;
    cap = 0;
    const size_t want = std::max(n, (size_t)1);
    CK(c, cudaMalloc((void**)&p, sizeof(T) * want));
    cap = want;
    return SPH_OK;
}

// ColorField::initializeData's slices per image row (ColorField.cpp:68), with
// its float functions: 2^ceil(log(ceil(sqrt(res)) / log 2)).
int mc_slices(int res) {
    return (int)(1u << static_cast<unsigned int>(std::ceil(std::log(std::ceil(std::sqrt((float)res)) / std::log(2.0f)))));
}

int mc_upload_table(sph_ctx* c) {
    if (c->mc_table) return SPH_OK;
    const McTable& T = mc_table();
    CK(c, cudaMalloc((void**)&c->mc_table, sizeof(T.tri) + sizeof(T.count)));
    CK(c, cudaMemcpyAsync(c->mc_table, T.tri, sizeof(T.tri), cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->mc_table + sizeof(T.tri), T.count, sizeof(T.count), cudaMemcpyHostToDevice, c->stream));
    return SPH_OK;
}

}  // namespace

extern "C" {

int sph_mc_case_table(signed char* tri, unsigned char* count, int* max_triangles) {
    const McTable& T = mc_table();
    if (tri) std::memcpy(tri, T.tri, sizeof(T.tri));
    if (count) std::memcpy(count, T.count, sizeof(T.count));
    if (max_triangles) *max_triangles = T.max_count;
    return SPH_OK;
}

int sph_colorfield(sph_ctx* c, int res) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (res < 2) res = 2;  // ColorField clamps the resolution (ColorField.cpp:45-48)
    if (res > kMaxSurfaceRes) return set_err(c, SPH_EINVAL, "sph_colorfield: res %d above %d", res, kMaxSurfaceRes);
    const size_t n = (size_t)res * res * res;
    if ((rc = grow(c, c->cf, c->cf_cap, n))) return rc;
    if (c->exact) {
        if ((rc = grow(c, c->cf_inv, c->cf_inv_cap, (size_t)c->max_num))) return rc;
        if (c->num_hint > 0)
            sphk::k_inv_density<<<(c->num_hint + sphk::kSurfThreads - 1) / sphk::kSurfThreads, sphk::kSurfThreads, 0,
                                  c->stream>>>(c->density, c->num_hint, c->cf_inv);
    }
    const unsigned long long chunks = (n + 31) / 32;
    unsigned long long stride = 7919;  // a prime; step past the chunk count's factors
    while (std::gcd(stride, chunks) != 1) stride += 2;
    const unsigned long long threads = chunks * 32;
    const unsigned blocks = (unsigned)((threads + sphk::kSurfThreads - 1) / sphk::kSurfThreads);
    const unsigned long long st = stride % chunks == 0 ? 1 : stride % chunks;
    if (c->exact)
        sphk::k_colorfield<true><<<blocks, sphk::kSurfThreads, 0, c->stream>>>(
            c->cf, res, chunks, st, c->pos_s, c->cf_inv, c->rec_vi, c->cell_start, c->cell_end, c->P);
    else
        sphk::k_colorfield<false><<<blocks, sphk::kSurfThreads, 0, c->stream>>>(
            c->cf, res, chunks, st, c->pos_s, c->cf_inv, c->rec_vi, c->cell_start, c->cell_end, c->P);
    CK_LAUNCH(c);
    c->cf_res = res;
    return SPH_OK;
}

int sph_marching_cubes(sph_ctx* c, const float* field, int res, float isolevel, int* ntri) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (ntri) *ntri = 0;
    if (res < 2 || res > kMaxSurfaceRes)
        return set_err(c, SPH_EINVAL, "sph_marching_cubes: res %d outside [2, %d]", res, kMaxSurfaceRes);
    if (!std::isfinite(isolevel)) return set_err(c, SPH_EINVAL, "sph_marching_cubes: isolevel not finite");
    if (!field) {
        if (!c->cf || c->cf_res != res)
            return set_err(c, SPH_ESTATE, "sph_marching_cubes: no colour field of resolution %d", res);
        field = c->cf;
    }
    if ((rc = mc_upload_table(c))) return rc;
    // the reference's image tiling (ColorField / MarchingCubes::initializeData),
    // widened where it would not hold every slice; its Morton walk covers the
    // next power of two
    int slices = mc_slices(res);
    while ((long long)slices * slices < res) slices *= 2;
    unsigned side = 1;
    while (side < (unsigned)(res * slices)) side *= 2;
    const unsigned items = side * side;
    const int nb = (int)((items + sphk::kSurfThreads - 1) / sphk::kSurfThreads);
    if ((rc = grow(c, c->mc_scan, c->mc_scan_cap, 2 * (size_t)nb + 1))) return rc;
    const sphk::McDev T{c->mc_table, (const unsigned char*)(c->mc_table + 256 * kMcMaxTriEdges)};
    unsigned* bsum = c->mc_scan;
    unsigned* off = c->mc_scan + nb;
    sphk::k_mc_count<<<nb, sphk::kSurfThreads, 0, c->stream>>>(field, res, slices, items, isolevel, T, bsum);
    sphk::k_mc_scan<<<1, 1024, 0, c->stream>>>(bsum, nb, off);
    CK_LAUNCH(c);
    unsigned total = 0;
    CK(c, cudaMemcpyAsync(&total, off + nb, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if ((rc = grow(c, c->mesh, c->mesh_cap, 18 * (size_t)total))) return rc;
    if (total > 0) {
        sphk::k_mc_emit<<<nb, sphk::kSurfThreads, 0, c->stream>>>(field, res, slices, items, isolevel, T, off,
                                                                 c->mesh, c->mesh + 9 * (size_t)total, total);
        CK_LAUNCH(c);
    }
    c->mesh_tri = (int)total;
    c->mesh_res = res;
    if (ntri) *ntri = (int)total;
    return SPH_OK;
}

int sph_post_process(sph_ctx* c, int res, int* ntri) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (ntri) *ntri = 0;
    if (res < 2) res = 2;
    if (c->num_hint == 0) {  // SPH::postProcess does nothing without particles
        c->mesh_tri = 0;
        return SPH_OK;
    }
    if ((rc = sph_colorfield(c, res))) return rc;
    // MarchingCubes::execute's isolevel (MarchingCubes.cpp:183)
    return sph_marching_cubes(c, nullptr, res, 0.0001f, ntri);
}

int sph_get_surface(sph_ctx* c, const float** field, const float** vertices, const float** normals, int* res,
                    int* ntri) {
    if (!c) return SPH_EINVAL;
    if (field) *field = c->cf;
    if (res) *res = c->cf_res;
    if (vertices) *vertices = c->mesh;
    if (normals) *normals = c->mesh ? c->mesh + 9 * (size_t)c->mesh_tri : nullptr;
    if (ntri) *ntri = c->mesh_tri;
    return SPH_OK;
}

int sph_download_surface(sph_ctx* c, float* field, float* vertices, float* normals, int cap_tri) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (cap_tri < 0) return set_err(c, SPH_EINVAL, "sph_download_surface: negative capacity");
    if (field && c->cf)
        CK(c, cudaMemcpyAsync(field, c->cf, sizeof(float) * (size_t)c->cf_res * c->cf_res * c->cf_res,
                              cudaMemcpyDeviceToHost, c->stream));
    const size_t k = (size_t)std::min(cap_tri, c->mesh_tri) * 9;
    if (k && vertices) CK(c, cudaMemcpyAsync(vertices, c->mesh, sizeof(float) * k, cudaMemcpyDeviceToHost, c->stream));
    if (k && normals)
        CK(c, cudaMemcpyAsync(normals, c->mesh + 9 * (size_t)c->mesh_tri, sizeof(float) * k, cudaMemcpyDeviceToHost,
                              c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

}  // extern "C"
