// sph_sort.cu — step prologue, grid hash, and the stable LSD radix sort on
// 32-bit cell keys that replaces the reference's bitonic sort.
//
//   hash:   rtpslib/system/common/cl_src/hash.cl:50-157 (+ cl_hash.h:33-114),
//           host Hash.cpp:42-75.  Fused here: the clear of cell_start
//           (CellIndices.cpp:58-62, a host upload of C+1 words in the
//           reference) and the digit histograms of every radix pass.
//   sort:   System::bitonic_sort (System.cpp:407-480, bitonic.cl:54-258) is an
//           unstable sort of nlpo2(N) padded keys.  Here: one pass per 8-bit
//           digit, each pass a single kernel (per-warp match_any ranking,
//           decoupled look-back across tiles, shared-memory reorder so the
//           global writes are runs of one digit).  Stable, so equal keys keep
//           ascending original index: the canonical order.
#include <cstdio>

#include "sph_device.cuh"

namespace sphk {

constexpr int kRadixBits = 8;
constexpr int kRadixSize = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys per tile
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1;
constexpr int kLookbackSpinLimit = 1 << 22;

int radix_tiles(int n) { return (n + kSortTile - 1) / kSortTile; }

// ---------------------------------------------------------------------------
// Prologue: apply the previous step's out-of-grid deletion to the particle
// count and zero the digit histograms the hash kernel accumulates.
__global__ void k_prologue(uint32_t* __restrict__ hist, int* __restrict__ info) {
    if (threadIdx.x == 0) {
        const int out = info[kOutStart];
        if (out >= 0) info[kNum] = out;
        info[kOutStart] = -1;
    }
    for (int k = threadIdx.x; k < 4 * kRadixSize; k += blockDim.x) hist[k] = 0;
}

void launch_prologue(uint32_t* hist, int* info, cudaStream_t st) { k_prologue<<<1, 256, 0, st>>>(hist, info); }

// Sort reset: zero the look-back status words and the tile counters.
__global__ void k_sort_reset(uint32_t* __restrict__ status, size_t words, int* __restrict__ tile_counters) {
    if (blockIdx.x == 0 && threadIdx.x < 4) tile_counters[threadIdx.x] = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    uint4* s4 = reinterpret_cast<uint4*>(status);
    const size_t w4 = words / 4;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < w4; k += stride) s4[k] = make_uint4(0, 0, 0, 0);
    for (size_t k = w4 * 4 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < words; k += stride) status[k] = 0;
}

void launch_sort_reset(uint32_t* status, size_t words, int* tile_counters, cudaStream_t st) {
    int blocks = (int)((words / 4 + 255) / 256);
    blocks = blocks < 1 ? 1 : (blocks > 1216 ? 1216 : blocks);
    k_sort_reset<<<blocks, 256, 0, st>>>(status, words, tile_counters);
}

// ---------------------------------------------------------------------------
// Hash.  Grid-stride over particles in original order (a few blocks per SM),
// so that the per-block digit histograms reach global memory with few atomics.
template <int PASSES>
__global__ void __launch_bounds__(256) k_hash(const float4* __restrict__ pos_u, uint32_t* __restrict__ keys,
                                              uint32_t* __restrict__ idx, uint32_t* __restrict__ cell_start,
                                              uint32_t* __restrict__ hist, const int* __restrict__ info,
                                              StepParams p, int clear_cells) {
    __shared__ uint32_t s_hist[PASSES > 0 ? PASSES : 1][kRadixSize];
    const int n = info[kNum];
    const int tid = threadIdx.x;
    for (int k = tid; k < PASSES * kRadixSize; k += blockDim.x) (&s_hist[0][0])[k] = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    // Fused cell_start clear (CellIndices.cpp:58-62).
    if (clear_cells) {
        for (size_t k = (size_t)blockIdx.x * blockDim.x + tid; k <= (size_t)p.nb_cells; k += stride)
            cell_start[k] = kEmpty;
    }
    __syncthreads();
    const unsigned lane = tid & 31;
    // The loop bound is uniform per warp (base is the warp's first index), so
    // match_any always sees the full warp.
    for (size_t base = (size_t)blockIdx.x * blockDim.x + (tid & ~31); base < (size_t)n; base += stride) {
        const size_t i = base + lane;
        const bool valid = i < (size_t)n;
        uint32_t key = 0;
        if (valid) {
            const float4 q = ldg4(pos_u + i);
            const int3 c = grid_cell(q.x, q.y, q.z, p.g_min, p.g_delta);
            int h = grid_hash_f(c.x, c.y, c.z, p.g_res);
            h = h > p.nb_cells ? p.nb_cells : h;
            h = h < 0 ? p.nb_cells : h;
            key = (uint32_t)h;
            keys[i] = key;
            idx[i] = (uint32_t)i;
        }
#pragma unroll
        for (int ps = 0; ps < PASSES; ++ps) {
            const uint32_t d = valid ? ((key >> (ps * kRadixBits)) & (kRadixSize - 1)) : 0x100u;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const int leader = 31 - __clz(peers);
            if (valid && (int)lane == leader) atomicAdd(&s_hist[ps][d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int k = tid; k < PASSES * kRadixSize; k += blockDim.x) {
        const uint32_t c = (&s_hist[0][0])[k];
        if (c) atomicAdd(hist + k, c);
    }
}

void launch_hash(const float4* pos_u, uint32_t* keys, uint32_t* idx, uint32_t* cell_start, uint32_t* hist,
                 const int* info, const StepParams& p, int grid_items, int passes, int clear_cells,
                 cudaStream_t st) {
    const int threads = 256;
    int blocks = (grid_items + threads - 1) / threads;
    const int cap = 152 * 8;  // a few resident blocks per SM
    blocks = blocks < 1 ? 1 : (blocks > cap ? cap : blocks);
    switch (passes) {
        case 0: k_hash<0><<<blocks, threads, 0, st>>>(pos_u, keys, idx, cell_start, hist, info, p, clear_cells); break;
        case 1: k_hash<1><<<blocks, threads, 0, st>>>(pos_u, keys, idx, cell_start, hist, info, p, clear_cells); break;
        case 2: k_hash<2><<<blocks, threads, 0, st>>>(pos_u, keys, idx, cell_start, hist, info, p, clear_cells); break;
        case 3: k_hash<3><<<blocks, threads, 0, st>>>(pos_u, keys, idx, cell_start, hist, info, p, clear_cells); break;
        default: k_hash<4><<<blocks, threads, 0, st>>>(pos_u, keys, idx, cell_start, hist, info, p, clear_cells); break;
    }
}

// ---------------------------------------------------------------------------
// Block-wide exclusive scan of one value per thread (256 threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < kSortWarps ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kSortWarps) s_warp[lane] = t;
    }
    __syncthreads();
    const uint32_t before = warp > 0 ? s_warp[warp - 1] : 0;
    __syncthreads();
    return before + x - v;
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One radix pass over digit bits [shift, shift+bits).
__global__ void __launch_bounds__(kSortThreads) k_radix_pass(const uint32_t* __restrict__ kin,
                                                             const uint32_t* __restrict__ vin,
                                                             uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                             const int* __restrict__ info,
                                                             const uint32_t* __restrict__ hist,
                                                             uint32_t* __restrict__ status, int* tile_counter,
                                                             int* err, int shift, int bits) {
    __shared__ uint32_t s_cnt[kSortWarps][kRadixSize];
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];
    __shared__ uint32_t s_tile_off[kRadixSize];
    __shared__ uint32_t s_gbase[kRadixSize];
    __shared__ uint32_t s_scan[kSortWarps];
    __shared__ int s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t mask = (1u << bits) - 1u;
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1);
    for (int k = tid; k < kSortWarps * kRadixSize; k += kSortThreads) (&s_cnt[0][0])[k] = 0;
    __syncthreads();
    const int tile = s_tile;
    if (tile >= (int)gridDim.x) {  // counters not reset: never index past the status rows
        if (tid == 0) atomicOr(err, kErrLookbackTimeout);
        return;
    }
    const int n = info[kNum];
    const int tile_base = tile * kSortTile;
    const int wbase = tile_base + warp * (32 * kSortItems);

    uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int i = wbase + k * 32 + lane;
        if (i < n) {
            key[k] = __ldg(kin + i);
            val[k] = __ldg(vin + i);
        } else {
            key[k] = 0xffffffffu;
            val[k] = 0;
        }
    }
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int i = wbase + k * 32 + lane;
        const bool valid = i < n;
        const uint32_t d = valid ? ((key[k] >> shift) & mask) : 0x100u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int leader = 31 - __clz(peers);
        uint32_t before = 0;
        if (valid) before = s_cnt[warp][d];
        rank[k] = before + (uint32_t)__popc(peers & lt_mask);
        __syncwarp();
        if (valid && lane == leader) s_cnt[warp][d] = before + (uint32_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();

    // Digit d = tid: warp-exclusive prefixes, tile total.
    const int d = tid;
    uint32_t total = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = s_cnt[w][d];
        s_cnt[w][d] = total;
        total += c;
    }
    // Decoupled look-back across tiles (bounded spin).
    uint32_t* row = status + (size_t)tile * kRadixSize;
    uint32_t excl = 0;
    if (tile == 0) {
        st_relaxed(row + d, kFlagInc | total);
    } else {
        st_relaxed(row + d, kFlagAgg | total);
        int j = tile - 1;
        int spins = 0;
        while (j >= 0) {
            const uint32_t v = ld_volatile(status + (size_t)j * kRadixSize + d);
            const uint32_t flag = v & ~kValueMask;
            if (flag == 0) {
                if (++spins > kLookbackSpinLimit) {
                    atomicOr(err, kErrLookbackTimeout);
                    break;
                }
                continue;
            }
            excl += v & kValueMask;
            if (flag == kFlagInc) break;
            --j;
        }
        st_relaxed(row + d, kFlagInc | (excl + total));
    }
    const uint32_t gstart = block_exclusive_scan(d < (1 << bits) ? hist[d] : 0u, s_scan);
    const uint32_t toff = block_exclusive_scan(total, s_scan);
    s_tile_off[d] = toff;
    s_gbase[d] = gstart + excl - toff;
    __syncthreads();

#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const int i = wbase + k * 32 + lane;
        if (i < n) {
            const uint32_t dd = (key[k] >> shift) & mask;
            const uint32_t lp = s_tile_off[dd] + s_cnt[warp][dd] + rank[k];
            s_keys[lp] = key[k];
            s_vals[lp] = val[k];
        }
    }
    __syncthreads();
    int m = n - tile_base;
    m = m < 0 ? 0 : (m > kSortTile ? kSortTile : m);
    for (int t = tid; t < m; t += kSortThreads) {
        const uint32_t kk = s_keys[t];
        const uint32_t dd = (kk >> shift) & mask;
        const uint32_t g = s_gbase[dd] + (uint32_t)t;
        kout[g] = kk;
        vout[g] = s_vals[t];
    }
}

void launch_radix_pass(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, const int* info,
                       const uint32_t* hist, uint32_t* status, int* tile_counter, int* err, int shift, int bits,
                       int grid_items, cudaStream_t st) {
    int tiles = radix_tiles(grid_items);
    if (tiles < 1) tiles = 1;
    k_radix_pass<<<tiles, kSortThreads, 0, st>>>(kin, vin, kout, vout, info, hist, status, tile_counter, err, shift,
                                                 bits);
}

}  // namespace sphk
