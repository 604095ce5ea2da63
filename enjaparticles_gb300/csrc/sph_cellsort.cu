// sph_cellsort.cu — the step's sort as a counting sort on the cell key.
//
// The reference hashes (hash.cl:50-157), sorts the (hash, index) pairs with
// System::bitonic_sort (System.cpp:407-480, bitonic.cl:54-258), finds the
// cell ranges (cellindices.cl:12-107 after the cell_start reset of
// CellIndices.cpp:58-62) and gathers the sorted arrays (permute.cl:10-46).
// The step produces what those stages leave, in the canonical order the
// stable radix sort of sph_sort.cu also gives (key ascending, equal keys by
// ascending particle index), in five passes:
//
//   count    the cell key of each particle (hash.cl, clamped to nb_cells like
//            k_hash) and an atomic count per cell; the count a particle finds
//            is its slot in the cell.
//   totals   the number of particles in each tile of 4096 cells (2048 or
//            8192 when the autotuner picks them); the first
//            thread also applies the previous step's out-of-grid deletion to
//            the particle count (count derives the same number on its own).
//            Grids of more than kDirectTiles tiles then scan the totals in
//            one block; smaller ones let every scan block sum the totals
//            before its tile itself (one launch fewer).
//   scan     an exclusive scan of the counts, one block per tile, its base the
//            sum of the totals of the tiles before it (no block waits on
//            another), writes cell_start (kEmpty for an empty cell) and
//            cell_end of the non-empty cells, the prefix of every cell (empty
//            ones included) for the neighbour passes' row runs, records where
//            the out-of-grid key nb_cells starts, and zeroes the counts for
//            the next step.
//   place    each particle's (index, key) at cell_start[key] + slot.
//   permute  slots within a cell come in atomic order, so each sorted
//            position ranks its particle index among the entries of its cell
//            and writes index, key and the gathered pos at cell_start + rank
//            (vel and veleval too for the staged update; the fused step
//            gathers veleval in its velocity pass, sph_integrate.cu).
//
// The batched step (sph_batch.cu) runs the totals and scan passes over the
// cells of all its scenes, with its own count, place and permute.
//
// The ranking reads every entry of a cell once per entry: quadratic in the
// occupancy of one cell, as the neighbour passes are (they walk every entry of
// the 27 cells around a particle).  The out-of-grid key nb_cells is the one
// cell they do not walk; a step in which k particles leave the grid together
// spends ~k^2/32 warp iterations here.
//
// Counts must be zero when a step starts: zeroed at allocation and re-zeroed
// by the scan of every step.
#include "sph_device.cuh"

namespace sphk {

namespace {

// The totals and scan passes take tiles of ST * kScanItems cells, ST threads
// per block: 2048, 4096 (the default) or 8192 cells, a launch shape the
// autotuner picks (the results are the same integers).
constexpr int kScanItems = 16;
constexpr int kItems = 4;                               // particles per thread in count and place
constexpr int kTileScanThreads = 1024;

}  // namespace

int cell_scan_tiles(int cells, int tile_cells) { return (cells + tile_cells - 1) / tile_cells; }

// ---------------------------------------------------------------------------
// Count: key and slot of every particle (original order).  A warp takes 4
// runs of 32 consecutive particles, all loads and atomics of the 4 in flight
// together.  The particle count is the previous step's after its out-of-grid
// deletion (k_cell_totals stores it once this pass is done).
__global__ void __launch_bounds__(256) k_cell_count(const float4* __restrict__ pos_u, uint32_t* __restrict__ key_of,
                                                    uint32_t* __restrict__ slot_of, uint32_t* __restrict__ count,
                                                    const int* __restrict__ info, StepParams p) {
    const int out = info[kOutStart];
    const int n = out >= 0 ? out : info[kNum];
    const unsigned lane = threadIdx.x & 31;
    const int wb = (blockIdx.x * blockDim.x + (threadIdx.x & ~31)) * kItems;  // first particle of the warp
    uint32_t key[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int i = wb + 32 * k + (int)lane;
        key[k] = 0xffffffffu;  // no valid key takes this value
        if (i < n) {
            const float4 q = ldg4(pos_u + i);
            const int3 c = grid_cell(q.x, q.y, q.z, p.g_min, p.g_delta);
            int h = grid_hash_f(c.x, c.y, c.z, p.g_res);
            h = h > p.nb_cells ? p.nb_cells : h;
            h = h < 0 ? p.nb_cells : h;
            key[k] = (uint32_t)h;
        }
    }
    uint32_t slot[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) slot[k] = key[k] != 0xffffffffu ? atomicAdd(count + key[k], 1u) : 0u;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int i = wb + 32 * k + (int)lane;
        if (i < n) {
            key_of[i] = key[k];
            slot_of[i] = slot[k];
        }
    }
}

// ---------------------------------------------------------------------------
// The 16 counts of cells [c0, c0 + 16): 128-bit loads when in range and the
// array is 16-byte aligned (c0 is a multiple of 16 cells).
__device__ __forceinline__ void load_counts(const uint32_t* __restrict__ count, uint32_t c0, uint32_t cells, bool vec,
                                            uint32_t (&v)[kScanItems]) {
    if (vec) {
        const uint4* q = reinterpret_cast<const uint4*>(count + c0);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) {
            const uint4 w = q[k];
            v[4 * k] = w.x;
            v[4 * k + 1] = w.y;
            v[4 * k + 2] = w.z;
            v[4 * k + 3] = w.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] = c0 + k < cells ? count[c0 + k] : 0u;
    }
}

// Totals: block b sums the counts of tile b.  info may be null (batches: no
// deletion).
template <int ST>
__global__ void __launch_bounds__(ST) k_cell_totals(const uint32_t* __restrict__ count,
                                                    uint32_t* __restrict__ tile_total, int* __restrict__ info,
                                                    uint32_t cells) {
    constexpr int kScanTile = ST * kScanItems;
    __shared__ uint32_t s_warp[ST / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (info != nullptr && blockIdx.x == 0 && tid == 0) {  // the step's particle count; the scan sets kOutStart anew
        const int out = info[kOutStart];
        if (out >= 0) info[kNum] = out;
        info[kOutStart] = -1;
    }
    const uint32_t c0 = (uint32_t)blockIdx.x * kScanTile + (uint32_t)tid * kScanItems;
    const bool vec = c0 + kScanItems <= cells && (reinterpret_cast<uintptr_t>(count) & 15u) == 0;
    uint32_t v[kScanItems];
    load_counts(count, c0, cells, vec, v);
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) s_warp[warp] = sum;
    __syncthreads();
    if (tid == 0) {
        uint32_t t = 0;
#pragma unroll
        for (int w = 0; w < ST / 32; ++w) t += s_warp[w];
        tile_total[blockIdx.x] = t;
    }
}

// Tile scan (grids of more than kDirectTiles tiles): tile_total becomes the
// exclusive prefix of the totals, in one block.
__global__ void __launch_bounds__(kTileScanThreads) k_cell_tile_scan(uint32_t* __restrict__ tile_total, int tiles) {
    __shared__ uint32_t s_warp[kTileScanThreads / 32];
    __shared__ uint32_t s_carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_carry = 0;
    for (int k0 = 0; k0 < tiles; k0 += kTileScanThreads) {
        const int k = k0 + tid;
        const uint32_t v = k < tiles ? tile_total[k] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        uint32_t before = s_carry, all = 0;
#pragma unroll
        for (int w = 0; w < kTileScanThreads / 32; ++w) {
            const uint32_t t = s_warp[w];
            before += w < warp ? t : 0u;
            all += t;
        }
        if (k < tiles) tile_total[k] = before + x - v;
        __syncthreads();
        if (tid == 0) s_carry += all;
        __syncthreads();
    }
}

// Scan: block b scans tile b (16 consecutive cells per thread) from the sum
// of the totals of tiles 0..b-1, or from tile_total[b] when the totals were
// scanned already (prescanned).  With info, the start of the last cell (the
// out-of-grid key) goes to info[kOutStart].
template <int ST>
__global__ void __launch_bounds__(ST) k_cell_scan(uint32_t* __restrict__ count, uint32_t* __restrict__ cell_start,
                                                  uint32_t* __restrict__ cell_end,
                                                  const uint32_t* __restrict__ tile_total, int* __restrict__ info,
                                                  uint32_t cells, int prescanned, uint32_t* __restrict__ pre) {
    constexpr int kScanTile = ST * kScanItems;
    __shared__ uint32_t s_warp[ST / 32];
    __shared__ uint32_t s_base[ST / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile = blockIdx.x;
    uint32_t before = 0;
    if (prescanned)
        before = tid == 0 ? __ldg(tile_total + tile) : 0u;
    else
        for (int t = tid; t < tile; t += ST) before += __ldg(tile_total + t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
    if (lane == 0) s_base[warp] = before;
    const uint32_t c0 = (uint32_t)tile * kScanTile + (uint32_t)tid * kScanItems;
    // a recorded rollout's cell arrays are packed at a stride of nb_cells + 1
    // words, so their base need not be 16-byte aligned
    const bool vec = c0 + kScanItems <= cells &&
                     ((reinterpret_cast<uintptr_t>(count) | reinterpret_cast<uintptr_t>(cell_start) |
                       reinterpret_cast<uintptr_t>(pre)) & 15u) == 0;
    uint32_t v[kScanItems];
    load_counts(count, c0, cells, vec, v);
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
    // block-wide exclusive scan of the thread sums
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t run = x - sum;
#pragma unroll
    for (int w = 0; w < ST / 32; ++w) run += (w < warp ? s_warp[w] : 0u) + s_base[w];
    uint32_t st[kScanItems], ex[kScanItems];
    const uint32_t last = cells - 1;  // the out-of-grid key
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        ex[k] = run;
        st[k] = v[k] ? run : kEmpty;
        if (v[k]) {
            cell_end[c0 + k] = run + v[k];
            if (info != nullptr && c0 + k == last) info[kOutStart] = (int)run;
        }
        run += v[k];
    }
    if (vec) {
        uint4* s4 = reinterpret_cast<uint4*>(cell_start + c0);
        uint4* z4 = reinterpret_cast<uint4*>(count + c0);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) {
            s4[k] = make_uint4(st[4 * k], st[4 * k + 1], st[4 * k + 2], st[4 * k + 3]);
            z4[k] = make_uint4(0u, 0u, 0u, 0u);
        }
        if (pre != nullptr) {
            uint4* p4 = reinterpret_cast<uint4*>(pre + c0);
#pragma unroll
            for (int k = 0; k < kScanItems / 4; ++k)
                p4[k] = make_uint4(ex[4 * k], ex[4 * k + 1], ex[4 * k + 2], ex[4 * k + 3]);
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (c0 + k < cells) {
                cell_start[c0 + k] = st[k];
                count[c0 + k] = 0u;
                if (pre != nullptr) pre[c0 + k] = ex[k];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Place: (index, key) of particle i at its cell's start + its slot; 4
// particles per thread, loads in flight together.
__global__ void __launch_bounds__(256) k_cell_place(const uint32_t* __restrict__ key_of,
                                                    const uint32_t* __restrict__ slot_of,
                                                    const uint32_t* __restrict__ cell_start,
                                                    uint2* __restrict__ entries, const int* __restrict__ info) {
    const int n = info[kNum];
    const int i0 = blockIdx.x * (blockDim.x * kItems) + threadIdx.x;
    uint32_t key[kItems], slot[kItems], cs[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int i = i0 + k * (int)blockDim.x;
        key[k] = i < n ? __ldg(key_of + i) : 0u;
        slot[k] = i < n ? __ldg(slot_of + i) : 0u;
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k) cs[k] = i0 + k * (int)blockDim.x < n ? __ldg(cell_start + key[k]) : 0u;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int i = i0 + k * (int)blockDim.x;
        if (i < n && in_bounds(cs[k] + slot[k], (uint32_t)n, const_cast<int*>(info) + kError))
            entries[cs[k] + slot[k]] = make_uint2((uint32_t)i, key[k]);
    }
}

// ---------------------------------------------------------------------------
// Permute: rank within the cell, then the sorted arrays.
// Gather: 0 = pos (the fused step gathers veleval later, beside the density
// pass), 1 = pos/veleval, 2 = pos/vel/veleval.
template <int Gather>
__global__ void __launch_bounds__(256) k_cell_permute(const uint2* __restrict__ entries,
                                                      const uint32_t* __restrict__ cell_start,
                                                      const uint32_t* __restrict__ cell_end,
                                                      uint32_t* __restrict__ keys, uint32_t* __restrict__ idx,
                                                      const float4* __restrict__ pos_u,
                                                      const float4* __restrict__ vel_u,
                                                      const float4* __restrict__ veleval_u,
                                                      float4* __restrict__ pos_s, float4* __restrict__ vel_s,
                                                      float4* __restrict__ veleval_s, const int* __restrict__ info,
                                                      float* __restrict__ pxy, float* __restrict__ pz) {
    const int n = info[kNum];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint2 e = __ldg(entries + s);
    const uint32_t id = e.x, key = e.y;
    int* err = const_cast<int*>(info) + kError;
    if (!in_bounds(id, (uint32_t)n, err)) return;
    // the gathers do not depend on the rank: in flight during the ranking
    const float4 pq = __ldg(pos_u + id);
    float4 vq = make_float4(0.f, 0.f, 0.f, 0.f), wq = vq;
    if (Gather >= 1) vq = __ldg(veleval_u + id);
    if (Gather == 2) wq = __ldg(vel_u + id);
    const uint32_t cs = __ldg(cell_start + key), ce = __ldg(cell_end + key);
    // every entry lies in a cell of [cs, ce) within [0, n) when the counts
    // were zero at the start of the step; never write outside it
    if (cs >= ce || ce > (uint32_t)n) {
        if (kChecked) atomicOr(err, kErrBounds);
        return;
    }
    const uint32_t* ids = reinterpret_cast<const uint32_t*>(entries);
    uint32_t rank = 0;
    for (uint32_t t = cs; t < ce; ++t) rank += __ldg(ids + 2 * t) < id ? 1u : 0u;
    const uint32_t p = cs + rank;
    keys[s] = key;  // one key over the whole cell
    idx[p] = id;
    pos_s[p] = pq;
    if (pxy != nullptr) {
        // the pair layout of k_density_pairs: (x, x', y, y') and (z, z')
        const uint32_t k = p >> 1, l = p & 1u;
        pxy[4 * k + l] = pq.x;
        pxy[4 * k + 2 + l] = pq.y;
        pz[2 * k + l] = pq.z;
        if (s == n - 1 && (n & 1)) {  // the last pair's unused lane
            pxy[4 * (n >> 1) + 1] = kFarAway;
            pxy[4 * (n >> 1) + 3] = kFarAway;
            pz[2 * (n >> 1) + 1] = kFarAway;
        }
    }
    if (Gather >= 1) veleval_s[p] = vq;
    if (Gather == 2) vel_s[p] = wq;
}

// ---------------------------------------------------------------------------
// Launchers, one per pass (the step profile times each).
void launch_cell_count(const float4* pos_u, uint32_t* key_of, uint32_t* slot_of, uint32_t* count, const int* info,
                       const StepParams& p, int grid_items, cudaStream_t st) {
    const int per = 256 * kItems;
    const int blocks = grid_items > 0 ? (grid_items + per - 1) / per : 1;
    k_cell_count<<<blocks, 256, 0, st>>>(pos_u, key_of, slot_of, count, info, p);
}

void launch_cell_totals(const uint32_t* count, uint32_t* tile_total, int* info, uint32_t cells, int tile_cells,
                        cudaStream_t st) {
    const int tiles = cell_scan_tiles((int)cells, tile_cells);
    if (tile_cells == 2048)
        k_cell_totals<128><<<tiles, 128, 0, st>>>(count, tile_total, info, cells);
    else if (tile_cells == 8192)
        k_cell_totals<512><<<tiles, 512, 0, st>>>(count, tile_total, info, cells);
    else
        k_cell_totals<256><<<tiles, 256, 0, st>>>(count, tile_total, info, cells);
}

void launch_cell_scan(uint32_t* count, uint32_t* cell_start, uint32_t* cell_end, uint32_t* tile_total, int* info,
                      uint32_t cells, int tile_cells, cudaStream_t st, uint32_t* pre) {
    const int tiles = cell_scan_tiles((int)cells, tile_cells);
    const int prescanned = tiles > kDirectTiles;
    if (prescanned) k_cell_tile_scan<<<1, kTileScanThreads, 0, st>>>(tile_total, tiles);
    if (tile_cells == 2048)
        k_cell_scan<128><<<tiles, 128, 0, st>>>(count, cell_start, cell_end, tile_total, info, cells, prescanned, pre);
    else if (tile_cells == 8192)
        k_cell_scan<512><<<tiles, 512, 0, st>>>(count, cell_start, cell_end, tile_total, info, cells, prescanned, pre);
    else
        k_cell_scan<256><<<tiles, 256, 0, st>>>(count, cell_start, cell_end, tile_total, info, cells, prescanned, pre);
}

void launch_cell_place(const uint32_t* key_of, const uint32_t* slot_of, const uint32_t* cell_start, uint2* entries,
                       const int* info, int grid_items, cudaStream_t st) {
    const int per = 256 * kItems;
    const int blocks = grid_items > 0 ? (grid_items + per - 1) / per : 1;
    k_cell_place<<<blocks, 256, 0, st>>>(key_of, slot_of, cell_start, entries, info);
}

void launch_cell_permute(const uint2* entries, const uint32_t* cell_start, const uint32_t* cell_end, uint32_t* keys,
                         uint32_t* idx, const float4* pos_u, const float4* vel_u, const float4* veleval_u,
                         float4* pos_s, float4* vel_s, float4* veleval_s, const int* info, int grid_items, int gather,
                         float4* pxy, float2* pz, cudaStream_t st) {
    const int blocks = grid_items > 0 ? (grid_items + 255) / 256 : 1;
    float* fxy = reinterpret_cast<float*>(pxy);
    float* fz = reinterpret_cast<float*>(pz);
    if (gather == 2)
        k_cell_permute<2><<<blocks, 256, 0, st>>>(entries, cell_start, cell_end, keys, idx, pos_u, vel_u, veleval_u,
                                                  pos_s, vel_s, veleval_s, info, fxy, fz);
    else if (gather == 1)
        k_cell_permute<1><<<blocks, 256, 0, st>>>(entries, cell_start, cell_end, keys, idx, pos_u, vel_u, veleval_u,
                                                  pos_s, vel_s, veleval_s, info, fxy, fz);
    else
        k_cell_permute<0><<<blocks, 256, 0, st>>>(entries, cell_start, cell_end, keys, idx, pos_u, vel_u, veleval_u,
                                                  pos_s, vel_s, veleval_s, info, fxy, fz);
}

}  // namespace sphk
