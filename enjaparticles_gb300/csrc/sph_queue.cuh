// sph_queue.cuh — the work queue of the batched step's persistent scheduler
// (sph_batch_set_scheduler(SPH_SCHED_QUEUE)).
//
// A pass (density, or force with the integrator) launches as many blocks of
// T threads as fit on the GPU at once.  Each block takes items from a device
// counter until none are left; an item is one tile of up to T consecutive
// sorted particles of one scene, so a block works on one scene at a time:
// the scene's parameter block sits in shared memory and its cell base,
// out-of-grid start and deletion bookkeeping are block-uniform.
//
// The items of scene s are tile_off[s] .. tile_off[s+1]-1, tile_off being the
// exclusive scan of ceil(n_s / T) over the scenes, n_s = seg[s+1] - seg[s]
// the scene's particles this step (seg: the scenes' first sorted indices,
// fixed for the step; the force pass lowers a scene's count as it deletes).  The first block to
// arrive computes it and publishes it with a flag; every block waits for the
// flag before taking items.  The wait is bounded: a block that polls more
// than spin_limit times sets kErrQueueTimeout in the error word and leaves
// (the step's result is then invalid and the next sph_batch_sync reports
// SPH_ETIMEOUT).  The first block is running when it arrives, so the flag is
// always set unless a test holds it back (hold).
#pragma once

#include <atomic>

#include "sph_device.cuh"

namespace sphk {

constexpr int kErrQueueTimeout = 2;  // bit of info[kError]

// Blocks of a persistent queue kernel: as many as fit on the current device
// at once (resident blocks per SM times SMs), cached per kernel and device.
// The cache entry is the one number, so host threads that fill it together
// store the same value and none reads half of it.
constexpr int kQueueMaxDevices = 64;
template <class Kernel>
int queue_grid(Kernel kernel, int threads, std::atomic<int> (&cache)[kQueueMaxDevices]) {
    int dev = 0;
    const bool cached = cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kQueueMaxDevices;
    if (cached) {
        const int g = cache[dev].load(std::memory_order_relaxed);
        if (g > 0) return g;
    }
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
    const int g = (per_sm < 1 ? 1 : per_sm) * (sms < 1 ? 1 : sms);
    if (cached) cache[dev].store(g, std::memory_order_relaxed);
    return g;
}

struct BatchQueue {
    unsigned* state;         // [0] next item, [1] blocks arrived, [2] table published; zeroed before a launch
    uint32_t* tile_off;      // [nscenes + 1]
    const uint32_t* seg;     // [nscenes + 1] first sorted index of every scene, then the total
    const uint32_t* slot_off;
    const uint32_t* cstart;  // cell_start of all scenes' cells
    const uint32_t* cbase;
    const StepParams* table;
    int* num_out;            // d_num (the force pass writes a scene's count after a deletion)
    int* del;                // d_del
    const float4* vel_s;     // sorted velocities of the scenes that delete
    int* err;                // info + kError
    int nscenes;
    unsigned spin_limit;
    int hold;
};

// One scene's tile as a scene resolver for the per-particle passes: the
// parameters in shared memory, everything else block-uniform.
struct TileScene {
    static constexpr bool kBatch = true;
    const StepParams* P;
    uint32_t sc, cb, os;  // scene, cell base, first out-of-grid sorted index (kEmpty: none)
    const uint32_t* seg;
    const uint32_t* slot_off;
    int* num;
    int* del;
    const float4* vel_s;
    __device__ __forceinline__ const StepParams& params(int) const { return *P; }
    __device__ __forceinline__ uint32_t cell_base(int) const { return cb; }
    __device__ __forceinline__ bool frozen(int i) const { return (uint32_t)i >= os; }
    __device__ __forceinline__ uint32_t scene(int) const { return sc; }
    __device__ __forceinline__ uint32_t out_start(uint32_t) const { return os; }
};

// Shared state of a queue block.
template <int T>
struct QueueShared {
    StepParams P;
    uint32_t scan[T / 32];
    uint32_t item, first, count, scene, cbase, out_start;
    int ok, is_first;
};

// The table and its publication (first block), then the bounded wait for it.
// Returns false when the block must leave.
template <int T>
__device__ __forceinline__ bool queue_start(const BatchQueue& Q, QueueShared<T>& S) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) S.is_first = atomicAdd(Q.state + 1, 1u) == 0u;
    __syncthreads();
    if (S.is_first) {
        uint32_t carry = 0;
        for (int base = 0; base < Q.nscenes; base += T) {
            const int s = base + tid;
            const uint32_t v =
                s < Q.nscenes ? (__ldg(Q.seg + s + 1) - __ldg(Q.seg + s) + (uint32_t)T - 1u) / (uint32_t)T : 0u;
            uint32_t x = v;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x += y;
            }
            if (lane == 31) S.scan[warp] = x;
            __syncthreads();
            uint32_t before = carry, all = 0;
#pragma unroll
            for (int w = 0; w < T / 32; ++w) {
                before += w < warp ? S.scan[w] : 0u;
                all += S.scan[w];
            }
            if (s < Q.nscenes) Q.tile_off[s] = before + x - v;
            carry += all;
            __syncthreads();
        }
        if (tid == 0) Q.tile_off[Q.nscenes] = carry;
        __threadfence();
        __syncthreads();
        if (tid == 0 && !Q.hold) atomicExch(Q.state + 2, 1u);
    }
    if (tid == 0) {
        int ok = 1;
        unsigned polls = 0;
        while (atomicAdd(Q.state + 2, 0u) == 0u) {
            if (++polls > Q.spin_limit) {
                atomicOr(Q.err, kErrQueueTimeout);
                ok = 0;
                break;
            }
            __nanosleep(256);
        }
        __threadfence();
        S.ok = ok;
    }
    __syncthreads();
    return S.ok != 0;
}

// The block's next item: its scene (parameters copied to shared memory),
// first sorted index and particle count.  Returns false when none are left.
template <int T>
__device__ __forceinline__ bool queue_next(const BatchQueue& Q, QueueShared<T>& S) {
    const int tid = threadIdx.x;
    __syncthreads();  // the previous item's readers of S are done
    if (tid == 0) {
        const uint32_t total = __ldcg(Q.tile_off + Q.nscenes);
        const uint32_t item = atomicAdd(Q.state, 1u);
        S.item = item;
        if (item < total) {
            // the scene s with tile_off[s] <= item < tile_off[s + 1]
            int lo = 0, hi = Q.nscenes;  // tile_off[lo] <= item < tile_off[hi]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (__ldcg(Q.tile_off + mid) <= item) lo = mid; else hi = mid;
            }
            const uint32_t t = item - __ldcg(Q.tile_off + lo);
            const uint32_t s0 = __ldg(Q.seg + lo), n = __ldg(Q.seg + lo + 1) - s0;
            S.scene = (uint32_t)lo;
            S.first = s0 + t * (uint32_t)T;
            S.count = n - t * (uint32_t)T < (uint32_t)T ? n - t * (uint32_t)T : (uint32_t)T;
            S.cbase = __ldg(Q.cbase + lo);
            S.out_start = __ldg(Q.cstart + S.cbase + (uint32_t)__ldg(&Q.table[lo].nb_cells));
        }
        S.ok = item < total;
    }
    __syncthreads();
    if (!S.ok) return false;
    // the scene's parameter block into shared memory
    const uint32_t* src = reinterpret_cast<const uint32_t*>(Q.table + S.scene);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&S.P);
    for (int k = tid; k < (int)(sizeof(StepParams) / 4); k += T) dst[k] = __ldg(src + k);
    __syncthreads();
    return true;
}

template <int T>
__device__ __forceinline__ TileScene queue_scene(const BatchQueue& Q, const QueueShared<T>& S) {
    return TileScene{&S.P, S.scene, S.cbase, S.out_start, Q.seg, Q.slot_off, Q.num_out, Q.del, Q.vel_s};
}

}  // namespace sphk
