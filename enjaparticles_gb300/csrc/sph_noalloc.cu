// sph_noalloc.cu — a key/value sort that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host application that owns all
// device memory through its own pool and forbids allocations behind its back,
// a real-time frame loop that cannot afford the implicit synchronisation an
// allocation may bring, or code running where the allocator is not reachable
// at all.  For them sph_sort_pairs_noalloc sorts caller-owned device arrays
// with the library's stable LSD radix sort, and keeps every byte of scratch
// it needs (digit histograms, look-back status words, one ping-pong key/value
// buffer, counters) in one file-scope __device__ array.  That array is part
// of the library image: every GPU that loads the library holds it (about
// 9 MiB) until the process exits.
#include <atomic>
#include <cstdio>

#include "sph_device.cuh"

namespace sphk {

namespace {

constexpr int kNoAllocMaxKeys = 1 << 20;                 // largest n accepted
constexpr int kNoAllocTiles = kNoAllocMaxKeys / 4096;    // radix tiles (4096 keys each)
constexpr int kNoAllocPasses = 4;                        // 8-bit digits of 32-bit keys
constexpr size_t kOffKeys = 0;
constexpr size_t kOffVals = kOffKeys + (size_t)kNoAllocMaxKeys;
constexpr size_t kOffHist = kOffVals + (size_t)kNoAllocMaxKeys;
constexpr size_t kOffStatus = kOffHist + (size_t)kNoAllocPasses * 256;
constexpr size_t kOffInfo = kOffStatus + (size_t)kNoAllocPasses * kNoAllocTiles * 256;
constexpr size_t kScratchWords = kOffInfo + (size_t)kInfoSlots;

// The scratch of every call.  Calls share it and it keeps the last call's
// contents; each call clears the parts that must start at zero.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

// Device address of g_noalloc_scratch per device, looked up on the first call
// made with that device current.  Two host threads making their first calls
// at once may both look it up: the runtime gives both the same address, and
// the atomic store makes the publication of either one safe to read.  A
// cudaDeviceReset unloads the library's module and with it this address (the
// header tells callers not to use the function after one); a call whose
// launches fail forgets the cached address, so that the next call looks it
// up again.
constexpr int kMaxDevices = 64;
std::atomic<uint32_t*> g_scratch_ptr[kMaxDevices];

__global__ void k_noalloc_reset(uint32_t* __restrict__ hist_status, size_t words, int* __restrict__ info, int n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < words; k += stride) hist_status[k] = 0;
    if (blockIdx.x == 0 && threadIdx.x < kInfoSlots) info[threadIdx.x] = threadIdx.x == kNum ? n : 0;
}

// Digit histograms of every pass, aggregated per warp with match_any.  Pass
// ps counts the digit (key >> 8 ps) masked to the pass's width, the digit the
// radix pass ranks by: the low key_bits bits of a key are its sort key.
__global__ void __launch_bounds__(256) k_noalloc_hist(const uint32_t* __restrict__ keys, int n, int passes,
                                                      int key_bits, uint32_t* __restrict__ hist) {
    __shared__ uint32_t s_hist[kNoAllocPasses][256];
    const int tid = threadIdx.x;
    for (int k = tid; k < kNoAllocPasses * 256; k += blockDim.x) (&s_hist[0][0])[k] = 0;
    __syncthreads();
    const unsigned lane = tid & 31;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t base = (size_t)blockIdx.x * blockDim.x + (tid & ~31); base < (size_t)n; base += stride) {
        const size_t i = base + lane;
        const bool valid = i < (size_t)n;
        const uint32_t key = valid ? __ldg(keys + i) : 0u;
        for (int ps = 0; ps < passes; ++ps) {
            const int bits = key_bits - 8 * ps < 8 ? key_bits - 8 * ps : 8;
            const uint32_t d = valid ? ((key >> (8 * ps)) & ((1u << bits) - 1u)) : 0x100u;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            if (valid && (int)lane == 31 - __clz(peers)) atomicAdd(&s_hist[ps][d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int k = tid; k < passes * 256; k += blockDim.x) {
        const uint32_t c = (&s_hist[0][0])[k];
        if (c) atomicAdd(hist + k, c);
    }
}

// [a, a+n) and [b, b+n) share an element.
bool overlaps(const uint32_t* a, const uint32_t* b, int n) {
    const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b, len = (uintptr_t)n * sizeof(uint32_t);
    return x < y + len && y < x + len;
}

}  // namespace

}  // namespace sphk

extern "C" int sph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                                      uint32_t* vals_out, int n, int key_bits, void* stream) {
    using namespace sphk;
    if (n < 0 || n > kNoAllocMaxKeys) return SPH_EINVAL;  // more than 1,048,576 pairs
    if (key_bits < 1 || key_bits > 32) return SPH_EINVAL;
    if (n > 0 && (!keys_in || !vals_in || !keys_out || !vals_out)) return SPH_EINVAL;
    if (n == 0) return SPH_OK;
    // not in place: no output may share an element with an input or with the
    // other output (the inputs are only read and may overlap each other)
    if (overlaps(keys_out, keys_in, n) || overlaps(keys_out, vals_in, n) || overlaps(keys_out, vals_out, n) ||
        overlaps(vals_out, keys_in, n) || overlaps(vals_out, vals_in, n))
        return SPH_EINVAL;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SPH_ECUDA;
    uint32_t* s = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!s) {
        // First call on this device: the host-side name of the array is not a
        // device address, so ask the runtime for the address on this device.
        if (cudaGetSymbolAddress((void**)&s, g_noalloc_scratch) != cudaSuccess || !s) {
            cudaGetLastError();
            return SPH_ECUDA;
        }
        g_scratch_ptr[dev].store(s, std::memory_order_release);
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int passes = (key_bits + 7) / 8;
    int* info = reinterpret_cast<int*>(s + kOffInfo);
    const size_t zero_words = (size_t)kNoAllocPasses * 256 + (size_t)passes * kNoAllocTiles * 256;
    k_noalloc_reset<<<256, 256, 0, st>>>(s + kOffHist, zero_words, info, n);
    int hblocks = (n + 255) / 256;
    hblocks = hblocks > 152 * 8 ? 152 * 8 : hblocks;
    k_noalloc_hist<<<hblocks, 256, 0, st>>>(keys_in, n, passes, key_bits, s + kOffHist);
    // Passes alternate between the caller's output and the scratch buffer so
    // that the last one lands in the output and the input is never written.
    const uint32_t *kin = keys_in, *vin = vals_in;
    for (int ps = 0; ps < passes; ++ps) {
        const bool to_out = ((passes - 1 - ps) % 2) == 0;
        uint32_t* kout = to_out ? keys_out : s + kOffKeys;
        uint32_t* vout = to_out ? vals_out : s + kOffVals;
        int bits = key_bits - 8 * ps;
        bits = bits > 8 ? 8 : bits;
        launch_radix_pass(kin, vin, kout, vout, info, s + kOffHist + (size_t)ps * 256,
                          s + kOffStatus + (size_t)ps * kNoAllocTiles * 256, info + kSortTiles + ps, info + kError,
                          8 * ps, bits, n, st);
        kin = kout;
        vin = vout;
    }
    // The error word is read on the caller's stream, so only that stream is
    // waited for (no device-wide synchronisation).
    int err = 0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&err, info + kError, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        g_scratch_ptr[dev].store(nullptr, std::memory_order_release);
        return SPH_ECUDA;
    }
    return err ? SPH_ETIMEOUT : SPH_OK;
}
