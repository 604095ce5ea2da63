// sph_cells.cu — cell ranges and the gather into sorted order.
//
//   cellindices: rtpslib/system/common/cl_src/cellindices.cl:12-107 with the
//                host side of CellIndices::execute (CellIndices.cpp:42-99).
//                The reference stages block+1 keys in local memory behind a
//                barrier; here the previous key comes from a warp shuffle
//                (lane 0 loads it), so there is no block barrier at all.
//   permute:     rtpslib/system/common/cl_src/permute.cl:10-46, fused into the
//                same pass: X_s[i] = X_u[sort_indices[i]] with 128-bit loads.
// The fused product path gathers pos and veleval only: the leapfrog reads
// each particle's own velocity straight from vel_u.
#include "sph_device.cuh"

namespace sphk {

// Gather: 0 = cell ranges only, 1 = + pos/veleval, 2 = + pos/vel/veleval.
template <int Gather>
__global__ void __launch_bounds__(256) k_cells_permute(const uint32_t* __restrict__ keys,
                                                       const uint32_t* __restrict__ idx,
                                                       uint32_t* __restrict__ cell_start,
                                                       uint32_t* __restrict__ cell_end,
                                                       const float4* __restrict__ pos_u,
                                                       const float4* __restrict__ vel_u,
                                                       const float4* __restrict__ veleval_u,
                                                       float4* __restrict__ pos_s, float4* __restrict__ vel_s,
                                                       float4* __restrict__ veleval_s, int* __restrict__ info,
                                                       int nb_cells) {
    const int n = info[kNum];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const uint32_t ncells = (uint32_t)nb_cells;
    const uint32_t key = i < n ? keys[i] : 0xffffffffu;
    uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
    if (lane == 0 && i > 0 && i < n) prev = keys[i - 1];
    if (i >= n) return;
    if (key <= ncells) {
        prev = prev < ncells ? prev : ncells;
        if (i == 0) {
            cell_start[key] = 0;
        } else if (prev != key) {
            cell_start[key] = (uint32_t)i;
            cell_end[prev] = (uint32_t)i;
        }
        if (i == n - 1) cell_end[key] = (uint32_t)n;
        if (key == ncells && (i == 0 || prev != key)) info[kOutStart] = i;
    }
    if (Gather == 0) return;
    const uint32_t o = __ldg(idx + i);
    if (!in_bounds(o, (uint32_t)n, info + kError)) return;
    pos_s[i] = __ldg(pos_u + o);
    veleval_s[i] = __ldg(veleval_u + o);
    if (Gather == 2) vel_s[i] = __ldg(vel_u + o);
}

void launch_cells_permute(const uint32_t* keys, const uint32_t* idx, uint32_t* cell_start, uint32_t* cell_end,
                          const float4* pos_u, const float4* vel_u, const float4* veleval_u, float4* pos_s,
                          float4* vel_s, float4* veleval_s, int* info, int nb_cells, int grid_items, int gather,
                          cudaStream_t st) {
    const int threads = 256;
    int blocks = (grid_items + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    if (gather == 2)
        k_cells_permute<2><<<blocks, threads, 0, st>>>(keys, idx, cell_start, cell_end, pos_u, vel_u, veleval_u, pos_s,
                                                       vel_s, veleval_s, info, nb_cells);
    else if (gather == 1)
        k_cells_permute<1><<<blocks, threads, 0, st>>>(keys, idx, cell_start, cell_end, pos_u, vel_u, veleval_u, pos_s,
                                                       vel_s, veleval_s, info, nb_cells);
    else
        k_cells_permute<0><<<blocks, threads, 0, st>>>(keys, idx, cell_start, cell_end, pos_u, vel_u, veleval_u, pos_s,
                                                       vel_s, veleval_s, info, nb_cells);
}

// Permute alone (the staged Permute::execute entry point).
__global__ void __launch_bounds__(256) k_permute(const uint32_t* __restrict__ idx, const float4* __restrict__ pos_u,
                                                 const float4* __restrict__ vel_u,
                                                 const float4* __restrict__ veleval_u, float4* __restrict__ pos_s,
                                                 float4* __restrict__ vel_s, float4* __restrict__ veleval_s,
                                                 const int* __restrict__ info) {
    const int n = info[kNum];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = __ldg(idx + i);
    if (!in_bounds(o, (uint32_t)n, const_cast<int*>(info) + kError)) return;
    pos_s[i] = __ldg(pos_u + o);
    vel_s[i] = __ldg(vel_u + o);
    veleval_s[i] = __ldg(veleval_u + o);
}

void launch_permute_only(const uint32_t* idx, const float4* pos_u, const float4* vel_u, const float4* veleval_u,
                         float4* pos_s, float4* vel_s, float4* veleval_s, const int* info, int grid_items,
                         cudaStream_t st) {
    const int threads = 256;
    int blocks = (grid_items + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    k_permute<<<blocks, threads, 0, st>>>(idx, pos_u, vel_u, veleval_u, pos_s, vel_s, veleval_s, info);
}

}  // namespace sphk
