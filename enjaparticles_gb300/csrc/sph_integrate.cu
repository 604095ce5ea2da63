// sph_integrate.cu — the staged (unfused) elementwise stages.
//   collision_wall: rtpslib/system/sph/cl_src/collision_wall.cl:31-118
//   leapfrog:       rtpslib/system/sph/cl_src/leapfrog.cl:30-121
//   gravity:        rtpslib/system/common/cl_src/gravity.cl:9-35
//   euler:          rtpslib/system/sph/cl_src/euler.cl:33-78
//   out-of-grid deletion bookkeeping of SPH::updateGPU (SPH.cpp:220-250)
// The fused step runs the same device functions (sph_physics.cuh) inside the
// force kernel.
#include "sph_physics.cuh"

namespace sphk {

__global__ void __launch_bounds__(256) k_collision(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                   float4* __restrict__ force_s, const int* __restrict__ info,
                                                   const StepParams P) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = scaled(__ldg(pos_s + i), P);
    force_s[i] = collide_walls(p, __ldg(vel_s + i), force_s[i], P);
}

void launch_collision(const float4* pos_s, const float4* vel_s, float4* force_s, const int* info,
                      const StepParams& p, int grid_items, cudaStream_t st) {
    int blocks = (grid_items + 255) / 256;
    if (blocks < 1) blocks = 1;
    k_collision<<<blocks, 256, 0, st>>>(pos_s, vel_s, force_s, info, p);
}

__global__ void __launch_bounds__(256) k_leapfrog(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                                  const float4* __restrict__ force_s,
                                                  const float4* __restrict__ xsph_s,
                                                  const uint32_t* __restrict__ idx, float4* __restrict__ pos_u,
                                                  float4* __restrict__ vel_u, float4* __restrict__ veleval_u,
                                                  const int* __restrict__ info, const StepParams P, float dt) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = scaled(__ldg(pos_s + i), P);
    float4 po, vo, eo;
    leapfrog_core(p, __ldg(vel_s + i), __ldg(force_s + i), __ldg(xsph_s + i), dt, P, po, vo, eo);
    const uint32_t o = __ldg(idx + i);
    if (!in_bounds(o, P.chk_cap, P.chk_err)) return;
    vel_u[o] = vo;
    veleval_u[o] = eo;
    pos_u[o] = po;
}

void launch_leapfrog(const float4* pos_s, const float4* vel_s, const float4* force_s, const float4* xsph_s,
                     uint32_t* idx, float4* pos_u, float4* vel_u, float4* veleval_u, const int* info,
                     const StepParams& p, float dt, int grid_items, cudaStream_t st) {
    int blocks = (grid_items + 255) / 256;
    if (blocks < 1) blocks = 1;
    k_leapfrog<<<blocks, 256, 0, st>>>(pos_s, vel_s, force_s, xsph_s, idx, pos_u, vel_u, veleval_u, info, p, dt);
}

template <bool Exact>
__global__ void __launch_bounds__(256) k_gravity(const float4* __restrict__ pos_s, float4* __restrict__ force_s,
                                                 const int* __restrict__ info, const StepParams P) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    force_s[i] = gravity_add<Exact>(force_s[i], __ldg(pos_s + i), P);
}

void launch_gravity(const float4* pos_s, float4* force_s, const int* info, const StepParams& p, int grid_items,
                    cudaStream_t st) {
    if (p.n_grav <= 0) return;
    int blocks = (grid_items + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (p.exact)
        k_gravity<true><<<blocks, 256, 0, st>>>(pos_s, force_s, info, p);
    else
        k_gravity<false><<<blocks, 256, 0, st>>>(pos_s, force_s, info, p);
}

__global__ void __launch_bounds__(256) k_euler(const float4* __restrict__ pos_s, const float4* __restrict__ vel_s,
                                               const float4* __restrict__ force_s, const uint32_t* __restrict__ idx,
                                               float4* __restrict__ pos_u, float4* __restrict__ vel_u,
                                               const int* __restrict__ info, const StepParams P, float dt) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 po, vo;
    euler_core(scaled(__ldg(pos_s + i), P), __ldg(vel_s + i), __ldg(force_s + i), dt, P, po, vo);
    const uint32_t o = __ldg(idx + i);
    if (!in_bounds(o, P.chk_cap, P.chk_err)) return;
    vel_u[o] = vo;
    pos_u[o] = po;
}

void launch_euler(const float4* pos_s, const float4* vel_s, const float4* force_s, uint32_t* idx, float4* pos_u,
                  float4* vel_u, const int* info, const StepParams& p, float dt, int grid_items, cudaStream_t st) {
    int blocks = (grid_items + 255) / 256;
    if (blocks < 1) blocks = 1;
    k_euler<<<blocks, 256, 0, st>>>(pos_s, vel_s, force_s, idx, pos_u, vel_u, info, p, dt);
}

// The fused step's velocity pass, once vel and veleval are uploaded, beside
// the density pass (which writes the 1/rho lane of rec_vi):
//   - the veleval lanes of the force pass's neighbour records, in sorted
//     order (the gather permute.cl:10-46 does into veleval_s);
//   - the out-of-grid deletion (SPH.cpp:220-250): the kept particles'
//     velocities in sorted order (call_prep copies vel_s to vel_u, done by the
//     force pass, which re-indexes them), the removed ones saved;
//   - with all_vel (the step with a triangle mesh, whose last kernel reads
//     vel_s), the sorted velocities of every kept particle, deletion or not.
__global__ void __launch_bounds__(256) k_step_velocities(const float4* __restrict__ pos_s,
                                                         const uint32_t* __restrict__ idx,
                                                         const float4* __restrict__ vel_u,
                                                         const float4* __restrict__ veleval_u,
                                                         float4* __restrict__ rec_vi, float4* __restrict__ vel_s,
                                                         float4* __restrict__ del_pos, float4* __restrict__ del_vel,
                                                         int* __restrict__ info, int all_vel) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_old) return;
    const uint32_t o = __ldg(idx + i);
    if (!in_bounds(o, (uint32_t)n_old, info + kError)) return;  // original indices are below the step's count
    if (i < n) {
        const float4 ve = __ldg(veleval_u + o);
        float* r = reinterpret_cast<float*>(rec_vi + i);
        *reinterpret_cast<float2*>(r) = make_float2(ve.x, ve.y);
        r[2] = ve.z;
    }
    if (out < 0 && !all_vel) return;
    const float4 v = __ldg(vel_u + o);
    if (i < n) {
        vel_s[i] = v;
    } else {
        del_pos[i - n] = __ldg(pos_s + i);
        del_vel[i - n] = v;
        if (i == n) info[kDeleted] = n_old - n;
    }
}

void launch_step_velocities(const float4* pos_s, const uint32_t* idx, const float4* vel_u, const float4* veleval_u,
                            float4* rec_vi, float4* vel_s, float4* del_pos, float4* del_vel, int* info, int all_vel,
                            int grid_items, cudaStream_t st) {
    const int blocks = grid_items > 0 ? (grid_items + 255) / 256 : 1;
    k_step_velocities<<<blocks, 256, 0, st>>>(pos_s, idx, vel_u, veleval_u, rec_vi, vel_s, del_pos, del_vel, info,
                                              all_vel);
}

// Staged deletion: after cellindices + permute, when some particles left the
// grid (cell_start[nb_cells] set), keep the first out_start sorted particles:
// save the removed ones, and re-index the kept ones in sorted order
// (call_prep(2) + hash_and_sort of SPH.cpp:236-247 give sort_indices = i,
// the keys being already sorted).
__global__ void __launch_bounds__(256) k_delete_staged(const float4* __restrict__ pos_s,
                                                       const float4* __restrict__ vel_s,
                                                       const float4* __restrict__ veleval_s,
                                                       uint32_t* __restrict__ idx, float4* __restrict__ pos_u,
                                                       float4* __restrict__ vel_u, float4* __restrict__ veleval_u,
                                                       float4* __restrict__ del_pos, float4* __restrict__ del_vel,
                                                       int* __restrict__ info) {
    int n_old, out;
    const int n = effective_num(info, n_old, out);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (out < 0 || i >= n_old) return;
    if (i < n) {
        idx[i] = (uint32_t)i;
        pos_u[i] = pos_s[i];
        vel_u[i] = vel_s[i];
        veleval_u[i] = veleval_s[i];
    } else {
        del_pos[i - n] = pos_s[i];
        del_vel[i - n] = vel_s[i];
        if (i == n) info[kDeleted] = n_old - n;
    }
}

void launch_delete_staged(const float4* pos_s, const float4* vel_s, const float4* veleval_s, uint32_t* idx,
                          float4* pos_u, float4* vel_u, float4* veleval_u, float4* del_pos, float4* del_vel, int* info,
                          int grid_items, cudaStream_t st) {
    int blocks = (grid_items + 255) / 256;
    if (blocks < 1) blocks = 1;
    k_delete_staged<<<blocks, 256, 0, st>>>(pos_s, vel_s, veleval_s, idx, pos_u, vel_u, veleval_u, del_pos, del_vel,
                                            info);
}

}  // namespace sphk
