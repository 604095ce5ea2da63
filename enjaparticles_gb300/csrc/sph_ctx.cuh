// sph_ctx.cuh — the single-system context behind the sph_ctx* handle of
// include/rtps_sph.h, shared by the translation units that drive it
// (sph_api.cu: buffers, stages and the step graph; sph_adjoint.cu: the
// differentiable rollout).
#pragma once

#include <string>
#include <vector>

#include "sph_device.cuh"

struct sph_adjoint;  // recorded rollout and its buffers (sph_adjoint.cu)

struct sph_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // sph_upload copies veleval and vel on up_stream after the position copy,
    // so that they overlap the fused step's sort and density passes; up_done
    // marks their end (the fused step's velocity pass waits for it; every
    // other call waits for it on entry).
    cudaStream_t up_stream = nullptr;
    cudaEvent_t up_start = nullptr, up_done = nullptr;
    // the fused step's velocity pass runs on side_stream beside the density
    // pass (after the permute and the velocity upload, before force)
    cudaStream_t side_stream = nullptr;
    cudaEvent_t side_fork = nullptr, side_join = nullptr;
    bool up_pending = false;
    SPHParams sp;
    GridParams gp, gps;
    sphk::StepParams P;
    int max_num = 0;
    int num_hint = 0;  // host upper bound of the particle count (grid sizing)
    int passes = 1;
    int exact = 0;
    // launch shapes (sph_set_launch_config / sph_autotune)
    sph_launch_config lc = {256, 128, 4096, 0};
    // device state
    float4 *pos_u = nullptr, *vel_u = nullptr, *veleval_u = nullptr;
    float4 *pos_s = nullptr, *vel_s = nullptr, *veleval_s = nullptr, *force_s = nullptr, *xsph_s = nullptr;
    float4 *del_pos = nullptr, *del_vel = nullptr;
    float* density = nullptr;
    float4* rec_pd = nullptr;    // (scaled pos, rho) per sorted particle
    float4* rec_vi = nullptr;    // (veleval, 1/rho) per sorted particle
    // sorted positions as pairs for the default arithmetic's density pass:
    // (x, x', y, y') and (z, z') of sorted particles 2k, 2k+1
    float4* pos_xy = nullptr;
    float2* pos_z = nullptr;
    uint32_t* nbr = nullptr;
    uint32_t* mask = nullptr;    // neighbour bitmask [kMaskWords][max_num]
    uint32_t *keys_a = nullptr, *idx_a = nullptr, *keys_b = nullptr, *idx_b = nullptr;
    uint32_t *keys_cur = nullptr, *idx_cur = nullptr;  // what SORT_HASHES / SORT_INDICES show
    uint32_t *cell_start = nullptr, *cell_end = nullptr;
    uint32_t* cell_pre = nullptr;  // the counting sort's prefix of the cell counts, every cell
    int* info = nullptr;
    uint32_t* scratch = nullptr;
    size_t scratch_words = 0;
    uint32_t* hist = nullptr;    // [4][256]
    uint32_t* status = nullptr;  // [passes][tiles][256]
    int tiles_cap = 0;
    // counting sort of the step (sph_cellsort.cu): particles per cell (zero
    // between steps), particles per tile of 4096 cells, (index, key) per slot
    uint32_t* cell_count = nullptr;
    uint32_t* cell_tile_total = nullptr;
    uint2* cell_entries = nullptr;
    int* host_info = nullptr;  // pinned
    // When set, the fused step also stores, per sorted particle, the SPH
    // force before the walls (keep_f) and the step's input velocity (keep_v):
    // the tape of the differentiable rollout.
    float4 *keep_f = nullptr, *keep_v = nullptr;
    // point gravity sources (device: positions, masses, alphas) and the integrator
    float4* grav = nullptr;
    int n_grav = 0;
    int integrator = 0;
    // triangle mesh: one allocation of tri_cap * 10 float4 (raw, geo, box)
    // and 2 float4 per 256 triangles (tile boxes)
    float4* tri = nullptr;
    int n_tri = 0;
    int tri_cap = 0;
    // hoses (SPH::addHose), sprayed at the start of every update
    std::vector<sph_hose*> hoses;
    // surface (sph_surface.cu): colour field, marching-cubes scan scratch, the
    // case table on the device, the mesh (vertices, then normals)
    float* cf = nullptr;
    size_t cf_cap = 0;
    double* cf_inv = nullptr;  // 1/rho per sorted particle, in double
    size_t cf_inv_cap = 0;
    int cf_res = 0;
    unsigned* mc_scan = nullptr;
    size_t mc_scan_cap = 0;
    signed char* mc_table = nullptr;
    float* mesh = nullptr;
    size_t mesh_cap = 0;
    int mesh_tri = 0;
    int mesh_res = 0;
    // graph of one fused step
    cudaGraphExec_t graph = nullptr;
    float graph_dt = 0.f;
    int graph_num = -1;
    int graph_exact = -1;
    unsigned params_version = 1, graph_version = 0;
    sph_adjoint* adj = nullptr;
    std::string err;
};

// Records the message (on the context, or as the last creation error when c
// is null) and returns code.
int set_err(sph_ctx* c, int code, const char* fmt, ...);
// Makes the context's device current and, unless join is false, orders
// the context stream after a pending upload's side-stream copies.
int check_ctx(sph_ctx* c, bool join = true);
// The step's wait for a pending upload, enqueued right before cells+permute
// (an external event wait node when the stream is being captured).
int join_upload(sph_ctx* c);
int join_upload_on(sph_ctx* c, cudaStream_t st);
// Enqueues one fused step (hash .. leapfrog) on c->stream.
int enqueue_fused_step(sph_ctx* c, float dt);
// Reads the device counters into c->host_info (synchronises the stream).
int read_info(sph_ctx* c);
// Frees the differentiable-rollout state of c (no-op when there is none).
void sph_adjoint_release(sph_ctx* c);

#define CK(ctx, call)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return set_err(ctx, SPH_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define CK_LAUNCH(ctx)                                                                                       \
    do {                                                                                                     \
        cudaError_t e_ = cudaGetLastError();                                                                 \
        if (e_ != cudaSuccess) return set_err(ctx, SPH_ECUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
    } while (0)
