// sph_batch.cuh — the batch behind the sph_batch* handle of
// include/rtps_sph.h, shared by sph_batch.cu (buffers, the batched step) and
// sph_adjoint.cu (the batched differentiable rollout).
#pragma once

#include <string>
#include <vector>

#include "sph_device.cuh"

constexpr int kBatchFrozen = 5;       // info slot: frozen particles seen by the last step
constexpr int kBatchFrozenTotal = 6;  // info slot: frozen particle-steps since the last reset

struct sph_batch_adjoint;  // recorded batched rollout (sph_adjoint.cu)

struct sph_batch {
    int device = 0, nscenes = 0, exact = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    std::vector<SPHParams> sp;
    std::vector<GridParams> gp, gps;
    std::vector<sphk::StepParams> P;
    std::vector<int> max_num, num;
    std::vector<uint32_t> slot_off, cbase;
    int nslots = 0, nvalid = 0, cell_bits = 0, scene_bits = 0, unit = 1;
    sph_launch_config lc = {256, 128, 4096, 0};  // launch shapes (sph_batch_autotune)
    // scheduler of the neighbour passes (SPH_SCHED_GRID / SPH_SCHED_QUEUE) and
    // the queue's state: [0..3] density, [4..7] force (sph_queue.cuh), its
    // tile tables, and the test hold of its table publication
    int sched = 0;
    unsigned* q_state = nullptr;
    uint32_t* q_tiles = nullptr;
    int q_hold = 0;
    unsigned q_spin = 1u << 22;
    size_t ncells_total = 0;
    uint32_t invalid_key = 0;
    unsigned params_version = 1;
    // device
    float4 *pos_u = nullptr, *vel_u = nullptr, *veleval_u = nullptr, *pos_s = nullptr, *veleval_s = nullptr;
    float4 *rec_pd = nullptr, *rec_vi = nullptr;
    float4* vel_s = nullptr;   // sorted velocities of the scenes that delete particles this step
    uint32_t* d_seg = nullptr;  // first sorted index of every scene (this step)
    int* d_del = nullptr;       // particles removed by every scene's last deletion
    float4* pos_xy = nullptr;  // sorted positions as pairs (default arithmetic's density pass)
    float2* pos_z = nullptr;
    float* density = nullptr;
    uint32_t* nbr = nullptr;   // neighbour counts (density pass) for the force pass
    uint32_t *mask = nullptr, *keys_a = nullptr, *idx_a = nullptr, *keys_b = nullptr, *idx_b = nullptr;
    uint32_t *cell_start = nullptr, *cell_end = nullptr;
    uint32_t* cell_pre = nullptr;  // prefix of the cell counts over every cell of every scene
    uint16_t* scene_of = nullptr;
    uint32_t *d_slot_off = nullptr, *d_cbase = nullptr;
    int* d_num = nullptr;
    sphk::StepParams* d_table = nullptr;
    int* info_nb = nullptr;
    // counting sort over the global cells: particles per cell (zero between
    // steps), per tile of 4096 cells, (slot index, key) per cell slot
    uint32_t *cell_count = nullptr, *cell_tile_total = nullptr;
    uint2* cell_entries = nullptr;
    int* host_info = nullptr;
    // tape outputs of the fused force pass (see sph_ctx::keep_f)
    float4 *keep_f = nullptr, *keep_v = nullptr;
    cudaGraphExec_t graph = nullptr;
    float graph_dt = 0.f;
    int graph_valid = -1, graph_exact = -1, graph_sched = -1;
    sph_launch_config graph_lc = {0, 0, 0, 0};
    sph_batch_adjoint* adj = nullptr;
    std::string err;
};

int berr(sph_batch* b, int code, const char* fmt, ...);
// Reads the per-scene particle counts back (they drop when a scene deletes
// particles that left its grid) into b->num and b->nvalid.  Blocking.
int batch_refresh_num(sph_batch* b);
sphk::ManyScenes batch_scenes(const sph_batch* b);
// ev (nullable): 5 events recorded around the cell totals+scan, the density
// pass and the force pass.
int batch_enqueue_step(sph_batch* b, float dt, cudaEvent_t* ev = nullptr);
void sph_batch_adjoint_release(sph_batch* b);

#define BCK(b, call)                                                                                  \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return berr(b, SPH_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));    \
    } while (0)
