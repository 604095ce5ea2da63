// sph_device.cuh — shared device-side definitions of the GB300 SPH step.
//
// Layout in HBM (one context, capacity max_num particles, C = nb_cells):
//   state, original order    pos_u, vel_u, veleval_u          float4[max_num]
//   sorted copies            pos_s, veleval_s (vel_s, force_s, xsph_s: staged
//                            path only)                          float4[max_num]
//   density_s, neighbour count                                  float/u32[max_num]
//   sort_hashes / sort_indices + radix ping-pong buffers        u32[max_num] x 4
//   cell_start, cell_end                                        u32[C+1]
//   counters (num, out-of-grid start, error word), radix scratch
// All particle arrays are float4 AoS, 16 B per particle, read with 128-bit
// loads.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rtps_sph.h"

namespace sphk {

constexpr uint32_t kEmpty = 0xffffffffu;
// Coordinate of the unused lane of the last position pair (never a neighbour).
constexpr float kFarAway = 1.0e18f;

// Device counters block (ctx->info).
enum InfoSlot : int {
    kNum = 0,        // particle count at the start of the step
    kOutStart = 1,   // first sorted index whose key is nb_cells, -1 if none
    kError = 2,      // bit flags, see kErr*
    kDeleted = 3,    // number of particles removed by the last out-of-grid deletion
    kSortTiles = 4,  // 4 slots: tile counters of the radix passes
    kInfoSlots = 16
};
constexpr int kErrLookbackTimeout = 1;
// Bit of the error word: a bounds-checked build found an index outside the
// array it addresses (the access was skipped).
constexpr int kErrBounds = 4;

// Bounds-checked builds (-DSPH_CHECKED: librtps_sph_checked.so).  Every
// gather and scatter index of the step's kernels is tested against the array
// it addresses before the access; a failed test sets kErrBounds in the
// context's error word and skips the access, so that an indexing error shows
// up as a status (SPH_EBOUNDS) where the default build would read or write
// out of bounds.  In the default build in_bounds is the constant true and the
// tests compile away.
#ifdef SPH_CHECKED
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif
__device__ __forceinline__ bool in_bounds(uint32_t i, uint32_t bound, int* err) {
    if constexpr (!kChecked) {
        return true;
    } else {
        if (i < bound) return true;
        atomicOr(err, kErrBounds);
        return false;
    }
}

// Neighbour bitmask written by the density pass: bit b of particle i says
// whether its b-th candidate (in walk order) is a neighbour other than itself;
// word w of particle i lives at mask[w * stride + i].
constexpr int kMaskWords = 16;
constexpr int kMaskBits = 32 * kMaskWords;

// Parameters every kernel of the step needs, passed by value.
struct StepParams {
    // SPHParams (floats copied once on the host)
    float sc, h, h2, rcut2, mass, rho0, K, eps, visc, wpoly6, wspiky_d, wvisc_dd, xsph_factor, vlimit;
    float kwall, cwall, bound;  // boundary stiffness, dampening, rest_distance*0.5
    float4 gravity;
    float dens_coef;   // wpoly6 * mass (float product, as density.cl:120)
    float coef_b;      // (float)(-0.5 * (double)wspiky_d)
    float coef_s;      // viscosity * wvisc_dd (float)
    float coef_d;      // (float)(2.0 * (double)mass * (double)wpoly6)
    float inv_eps;     // 1 / eps, correctly rounded (the force pass's clamp)
    // unscaled grid (hash) and scaled grid (neighbour walk, walls)
    float4 g_min, g_delta, g_res;
    float4 gs_min, gs_delta, gs_res, gs_bnd_min, gs_bnd_max;
    int nb_cells;
    int res_x, res_y, res_z;      // integer grid_res of the scaled grid
    int int_hash_ok;              // integer neighbour hashing equals the float formula
    int unit_scale;               // simulation_scale == 1.0f
    // point gravity sources (gravity.cl), none by default
    int n_grav;
    const float4* grav_pos;
    const float* grav_mass;
    const float* grav_alpha;
    int integrator;               // kIntegratorLeapfrog or kIntegratorEuler
    int exact;                    // exact arithmetic in the elementwise stages
    // triangle mesh (collision_tri.cl), none by default
    int n_tri;
    float tri_bound;              // boundary_distance
    const float4* tri_raw;        // 4 float4 per triangle, as loaded
    float4* tri_geo;              // 4 float4 per triangle (sph_triangles.cu)
    float4* tri_box;              // 2 float4 per triangle
    float4* tri_tile;             // 2 float4 per 256 triangles
    // bounds-checked builds: slots of the particle arrays (a batch: of all
    // scenes) and the error word that in_bounds reports to
    uint32_t chk_cap;
    int* chk_err;
};
constexpr int kIntegratorLeapfrog = 0;
constexpr int kIntegratorEuler = 1;
constexpr int kMaxGravitySources = 64;
constexpr int kMaxTriangles = 1 << 20;

// Scenes of the neighbour passes.
//   OneScene: one particle system; the step parameters are the kernel
//   argument and the cell arrays are the context's.
//   ManyScenes: a batch of independent systems sorted together; the scene of
//   sorted particle i is the high part of its key (key = scene << cell_bits |
//   cell), each scene has its own parameter block and its own segment of the
//   cell arrays.  A particle in its scene's out-of-grid cell is left out of
//   the neighbour passes (`frozen`) and deleted by the force pass, as a lone
//   system deletes it (SPH.cpp:220-250): the scene keeps its first sorted
//   particles, re-indexed in sorted order, and the removed ones go to the
//   slots after them.
struct OneScene {
    static constexpr bool kBatch = false;
    StepParams P;
    __device__ __forceinline__ const StepParams& params(int) const { return P; }
    __device__ __forceinline__ uint32_t cell_base(int) const { return 0u; }
    __device__ __forceinline__ bool frozen(int) const { return false; }
    __device__ __forceinline__ uint32_t scene(int) const { return 0u; }
};
struct ManyScenes {
    static constexpr bool kBatch = true;
    const StepParams* table;
    const uint32_t* cbase;
    const uint32_t* keys;
    int cell_bits;
    // deletion (the force pass of the batched step; null elsewhere)
    const uint32_t* seg;       // first sorted index of every scene this step
    const uint32_t* slot_off;  // first particle slot of every scene
    const uint32_t* cstart;    // cell_start of all scenes' cells
    int* num;                  // particles per scene
    int* del;                  // particles removed by the scene's last deletion
    const float4* vel_s;       // sorted velocities of the scenes that delete
    __device__ __forceinline__ uint32_t scene(int i) const { return __ldg(keys + i) >> cell_bits; }
    __device__ __forceinline__ const StepParams& params(int i) const { return table[scene(i)]; }
    __device__ __forceinline__ uint32_t cell_base(int i) const { return __ldg(cbase + scene(i)); }
    __device__ __forceinline__ bool frozen(int i) const {
        const uint32_t k = __ldg(keys + i);
        return (k & ((1u << cell_bits) - 1u)) == (uint32_t)table[k >> cell_bits].nb_cells;
    }
    // First out-of-grid sorted index of scene s, kEmpty when it has none.
    __device__ __forceinline__ uint32_t out_start(uint32_t s) const {
        return __ldg(cstart + __ldg(cbase + s) + (uint32_t)table[s].nb_cells);
    }
};

// float -> int as the kernels' (int) cast, truncating toward zero; the
// hardware conversion saturates and maps NaN to 0.
__device__ __forceinline__ int f2i_rz(float v) { return __float2int_rz(v); }

// calcGridCell (system/common/cl_src/cl_hash.h:33-54), exact float ops.
__device__ __forceinline__ int3 grid_cell(float px, float py, float pz, const float4& gmin, const float4& gdelta) {
    int3 c;
    c.x = f2i_rz(__fmul_rn(__fsub_rn(px, gmin.x), gdelta.x));
    c.y = f2i_rz(__fmul_rn(__fsub_rn(py, gmin.y), gdelta.y));
    c.z = f2i_rz(__fmul_rn(__fsub_rn(pz, gmin.z), gdelta.z));
    return c;
}

// calcGridHash (cl_hash.h:57-114): ((gz*res.y + gy)*res.x + gx) in float,
// every operation separately rounded, then (int).
__device__ __forceinline__ int grid_hash_f(int gx, int gy, int gz, const float4& res) {
    float a = __fmul_rn((float)gz, res.y);
    float b = __fadd_rn(a, (float)gy);
    float c = __fmul_rn(b, res.x);
    float d = __fadd_rn(c, (float)gx);
    return f2i_rz(d);
}

// |r|^2 with the reference's association ((x*x + y*y) + z*z), no contraction.
__device__ __forceinline__ float dist2_exact(float dx, float dy, float dz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }



// Launch helpers implemented in the .cu files.
void launch_prologue(uint32_t* hist, int* info, cudaStream_t st);
void launch_sort_reset(uint32_t* status, size_t words, int* tile_counters, cudaStream_t st);
void launch_hash(const float4* pos_u, uint32_t* keys, uint32_t* idx, uint32_t* cell_start, uint32_t* hist,
                 const int* info, const StepParams& p, int grid_items, int passes, int clear_cells,
                 cudaStream_t st);
void launch_radix_pass(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, const int* info,
                       const uint32_t* hist, uint32_t* status, int* tile_counter, int* err, int shift, int bits,
                       int grid_items, cudaStream_t st);
int radix_tiles(int n);
// Counting sort on the cell key (sph_cellsort.cu): count, totals, scan,
// place, then permute (which reads veleval_u/vel_u: after any upload join).
int cell_scan_tiles(int cells, int tile_cells);
void launch_cell_count(const float4* pos_u, uint32_t* key_of, uint32_t* slot_of, uint32_t* count, const int* info,
                       const StepParams& p, int grid_items, cudaStream_t st);
// totals and scan over cells [0, cells); info null for a batch.  Above
// kDirectTiles tiles of 4096 cells the scan first scans the tile totals in
// one block (one more launch) instead of summing them in every block.
constexpr int kDirectTiles = 2048;
// tile_cells: cells per scan tile (2048, 4096 or 8192); tile_total holds
// cell_scan_tiles(cells, 2048) words, enough for any of them.
constexpr int kScanTileMin = 2048;
void launch_cell_totals(const uint32_t* count, uint32_t* tile_total, int* info, uint32_t cells, int tile_cells,
                        cudaStream_t st);
// pre (nullable): the exclusive prefix of the counts over every cell, empty
// ones included (pre[k]: sorted particles with a key below k), so that the
// sorted particles of cells lo..hi are pre[lo] .. pre[hi + 1] - 1.
void launch_cell_scan(uint32_t* count, uint32_t* cell_start, uint32_t* cell_end, uint32_t* tile_total, int* info,
                      uint32_t cells, int tile_cells, cudaStream_t st, uint32_t* pre = nullptr);
void launch_cell_place(const uint32_t* key_of, const uint32_t* slot_of, const uint32_t* cell_start, uint2* entries,
                       const int* info, int grid_items, cudaStream_t st);
// pxy / pz (nullable): the sorted positions also as pairs (launch_density).
void launch_cell_permute(const uint2* entries, const uint32_t* cell_start, const uint32_t* cell_end, uint32_t* keys,
                         uint32_t* idx, const float4* pos_u, const float4* vel_u, const float4* veleval_u,
                         float4* pos_s, float4* vel_s, float4* veleval_s, const int* info, int grid_items, int gather,
                         float4* pxy, float2* pz, cudaStream_t st);
void launch_cells_permute(const uint32_t* keys, const uint32_t* idx, uint32_t* cell_start, uint32_t* cell_end,
                          const float4* pos_u, const float4* vel_u, const float4* veleval_u, float4* pos_s,
                          float4* vel_s, float4* veleval_s, int* info, int nb_cells, int grid_items, int gather,
                          cudaStream_t st);
// pxy / pz: the sorted positions as pairs (k_density_pairs, sph_density.cu),
// used by the default arithmetic at unit simulation scale (nullable: the
// scalar pass then runs); pack: write them from pos_s first (for sorts
// whose permute does not).
void launch_density(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd, float4* rec_vi,
                    uint32_t* nbr, uint32_t* mask, size_t mask_stride, const uint32_t* cell_start,
                    const uint32_t* cell_end, const int* info, const StepParams& p, int grid_items, float4* pxy,
                    float2* pz, bool pack, int threads, cudaStream_t st, const uint32_t* keys = nullptr,
                    const uint32_t* cell_pre = nullptr);
// The fused step's velocity pass, beside density and before force (the first
// passes that need the uploaded velocities): the veleval lanes of rec_vi in
// sorted order, and the out-of-grid bookkeeping (kept velocities into vel_s
// in sorted order, removed particles into del_pos/del_vel); all_vel: vel_s of
// every kept particle in every step.
void launch_step_velocities(const float4* pos_s, const uint32_t* idx, const float4* vel_u, const float4* veleval_u,
                            float4* rec_vi, float4* vel_s, float4* del_pos, float4* del_vel, int* info, int all_vel,
                            int grid_items, cudaStream_t st);
// keep_f / keep_v (fused only, nullable): per sorted particle, the SPH force
// before the walls and the velocity the step integrates.
// nbr: the density pass's neighbour counts (itself included), which give the
// force pass the length of its neighbour loop.
void launch_force(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                  size_t mask_stride, const uint32_t* nbr, const uint32_t* cell_start, const uint32_t* cell_end, const int* info,
                  float4* force_s, float4* xsph_s, uint32_t* idx, const float4* vel_s, float4* pos_u, float4* vel_u,
                  float4* veleval_u, float4* keep_f, float4* keep_v, const StepParams& p, float dt, int fused,
                  int exact, int grid_items, int threads, cudaStream_t st, const uint32_t* cell_pre = nullptr);
// Batch forms of the neighbour passes (fused force only).
void launch_density_batch(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd,
                          float4* rec_vi, uint32_t* nbr, uint32_t* mask, size_t mask_stride,
                          const uint32_t* cell_start, const uint32_t* cell_end, const int* info,
                          const ManyScenes& scenes, bool unit, int exact, int grid_items, float4* pxy, float2* pz,
                          bool pack, int threads, cudaStream_t st, const uint32_t* cell_pre = nullptr);
void launch_force_batch(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                        size_t mask_stride, const uint32_t* nbr, const uint32_t* cell_start, const uint32_t* cell_end, const int* info,
                        uint32_t* idx, float4* pos_u, float4* vel_u, float4* veleval_u, float4* keep_f,
                        float4* keep_v, const ManyScenes& scenes, bool unit, float dt, int exact, int grid_items,
                        int threads, cudaStream_t st, const uint32_t* cell_pre = nullptr);
// The batch's neighbour passes under the queue scheduler (sph_queue.cuh):
// persistent blocks taking (scene, tile) items from Q.
struct BatchQueue;
void launch_density_queue(const float4* pos_s, const float4* veleval_s, float* density, float4* rec_pd,
                          float4* rec_vi, uint32_t* nbr, uint32_t* mask, size_t mask_stride,
                          const uint32_t* cell_start, const uint32_t* cell_end, float4* pxy, float2* pz,
                          const BatchQueue& Q, bool unit, int exact, int threads, cudaStream_t st);
void launch_force_queue(const float4* pos_s, const float4* rec_pd, const float4* rec_vi, const uint32_t* mask,
                        size_t mask_stride, const uint32_t* nbr, const uint32_t* cell_start,
                        const uint32_t* cell_end, uint32_t* idx, float4* pos_u, float4* vel_u, float4* veleval_u,
                        float4* keep_f, float4* keep_v, const BatchQueue& Q, bool unit, float dt, int exact,
                        int threads, cudaStream_t st);
void launch_collision(const float4* pos_s, const float4* vel_s, float4* force_s, const int* info,
                      const StepParams& p, int grid_items, cudaStream_t st);
void launch_leapfrog(const float4* pos_s, const float4* vel_s, const float4* force_s, const float4* xsph_s,
                     uint32_t* idx, float4* pos_u, float4* vel_u, float4* veleval_u, const int* info,
                     const StepParams& p, float dt, int grid_items, cudaStream_t st);
void launch_gravity(const float4* pos_s, float4* force_s, const int* info, const StepParams& p, int grid_items,
                    cudaStream_t st);
// collision_triangle after the walls; no-op without a mesh.
void launch_triangles(const float4* pos_s, const float4* vel_s, float4* force_s, const int* info, const StepParams& p,
                      int grid_items, cudaStream_t st);
// The end of the step with a mesh: gravity, walls, triangles and the
// integrator in one kernel after the (unfused) force pass.
void launch_triangles_step(const float4* pos_s, const float4* vel_s, const float4* force_s, const float4* xsph_s,
                           uint32_t* idx, float4* pos_u, float4* vel_u, float4* veleval_u, const int* info,
                           const StepParams& p, float dt, int grid_items, cudaStream_t st);
void launch_euler(const float4* pos_s, const float4* vel_s, const float4* force_s, uint32_t* idx, float4* pos_u,
                  float4* vel_u, const int* info, const StepParams& p, float dt, int grid_items, cudaStream_t st);
void launch_delete_staged(const float4* pos_s, const float4* vel_s, const float4* veleval_s, uint32_t* idx,
                          float4* pos_u, float4* vel_u, float4* veleval_u, float4* del_pos, float4* del_vel, int* info,
                          int grid_items, cudaStream_t st);
void launch_permute_only(const uint32_t* idx, const float4* pos_u, const float4* vel_u, const float4* veleval_u,
                         float4* pos_s, float4* vel_s, float4* veleval_s, const int* info, int grid_items,
                         cudaStream_t st);

}  // namespace sphk

// Host helpers shared by the single-system and batch APIs (sph_api.cu).
#include <string>
#include <tuple>

// The autotuner's candidate launch shapes, its per-process results keyed by
// (kind: 0 one system, 1 batch; particle slots; cells; arithmetic mode), and
// its choice per knob from the candidates' times t[k] = (density, force,
// cell totals + scan).
struct SphTuneKey {
    int kind;
    long long slots, cells;
    int exact;
    bool operator<(const SphTuneKey& o) const {
        return std::tie(kind, slots, cells, exact) < std::tie(o.kind, o.slots, o.cells, o.exact);
    }
};
extern const sph_launch_config sph_tune_candidates[3];
bool sph_launch_config_valid(const sph_launch_config& g);
bool sph_tune_cache_get(const SphTuneKey& k, sph_launch_config& out);
void sph_tune_cache_put(const SphTuneKey& k, const sph_launch_config& v);
sph_launch_config sph_tune_pick(const double t[3][3]);
int sph_make_step_params(const SPHParams& s, const GridParams& gp, const GridParams& gps, sphk::StepParams& P,
                         std::string& err);
GridParams sph_scaled_grid(const GridParams& g, float sc);
