// sph_api.cu — the C ABI of include/rtps_sph.h: context, buffers, stages, and
// the CUDA-graph step.  Replaces the reference's OpenCL host layer
// (rtpslib/opencl/{CLL,Kernel,Buffer}) and the buffer setup of
// System::prepareSorted / SPH::prepareSorted (System.cpp:198-291,
// SPH.cpp:482-520).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "sph_ctx.cuh"

using sphk::StepParams;

// the message of the last failed sph_create on this host thread
static thread_local std::string g_create_error;

int set_err(sph_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c)
        c->err = buf;
    else
        g_create_error = buf;
    return code;
}

namespace {

__global__ void k_fill_u32(uint32_t* p, size_t n, uint32_t v) {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) p[k] = v;
}
__global__ void k_set_num(int* info, int n) {
    info[sphk::kNum] = n;
    info[sphk::kOutStart] = -1;
    info[sphk::kDeleted] = 0;
    info[sphk::kError] = 0;
}

void fill_u32(uint32_t* p, size_t n, uint32_t v, cudaStream_t st) {
    int blocks = (int)((n + 255) / 256);
    blocks = blocks < 1 ? 1 : (blocks > 4096 ? 4096 : blocks);
    k_fill_u32<<<blocks, 256, 0, st>>>(p, n, v);
}

int bit_width(uint32_t v) {
    int b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

float next_up(float x) { return std::nextafter(x, INFINITY); }
float next_down(float x) { return std::nextafter(x, -INFINITY); }

// Largest float t with sqrtf(t) <= h: |r| <= h  <=>  r2 <= t.
float cutoff_r2(float h) {
    float t = h * h;
    while (t > 0.f && std::sqrt(t) > h) t = next_down(t);
    while (std::sqrt(next_up(t)) <= h) t = next_up(t);
    return t;
}

bool finite_params(const SPHParams& s) {
    const float* f = reinterpret_cast<const float*>(&s);
    for (int k = 0; k < 27; ++k)
        if (!std::isfinite(f[k])) return false;
    return std::isfinite(s.gravity.x) && std::isfinite(s.gravity.y) && std::isfinite(s.gravity.z) &&
           std::isfinite(s.gravity.w);
}

float4 to_f4(const sph_float4& v) { return make_float4(v.x, v.y, v.z, v.w); }

}  // namespace

// Per-step kernel parameters of one system (also used by the batch API).
int sph_make_step_params(const SPHParams& s, const GridParams& gp, const GridParams& gps, StepParams& P,
                         std::string& err) {
    if (!finite_params(s)) {
        err = "SPHParams holds a non-finite value";
        return SPH_EINVAL;
    }
    if (!(s.smoothing_distance > 0.f)) {
        err = "smoothing_distance must be > 0";
        return SPH_EINVAL;
    }
    if (!(s.simulation_scale > 0.f)) {
        err = "simulation_scale must be > 0";
        return SPH_EINVAL;
    }
    P.sc = s.simulation_scale;
    P.h = s.smoothing_distance;
    P.h2 = s.smoothing_distance * s.smoothing_distance;
    P.rcut2 = cutoff_r2(s.smoothing_distance);
    P.mass = s.mass;
    P.rho0 = s.rest_density;
    P.K = s.K;
    P.eps = s.EPSILON;
    P.inv_eps = 1.0f / s.EPSILON;
    P.visc = s.viscosity;
    P.wpoly6 = s.wpoly6_coef;
    P.wspiky_d = s.wspiky_d_coef;
    P.wvisc_dd = s.wvisc_dd_coef;
    P.xsph_factor = s.xsph_factor;
    P.vlimit = s.velocity_limit;
    P.kwall = s.boundary_stiffness;
    P.cwall = s.boundary_dampening;
    P.bound = s.rest_distance * .5f;
    P.gravity = to_f4(s.gravity);
    P.dens_coef = s.wpoly6_coef * s.mass;
    P.coef_b = (float)(-0.5 * (double)s.wspiky_d_coef);
    P.coef_s = s.viscosity * s.wvisc_dd_coef;
    P.coef_d = (float)(2.0 * (double)s.mass * (double)s.wpoly6_coef);
    P.g_min = to_f4(gp.grid_min);
    P.g_delta = to_f4(gp.grid_delta);
    P.g_res = to_f4(gp.grid_res);
    P.gs_min = to_f4(gps.grid_min);
    P.gs_delta = to_f4(gps.grid_delta);
    P.gs_res = to_f4(gps.grid_res);
    P.gs_bnd_min = to_f4(gps.bnd_min);
    P.gs_bnd_max = to_f4(gps.bnd_max);
    P.nb_cells = gp.nb_cells;
    P.res_x = (int)gps.grid_res.x;
    P.res_y = (int)gps.grid_res.y;
    P.res_z = (int)gps.grid_res.z;
    const bool integral = (float)P.res_x == gps.grid_res.x && (float)P.res_y == gps.grid_res.y &&
                          (float)P.res_z == gps.grid_res.z && P.res_x > 0 && P.res_y > 0 && P.res_z > 0;
    const double span = (double)(P.res_x + 4) * (P.res_y + 4) * (P.res_z + 4);
    P.int_hash_ok = (integral && span < 16777216.0) ? 1 : 0;
    P.unit_scale = s.simulation_scale == 1.0f ? 1 : 0;
    P.n_grav = 0;
    P.grav_pos = nullptr;
    P.grav_mass = nullptr;
    P.grav_alpha = nullptr;
    P.integrator = sphk::kIntegratorLeapfrog;
    P.exact = 0;
    P.n_tri = 0;
    P.tri_bound = s.boundary_distance;
    P.tri_raw = nullptr;
    P.tri_geo = nullptr;
    P.tri_box = nullptr;
    P.tri_tile = nullptr;
    return SPH_OK;
}

// System::setupDomain's scaled copy (System.cpp:318-325): lanes times
// sim_scale, delta times the float reciprocal of sim_scale.
GridParams sph_scaled_grid(const GridParams& g, float sc) {
    auto mul = [sc](sph_float4 v) {
        v.x = sc * v.x; v.y = sc * v.y; v.z = sc * v.z; v.w = sc * v.w;
        return v;
    };
    auto div = [sc](sph_float4 v) {
        const float d = 1.f / sc;
        v.x = d * v.x; v.y = d * v.y; v.z = d * v.z; v.w = d * v.w;
        return v;
    };
    GridParams s = g;
    s.grid_min = mul(g.grid_min);
    s.grid_max = mul(g.grid_max);
    s.bnd_min = mul(g.bnd_min);
    s.bnd_max = mul(g.bnd_max);
    s.grid_size = mul(g.grid_size);
    s.grid_delta = div(g.grid_delta);
    return s;
}

namespace {

int build_step_params(sph_ctx* c) {
    std::string err;
    const int rc = sph_make_step_params(c->sp, c->gp, c->gps, c->P, err);
    if (rc != SPH_OK) return set_err(c, rc, "%s", err.c_str());
    c->P.n_grav = c->n_grav;
    c->P.grav_pos = c->grav;
    c->P.grav_mass = reinterpret_cast<const float*>(c->grav + sphk::kMaxGravitySources);
    c->P.grav_alpha = c->P.grav_mass + sphk::kMaxGravitySources;
    c->P.integrator = c->integrator;
    c->P.exact = c->exact;
    c->P.n_tri = c->n_tri;
    c->P.chk_cap = (uint32_t)c->max_num;
    c->P.chk_err = c->info ? c->info + sphk::kError : nullptr;
    if (c->tri) {
        c->P.tri_raw = c->tri;
        c->P.tri_geo = c->tri + 4 * (size_t)c->tri_cap;
        c->P.tri_box = c->tri + 8 * (size_t)c->tri_cap;
        c->P.tri_tile = c->tri + 10 * (size_t)c->tri_cap;
    }
    c->params_version++;
    return SPH_OK;
}

size_t field_elem_bytes(int field) {
    switch (field) {
        case SPH_FIELD_DENSITY_S:
        case SPH_FIELD_SORT_HASHES:
        case SPH_FIELD_SORT_INDICES:
        case SPH_FIELD_CELL_START:
        case SPH_FIELD_CELL_END:
        case SPH_FIELD_NEIGHBOR_COUNT:
            return 4;
        default:
            return 16;
    }
}

void* field_ptr(sph_ctx* c, int field) {
    switch (field) {
        case SPH_FIELD_POS_U: return c->pos_u;
        case SPH_FIELD_VEL_U: return c->vel_u;
        case SPH_FIELD_VELEVAL_U: return c->veleval_u;
        case SPH_FIELD_POS_S: return c->pos_s;
        case SPH_FIELD_VEL_S: return c->vel_s;
        case SPH_FIELD_VELEVAL_S: return c->veleval_s;
        case SPH_FIELD_DENSITY_S: return c->density;
        case SPH_FIELD_FORCE_S: return c->force_s;
        case SPH_FIELD_XSPH_S: return c->xsph_s;
        case SPH_FIELD_SORT_HASHES: return c->keys_cur;
        case SPH_FIELD_SORT_INDICES: return c->idx_cur;
        case SPH_FIELD_CELL_START: return c->cell_start;
        case SPH_FIELD_CELL_END: return c->cell_end;
        case SPH_FIELD_NEIGHBOR_COUNT: return c->nbr;
        default: return nullptr;
    }
}

int field_capacity(sph_ctx* c, int field) {
    return (field == SPH_FIELD_CELL_START || field == SPH_FIELD_CELL_END) ? c->gp.nb_cells + 1 : c->max_num;
}

void free_all(sph_ctx* c) {
    sph_adjoint_release(c);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    void* ptrs[] = {c->pos_u, c->vel_u, c->veleval_u, c->pos_s, c->vel_s, c->veleval_s, c->force_s, c->xsph_s,
                    c->del_pos, c->del_vel, c->density, c->rec_pd, c->rec_vi, c->nbr, c->mask, c->keys_a, c->idx_a, c->keys_b, c->idx_b,
                    c->cell_start, c->cell_end, c->info, c->scratch, c->grav, c->tri, c->cf, c->cf_inv,
                    c->mc_scan, c->mc_table, c->mesh, c->cell_count, c->cell_tile_total, c->cell_entries,
                    c->pos_xy, c->pos_z, c->cell_pre};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->host_info) cudaFreeHost(c->host_info);
    if (c->up_done) cudaEventDestroy(c->up_done);
    if (c->side_fork) cudaEventDestroy(c->side_fork);
    if (c->side_join) cudaEventDestroy(c->side_join);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    if (c->up_start) cudaEventDestroy(c->up_start);
    if (c->up_stream) cudaStreamDestroy(c->up_stream);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
}

// Buffers the hash writes and the sort reads first, so that the last radix
// pass lands in keys_a / idx_a.
uint32_t* hash_keys(sph_ctx* c) { return (c->passes & 1) ? c->keys_b : c->keys_a; }
uint32_t* hash_idx(sph_ctx* c) { return (c->passes & 1) ? c->idx_b : c->idx_a; }

// --- launch sequences ------------------------------------------------------
int enqueue_hash(sph_ctx* c) {
    sphk::launch_prologue(c->hist, c->info, c->stream);
    sphk::launch_hash(c->pos_u, hash_keys(c), hash_idx(c), c->cell_start, c->hist, c->info, c->P, c->num_hint,
                      c->passes, 1, c->stream);
    c->keys_cur = hash_keys(c);
    c->idx_cur = hash_idx(c);
    CK_LAUNCH(c);
    return SPH_OK;
}

int enqueue_sort(sph_ctx* c) {
    sphk::launch_sort_reset(c->status, (size_t)c->passes * c->tiles_cap * 256, c->info + sphk::kSortTiles,
                            c->stream);
    uint32_t *kin = hash_keys(c), *vin = hash_idx(c);
    uint32_t *kout = (kin == c->keys_a) ? c->keys_b : c->keys_a, *vout = (vin == c->idx_a) ? c->idx_b : c->idx_a;
    const int total_bits = bit_width((uint32_t)c->gp.nb_cells);
    for (int ps = 0; ps < c->passes; ++ps) {
        const int shift = ps * 8;
        int bits = total_bits - shift;
        bits = bits > 8 ? 8 : (bits < 1 ? 1 : bits);
        sphk::launch_radix_pass(kin, vin, kout, vout, c->info, c->hist + ps * 256,
                                c->status + (size_t)ps * c->tiles_cap * 256, c->info + sphk::kSortTiles + ps,
                                c->info + sphk::kError, shift, bits, c->num_hint, c->stream);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    c->keys_cur = c->keys_a;
    c->idx_cur = c->idx_a;
    CK_LAUNCH(c);
    return SPH_OK;
}

// The step's sort: counting sort on the cell key up to the sorted arrays,
// cell ranges and the gather (gather 0: pos, 2: pos/vel/veleval).
int enqueue_cell_sort(sph_ctx* c, int gather) {
    cudaStream_t st = c->stream;
    sphk::launch_cell_count(c->pos_u, c->keys_b, c->idx_b, c->cell_count, c->info, c->P, c->num_hint, st);
    const uint32_t cells = (uint32_t)c->gp.nb_cells + 1u;
    sphk::launch_cell_totals(c->cell_count, c->cell_tile_total, c->info, cells, c->lc.scan_tile_cells, st);
    sphk::launch_cell_scan(c->cell_count, c->cell_start, c->cell_end, c->cell_tile_total, c->info, cells,
                           c->lc.scan_tile_cells, st, c->cell_pre);
    sphk::launch_cell_place(c->keys_b, c->idx_b, c->cell_start, c->cell_entries, c->info, c->num_hint, st);
    // the permute gathers the velocities when gather == 2
    if (gather == 2) {
        const int rc = join_upload(c);
        if (rc) return rc;
    }
    sphk::launch_cell_permute(c->cell_entries, c->cell_start, c->cell_end, c->keys_a, c->idx_a, c->pos_u, c->vel_u,
                              c->veleval_u, c->pos_s, c->vel_s, c->veleval_s, c->info, c->num_hint, gather, c->pos_xy,
                              c->pos_z, st);
    c->keys_cur = c->keys_a;
    c->idx_cur = c->idx_a;
    CK_LAUNCH(c);
    return SPH_OK;
}

// Density over the sorted arrays (with the neighbour counts the force pass
// reads); the fused step leaves the veleval lanes of rec_vi to its velocity
// pass.  pack: the
// position pairs of the default arithmetic are written from pos_s first
// (the stage API's permutes do not write them; the counting sort's does).
// sorted_keys: the cell key of every sorted particle, as the counting sort
// of the same enqueue wrote it (keys_a), for the default arithmetic's
// cell-pair pass; null where the keys are not known to match pos_s (the
// stage API's density, which the caller may run after any stage), which
// then takes the one-particle pass.  The same enqueue's counting sort also
// wrote cell_pre, which the cell-pair pass then takes its row runs from.
void density_launch(sph_ctx* c, bool fused, cudaStream_t st, bool pack = false,
                    const uint32_t* sorted_keys = nullptr) {
    sphk::launch_density(c->pos_s, fused ? nullptr : c->veleval_s, c->density, c->rec_pd, c->rec_vi,
                         c->nbr, c->mask,
                         (size_t)c->max_num, c->cell_start, c->cell_end, c->info, c->P, c->num_hint, c->pos_xy,
                         c->pos_z, pack, c->lc.density_threads, st, sorted_keys,
                         sorted_keys != nullptr ? c->cell_pre : nullptr);
}

// cell_pre: the prefix of the cell counts when the same enqueue's counting
// sort wrote it (null for the stage API, whose cell ranges come from its own
// cellindices pass).
void force_launch(sph_ctx* c, uint32_t* idx, bool fused, float dt, cudaStream_t st,
                  const uint32_t* cell_pre = nullptr) {
    sphk::launch_force(c->pos_s, c->rec_pd, c->rec_vi, c->mask, (size_t)c->max_num, c->nbr, c->cell_start, c->cell_end,
                       c->info, c->force_s, c->xsph_s, idx, c->vel_s, c->pos_u, c->vel_u, c->veleval_u,
                       fused ? c->keep_f : nullptr, fused ? c->keep_v : nullptr, c->P, dt, fused ? 1 : 0, c->exact,
                       c->num_hint, c->lc.force_threads, st, cell_pre);
}

}  // namespace

// SPH::update as staged launches up to the force pass: hash, sort,
// cellindices+permute, out-of-grid deletion, density, force.
static int enqueue_to_force(sph_ctx* c) {
    int rc = enqueue_cell_sort(c, 2);
    if (rc) return rc;
    sphk::launch_delete_staged(c->pos_s, c->vel_s, c->veleval_s, c->idx_a, c->pos_u, c->vel_u, c->veleval_u,
                               c->del_pos, c->del_vel, c->info, c->num_hint, c->stream);
    density_launch(c, false, c->stream, false, c->keys_a);
    force_launch(c, c->idx_a, false, 0.f, c->stream, c->cell_pre);
    return SPH_OK;
}

// SPH::update as staged launches: up to force, then gravity, walls, triangles.
static int enqueue_update(sph_ctx* c) {
    int rc = enqueue_to_force(c);
    if (rc) return rc;
    sphk::launch_gravity(c->pos_s, c->force_s, c->info, c->P, c->num_hint, c->stream);
    sphk::launch_collision(c->pos_s, c->vel_s, c->force_s, c->info, c->P, c->num_hint, c->stream);
    sphk::launch_triangles(c->pos_s, c->vel_s, c->force_s, c->info, c->P, c->num_hint, c->stream);
    CK_LAUNCH(c);
    return SPH_OK;
}

int enqueue_fused_step(sph_ctx* c, float dt) {
    const bool mesh = c->n_tri > 0;
    int rc = enqueue_cell_sort(c, 0);
    if (rc) return rc;
    // beside the density pass, on the side stream, once the velocities are
    // in: the veleval lanes of the neighbour records and the deletion
    // bookkeeping (they and the integrator are the step's only readers of
    // the uploaded velocities; with a mesh, also the sorted velocities the
    // triangle kernel reads)
    CK(c, cudaEventRecord(c->side_fork, c->stream));
    CK(c, cudaStreamWaitEvent(c->side_stream, c->side_fork, 0));
    density_launch(c, true, c->stream, false, c->keys_a);
    if ((rc = join_upload_on(c, c->side_stream))) return rc;
    sphk::launch_step_velocities(c->pos_s, c->idx_a, c->vel_u, c->veleval_u, c->rec_vi, c->vel_s, c->del_pos,
                                 c->del_vel, c->info, mesh ? 1 : 0, c->num_hint, c->side_stream);
    CK(c, cudaEventRecord(c->side_join, c->side_stream));
    CK(c, cudaStreamWaitEvent(c->stream, c->side_join, 0));
    if (mesh) {
        // the triangle stage sits between the walls and the integrator: the
        // force pass without them, then one kernel for gravity, walls,
        // triangles and the integrator
        force_launch(c, c->idx_a, false, 0.f, c->stream, c->cell_pre);
        sphk::launch_triangles_step(c->pos_s, c->vel_s, c->force_s, c->xsph_s, c->idx_a, c->pos_u, c->vel_u,
                                    c->veleval_u, c->info, c->P, dt, c->num_hint, c->stream);
    } else {
        force_launch(c, c->idx_a, true, dt, c->stream, c->cell_pre);
    }
    CK_LAUNCH(c);
    return SPH_OK;
}

int read_info(sph_ctx* c) {
    CK(c, cudaMemcpyAsync(c->host_info, c->info, sizeof(int) * sphk::kInfoSlots, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (c->host_info[sphk::kError] & sphk::kErrLookbackTimeout) {
        return set_err(c, SPH_ETIMEOUT, "sort look-back wait expired; the step result is invalid");
    }
    if (c->host_info[sphk::kError] & sphk::kErrBounds) {
        return set_err(c, SPH_EBOUNDS, "an index of a kernel fell outside its array (bounds-checked library); "
                       "the results are invalid");
    }
    return SPH_OK;
}

int check_ctx(sph_ctx* c, bool join) {
    if (!c) return SPH_EINVAL;
    int dev = -1;
    if (cudaGetDevice(&dev) == cudaSuccess && dev != c->device) CK(c, cudaSetDevice(c->device));
    if (join && c->up_pending) {
        CK(c, cudaStreamWaitEvent(c->stream, c->up_done, 0));
        c->up_pending = false;
    }
    return SPH_OK;
}

// Stream st waits for the latest upload (st is the context stream, or a
// stream the context stream later waits for).
int join_upload_on(sph_ctx* c, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(c, cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusActive) {
        // in the step graph for good: every replay waits for the latest upload
        CK(c, cudaStreamWaitEvent(st, c->up_done, cudaEventWaitExternal));
    } else if (c->up_pending) {
        CK(c, cudaStreamWaitEvent(st, c->up_done, 0));
        c->up_pending = false;
    }
    return SPH_OK;
}

int join_upload(sph_ctx* c) { return join_upload_on(c, c->stream); }


// --- launch shapes and the autotuner (helpers shared with the batch) -------

bool sph_launch_config_valid(const sph_launch_config& g) {
    return (g.density_threads == 128 || g.density_threads == 256 || g.density_threads == 512) &&
           (g.force_threads == 64 || g.force_threads == 128 || g.force_threads == 256) &&
           (g.scan_tile_cells == 2048 || g.scan_tile_cells == 4096 || g.scan_tile_cells == 8192) && g.reserved == 0;
}

// The tuner's candidates: every knob has three values; candidate k takes the
// k-th of each (the knobs are separate kernels, timed separately).
const sph_launch_config sph_tune_candidates[3] = {{128, 64, 2048, 0}, {256, 128, 4096, 0}, {512, 256, 8192, 0}};

namespace {
std::mutex g_tune_mutex;
std::map<SphTuneKey, sph_launch_config> g_tune_cache;  // results of the tuner in this process
}  // namespace

bool sph_tune_cache_get(const SphTuneKey& k, sph_launch_config& out) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    const auto it = g_tune_cache.find(k);
    if (it == g_tune_cache.end()) return false;
    out = it->second;
    return true;
}

void sph_tune_cache_put(const SphTuneKey& k, const sph_launch_config& v) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[k] = v;
}

sph_launch_config sph_tune_pick(const double t[3][3]) {
    sph_launch_config best = sph_tune_candidates[1];
    int bd = 1, bf = 1, bs = 1;
    for (int k = 0; k < 3; ++k) {
        if (t[k][0] < t[bd][0]) bd = k;
        if (t[k][1] < t[bf][1]) bf = k;
        if (t[k][2] < t[bs][2]) bs = k;
    }
    best.density_threads = sph_tune_candidates[bd].density_threads;
    best.force_threads = sph_tune_candidates[bf].force_threads;
    best.scan_tile_cells = sph_tune_candidates[bs].scan_tile_cells;
    return best;
}


extern "C" {

#define SPH_STR_(x) #x
#define SPH_STR(x) SPH_STR_(x)
const char* sph_build_info(void) {
    return "librtps_sph: GB300 sm_103a SPH step (hash, 8-bit LSD radix sort, cellindices+permute, density, "
           "force+collision+leapfrog); CUDART " SPH_STR(CUDART_VERSION)
#ifdef SPH_CHECKED
           "; bounds-checked (SPH_CHECKED)"
#endif
        ;
}

int sph_create(const SPHParams* sphp, const GridParams* grid, const GridParams* grid_scaled, int max_num,
               sph_ctx** out) {
    if (!sphp || !grid || !out) return set_err(nullptr, SPH_EINVAL, "null argument");
    *out = nullptr;
    if (max_num <= 0 || max_num >= (1 << 30)) return set_err(nullptr, SPH_EINVAL, "max_num out of range: %d", max_num);
    if (grid->nb_cells <= 0 || grid->nb_cells + 1 >= (1 << 24))
        return set_err(nullptr, SPH_EINVAL, "nb_cells must be in [1, 2^24-2] (float cell hashes), got %d",
                       grid->nb_cells);
    sph_ctx* c = new sph_ctx();
    c->sp = *sphp;
    c->gp = *grid;
    c->gps = grid_scaled ? *grid_scaled : sph_scaled_grid(*grid, sphp->simulation_scale);
    if (c->gps.nb_cells != c->gp.nb_cells) {
        delete c;
        return set_err(nullptr, SPH_EINVAL, "scaled grid nb_cells differs");
    }
    c->max_num = max_num;
    c->sp.max_num = max_num;
    if (build_step_params(c) != SPH_OK) {
        g_create_error = c->err;
        delete c;
        return SPH_EINVAL;
    }
    cudaError_t e = cudaGetDevice(&c->device);
    if (e != cudaSuccess) {
        delete c;
        return set_err(nullptr, SPH_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    }
    const int total_bits = bit_width((uint32_t)c->gp.nb_cells);
    c->passes = (total_bits + 7) / 8;
    if (c->passes < 1) c->passes = 1;
    c->tiles_cap = sphk::radix_tiles(max_num);
    const size_t N = (size_t)max_num, C1 = (size_t)c->gp.nb_cells + 1;
    int rc = SPH_OK;
#define ALLOC(ptr, bytes)                                                                                 \
    do {                                                                                                  \
        if (rc == SPH_OK) {                                                                               \
            cudaError_t ae = cudaMalloc((void**)&(ptr), (bytes));                                         \
            if (ae != cudaSuccess) {                                                                      \
                rc = set_err(nullptr, SPH_ENOMEM, "cudaMalloc(%zu): %s", (size_t)(bytes), cudaGetErrorString(ae)); \
                cudaGetLastError();                                                                       \
            }                                                                                             \
        }                                                                                                 \
    } while (0)
    ALLOC(c->pos_u, N * 16);
    ALLOC(c->vel_u, N * 16);
    ALLOC(c->veleval_u, N * 16);
    ALLOC(c->pos_s, N * 16);
    ALLOC(c->vel_s, N * 16);
    ALLOC(c->veleval_s, N * 16);
    ALLOC(c->force_s, N * 16);
    ALLOC(c->xsph_s, N * 16);
    ALLOC(c->del_pos, N * 16);
    ALLOC(c->del_vel, N * 16);
    ALLOC(c->density, N * 4);
    ALLOC(c->nbr, N * 4);
    ALLOC(c->rec_pd, N * 16);
    ALLOC(c->rec_vi, N * 16);
    ALLOC(c->pos_xy, (N / 2 + 1) * 16);
    ALLOC(c->pos_z, (N / 2 + 1) * 8);
    ALLOC(c->mask, N * 4 * sphk::kMaskWords);
    ALLOC(c->keys_a, N * 4);
    ALLOC(c->idx_a, N * 4);
    ALLOC(c->keys_b, N * 4);
    ALLOC(c->idx_b, N * 4);
    ALLOC(c->cell_start, C1 * 4);
    ALLOC(c->cell_end, C1 * 4);
    ALLOC(c->cell_pre, C1 * 4);
    ALLOC(c->cell_count, C1 * 4);
    ALLOC(c->cell_tile_total, (size_t)sphk::cell_scan_tiles((int)C1, sphk::kScanTileMin) * 4);
    ALLOC(c->cell_entries, N * 8);
    ALLOC(c->info, sizeof(int) * sphk::kInfoSlots);
    // point sources: kMaxGravitySources float4 positions, then masses, then alphas
    ALLOC(c->grav, sizeof(float4) * sphk::kMaxGravitySources + 2 * sizeof(float) * sphk::kMaxGravitySources);
    c->scratch_words = 4 * 256 + (size_t)c->passes * c->tiles_cap * 256;
    ALLOC(c->scratch, c->scratch_words * 4);
#undef ALLOC
    if (rc == SPH_OK && cudaMallocHost((void**)&c->host_info, sizeof(int) * sphk::kInfoSlots) != cudaSuccess)
        rc = set_err(nullptr, SPH_ENOMEM, "cudaMallocHost failed");
    if (rc == SPH_OK && (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
                         cudaStreamCreateWithFlags(&c->up_stream, cudaStreamNonBlocking) != cudaSuccess ||
                         cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking) != cudaSuccess ||
                         cudaEventCreateWithFlags(&c->side_fork, cudaEventDisableTiming) != cudaSuccess ||
                         cudaEventCreateWithFlags(&c->side_join, cudaEventDisableTiming) != cudaSuccess ||
                         cudaEventCreateWithFlags(&c->up_start, cudaEventDisableTiming) != cudaSuccess ||
                         cudaEventCreateWithFlags(&c->up_done, cudaEventDisableTiming) != cudaSuccess))
        rc = set_err(nullptr, SPH_ECUDA, "cudaStreamCreate / cudaEventCreate failed");
    if (rc != SPH_OK) {
        free_all(c);
        delete c;
        return rc;
    }
    c->stream = c->own_stream;
    c->P.chk_err = c->info + sphk::kError;
    c->hist = c->scratch;
    c->status = c->scratch + 4 * 256;
    c->keys_cur = c->keys_a;
    c->idx_cur = c->idx_a;
    // Initial contents as SPH::prepareSorted / System::prepareSorted leave them.
    cudaStream_t st = c->stream;
    cudaMemsetAsync(c->info, 0, sizeof(int) * sphk::kInfoSlots, st);
    k_set_num<<<1, 1, 0, st>>>(c->info, 0);
    const void* zero_f4[] = {c->pos_u, c->vel_u, c->veleval_u, c->pos_s, c->vel_s, c->veleval_s, c->force_s,
                             c->xsph_s, c->del_pos, c->del_vel};
    for (const void* p : zero_f4) cudaMemsetAsync((void*)p, 0, N * 16, st);
    cudaMemsetAsync(c->density, 0, N * 4, st);
    cudaMemsetAsync(c->nbr, 0, N * 4, st);
    cudaMemsetAsync(c->rec_pd, 0, N * 16, st);
    cudaMemsetAsync(c->rec_vi, 0, N * 16, st);
    cudaMemsetAsync(c->pos_xy, 0, (N / 2 + 1) * 16, st);
    cudaMemsetAsync(c->pos_z, 0, (N / 2 + 1) * 8, st);
    cudaMemsetAsync(c->mask, 0, N * 4 * sphk::kMaskWords, st);
    fill_u32(c->keys_a, N, 0x7fffffffu, st);
    fill_u32(c->idx_a, N, 0x7fffffffu, st);
    fill_u32(c->keys_b, N, 0x7fffffffu, st);
    fill_u32(c->idx_b, N, 0x7fffffffu, st);
    fill_u32(c->cell_start, C1, 666u, st);
    fill_u32(c->cell_end, C1, 666u, st);
    cudaMemsetAsync(c->cell_count, 0, C1 * 4, st);
    cudaMemsetAsync(c->cell_entries, 0, N * 8, st);
    cudaMemsetAsync(c->scratch, 0, c->scratch_words * 4, st);
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_err(nullptr, SPH_ECUDA, "context init: %s", cudaGetErrorString(e));
        free_all(c);
        delete c;
        return SPH_ECUDA;
    }
    *out = c;
    return SPH_OK;
}

int sph_destroy(sph_ctx* c) {
    if (!c) return SPH_EINVAL;
    cudaSetDevice(c->device);
    if (c->up_stream) cudaStreamSynchronize(c->up_stream);
    if (c->side_stream) cudaStreamSynchronize(c->side_stream);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (sph_hose* h : c->hoses) sph_hose_destroy(h);
    free_all(c);
    delete c;
    return SPH_OK;
}

int sph_set_params(sph_ctx* c, const SPHParams* sphp) {
    if (!c || !sphp) return SPH_EINVAL;
    SPHParams old = c->sp;
    c->sp = *sphp;
    c->sp.max_num = c->max_num;
    int rc = build_step_params(c);
    if (rc != SPH_OK) {
        c->sp = old;
        build_step_params(c);
        return rc;
    }
    return SPH_OK;
}

int sph_get_params(sph_ctx* c, SPHParams* sphp, GridParams* grid, GridParams* grid_scaled) {
    if (!c) return SPH_EINVAL;
    if (sphp) *sphp = c->sp;
    if (grid) *grid = c->gp;
    if (grid_scaled) *grid_scaled = c->gps;
    return SPH_OK;
}

int sph_set_stream(sph_ctx* c, void* stream) {
    if (!c) return SPH_EINVAL;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    return SPH_OK;
}

int sph_set_exact(sph_ctx* c, int exact) {
    if (!c) return SPH_EINVAL;
    c->exact = exact ? 1 : 0;
    c->P.exact = c->exact;
    return SPH_OK;
}

int sph_set_gravity_sources(sph_ctx* c, int count, const sph_float4* points, const float* masses,
                            const float* alphas) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (count < 0 || count > sphk::kMaxGravitySources)
        return set_err(c, SPH_EINVAL, "sph_set_gravity_sources: count %d outside [0, %d]", count,
                       sphk::kMaxGravitySources);
    if (count > 0 && (!points || !masses || !alphas))
        return set_err(c, SPH_EINVAL, "sph_set_gravity_sources: null array");
    for (int k = 0; k < count; ++k)
        if (!std::isfinite(points[k].x) || !std::isfinite(points[k].y) || !std::isfinite(points[k].z) ||
            !std::isfinite(points[k].w) || !std::isfinite(masses[k]) || !std::isfinite(alphas[k]))
            return set_err(c, SPH_EINVAL, "sph_set_gravity_sources: source %d is not finite", k);
    if (count > 0) {
        float* m = reinterpret_cast<float*>(c->grav + sphk::kMaxGravitySources);
        CK(c, cudaMemcpyAsync(c->grav, points, sizeof(float4) * count, cudaMemcpyHostToDevice, c->stream));
        CK(c, cudaMemcpyAsync(m, masses, sizeof(float) * count, cudaMemcpyHostToDevice, c->stream));
        CK(c, cudaMemcpyAsync(m + sphk::kMaxGravitySources, alphas, sizeof(float) * count, cudaMemcpyHostToDevice,
                              c->stream));
        CK(c, cudaStreamSynchronize(c->stream));  // host arrays may go away
    }
    c->n_grav = count;
    return build_step_params(c);
}

int sph_load_triangles(sph_ctx* c, const sph_float4* tris, int count) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (count < 0 || count > sphk::kMaxTriangles)
        return set_err(c, SPH_EINVAL, "sph_load_triangles: count %d outside [0, %d]", count, sphk::kMaxTriangles);
    if (count > 0 && !tris) return set_err(c, SPH_EINVAL, "sph_load_triangles: null array");
    for (int j = 0; j < count; ++j)
        for (int k = 0; k < 3; ++k) {
            const sph_float4& v = tris[4 * (size_t)j + k];
            if (!std::isfinite(v.x) || !std::isfinite(v.y) || !std::isfinite(v.z) || !std::isfinite(v.w))
                return set_err(c, SPH_EINVAL, "sph_load_triangles: vertex %d of triangle %d is not finite", k, j);
        }
    if (count > c->tri_cap) {
        CK(c, cudaStreamSynchronize(c->stream));  // queued work may still read the old mesh
        if (c->tri) CK(c, cudaFree(c->tri));
        c->tri = nullptr;
        c->tri_cap = 0;
        c->n_tri = 0;
        CK(c, cudaMalloc(&c->tri, sizeof(float4) * (10 * (size_t)count + 2 * (size_t)((count + 255) / 256))));
        c->tri_cap = count;
    }
    if (count > 0) {
        CK(c, cudaMemcpyAsync(c->tri, tris, sizeof(float4) * 4 * (size_t)count, cudaMemcpyHostToDevice, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));  // the host array may go away
    }
    c->n_tri = count;
    return build_step_params(c);
}

int sph_set_integrator(sph_ctx* c, int integrator) {
    if (!c) return SPH_EINVAL;
    if (integrator != SPH_INTEGRATOR_LEAPFROG && integrator != SPH_INTEGRATOR_EULER)
        return set_err(c, SPH_EINVAL, "sph_set_integrator: unknown integrator %d", integrator);
    c->integrator = integrator;
    return build_step_params(c);
}

int sph_upload(sph_ctx* c, const sph_float4* pos, const sph_float4* vel, const sph_float4* veleval, int n) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!pos || !vel || n < 0 || n > c->max_num) return set_err(c, SPH_EINVAL, "sph_upload: bad arguments (n=%d)", n);
    const size_t b = (size_t)n * 16;
    if (n > 0) {
        CK(c, cudaMemcpyAsync(c->pos_u, pos, b, cudaMemcpyHostToDevice, c->stream));
        // veleval and vel follow on the side stream once pos is in (the link
        // is not shared with it): the next fused step's hash, sort, permute
        // and density, which read only pos, run meanwhile
        CK(c, cudaEventRecord(c->up_start, c->stream));
        CK(c, cudaStreamWaitEvent(c->up_stream, c->up_start, 0));
        if (veleval)
            CK(c, cudaMemcpyAsync(c->veleval_u, veleval, b, cudaMemcpyHostToDevice, c->up_stream));
        else
            CK(c, cudaMemsetAsync(c->veleval_u, 0, b, c->up_stream));
        CK(c, cudaMemcpyAsync(c->vel_u, vel, b, cudaMemcpyHostToDevice, c->up_stream));
        CK(c, cudaEventRecord(c->up_done, c->up_stream));
        c->up_pending = true;
    }
    k_set_num<<<1, 1, 0, c->stream>>>(c->info, n);
    CK_LAUNCH(c);
    c->num_hint = n;
    return SPH_OK;
}

int sph_get_num(sph_ctx* c, int* num) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!num) return SPH_EINVAL;
    rc = read_info(c);
    const int out = c->host_info[sphk::kOutStart];
    const int n = c->host_info[sphk::kNum];
    *num = out >= 0 ? (out < n ? out : n) : n;
    return rc;
}

int sph_push_particles(sph_ctx* c, const sph_float4* pos, const sph_float4* vel, int n) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!pos || !vel || n < 0) return set_err(c, SPH_EINVAL, "sph_push_particles: bad arguments");
    int cur = 0;
    rc = sph_get_num(c, &cur);
    if (rc) return rc;
    if (cur + n > c->max_num)
        return set_err(c, SPH_EINVAL, "pushParticles: exceeded max nb (%d) of particles allowed", c->max_num);
    if (n == 0) return SPH_OK;
    const size_t b = (size_t)n * 16;
    CK(c, cudaMemcpyAsync(c->pos_u + cur, pos, b, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->vel_u + cur, vel, b, cudaMemcpyHostToDevice, c->stream));
    k_set_num<<<1, 1, 0, c->stream>>>(c->info, cur + n);
    CK_LAUNCH(c);
    c->num_hint = cur + n;
    CK(c, cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

int sph_set_num(sph_ctx* c, int num) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (num < 0 || num > c->max_num) return set_err(c, SPH_EINVAL, "sph_set_num: %d out of range", num);
    k_set_num<<<1, 1, 0, c->stream>>>(c->info, num);
    CK_LAUNCH(c);
    c->num_hint = num;
    return SPH_OK;
}

int sph_download_async(sph_ctx* c, int field, void* host, int n) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!host || n < 0) return set_err(c, SPH_EINVAL, "sph_download: bad arguments");
    if (field < 0 || field >= SPH_FIELD_COUNT_) return set_err(c, SPH_EINVAL, "unknown field %d", field);
    if (n > field_capacity(c, field)) return set_err(c, SPH_EINVAL, "n=%d exceeds field capacity", n);
    if (n == 0) return SPH_OK;
    CK(c, cudaMemcpyAsync(host, field_ptr(c, field), (size_t)n * field_elem_bytes(field), cudaMemcpyDeviceToHost,
                          c->stream));
    return SPH_OK;
}

int sph_download(sph_ctx* c, int field, void* host, int n) {
    int rc = sph_download_async(c, field, host, n);
    if (rc) return rc;
    return read_info(c);
}

int sph_get_device_ptr(sph_ctx* c, int field, void** dptr) {
    if (!c || !dptr) return SPH_EINVAL;
    void* p = field_ptr(c, field);
    if (!p) return set_err(c, SPH_EINVAL, "unknown field %d", field);
    *dptr = p;
    return SPH_OK;
}

int sph_get_deleted(sph_ctx* c, sph_float4* pos, sph_float4* vel, int cap, int* count) {
    int rc = check_ctx(c);
    if (rc) return rc;
    rc = read_info(c);
    if (rc) return rc;
    const int nd = c->host_info[sphk::kDeleted];
    if (count) *count = nd;
    const int k = nd < cap ? nd : cap;
    // on the context's stream only: no wait for other streams of the device
    if (k > 0 && pos) CK(c, cudaMemcpyAsync(pos, c->del_pos, (size_t)k * 16, cudaMemcpyDeviceToHost, c->stream));
    if (k > 0 && vel) CK(c, cudaMemcpyAsync(vel, c->del_vel, (size_t)k * 16, cudaMemcpyDeviceToHost, c->stream));
    if (k > 0 && (pos || vel)) CK(c, cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

// --- stages ----------------------------------------------------------------
int sph_stage_hash(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    return enqueue_hash(c);
}

int sph_stage_sort(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    return enqueue_sort(c);
}

int sph_stage_cellindices(sph_ctx* c, int* nc) {
    int rc = check_ctx(c);
    if (rc) return rc;
    sphk::launch_cells_permute(c->keys_cur, c->idx_cur, c->cell_start, c->cell_end, c->pos_u, c->vel_u,
                               c->veleval_u, c->pos_s, c->vel_s, c->veleval_s, c->info, c->gp.nb_cells, c->num_hint,
                               0, c->stream);
    CK_LAUNCH(c);
    if (nc) {
        uint32_t v = 0;
        CK(c, cudaMemcpyAsync(&v, c->cell_start + c->gp.nb_cells, 4, cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        *nc = (int)v;
    }
    return SPH_OK;
}

int sph_stage_permute(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    sphk::launch_permute_only(c->idx_cur, c->pos_u, c->vel_u, c->veleval_u, c->pos_s, c->vel_s, c->veleval_s, c->info,
                              c->num_hint, c->stream);
    CK_LAUNCH(c);
    return SPH_OK;
}

int sph_stage_density(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    density_launch(c, false, c->stream, true);
    CK_LAUNCH(c);
    return SPH_OK;
}

int sph_stage_force(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    force_launch(c, c->idx_cur, false, 0.f, c->stream);
    CK_LAUNCH(c);
    return SPH_OK;
}

int sph_stage_collision(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    sphk::launch_collision(c->pos_s, c->vel_s, c->force_s, c->info, c->P, c->num_hint, c->stream);
    CK_LAUNCH(c);
    return SPH_OK;
}

int sph_stage_gravity(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    sphk::launch_gravity(c->pos_s, c->force_s, c->info, c->P, c->num_hint, c->stream);
    CK_LAUNCH(c);
    return SPH_OK;
}

int sph_stage_collision_triangles(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    sphk::launch_triangles(c->pos_s, c->vel_s, c->force_s, c->info, c->P, c->num_hint, c->stream);
    CK_LAUNCH(c);
    return SPH_OK;
}

int sph_stage_euler(sph_ctx* c, float dt) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!std::isfinite(dt)) return set_err(c, SPH_EINVAL, "dt must be finite");
    sphk::launch_euler(c->pos_s, c->vel_s, c->force_s, c->idx_cur, c->pos_u, c->vel_u, c->info, c->P, dt,
                       c->num_hint, c->stream);
    CK_LAUNCH(c);
    return SPH_OK;
}

int sph_stage_leapfrog(sph_ctx* c, float dt) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!std::isfinite(dt)) return set_err(c, SPH_EINVAL, "dt must be finite");
    sphk::launch_leapfrog(c->pos_s, c->vel_s, c->force_s, c->xsph_s, c->idx_cur, c->pos_u, c->vel_u, c->veleval_u,
                          c->info, c->P, dt, c->num_hint, c->stream);
    CK_LAUNCH(c);
    return SPH_OK;
}

int sph_update(sph_ctx* c) {
    int rc = check_ctx(c, false);  // the upload is joined before cells+permute
    if (rc) return rc;
    if (!c->hoses.empty() && (rc = sph_spray_hoses(c, nullptr))) return rc;
    return enqueue_update(c);
}

// --- hoses (SPH.cpp:523-558) ---------------------------------------------------
namespace {
// The "spacing" setting (SPHSettings.cpp:94-97): rest_distance over
// simulation_scale, through the settings' 6-digit round trip.
float sph_spacing(const sph_ctx* c) { return sph_settings_round(c->sp.rest_distance / c->sp.simulation_scale); }
}  // namespace

int sph_add_hose(sph_ctx* c, int total_n, sph_float4 center, sph_float4 velocity, float radius, float dt,
                 int* index) {
    int rc = check_ctx(c);
    if (rc) return rc;
    const float spacing = sph_spacing(c);
    sph_hose* h = nullptr;
    rc = sph_hose_create(dt, total_n, center, velocity, radius * spacing, spacing, &h);
    if (rc) return set_err(c, rc, "sph_add_hose: bad arguments");
    c->hoses.push_back(h);
    if (index) *index = (int)c->hoses.size() - 1;
    return SPH_OK;
}

int sph_update_hose(sph_ctx* c, int index, sph_float4 center, sph_float4 velocity, float radius) {
    if (!c) return SPH_EINVAL;
    if (index < 0 || index >= (int)c->hoses.size()) return set_err(c, SPH_EINVAL, "no hose %d", index);
    const float spacing = sph_spacing(c);
    const int rc = sph_hose_update(c->hoses[index], center, velocity, radius * spacing, spacing);
    return rc ? set_err(c, rc, "sph_update_hose: bad arguments") : SPH_OK;
}

int sph_refill_hose(sph_ctx* c, int index, int n) {
    if (!c) return SPH_EINVAL;
    if (index < 0 || index >= (int)c->hoses.size()) return set_err(c, SPH_EINVAL, "no hose %d", index);
    const int rc = sph_hose_refill(c->hoses[index], n);
    return rc ? set_err(c, rc, "sph_refill_hose: bad arguments") : SPH_OK;
}

int sph_spray_hoses(sph_ctx* c, int* added) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (added) *added = 0;
    const int hint0 = c->num_hint;
    bool pushed = false;
    for (sph_hose* h : c->hoses) {
        int k = 0;
        sph_hose_spray(h, &k);
        if (k == 0) continue;
        std::vector<sph_float4> pos((size_t)k), vel((size_t)k);
        sph_float4 v;
        sph_hose_particles(h, pos.data(), k, &v);
        for (auto& e : vel) e = v;
        int cur = 0;
        if ((rc = sph_get_num(c, &cur))) return rc;
        if (cur + k > c->max_num) continue;  // dropped, as SPH::pushParticles does (SPH.cpp:562-567)
        if ((rc = sph_push_particles(c, pos.data(), vel.data(), k))) return rc;
        pushed = true;
        if (added) *added += k;
    }
    if (pushed) {
        // An upper bound of the count that stays put while the hoses empty
        // (pushes move particles from the hoses into the system), so that
        // the step graph, sized by it, is not re-captured at every spray.
        long pending = 0;
        for (sph_hose* h : c->hoses) {
            int r = 0;
            sph_hose_remaining(h, &r);
            pending += r;
        }
        const long bound = std::min<long>(c->max_num, (long)c->num_hint + pending);
        c->num_hint = (int)std::max<long>(hint0, bound);
    }
    return SPH_OK;
}

int sph_integrate(sph_ctx* c, float dt) {
    if (!c) return SPH_EINVAL;
    return c->integrator == SPH_INTEGRATOR_EULER ? sph_stage_euler(c, dt) : sph_stage_leapfrog(c, dt);
}

static int ensure_step_graph(sph_ctx* c, float dt);

int sph_step(sph_ctx* c, float dt, int nsteps) {
    int rc = check_ctx(c, false);  // the upload is joined inside the step, before cells+permute
    if (rc) return rc;
    if (nsteps < 0 || !std::isfinite(dt)) return set_err(c, SPH_EINVAL, "sph_step: bad arguments");
    if (!c->hoses.empty()) {
        // SPH::updateGPU sprays the hoses before every step (SPH.cpp:162-166)
        for (int k = 0; k < nsteps; ++k) {
            if ((rc = sph_spray_hoses(c, nullptr))) return rc;
            if (c->num_hint == 0) continue;
            if ((rc = ensure_step_graph(c, dt))) return rc;
            CK(c, cudaGraphLaunch(c->graph, c->stream));
            c->up_pending = false;  // the graph waited for it
        }
    } else {
        if (nsteps == 0 || c->num_hint == 0) return SPH_OK;
        if ((rc = ensure_step_graph(c, dt))) return rc;
        for (int k = 0; k < nsteps; ++k) CK(c, cudaGraphLaunch(c->graph, c->stream));
        c->up_pending = false;  // the graph waited for it
    }
    c->keys_cur = c->keys_a;
    c->idx_cur = c->idx_a;
    return SPH_OK;
}

// (Re-)captures the graph of one step when dt, the particle bound, the
// arithmetic mode or the parameters changed since the last capture.
static int ensure_step_graph(sph_ctx* c, float dt) {
    int rc = SPH_OK;
    const bool stale = !c->graph || c->graph_dt != dt || c->graph_num != c->num_hint || c->graph_exact != c->exact ||
                       c->graph_version != c->params_version;
    if (stale) {
        if (c->graph) {
            cudaGraphExecDestroy(c->graph);
            c->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_fused_step(c, dt);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return set_err(c, SPH_ECUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            c->graph = nullptr;
            return set_err(c, SPH_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
        }
        c->graph_dt = dt;
        c->graph_num = c->num_hint;
        c->graph_exact = c->exact;
        c->graph_version = c->params_version;
    }
    return SPH_OK;
}

int sph_step_eager(sph_ctx* c, float dt, int nsteps) {
    int rc = check_ctx(c, false);
    if (rc) return rc;
    if (nsteps < 0 || !std::isfinite(dt)) return set_err(c, SPH_EINVAL, "sph_step_eager: bad arguments");
    for (int k = 0; k < nsteps; ++k) {
        if (!c->hoses.empty() && (rc = sph_spray_hoses(c, nullptr))) return rc;
        if (c->num_hint == 0) continue;
        if ((rc = enqueue_fused_step(c, dt))) return rc;
    }
    return SPH_OK;
}

int sph_step_profile(sph_ctx* c, float dt, int nsteps, float* kernel_ms, int cap, int* nkernels) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (nsteps < 0 || !std::isfinite(dt) || !kernel_ms || cap <= 0)
        return set_err(c, SPH_EINVAL, "sph_step_profile: bad arguments");
    if (c->n_tri > 0)
        return set_err(c, SPH_ESTATE, "sph_step_profile times the fused step without a triangle mesh");
    if (!c->hoses.empty()) return set_err(c, SPH_ESTATE, "sph_step_profile times the fused step without hoses");
    // Launches of one fused step: count, totals, scan, place, permute,
    // density, velocity pass, force+collision+leapfrog.
    const int nk = 8;
    if (nkernels) *nkernels = nk;
    for (int k = 0; k < cap; ++k) kernel_ms[k] = 0.f;
    cudaEvent_t ev[nk + 1];
    for (int k = 0; k <= nk; ++k) CK(c, cudaEventCreate(&ev[k]));
    cudaStream_t st = c->stream;
    for (int step = 0; step < nsteps && c->num_hint > 0; ++step) {
        int e = 0;
        CK(c, cudaEventRecord(ev[e++], st));
        sphk::launch_cell_count(c->pos_u, c->keys_b, c->idx_b, c->cell_count, c->info, c->P, c->num_hint, st);
        CK(c, cudaEventRecord(ev[e++], st));
        sphk::launch_cell_totals(c->cell_count, c->cell_tile_total, c->info, (uint32_t)c->gp.nb_cells + 1u,
                                 c->lc.scan_tile_cells, st);
        CK(c, cudaEventRecord(ev[e++], st));
        sphk::launch_cell_scan(c->cell_count, c->cell_start, c->cell_end, c->cell_tile_total, c->info,
                               (uint32_t)c->gp.nb_cells + 1u, c->lc.scan_tile_cells, st, c->cell_pre);
        CK(c, cudaEventRecord(ev[e++], st));
        sphk::launch_cell_place(c->keys_b, c->idx_b, c->cell_start, c->cell_entries, c->info, c->num_hint, st);
        CK(c, cudaEventRecord(ev[e++], st));
        sphk::launch_cell_permute(c->cell_entries, c->cell_start, c->cell_end, c->keys_a, c->idx_a, c->pos_u,
                                  c->vel_u, c->veleval_u, c->pos_s, c->vel_s, c->veleval_s, c->info, c->num_hint, 0,
                                  c->pos_xy, c->pos_z, st);
        CK(c, cudaEventRecord(ev[e++], st));
        density_launch(c, true, st, false, c->keys_a);
        CK(c, cudaEventRecord(ev[e++], st));
        sphk::launch_step_velocities(c->pos_s, c->idx_a, c->vel_u, c->veleval_u, c->rec_vi, c->vel_s, c->del_pos,
                                     c->del_vel, c->info, 0, c->num_hint, st);
        CK(c, cudaEventRecord(ev[e++], st));
        force_launch(c, c->idx_a, true, dt, st, c->cell_pre);
        CK(c, cudaEventRecord(ev[e++], st));
        CK_LAUNCH(c);
        CK(c, cudaEventSynchronize(ev[nk]));
        for (int k = 0; k < nk && k < cap; ++k) {
            float ms = 0.f;
            CK(c, cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
            kernel_ms[k] += ms;
        }
    }
    for (int k = 0; k <= nk; ++k) cudaEventDestroy(ev[k]);
    c->keys_cur = c->keys_a;
    c->idx_cur = c->idx_a;
    return read_info(c);
}

const char* sph_profile_kernel_name(sph_ctx* c, int k) {
    static const char* names[] = {"k_cell_count", "k_cell_totals", "k_cell_scan", "k_cell_place",
                                  "k_cell_permute", "k_density", "k_step_velocities",
                                  "k_force(fused collision+leapfrog)"};
    if (!c || k < 0 || k >= 8) return "";
    return names[k];
}

// --- launch shapes and the autotuner ----------------------------------------

int sph_get_launch_config(sph_ctx* c, sph_launch_config* cfg) {
    if (!c || !cfg) return SPH_EINVAL;
    *cfg = c->lc;
    return SPH_OK;
}

int sph_set_launch_config(sph_ctx* c, const sph_launch_config* cfg) {
    if (!c || !cfg) return SPH_EINVAL;
    if (!sph_launch_config_valid(*cfg))
        return set_err(c, SPH_EINVAL, "sph_set_launch_config: shape (%d, %d, %d) not among the candidates",
                       cfg->density_threads, cfg->force_threads, cfg->scan_tile_cells);
    c->lc = *cfg;
    c->params_version++;  // the step graph is captured anew
    return SPH_OK;
}

int sph_autotune(sph_ctx* c, float dt, int steps, int flags, sph_launch_config* chosen) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (steps < 1 || !std::isfinite(dt)) return set_err(c, SPH_EINVAL, "sph_autotune: bad arguments");
    const SphTuneKey key{0, c->max_num, c->gp.nb_cells, c->exact};
    sph_launch_config best;
    if (!(flags & SPH_TUNE_RETIME) && sph_tune_cache_get(key, best)) {
        c->lc = best;
        c->params_version++;
        if (chosen) *chosen = best;
        return SPH_OK;
    }
    if (c->n_tri > 0 || !c->hoses.empty())
        return set_err(c, SPH_ESTATE, "sph_autotune times the fused step without a triangle mesh or hoses");
    if ((rc = read_info(c))) return rc;
    const int num = c->host_info[sphk::kNum];
    if (num <= 0 || c->num_hint <= 0) return set_err(c, SPH_ESTATE, "sph_autotune: no particles");
    // Save the state the steps change: pos/vel/veleval, the device counters
    // and the last deletion's particles.
    int saved_info[sphk::kInfoSlots];
    std::memcpy(saved_info, c->host_info, sizeof(saved_info));
    const int ndel = std::min(std::max(saved_info[sphk::kDeleted], 0), c->max_num);
    const size_t bytes = (size_t)num * 16, dbytes = (size_t)ndel * 16;
    float4* save = nullptr;
    if (cudaMalloc((void**)&save, 3 * bytes + 2 * dbytes + 16) != cudaSuccess) {
        cudaGetLastError();
        return set_err(c, SPH_ENOMEM, "sph_autotune: %zu bytes of scratch", 3 * bytes + 2 * dbytes);
    }
    float4* const fields[5] = {c->pos_u, c->vel_u, c->veleval_u, c->del_pos, c->del_vel};
    const size_t sizes[5] = {bytes, bytes, bytes, dbytes, dbytes};
    auto copy_all = [&](bool to_save) -> cudaError_t {
        size_t off = 0;
        for (int f = 0; f < 5; ++f) {
            if (sizes[f] == 0) continue;
            char* sp = reinterpret_cast<char*>(save) + off;
            cudaError_t e = to_save ? cudaMemcpyAsync(sp, fields[f], sizes[f], cudaMemcpyDeviceToDevice, c->stream)
                                    : cudaMemcpyAsync(fields[f], sp, sizes[f], cudaMemcpyDeviceToDevice, c->stream);
            if (e != cudaSuccess) return e;
            off += sizes[f];
        }
        if (!to_save) {
            std::memcpy(c->host_info, saved_info, sizeof(saved_info));
            return cudaMemcpyAsync(c->info, c->host_info, sizeof(saved_info), cudaMemcpyHostToDevice, c->stream);
        }
        return cudaSuccess;
    };
    const sph_launch_config keep = c->lc;
    double t[3][3] = {{0}};
    cudaError_t e = copy_all(true);
    for (int k = 0; k < 3 && e == cudaSuccess && rc == SPH_OK; ++k) {
        c->lc = sph_tune_candidates[k];
        float ms[8];
        int nk = 0;
        // one untimed step per candidate (first launches), then the timed ones
        if ((e = copy_all(false)) != cudaSuccess) break;
        if ((rc = sph_step_profile(c, dt, 1, ms, 8, &nk))) break;
        if ((e = copy_all(false)) != cudaSuccess) break;
        if ((rc = sph_step_profile(c, dt, steps, ms, 8, &nk))) break;
        t[k][0] = ms[5];
        t[k][1] = ms[7];
        t[k][2] = (double)ms[1] + ms[2];
    }
    if (e == cudaSuccess) e = copy_all(false);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(save);
    if (rc || e != cudaSuccess) {
        c->lc = keep;
        c->params_version++;
        if (rc) return rc;
        return set_err(c, SPH_ECUDA, "sph_autotune: %s", cudaGetErrorString(e));
    }
    best = sph_tune_pick(t);
    c->lc = best;
    c->params_version++;
    sph_tune_cache_put(key, best);
    if (chosen) *chosen = best;
    return SPH_OK;
}

int sph_sync(sph_ctx* c) {
    int rc = check_ctx(c);
    if (rc) return rc;
    return read_info(c);
}

int sph_last_error(sph_ctx* c, char* buf, int len) {
    if (!buf || len <= 0) return SPH_EINVAL;
    const std::string& s = c ? c->err : g_create_error;
    std::snprintf(buf, (size_t)len, "%s", s.c_str());
    return SPH_OK;
}

}  // extern "C"
