// sph_batch.cu — many independent SPH systems ("scenes") stepped together.
//
// No counterpart in the reference, which steps one system per SPH object; a
// batch gives each scene its own SPHParams and grid and advances all of them
// with one launch sequence per step (captured in one CUDA graph):
//
//   hash     every particle slot of every scene; key = scene << cell_bits |
//            cell (the scene's own grid and out-of-grid cell C_s); the
//            scene's cells are one segment of a cell array shared by all
//            scenes (global cell = cbase[scene] + cell)
//   sort     the counting sort of the single system (sph_cellsort.cu) over
//            the global cells: an atomic count per cell gives each particle a
//            slot, the scan gives the cell ranges (per-scene segments), each
//            particle goes to its cell's start + slot, and the permute ranks
//            it by slot index among its cell's entries.  Scenes come out in
//            order, each in its own cell order with equal keys by slot, the
//            order a stable sort of the keys gives; unused slots take no
//            part
//   density, force+collision+leapfrog: the neighbour passes with the scene of
//            each particle looked up from its key (ManyScenes)
//
// Per particle the arithmetic is the single-system one, so every scene of a
// batch steps exactly as it would alone.  Particles that leave their scene's
// grid are deleted as a lone system deletes them (SPH.cpp:220-250): the
// scene keeps its first sorted particles, re-indexed in sorted order, its
// count drops, and the removed particles are kept after them in the scene's
// slots (sph_batch_get_deleted).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sph_batch.cuh"
#include "sph_queue.cuh"

using sphk::StepParams;

namespace {

// Count: key and cell slot of every used particle slot; unused slots get
// invalid_key.
__global__ void __launch_bounds__(256) k_bcount(const float4* __restrict__ pos_u, uint32_t* __restrict__ key_of,
                                                uint32_t* __restrict__ slot_of, uint32_t* __restrict__ count,
                                                const uint16_t* __restrict__ scene_of,
                                                const uint32_t* __restrict__ slot_off,
                                                const uint32_t* __restrict__ cbase, const int* __restrict__ num,
                                                const StepParams* __restrict__ table, int nslots, int cell_bits,
                                                uint32_t invalid_key) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nslots) return;
    const uint32_t s = scene_of[t];
    uint32_t key = invalid_key;
    if ((int)((uint32_t)t - slot_off[s]) < num[s]) {
        const StepParams& P = table[s];
        const float4 q = __ldg(pos_u + t);
        const int3 c = sphk::grid_cell(q.x, q.y, q.z, P.g_min, P.g_delta);
        int h = sphk::grid_hash_f(c.x, c.y, c.z, P.g_res);
        h = h > P.nb_cells ? P.nb_cells : h;
        h = h < 0 ? P.nb_cells : h;
        key = (s << cell_bits) | (uint32_t)h;
        slot_of[t] = atomicAdd(count + cbase[s] + (uint32_t)h, 1u);
    }
    key_of[t] = key;
}

// Place: (slot index, key) at the start of the particle's cell + its slot.
__global__ void __launch_bounds__(256) k_bplace(const uint32_t* __restrict__ key_of,
                                                const uint32_t* __restrict__ slot_of,
                                                const uint32_t* __restrict__ cell_start,
                                                const uint32_t* __restrict__ cbase, uint2* __restrict__ entries,
                                                int nslots, int cell_bits, uint32_t invalid_key) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nslots) return;
    const uint32_t key = __ldg(key_of + t);
    if (key == invalid_key) return;
    const uint32_t g = __ldg(cbase + (key >> cell_bits)) + (key & ((1u << cell_bits) - 1u));
    entries[__ldg(cell_start + g) + __ldg(slot_of + t)] = make_uint2((uint32_t)t, key);
}

// Scenes' first sorted indices: the exclusive scan of the particle counts
// (scene after scene in sorted order; seg[nscenes] = the batch's particle
// total, also the step's info[kNum]).
__global__ void __launch_bounds__(1024) k_bscene_scan(const int* __restrict__ num, uint32_t* __restrict__ seg,
                                                      int* __restrict__ info, int nscenes) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    if (t == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < nscenes; base += 1024) {
        const int k = base + t;
        const uint32_t v = k < nscenes ? (uint32_t)num[k] : 0u;
        uint32_t x = v;
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) s_warp[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = s_warp[lane];
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= d) w += y;
            }
            s_warp[lane] = w;
        }
        __syncthreads();
        const uint32_t before = s_carry + (wid > 0 ? s_warp[wid - 1] : 0u) + x - v;
        if (k < nscenes) seg[k] = before;
        __syncthreads();
        if (t == 1023) s_carry = before + v;
        __syncthreads();
    }
    if (t == 0) {
        info[sphk::kNum] = (int)s_carry;
        seg[nscenes] = s_carry;
    }
}

// Permute: rank within the cell, sorted keys (the scene resolver reads them),
// indices, the gather of pos / veleval (and vel, for a scene that deletes
// particles this step: its kept particles are re-indexed by the force pass,
// which then reads no velocity by slot); particles in their scene's
// out-of-grid cell are counted as frozen.
__global__ void __launch_bounds__(256) k_bpermute(const uint2* __restrict__ entries,
                                                  const uint32_t* __restrict__ cell_start,
                                                  const uint32_t* __restrict__ cell_end,
                                                  const uint32_t* __restrict__ cbase,
                                                  const StepParams* __restrict__ table, uint32_t* __restrict__ keys,
                                                  uint32_t* __restrict__ idx, const float4* __restrict__ pos_u,
                                                  const float4* __restrict__ veleval_u, float4* __restrict__ pos_s,
                                                  float4* __restrict__ veleval_s, int* __restrict__ info,
                                                  int cell_bits, float* __restrict__ pxy, float* __restrict__ pz,
                                                  const float4* __restrict__ vel_u, float4* __restrict__ vel_s) {
    const int nvalid = info[sphk::kNum];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nvalid) return;
    const uint2 e = __ldg(entries + i);
    const uint32_t id = e.x, key = e.y;
    if (!sphk::in_bounds(id, table[0].chk_cap, table[0].chk_err)) return;
    const float4 pq = __ldg(pos_u + id);
    const float4 vq = __ldg(veleval_u + id);
    const uint32_t s = key >> cell_bits, cell = key & ((1u << cell_bits) - 1u);
    const uint32_t g = __ldg(cbase + s) + cell;
    const uint32_t cs = __ldg(cell_start + g), ce = __ldg(cell_end + g);
    if (cs >= ce || ce > (uint32_t)nvalid) {  // never write outside the cell
        if (sphk::kChecked) atomicOr(table[0].chk_err, sphk::kErrBounds);
        return;
    }
    const uint32_t* ids = reinterpret_cast<const uint32_t*>(entries);
    uint32_t rank = 0;
    for (uint32_t t = cs; t < ce; ++t) rank += __ldg(ids + 2 * t) < id ? 1u : 0u;
    const uint32_t p = cs + rank;
    keys[i] = key;
    idx[p] = id;
    pos_s[p] = pq;
    {
        // the pair layout of the default arithmetic's density pass
        const uint32_t k = p >> 1, l = p & 1u;
        pxy[4 * k + l] = pq.x;
        pxy[4 * k + 2 + l] = pq.y;
        pz[2 * k + l] = pq.z;
        if (i == nvalid - 1 && (nvalid & 1)) {  // the last pair's unused lane
            pxy[4 * (nvalid >> 1) + 1] = sphk::kFarAway;
            pxy[4 * (nvalid >> 1) + 3] = sphk::kFarAway;
            pz[2 * (nvalid >> 1) + 1] = sphk::kFarAway;
        }
    }
    veleval_s[p] = vq;
    if (__ldg(cell_start + __ldg(cbase + s) + (uint32_t)table[s].nb_cells) != sphk::kEmpty) vel_s[p] = __ldg(vel_u + id);
    if (cell == (uint32_t)table[s].nb_cells) {
        atomicAdd(info + kBatchFrozen, 1);
        atomicAdd(info + kBatchFrozenTotal, 1);
    }
}

__global__ void k_bset(int* p, int v) { *p = v; }
__global__ void k_bzero_int(int* p) { *p = 0; }

int bit_width_u(uint32_t v) {
    int b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

}  // namespace

// the message of the last failed sph_batch_create on this host thread
static thread_local std::string g_batch_create_error;

int berr(sph_batch* b, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    (b ? b->err : g_batch_create_error) = buf;
    return code;
}

static void batch_free(sph_batch* b) {
    sph_batch_adjoint_release(b);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    void* ptrs[] = {b->pos_u, b->vel_u, b->veleval_u, b->pos_s, b->veleval_s, b->rec_pd, b->rec_vi, b->density,
                    b->mask, b->keys_a, b->idx_a, b->keys_b, b->idx_b, b->cell_start, b->cell_end, b->scene_of,
                    b->d_slot_off, b->d_cbase, b->d_num, b->d_table, b->info_nb, b->cell_count, b->cell_tile_total,
                    b->cell_entries, b->pos_xy, b->pos_z, b->vel_s, b->d_seg, b->d_del, b->nbr, b->q_state,
                    b->q_tiles, b->cell_pre};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b->host_info) cudaFreeHost(b->host_info);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
}

sphk::ManyScenes batch_scenes(const sph_batch* b) {
    return sphk::ManyScenes{b->d_table, b->d_cbase, b->keys_a, b->cell_bits, b->d_seg, b->d_slot_off,
                            b->cell_start, b->d_num, b->d_del, b->vel_s};
}

int batch_refresh_num(sph_batch* b) {
    std::vector<int> n(b->nscenes);
    BCK(b, cudaMemcpyAsync(n.data(), b->d_num, sizeof(int) * b->nscenes, cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    int total = 0;
    for (int s = 0; s < b->nscenes; ++s) {
        b->num[s] = n[s];
        total += n[s];
    }
    b->nvalid = total;
    return SPH_OK;
}

int batch_enqueue_step(sph_batch* b, float dt, cudaEvent_t* ev) {
    cudaStream_t st = b->stream;
    const int blocks = (b->nslots + 255) / 256;
    const uint32_t cells = (uint32_t)b->ncells_total;
    k_bzero_int<<<1, 1, 0, st>>>(b->info_nb + kBatchFrozen);
    k_bcount<<<blocks < 1 ? 1 : blocks, 256, 0, st>>>(b->pos_u, b->keys_b, b->idx_b, b->cell_count, b->scene_of,
                                                       b->d_slot_off, b->d_cbase, b->d_num, b->d_table, b->nslots,
                                                       b->cell_bits, b->invalid_key);
    k_bscene_scan<<<1, 1024, 0, st>>>(b->d_num, b->d_seg, b->info_nb, b->nscenes);
    // ev (nullable, sph_batch_autotune): events around the cell totals+scan,
    // the density pass and the force pass
    if (ev) BCK(b, cudaEventRecord(ev[0], st));
    sphk::launch_cell_totals(b->cell_count, b->cell_tile_total, nullptr, cells, b->lc.scan_tile_cells, st);
    sphk::launch_cell_scan(b->cell_count, b->cell_start, b->cell_end, b->cell_tile_total, nullptr, cells,
                           b->lc.scan_tile_cells, st, b->cell_pre);
    if (ev) BCK(b, cudaEventRecord(ev[1], st));
    k_bplace<<<blocks < 1 ? 1 : blocks, 256, 0, st>>>(b->keys_b, b->idx_b, b->cell_start, b->d_cbase, b->cell_entries,
                                                       b->nslots, b->cell_bits, b->invalid_key);
    const int cb = (b->nvalid + 255) / 256;
    k_bpermute<<<cb < 1 ? 1 : cb, 256, 0, st>>>(b->cell_entries, b->cell_start, b->cell_end, b->d_cbase, b->d_table,
                                                b->keys_a, b->idx_a, b->pos_u, b->veleval_u, b->pos_s, b->veleval_s,
                                                b->info_nb, b->cell_bits, reinterpret_cast<float*>(b->pos_xy),
                                                reinterpret_cast<float*>(b->pos_z), b->vel_u, b->vel_s);
    const sphk::ManyScenes scenes = batch_scenes(b);
    if (ev) BCK(b, cudaEventRecord(ev[2], st));
    if (b->sched == SPH_SCHED_QUEUE) {
        // persistent blocks over (scene, tile) items (sph_queue.cuh)
        BCK(b, cudaMemsetAsync(b->q_state, 0, 8 * sizeof(unsigned), st));
        sphk::BatchQueue Q{b->q_state, b->q_tiles, b->d_seg, b->d_slot_off, b->cell_start, b->d_cbase,
                           b->d_table, b->d_num, b->d_del, b->vel_s, b->info_nb + sphk::kError, b->nscenes,
                           b->q_spin, b->q_hold};
        sphk::launch_density_queue(b->pos_s, b->veleval_s, b->density, b->rec_pd, b->rec_vi, b->nbr, b->mask,
                                   (size_t)b->nslots, b->cell_start, b->cell_end, b->pos_xy, b->pos_z, Q,
                                   b->unit != 0, b->exact, b->lc.density_threads, st);
        if (ev) BCK(b, cudaEventRecord(ev[3], st));
        Q.state = b->q_state + 4;
        Q.tile_off = b->q_tiles + (b->nscenes + 1);
        sphk::launch_force_queue(b->pos_s, b->rec_pd, b->rec_vi, b->mask, (size_t)b->nslots, b->nbr, b->cell_start,
                                 b->cell_end, b->idx_a, b->pos_u, b->vel_u, b->veleval_u, b->keep_f, b->keep_v, Q,
                                 b->unit != 0, dt, b->exact, b->lc.force_threads, st);
        if (ev) BCK(b, cudaEventRecord(ev[4], st));
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return berr(b, SPH_ECUDA, "kernel launch: %s", cudaGetErrorString(e));
        return SPH_OK;
    }
    sphk::launch_density_batch(b->pos_s, b->veleval_s, b->density, b->rec_pd, b->rec_vi, b->nbr, b->mask,
                               (size_t)b->nslots, b->cell_start, b->cell_end, b->info_nb, scenes, b->unit != 0,
                               b->exact, b->nvalid, b->pos_xy, b->pos_z, false, b->lc.density_threads, st,
                               b->cell_pre);
    if (ev) BCK(b, cudaEventRecord(ev[3], st));
    sphk::launch_force_batch(b->pos_s, b->rec_pd, b->rec_vi, b->mask, (size_t)b->nslots, b->nbr, b->cell_start, b->cell_end,
                             b->info_nb, b->idx_a, b->pos_u, b->vel_u, b->veleval_u, b->keep_f, b->keep_v, scenes,
                             b->unit != 0, dt, b->exact, b->nvalid, b->lc.force_threads, st, b->cell_pre);
    if (ev) BCK(b, cudaEventRecord(ev[4], st));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return berr(b, SPH_ECUDA, "kernel launch: %s", cudaGetErrorString(e));
    return SPH_OK;
}

extern "C" {

int sph_batch_create(int nscenes, const SPHParams* sphp, const GridParams* grids, const GridParams* grids_scaled,
                     const int* max_num, sph_batch** out) {
    if (!out || !sphp || !grids || !max_num || nscenes <= 0 || nscenes > 65536)
        return berr(nullptr, SPH_EINVAL, "sph_batch_create: bad arguments");
    *out = nullptr;
    sph_batch* b = new sph_batch();
    b->nscenes = nscenes;
    uint32_t maxc = 0;
    size_t slots = 0, cells = 0;
    for (int s = 0; s < nscenes; ++s) {
        if (max_num[s] <= 0 || grids[s].nb_cells <= 0 || grids[s].nb_cells + 1 >= (1 << 24)) {
            delete b;
            return berr(nullptr, SPH_EINVAL, "scene %d: bad max_num or nb_cells", s);
        }
        b->sp.push_back(sphp[s]);
        b->gp.push_back(grids[s]);
        b->gps.push_back(grids_scaled ? grids_scaled[s] : sph_scaled_grid(grids[s], sphp[s].simulation_scale));
        StepParams P;
        std::string e;
        if (sph_make_step_params(b->sp[s], b->gp[s], b->gps[s], P, e) != SPH_OK) {
            delete b;
            return berr(nullptr, SPH_EINVAL, "scene %d: %s", s, e.c_str());
        }
        if (!P.unit_scale) b->unit = 0;
        b->P.push_back(P);
        b->max_num.push_back(max_num[s]);
        b->num.push_back(0);
        b->slot_off.push_back((uint32_t)slots);
        b->cbase.push_back((uint32_t)cells);
        slots += (size_t)max_num[s];
        cells += (size_t)grids[s].nb_cells + 1;
        if ((uint32_t)grids[s].nb_cells > maxc) maxc = (uint32_t)grids[s].nb_cells;
    }
    if (slots >= (1u << 30)) {
        delete b;
        return berr(nullptr, SPH_EINVAL, "too many particle slots");
    }
    b->nslots = (int)slots;
    b->ncells_total = cells;
    b->cell_bits = bit_width_u(maxc + 1u);
    b->scene_bits = bit_width_u((uint32_t)(nscenes - 1));
    if (b->cell_bits + b->scene_bits > 32) {
        delete b;
        return berr(nullptr, SPH_EINVAL, "scene and cell bits exceed a 32-bit key");
    }
    b->invalid_key = (uint32_t)(((uint64_t)nscenes << b->cell_bits) - 1u);
    cudaGetDevice(&b->device);
    const size_t N = slots;
    int rc = SPH_OK;
#define BALLOC(ptr, bytes)                                                                                   \
    do {                                                                                                     \
        if (rc == SPH_OK && cudaMalloc((void**)&(ptr), (bytes)) != cudaSuccess) {                            \
            cudaGetLastError();                                                                              \
            rc = berr(nullptr, SPH_ENOMEM, "cudaMalloc(%zu) failed", (size_t)(bytes));                       \
        }                                                                                                    \
    } while (0)
    BALLOC(b->pos_u, N * 16);
    BALLOC(b->vel_u, N * 16);
    BALLOC(b->veleval_u, N * 16);
    BALLOC(b->pos_s, N * 16);
    BALLOC(b->veleval_s, N * 16);
    BALLOC(b->rec_pd, N * 16);
    BALLOC(b->rec_vi, N * 16);
    BALLOC(b->pos_xy, (N / 2 + 1) * 16);
    BALLOC(b->vel_s, N * 16);
    BALLOC(b->q_state, 8 * sizeof(unsigned));
    BALLOC(b->q_tiles, 2 * (nscenes + 1) * 4);
    BALLOC(b->d_seg, (nscenes + 1) * 4);
    BALLOC(b->d_del, nscenes * 4);
    BALLOC(b->pos_z, (N / 2 + 1) * 8);
    BALLOC(b->density, N * 4);
    BALLOC(b->nbr, N * 4);
    BALLOC(b->mask, N * 4 * sphk::kMaskWords);
    BALLOC(b->keys_a, N * 4);
    BALLOC(b->idx_a, N * 4);
    BALLOC(b->keys_b, N * 4);
    BALLOC(b->idx_b, N * 4);
    BALLOC(b->cell_start, cells * 4);
    BALLOC(b->cell_end, cells * 4);
    BALLOC(b->cell_pre, cells * 4);
    BALLOC(b->scene_of, N * 2);
    BALLOC(b->d_slot_off, nscenes * 4);
    BALLOC(b->d_cbase, nscenes * 4);
    BALLOC(b->d_num, nscenes * 4);
    BALLOC(b->d_table, nscenes * sizeof(StepParams));
    BALLOC(b->info_nb, sizeof(int) * sphk::kInfoSlots);
    BALLOC(b->cell_count, cells * 4);
    BALLOC(b->cell_tile_total, (size_t)sphk::cell_scan_tiles((int)cells, sphk::kScanTileMin) * 4);
    BALLOC(b->cell_entries, N * 8);
#undef BALLOC
    if (rc == SPH_OK && cudaMallocHost((void**)&b->host_info, sizeof(int) * sphk::kInfoSlots) != cudaSuccess)
        rc = berr(nullptr, SPH_ENOMEM, "cudaMallocHost failed");
    if (rc == SPH_OK && cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = berr(nullptr, SPH_ECUDA, "cudaStreamCreate failed");
    if (rc != SPH_OK) {
        batch_free(b);
        delete b;
        return rc;
    }
    b->stream = b->own_stream;
    std::vector<uint16_t> sof(N);
    for (int s = 0; s < nscenes; ++s)
        for (int k = 0; k < max_num[s]; ++k) sof[b->slot_off[s] + k] = (uint16_t)s;
    cudaStream_t st = b->stream;
    cudaError_t e = cudaMemcpy(b->scene_of, sof.data(), N * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_slot_off, b->slot_off.data(), nscenes * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_cbase, b->cbase.data(), nscenes * 4, cudaMemcpyHostToDevice);
    for (StepParams& P : b->P) {
        P.chk_cap = (uint32_t)N;
        P.chk_err = b->info_nb + sphk::kError;
    }
    if (e == cudaSuccess) e = cudaMemcpy(b->d_table, b->P.data(), nscenes * sizeof(StepParams), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->d_num, 0, nscenes * 4);
    if (e == cudaSuccess) e = cudaMemset(b->d_del, 0, nscenes * 4);
    if (e == cudaSuccess) e = cudaMemset(b->d_seg, 0, (nscenes + 1) * 4);
    if (e == cudaSuccess) e = cudaMemset(b->info_nb, 0, sizeof(int) * sphk::kInfoSlots);
    if (e == cudaSuccess) e = cudaMemset(b->cell_count, 0, cells * 4);
    if (e == cudaSuccess) e = cudaMemset(b->cell_entries, 0, N * 8);
    const void* zero[] = {b->pos_u, b->vel_u, b->veleval_u, b->pos_s, b->veleval_s, b->rec_pd, b->rec_vi, b->vel_s};
    for (const void* p : zero)
        if (e == cudaSuccess) e = cudaMemset((void*)p, 0, N * 16);
    if (e == cudaSuccess) e = cudaMemset(b->cell_start, 0xff, cells * 4);
    if (e == cudaSuccess) e = cudaMemset(b->cell_end, 0, cells * 4);
    if (e == cudaSuccess) {
        k_bset<<<1, 1, 0, st>>>(b->info_nb + sphk::kOutStart, -1);
        e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) {
        berr(nullptr, SPH_ECUDA, "batch init: %s", cudaGetErrorString(e));
        batch_free(b);
        delete b;
        return SPH_ECUDA;
    }
    *out = b;
    return SPH_OK;
}

int sph_batch_destroy(sph_batch* b) {
    if (!b) return SPH_EINVAL;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_free(b);
    delete b;
    return SPH_OK;
}

int sph_batch_set_stream(sph_batch* b, void* stream) {
    if (!b) return SPH_EINVAL;
    b->stream = stream ? (cudaStream_t)stream : b->own_stream;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return SPH_OK;
}

int sph_batch_set_params(sph_batch* b, int scene, const SPHParams* sphp) {
    if (!b || !sphp || scene < 0 || scene >= b->nscenes) return berr(b, SPH_EINVAL, "sph_batch_set_params: bad arguments");
    if (sphp->simulation_scale != b->sp[scene].simulation_scale)
        return berr(b, SPH_EINVAL, "sph_batch_set_params: simulation_scale cannot change (it sets the grid)");
    cudaSetDevice(b->device);
    SPHParams sp = *sphp;
    sp.max_num = b->max_num[scene];
    sp.num = b->num[scene];
    StepParams P;
    std::string e;
    if (sph_make_step_params(sp, b->gp[scene], b->gps[scene], P, e) != SPH_OK)
        return berr(b, SPH_EINVAL, "scene %d: %s", scene, e.c_str());
    P.chk_cap = b->P[scene].chk_cap;
    P.chk_err = b->P[scene].chk_err;
    b->sp[scene] = sp;
    b->P[scene] = P;
    BCK(b, cudaMemcpyAsync(b->d_table + scene, &b->P[scene], sizeof(StepParams), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    b->params_version++;
    return SPH_OK;
}

int sph_batch_get_params(sph_batch* b, int scene, SPHParams* sphp) {
    if (!b || !sphp || scene < 0 || scene >= b->nscenes) return berr(b, SPH_EINVAL, "sph_batch_get_params: bad arguments");
    *sphp = b->sp[scene];
    return SPH_OK;
}

int sph_batch_get_device_ptr(sph_batch* b, int field, void** dptr) {
    if (!b || !dptr) return SPH_EINVAL;
    switch (field) {
        case SPH_FIELD_POS_U: *dptr = b->pos_u; return SPH_OK;
        case SPH_FIELD_VEL_U: *dptr = b->vel_u; return SPH_OK;
        case SPH_FIELD_VELEVAL_U: *dptr = b->veleval_u; return SPH_OK;
        default: return berr(b, SPH_EINVAL, "sph_batch_get_device_ptr: only pos_u, vel_u, veleval_u");
    }
}

int sph_batch_slot_offset(sph_batch* b, int scene, int* offset) {
    if (!b || !offset || scene < 0 || scene >= b->nscenes) return SPH_EINVAL;
    *offset = (int)b->slot_off[scene];
    return SPH_OK;
}

int sph_batch_set_exact(sph_batch* b, int exact) {
    if (!b) return SPH_EINVAL;
    b->exact = exact ? 1 : 0;
    return SPH_OK;
}

int sph_batch_upload(sph_batch* b, int scene, const sph_float4* pos, const sph_float4* vel,
                     const sph_float4* veleval, int n) {
    if (!b || scene < 0 || scene >= b->nscenes || !pos || !vel || n < 0 || n > b->max_num[scene])
        return berr(b, SPH_EINVAL, "sph_batch_upload: bad arguments");
    cudaStream_t st = b->stream;
    int rc = batch_refresh_num(b);  // earlier steps may have deleted particles
    if (rc) return rc;
    const size_t off = b->slot_off[scene], bytes = (size_t)n * 16;
    if (n > 0) {
        BCK(b, cudaMemcpyAsync(b->pos_u + off, pos, bytes, cudaMemcpyHostToDevice, st));
        BCK(b, cudaMemcpyAsync(b->vel_u + off, vel, bytes, cudaMemcpyHostToDevice, st));
        if (veleval)
            BCK(b, cudaMemcpyAsync(b->veleval_u + off, veleval, bytes, cudaMemcpyHostToDevice, st));
        else
            BCK(b, cudaMemsetAsync(b->veleval_u + off, 0, bytes, st));
    }
    k_bset<<<1, 1, 0, st>>>(b->d_num + scene, n);
    k_bset<<<1, 1, 0, st>>>(b->d_del + scene, 0);
    b->nvalid += n - b->num[scene];
    b->num[scene] = n;
    k_bset<<<1, 1, 0, st>>>(b->info_nb + sphk::kNum, b->nvalid);
    BCK(b, cudaGetLastError());
    BCK(b, cudaStreamSynchronize(st));
    return SPH_OK;
}

int sph_batch_step(sph_batch* b, float dt, int nsteps) {
    if (!b || nsteps < 0 || !std::isfinite(dt)) return berr(b, SPH_EINVAL, "sph_batch_step: bad arguments");
    cudaSetDevice(b->device);
    if (nsteps == 0 || b->nvalid == 0) return SPH_OK;
    if (!b->graph || b->graph_dt != dt || b->graph_valid != b->nvalid || b->graph_exact != b->exact ||
        b->graph_sched != b->sched || std::memcmp(&b->graph_lc, &b->lc, sizeof(b->lc)) != 0) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = batch_enqueue_step(b, dt, nullptr);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc != SPH_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return berr(b, SPH_ECUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return berr(b, SPH_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
        }
        b->graph_dt = dt;
        b->graph_valid = b->nvalid;
        b->graph_exact = b->exact;
        b->graph_lc = b->lc;
        b->graph_sched = b->sched;
    }
    for (int k = 0; k < nsteps; ++k) BCK(b, cudaGraphLaunch(b->graph, b->stream));
    return SPH_OK;
}

int sph_batch_sync(sph_batch* b) {
    if (!b) return SPH_EINVAL;
    // a bounded wait of the queue scheduler that ran out (sph_queue.cuh), or
    // an index out of bounds (bounds-checked library); read on the batch's
    // stream, so that no other stream of the device is waited for
    int err = 0;
    BCK(b, cudaMemcpyAsync(&err, b->info_nb + sphk::kError, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    if (err) {
        BCK(b, cudaMemsetAsync(b->info_nb + sphk::kError, 0, sizeof(int), b->stream));
        BCK(b, cudaStreamSynchronize(b->stream));
        if (err & sphk::kErrBounds)
            return berr(b, SPH_EBOUNDS, "an index of a kernel fell outside its array (bounds-checked library, "
                        "error word %d); the steps since the last sync are invalid", err);
        return berr(b, SPH_ETIMEOUT, "a bounded wait of the queue scheduler expired (error word %d); the steps "
                    "since the last sync are invalid", err);
    }
    return SPH_OK;
}

int sph_batch_set_scheduler(sph_batch* b, int scheduler) {
    if (!b || (scheduler != SPH_SCHED_GRID && scheduler != SPH_SCHED_QUEUE))
        return berr(b, SPH_EINVAL, "sph_batch_set_scheduler: %d is not a scheduler", scheduler);
    b->sched = scheduler;
    return SPH_OK;
}

int sph_batch_get_scheduler(sph_batch* b, int* scheduler) {
    if (!b || !scheduler) return SPH_EINVAL;
    *scheduler = b->sched;
    return SPH_OK;
}

int sph_batch_queue_test_hold(sph_batch* b, int hold, unsigned spin_limit) {
    if (!b || spin_limit == 0) return berr(b, SPH_EINVAL, "sph_batch_queue_test_hold: bad arguments");
    b->q_hold = hold ? 1 : 0;
    b->q_spin = spin_limit;
    b->graph_valid = -1;  // captured anew with the new queue arguments
    return SPH_OK;
}

int sph_batch_out_of_grid(sph_batch* b, int* count) {
    if (!b || !count) return SPH_EINVAL;
    int v = 0;
    BCK(b, cudaMemcpyAsync(&v, b->info_nb + kBatchFrozen, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    *count = v;
    return SPH_OK;
}

int sph_batch_get_launch_config(sph_batch* b, sph_launch_config* cfg) {
    if (!b || !cfg) return SPH_EINVAL;
    *cfg = b->lc;
    return SPH_OK;
}

int sph_batch_set_launch_config(sph_batch* b, const sph_launch_config* cfg) {
    if (!b || !cfg) return SPH_EINVAL;
    if (!sph_launch_config_valid(*cfg))
        return berr(b, SPH_EINVAL, "sph_batch_set_launch_config: shape (%d, %d, %d) not among the candidates",
                    cfg->density_threads, cfg->force_threads, cfg->scan_tile_cells);
    b->lc = *cfg;
    return SPH_OK;
}

int sph_batch_autotune(sph_batch* b, float dt, int steps, int flags, sph_launch_config* chosen) {
    if (!b || steps < 1 || !std::isfinite(dt)) return berr(b, SPH_EINVAL, "sph_batch_autotune: bad arguments");
    cudaSetDevice(b->device);
    int rc = batch_refresh_num(b);
    if (rc) return rc;
    const SphTuneKey key{1, b->nslots, (long long)b->ncells_total, b->exact};
    sph_launch_config best;
    if (!(flags & SPH_TUNE_RETIME) && sph_tune_cache_get(key, best)) {
        b->lc = best;
        if (chosen) *chosen = best;
        return SPH_OK;
    }
    if (b->nvalid <= 0) return berr(b, SPH_ESTATE, "sph_batch_autotune: no particles");
    // Save what the steps change: every slot's pos/vel/veleval, the scene
    // counts and deletions, the counters.
    const size_t fb = (size_t)b->nslots * 16, sb = (size_t)b->nscenes * 4, ib = sizeof(int) * sphk::kInfoSlots;
    char* save = nullptr;
    if (cudaMalloc((void**)&save, 3 * fb + 2 * sb + ib) != cudaSuccess) {
        cudaGetLastError();
        return berr(b, SPH_ENOMEM, "sph_batch_autotune: %zu bytes of scratch", 3 * fb + 2 * sb + ib);
    }
    void* const fields[6] = {b->pos_u, b->vel_u, b->veleval_u, b->d_num, b->d_del, b->info_nb};
    const size_t sizes[6] = {fb, fb, fb, sb, sb, ib};
    auto copy_all = [&](bool to_save) -> cudaError_t {
        size_t off = 0;
        for (int f = 0; f < 6; ++f) {
            cudaError_t e = to_save ? cudaMemcpyAsync(save + off, fields[f], sizes[f], cudaMemcpyDeviceToDevice,
                                                      b->stream)
                                    : cudaMemcpyAsync(fields[f], save + off, sizes[f], cudaMemcpyDeviceToDevice,
                                                      b->stream);
            if (e != cudaSuccess) return e;
            off += sizes[f];
        }
        return cudaSuccess;
    };
    cudaEvent_t ev[5];
    for (auto& x : ev) x = nullptr;
    cudaError_t e = cudaSuccess;
    for (auto& x : ev)
        if (e == cudaSuccess) e = cudaEventCreate(&x);
    const sph_launch_config keep = b->lc;
    double t[3][3] = {{0}};
    if (e == cudaSuccess) e = copy_all(true);
    for (int k = 0; k < 3 && e == cudaSuccess && rc == SPH_OK; ++k) {
        b->lc = sph_tune_candidates[k];
        if ((e = copy_all(false)) != cudaSuccess) break;
        if ((rc = batch_enqueue_step(b, dt, nullptr))) break;  // first launches, untimed
        if ((e = copy_all(false)) != cudaSuccess) break;
        for (int it = 0; it < steps && e == cudaSuccess && rc == SPH_OK; ++it) {
            if ((rc = batch_enqueue_step(b, dt, ev))) break;
            if ((e = cudaEventSynchronize(ev[4])) != cudaSuccess) break;
            float ms[4];
            for (int q = 0; q < 4 && e == cudaSuccess; ++q) e = cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]);
            t[k][0] += ms[2];
            t[k][1] += ms[3];
            t[k][2] += ms[0];
        }
    }
    if (e == cudaSuccess) e = copy_all(false);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    for (auto& x : ev)
        if (x) cudaEventDestroy(x);
    cudaFree(save);
    if (rc || e != cudaSuccess) {
        b->lc = keep;
        if (rc) return rc;
        return berr(b, SPH_ECUDA, "sph_batch_autotune: %s", cudaGetErrorString(e));
    }
    best = sph_tune_pick(t);
    b->lc = best;
    sph_tune_cache_put(key, best);
    if (chosen) *chosen = best;
    return SPH_OK;
}

int sph_batch_get_num(sph_batch* b, int scene, int* n) {
    if (!b || !n || scene < 0 || scene >= b->nscenes) return berr(b, SPH_EINVAL, "sph_batch_get_num: bad arguments");
    cudaSetDevice(b->device);
    const int rc = batch_refresh_num(b);
    if (rc) return rc;
    *n = b->num[scene];
    return SPH_OK;
}

int sph_batch_get_deleted(sph_batch* b, int scene, sph_float4* pos, sph_float4* vel, int cap, int* count) {
    if (!b || !count || scene < 0 || scene >= b->nscenes || cap < 0 || (cap > 0 && (!pos || !vel)))
        return berr(b, SPH_EINVAL, "sph_batch_get_deleted: bad arguments");
    cudaSetDevice(b->device);
    int rc = batch_refresh_num(b);
    if (rc) return rc;
    int del = 0;
    BCK(b, cudaMemcpyAsync(&del, b->d_del + scene, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    *count = del;
    const int k = del < cap ? del : cap;
    if (k > 0) {
        const size_t off = (size_t)b->slot_off[scene] + (size_t)b->num[scene];
        BCK(b, cudaMemcpyAsync(pos, b->pos_u + off, (size_t)k * 16, cudaMemcpyDeviceToHost, b->stream));
        BCK(b, cudaMemcpyAsync(vel, b->vel_u + off, (size_t)k * 16, cudaMemcpyDeviceToHost, b->stream));
    }
    return sph_batch_sync(b);
}

int sph_batch_download(sph_batch* b, int scene, int field, void* host, int n) {
    if (!b || scene < 0 || scene >= b->nscenes || !host || n < 0 || n > b->max_num[scene])
        return berr(b, SPH_EINVAL, "sph_batch_download: bad arguments");
    const float4* src = nullptr;
    switch (field) {
        case SPH_FIELD_POS_U: src = b->pos_u; break;
        case SPH_FIELD_VEL_U: src = b->vel_u; break;
        case SPH_FIELD_VELEVAL_U: src = b->veleval_u; break;
        default: return berr(b, SPH_EINVAL, "sph_batch_download: only pos_u, vel_u, veleval_u");
    }
    if (n > 0)
        BCK(b, cudaMemcpyAsync(host, src + b->slot_off[scene], (size_t)n * 16, cudaMemcpyDeviceToHost, b->stream));
    return sph_batch_sync(b);
}

int sph_batch_last_error(sph_batch* b, char* buf, int len) {
    if (!buf || len <= 0) return SPH_EINVAL;
    std::snprintf(buf, (size_t)len, "%s", (b ? b->err : g_batch_create_error).c_str());
    return SPH_OK;
}

}  // extern "C"
