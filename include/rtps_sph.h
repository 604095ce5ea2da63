/*
 * rtps_sph.h — C ABI of librtps_sph.so, the GB300 (sm_103a) SPH particle step.
 *
 * This boundary replaces the OpenCL host layer of the RTPS / EnjaParticles
 * reference (rtpslib/opencl: CL context CLL.h:46-87, Kernel::execute/setArg
 * Kernel.h:46-77, Buffer<T> copies Buffer.h:44-106) for the SPH path
 * SPH::updateGPU (rtpslib/system/SPH.cpp:149-300) + SPH::integrate
 * (SPH.cpp:389-441).  Every stage object of that path has one entry point
 * here, and the whole per-frame sequence has one more (sph_step).
 *
 * Conventions
 *   - Plain C: no C++ or torch types.  All particle arrays are float4
 *     array-of-structs (16 bytes per particle), as in the reference.
 *   - "_u" fields are in original (unsorted) particle order, "_s" fields in
 *     the order of the last sort (cell key, then original index).
 *   - Every function returns an int status: SPH_OK (0) or a negative code.
 *     sph_last_error() gives the message of the last failure on a context.
 *   - A context owns one CUDA stream and all device memory of one particle
 *     system.  Calls are asynchronous with respect to the host unless their
 *     comment says otherwise; sph_sync() waits.  A context is not
 *     thread-safe: one host thread drives it at a time.
 */
#ifndef RTPS_SPH_H
#define RTPS_SPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__) || defined(__clang__)
#define SPH_ALIGN16 __attribute__((aligned(16)))
#else
#define SPH_ALIGN16
#endif

/* rtpslib/structs.h:403-578 — float4, 16-byte aligned. */
typedef struct sph_float4 {
    float x, y, z, w;
} SPH_ALIGN16 sph_float4;

/* SPHParams, byte-compatible with rtpslib/system/SPHSettings.h:38-136 and its
 * OpenCL copy rtpslib/system/sph/cl_src/cl_sph_structs.h:30-75 (144 bytes). */
typedef struct SPHParams {
    float rest_density;        /*   0 */
    float mass;                /*   4 */
    float rest_distance;       /*   8 */
    float smoothing_distance;  /*  12  h */
    float simulation_scale;    /*  16 */
    float boundary_stiffness;  /*  20 */
    float boundary_dampening;  /*  24 */
    float boundary_distance;   /*  28 */
    float K;                   /*  32  gas constant */
    float viscosity;           /*  36 */
    float velocity_limit;      /*  40  (clamps the acceleration norm) */
    float xsph_factor;         /*  44 */
    float friction_coef;       /*  48 */
    float restitution_coef;    /*  52 */
    float shear;               /*  56 */
    float attraction;          /*  60 */
    float spring;              /*  64 */
    float EPSILON;             /*  68 */
    float wpoly6_coef;         /*  72 */
    float wpoly6_d_coef;       /*  76 */
    float wpoly6_dd_coef;      /*  80 */
    float wspiky_coef;         /*  84 */
    float wspiky_d_coef;       /*  88 */
    float wspiky_dd_coef;      /*  92 */
    float wvisc_coef;          /*  96 */
    float wvisc_d_coef;        /* 100 */
    float wvisc_dd_coef;       /* 104 */
    int   num;                 /* 108 */
    int   max_num;             /* 112 */
    sph_float4 gravity;        /* 128 */
} SPH_ALIGN16 SPHParams;

/* GridParams, byte-compatible with rtpslib/domain/Domain.h:144-158 and
 * rtpslib/system/common/cl_src/cl_structs.h:29-43 (128 bytes).  grid_res is
 * float, as in the reference. */
typedef struct GridParams {
    sph_float4 grid_size;   /*   0 */
    sph_float4 grid_min;    /*  16 */
    sph_float4 grid_max;    /*  32 */
    sph_float4 bnd_min;     /*  48 */
    sph_float4 bnd_max;     /*  64 */
    sph_float4 grid_res;    /*  80 */
    sph_float4 grid_delta;  /*  96  cells per unit length */
    int        nb_cells;    /* 112 */
} SPH_ALIGN16 GridParams;

#ifdef __cplusplus
static_assert(sizeof(SPHParams) == 144, "SPHParams must be 144 bytes");
static_assert(offsetof(SPHParams, EPSILON) == 68, "SPHParams.EPSILON offset");
static_assert(offsetof(SPHParams, wvisc_dd_coef) == 104, "SPHParams.wvisc_dd_coef offset");
static_assert(offsetof(SPHParams, num) == 108, "SPHParams.num offset");
static_assert(offsetof(SPHParams, max_num) == 112, "SPHParams.max_num offset");
static_assert(offsetof(SPHParams, gravity) == 128, "SPHParams.gravity offset");
static_assert(sizeof(GridParams) == 128, "GridParams must be 128 bytes");
static_assert(offsetof(GridParams, grid_res) == 80, "GridParams.grid_res offset");
static_assert(offsetof(GridParams, grid_delta) == 96, "GridParams.grid_delta offset");
static_assert(offsetof(GridParams, nb_cells) == 112, "GridParams.nb_cells offset");
#else
_Static_assert(sizeof(SPHParams) == 144, "SPHParams must be 144 bytes");
_Static_assert(sizeof(GridParams) == 128, "GridParams must be 128 bytes");
#endif

/* Status codes. */
#define SPH_OK         0
#define SPH_EINVAL    -1  /* bad argument (null pointer, n > capacity, NaN parameter, ...) */
#define SPH_ENOMEM    -2  /* device allocation failed */
#define SPH_ECUDA     -3  /* a CUDA runtime call failed; see sph_last_error */
#define SPH_EOOB      -4  /* particles left the grid (reported, not trapped) */
#define SPH_ETIMEOUT  -5  /* a bounded device-side wait expired; the step is invalid */
#define SPH_ESTATE    -6  /* call not valid in the context's current state */
#define SPH_EBOUNDS   -7  /* bounds-checked library only: a kernel index fell outside its array (the access
                             was skipped); the results since the last check are invalid */

/* Value of an empty cell in cell_start (CellIndices.cpp:58-62). */
#define SPH_EMPTY_CELL 0xffffffffu

/* Fields for sph_download / sph_get_device_ptr. */
enum sph_field {
    SPH_FIELD_POS_U = 0,      /* float4[max_num] original order */
    SPH_FIELD_VEL_U = 1,      /* float4[max_num] */
    SPH_FIELD_VELEVAL_U = 2,  /* float4[max_num] */
    SPH_FIELD_POS_S = 3,      /* float4[max_num] sorted order */
    SPH_FIELD_VEL_S = 4,      /* float4[max_num] (written by sph_stage_permute only) */
    SPH_FIELD_VELEVAL_S = 5,  /* float4[max_num] */
    SPH_FIELD_DENSITY_S = 6,  /* float[max_num] */
    SPH_FIELD_FORCE_S = 7,    /* float4[max_num] (written by the staged path only) */
    SPH_FIELD_XSPH_S = 8,     /* float4[max_num] (written by the staged path only) */
    SPH_FIELD_SORT_HASHES = 9,   /* uint32[max_num] */
    SPH_FIELD_SORT_INDICES = 10, /* uint32[max_num] */
    SPH_FIELD_CELL_START = 11,   /* uint32[nb_cells+1] */
    SPH_FIELD_CELL_END = 12,     /* uint32[nb_cells+1] */
    SPH_FIELD_NEIGHBOR_COUNT = 13, /* uint32[max_num] neighbours within h, self included (staged density only) */
    SPH_FIELD_COUNT_ = 14
};

typedef struct sph_ctx sph_ctx;

/* ---------------------------------------------------------------------------
 * Host-side parameter helpers (no device work; usable without a GPU).
 * ------------------------------------------------------------------------- */

/* Domain::calculateCells + System::setupDomain (rtpslib/domain/Domain.cpp:38-81,
 * rtpslib/system/System.cpp:294-329): pad [bnd_min, bnd_max] by 2*cell_size,
 * res = ceil(size/cell), delta = res/size, nb_cells = res.x*res.y*res.z.
 * Writes the unscaled grid and the copy scaled by sim_scale. */
int sph_setup_domain(const sph_float4* bnd_min, const sph_float4* bnd_max,
                     float cell_size, float sim_scale,
                     GridParams* grid, GridParams* grid_scaled);

/* The settings store of the reference keeps every derived number as a string
 * written at 6 significant digits (rtpslib/RTPSSettings.h:78-85); this returns
 * the float that such a round trip yields. */
float sph_settings_round(float value);

/* Kernel coefficients of SPH::calculate (rtpslib/system/SPHSettings.cpp:111-119)
 * for smoothing distance h, each passed through sph_settings_round. */
int sph_kernel_coefficients(float h, SPHParams* sphp);

/* The dam-break parameter set of the benchmark configurations: lattice
 * spacing s, h = 2s, rest_distance = s, mass = rest_density*s^3, unit-box
 * domain, with the constants given (viscosity, gas constant, wall stiffness
 * and damping, velocity limit, XSPH factor, gravity z).  Coefficients and
 * derived values are rounded as sph_settings_round does. */
int sph_dambreak_params(int num, float spacing, float viscosity,
                        SPHParams* sphp, GridParams* grid, GridParams* grid_scaled);

/* The parameter block and grids the reference gives an SPH system built from
 * its settings map (RTPS::generateSystemInstance -> SPH::SPH, SPH.cpp:50-58):
 * SPH::calculate (SPHSettings.cpp:30-144), SPH::updateParams (:150-199) and
 * System::setupDomain (System.cpp:294-329), with every derived value passed
 * through the map's 6-significant-digit strings (RTPSSettings.h:65-85).
 * keys/values: count (key, value) strings as an RTPSSettings holds them (a
 * later entry of a key replaces an earlier one; a missing key reads as "0").
 * The path reads rest_density, max_num_particles (>= 2), domain_min and
 * domain_max ("x y z w"), gas_constant, viscosity, velocity_limit,
 * xsph_factor, gravity ("x y z w"), boundary_stiffness, boundary_dampening,
 * friction_kinetic, restitution, shear, attraction, spring.  spacing
 * (nullable) receives SPH::spacing, the lattice spacing System::addBox
 * uses.  SPH_EINVAL for a non-positive rest density or domain volume. */
int sph_params_from_settings(int count, const char* const* keys, const char* const* values, SPHParams* sphp,
                             GridParams* grid, GridParams* grid_scaled, float* spacing);

/* ---------------------------------------------------------------------------
 * Context lifetime (System::System / SPH::SPH / prepareSorted,
 * System.cpp:47-89,198-291, SPH.cpp:50-99,482-520).
 * ------------------------------------------------------------------------- */

/* Allocate a context for up to max_num particles on the current CUDA device.
 * grid_scaled may be NULL, in which case it is derived from grid and
 * sphp->simulation_scale as System::setupDomain does.  Requires
 * grid->nb_cells + 1 < 2^24 (the reference computes cell hashes in float).
 * Blocking. */
int sph_create(const SPHParams* sphp, const GridParams* grid,
               const GridParams* grid_scaled, int max_num, sph_ctx** out);
int sph_destroy(sph_ctx* ctx);

/* SPH::updateParams (SPHSettings.cpp:149-200): replace the parameter block.
 * sphp->num is ignored (the particle count is owned by the context). */
int sph_set_params(sph_ctx* ctx, const SPHParams* sphp);
int sph_get_params(sph_ctx* ctx, SPHParams* sphp, GridParams* grid, GridParams* grid_scaled);

/* Use an external CUDA stream (cudaStream_t passed as void*); NULL restores the
 * context's own stream. */
int sph_set_stream(sph_ctx* ctx, void* stream);

/* ---------------------------------------------------------------------------
 * Particle data (Buffer<T>::copyToDevice/copyToHost, SPH::pushParticles
 * SPH.cpp:560-602).
 * ------------------------------------------------------------------------- */

/* Replace the state with n particles.  veleval may be NULL: it is then zero,
 * as in the reference, where pushParticles never writes veleval.  Host
 * pointers; pinned memory makes the copy asynchronous.  pos is copied on the
 * context stream, veleval and vel after it on a side stream: the next fused
 * step waits for them only in its velocity pass, which runs beside its
 * density pass, so they overlap its hash, sort, permute and density; every
 * other call waits for them on entry.  Host arrays must stay
 * valid until the next call that waits (sph_sync, a download, ...). */
int sph_upload(sph_ctx* ctx, const sph_float4* pos, const sph_float4* vel,
               const sph_float4* veleval, int n);
/* Append n particles after the current ones (pushParticles; veleval of the
 * new particles keeps whatever the buffer held, zero on a fresh context). */
int sph_push_particles(sph_ctx* ctx, const sph_float4* pos, const sph_float4* vel, int n);
/* Copy n elements of a field to host memory.  Blocking. */
int sph_download(sph_ctx* ctx, int field, void* host, int n);
/* Same, without waiting: the copy is ordered on the context stream; call
 * sph_sync before reading host memory (which should be pinned). */
int sph_download_async(sph_ctx* ctx, int field, void* host, int n);
/* Device address of a field, for zero-copy use (e.g. torch.from_blob). */
int sph_get_device_ptr(sph_ctx* ctx, int field, void** dptr);
/* Current particle count (after any out-of-grid deletion).  Blocking. */
int sph_get_num(sph_ctx* ctx, int* num);
/* Set the particle count after writing state through sph_get_device_ptr. */
int sph_set_num(sph_ctx* ctx, int num);

/* ---------------------------------------------------------------------------
 * Stages.  One entry point per stage object of SPH::updateGPU / integrate.
 * ------------------------------------------------------------------------- */

/* Hash::execute (Hash.cpp:42-75; hash.cl:50-157): sort_hashes[i] = cell key of
 * pos_u[i] from the unscaled grid (nb_cells when outside), sort_indices[i] = i. */
int sph_stage_hash(sph_ctx* ctx);
/* System::bitonic_sort (System.cpp:407-480), replaced by a stable LSD radix
 * sort: ascending keys, equal keys in ascending original index. */
int sph_stage_sort(sph_ctx* ctx);
/* CellIndices::execute (CellIndices.cpp:42-169; cellindices.cl:12-107).
 * cell_start = first sorted index of each cell (SPH_EMPTY_CELL if empty),
 * cell_end = one past the last (only written for occupied cells).  *nc gets
 * cell_start[nb_cells] as int (-1 when no particle is outside the grid).
 * nc may be NULL; when not NULL the call blocks. */
int sph_stage_cellindices(sph_ctx* ctx, int* nc);
/* Permute::execute (Permute.cpp:45-108; permute.cl:10-46): X_s[i] = X_u[idx[i]]
 * for pos, vel, veleval. */
int sph_stage_permute(sph_ctx* ctx);
/* Density::execute (sph/Density.cpp:52-92; density.cl:44-126). */
int sph_stage_density(sph_ctx* ctx);
/* Force::execute (sph/Force.cpp:52-94; force.cl:43-186): force_s, xsph_s. */
int sph_stage_force(sph_ctx* ctx);
/* CollisionWall::execute (sph/Collision_wall.cpp:39-67; collision_wall.cl:31-118):
 * force_s += wall repulsion and friction. */
int sph_stage_collision(sph_ctx* ctx);
/* LeapFrog::execute (sph/LeapFrog.cpp:42-83; leapfrog.cl:30-121): integrate and
 * scatter to pos_u, vel_u, veleval_u. */
int sph_stage_leapfrog(sph_ctx* ctx, float dt);
/* Gravity::execute (common/Gravity.cpp:43-75; gravity.cl:9-35) as
 * SPH::updateGPU calls it after force (SPH.cpp:289-296): force_s += the pull
 * of the point sources set by sph_set_gravity_sources on the sorted
 * positions.  No-op without sources. */
int sph_stage_gravity(sph_ctx* ctx);
/* Euler::execute (sph/cl_src/euler.cl:33-78): the SPH Euler integrator.  Its
 * gravity is the constant -9.8 in z and its acceleration limit the constant
 * 600, as in the reference; it writes pos_u and vel_u and leaves veleval_u. */
int sph_stage_euler(sph_ctx* ctx, float dt);
/* CollisionTriangle::execute (sph/Collision_triangle.cpp:84-116;
 * collision_tri.cl:436-520), the second half of SPH::collision (SPH.cpp:
 * 303-336): force_s += the repulsion and friction of the triangles of the
 * mesh loaded by sph_load_triangles whose segment test (particle position
 * -+ boundary_distance along the velocity) hits them, and force_s.w += the
 * triangle count.  Always in exact arithmetic.  No-op without a mesh. */
int sph_stage_collision_triangles(sph_ctx* ctx);

/* Point gravity sources: the settings gravity_sources / gravity_mass /
 * gravity_alphas of System::prepareSorted (System.cpp:260-272).  count
 * sources (0 removes them, at most SPH_MAX_GRAVITY_SOURCES) with positions
 * points[k] (unscaled), masses[k] and strengths alphas[k]; each pulls a
 * particle at squared scaled distance d with alpha*mass/d, and pushes it with
 * alpha*mass/(0.5*simulation_scale)^2 inside that radius.  Blocking. */
#define SPH_MAX_GRAVITY_SOURCES 64
int sph_set_gravity_sources(sph_ctx* ctx, int count, const sph_float4* points, const float* masses,
                            const float* alphas);

/* The integrator of SPH::integrate (SPH.cpp:392-436), the setting
 * "integrator": leapfrog (the default) or euler.  Used by sph_integrate and
 * the fused step. */
#define SPH_INTEGRATOR_LEAPFROG 0
#define SPH_INTEGRATOR_EULER 1
int sph_set_integrator(sph_ctx* ctx, int integrator);

/* SPH::loadTriangles -> CollisionTriangle::loadTriangles (sph/
 * Collision_triangle.cpp:44-82).  count triangles of four sph_float4 each
 * (three vertices, unscaled, and a normal: rtps Triangle, structs.h:586-590);
 * the stored normal is not read, the kernel uses (b-a)x(c-a) normalised.
 * count 0 unloads the mesh.  The reference's buffer holds 2048 triangles;
 * this one grows to SPH_MAX_TRIANGLES.  Non-finite vertices are rejected.
 * Blocking. */
#define SPH_MAX_TRIANGLES (1 << 20)
int sph_load_triangles(sph_ctx* ctx, const sph_float4* tris, int count);

/* Hoses: a disc of new particles pushed into the system every few steps.
 *
 * sph_hose is the reference's Hose (common/Hose.cpp:30-130) on its own, a
 * host object: total_n particles, emitted from a disc of the given radius
 * around center, normal to velocity, on a jittered grid of the given
 * spacing (addDiscRandom, domain/IV.cpp:313-367), every
 * 1 + spacing/dt/|velocity|/10 sprays.  The jitter comes from the C
 * library's rand(), as in the reference (seed it with srand).  A zero y or z
 * velocity is replaced by 1e-7, as the reference does.  No GPU is involved. */
typedef struct sph_hose sph_hose;
int sph_hose_create(float dt, int total_n, sph_float4 center, sph_float4 velocity, float radius, float spacing,
                    sph_hose** out);
/* Hose::update and Hose::refill. */
int sph_hose_update(sph_hose* hose, sph_float4 center, sph_float4 velocity, float radius, float spacing);
int sph_hose_refill(sph_hose* hose, int n);
/* Hose::spray: one tick of the emission clock; *count = the particles this
 * tick emits (0 between emissions), kept until the next spray. */
int sph_hose_spray(sph_hose* hose, int* count);
/* The last spray's particles (at most cap) and the velocity they are pushed
 * with (Hose::getVelocity). */
int sph_hose_particles(const sph_hose* hose, sph_float4* pos, int cap, sph_float4* velocity);
/* Particles left in the hose. */
int sph_hose_remaining(const sph_hose* hose, int* n);
void sph_hose_destroy(sph_hose* hose);

/* SPH::addHose / updateHose / refillHose (SPH.cpp:523-545): hoses owned by
 * the context.  radius is in particle spacings: it is multiplied by the
 * "spacing" setting, rest_distance / simulation_scale.  dt is the time step
 * the emission rate is computed for (the setting time_step). *index gets the
 * hose's index. */
int sph_add_hose(sph_ctx* ctx, int total_n, sph_float4 center, sph_float4 velocity, float radius, float dt,
                 int* index);
int sph_update_hose(sph_ctx* ctx, int index, sph_float4 center, sph_float4 velocity, float radius);
int sph_refill_hose(sph_ctx* ctx, int index, int n);
/* SPH::sprayHoses (SPH.cpp:547-558): every hose sprays once and what it
 * emits is appended with sph_push_particles at the hose's velocity; a spray
 * that would pass max_num is dropped, as SPH::pushParticles drops it
 * (SPH.cpp:562-567).  sph_update, and sph_step and sph_step_eager before
 * every step, call it first when the context has hoses, as SPH::updateGPU
 * does (SPH.cpp:162-166).  *added (may be null) gets the particles added.
 * Blocking when a hose emits. */
int sph_spray_hoses(sph_ctx* ctx, int* added);

/* SPH::postProcess (SPH.cpp:338-386), headless: the colour field and its
 * marching-cubes surface, kept in device buffers owned by the context.
 *
 * sph_colorfield: ColorField::execute (sph/ColorField.cpp:84-121;
 * colorfield.cl): res^3 samples spanning the scaled grid's bounds, sample
 * (s, t, r) at index s + t*res + r*res^2, value mass * sum over particles within
 * h of Wspiky(max(|r|, EPSILON)) / rho_j, from the sorted state of the last
 * update.  res below 2 becomes 2; at most 512.  Asynchronous. */
int sph_colorfield(sph_ctx* ctx, int res);
/* MarchingCubes::execute (common/MarchingCubes.cpp:166-370; classifycubes.cl,
 * constructhp.cl, traversehp.cl) on a res^3 field: the device array `field`
 * (s + t*res + r*res^2 order), or the context's colour field when field is
 * null.  Writes the context's mesh: *ntri triangles, 9 floats each for the
 * vertices (grid position / (res - 1) * 10, the reference's render box) and
 * 9 for the vertex normals, in the reference's cube order.  The per-case
 * triangulation is sph_mc_case_table's: per cube the triangle count and the
 * vertices equal the reference's; which diagonal splits a quad can differ.
 * Blocking (reads the count). */
int sph_marching_cubes(sph_ctx* ctx, const float* field, int res, float isolevel, int* ntri);
/* Colour field + marching cubes at the reference's isolevel 0.0001;
 * nothing (0 triangles) without particles. */
int sph_post_process(sph_ctx* ctx, int res, int* ntri);
/* Device views of the colour field (res^3 floats), the mesh vertices and
 * normals (ntri*9 floats each); valid until the next surface call. */
int sph_get_surface(sph_ctx* ctx, const float** field, const float** vertices, const float** normals, int* res,
                    int* ntri);
/* Host copies of the field (res^3 floats) and of at most cap_tri triangles'
 * vertices and normals; any pointer may be null.  Blocking. */
int sph_download_surface(sph_ctx* ctx, float* field, float* vertices, float* normals, int cap_tri);
/* The marching-cubes case table, no reference counterpart (the reference
 * uses a published table): for case c (bit k set when corner k is above the
 * isolevel, corners in the reference's order), count[c] triangles given by
 * tri[c*18 .. c*18+3*count[c]-1] as local edge numbers (the reference's edge
 * list); *max_triangles gets the largest count.  Host only. */
#define SPH_MC_CASE_EDGES 18
int sph_mc_case_table(signed char* tri, unsigned char* count, int* max_triangles);

/* SPH::update (SPH.cpp:117-125 -> updateGPU :149-300) with SPH::collision
 * (SPH.cpp:303-336) enabled after gravity: hash, sort, cellindices, permute,
 * out-of-grid deletion, density, force, point-source gravity, walls, and the
 * triangle mesh when one is loaded. */
int sph_update(sph_ctx* ctx);
/* SPH::integrate (SPH.cpp:389-441): the integrator sph_set_integrator chose. */
int sph_integrate(sph_ctx* ctx, float dt);

/* nsteps x (update + integrate) on the fused path: hash and sort (a counting
 * sort on the cell key, with the same canonical order as sph_stage_sort) ->
 * cellindices+permute -> density -> force+gravity+collision+integrator,
 * replayed from a captured CUDA graph.  With a triangle mesh loaded the force
 * pass leaves out the walls and the integrator, and one triangle kernel
 * applies gravity, walls, triangles and the integrator.  Results equal
 * nsteps staged update()+integrate() calls.  Asynchronous. */
int sph_step(sph_ctx* ctx, float dt, int nsteps);

/* The same fused step launched kernel by kernel, without a graph (for
 * profiling and for callers that capture their own graphs). */
int sph_step_eager(sph_ctx* ctx, float dt, int nsteps);

/* nsteps fused steps launched kernel by kernel with a CUDA event between
 * launches on the context stream, for per-kernel timing.  kernel_ms[k]
 * accumulates the device time of launch k of the step (k < cap); *nkernels
 * gets the number of launches per step; names come from
 * sph_profile_kernel_name.  SPH_ESTATE with a triangle mesh loaded.
 * Blocking. */
int sph_step_profile(sph_ctx* ctx, float dt, int nsteps, float* kernel_ms, int cap, int* nkernels);
const char* sph_profile_kernel_name(sph_ctx* ctx, int k);

/* Launch shapes of the step's kernels.  No counterpart in the reference,
 * whose work-group sizes are constants of its host code
 * (rtpslib/system/sph/Density.cpp:80, Force.cpp:82).  Every shape gives the
 * same results bit for bit; only the time differs. */
typedef struct {
    int density_threads; /* threads per block of the density pass: 128, 256 (default) or 512 */
    int force_threads;   /* of the fused force pass: 64, 128 (default) or 256 */
    int scan_tile_cells; /* cells per block of the cell totals and scan: 2048, 4096 (default) or 8192 */
    int reserved;        /* 0 */
} sph_launch_config;

/* The context's launch shapes.  set: SPH_EINVAL for a value outside the
 * listed ones (the context keeps its shapes). */
int sph_get_launch_config(sph_ctx* ctx, sph_launch_config* cfg);
int sph_set_launch_config(sph_ctx* ctx, const sph_launch_config* cfg);

#define SPH_TUNE_RETIME 1 /* time the candidates even when the process has a result for this key */

/* Autotuner.  Times the candidate shapes of the density pass, the force
 * pass and the cell scan over `steps` fused steps each, from the current
 * state (saved before and restored after, so the simulation does not
 * advance), keeps the fastest of each and sets them on the context.  The
 * result is remembered in the process per (max_num, nb_cells, arithmetic
 * mode): a later call on any context with the same key takes it without
 * timing, unless flags has SPH_TUNE_RETIME.  chosen (nullable) receives the
 * shapes.  Needs particles (SPH_ESTATE without); times the step without a
 * triangle mesh or hoses (SPH_ESTATE with one).  Blocking; allocates
 * 48 bytes per particle of scratch while it runs. */
int sph_autotune(sph_ctx* ctx, float dt, int steps, int flags, sph_launch_config* chosen);

/* Force-stage arithmetic.  0 (default): FMA and reciprocals, within the
 * FP32 tolerance of the oracle.  1: the oracle's exact operation sequence
 * (IEEE divisions and square roots, no contraction), bitwise equal to the
 * FP32 oracle.  Hash, sort, cell ranges, permute, density, collision and
 * leapfrog are always exact. */
int sph_set_exact(sph_ctx* ctx, int exact);

/* Particles removed by the last out-of-grid deletion (SPH.cpp:220-250 keeps
 * them in deleted_pos / deleted_vel, getDeletedPos/Vel SPH.h:83-84): copies up
 * to cap of them and stores their number in *count.  Blocking. */
int sph_get_deleted(sph_ctx* ctx, sph_float4* pos, sph_float4* vel, int cap, int* count);

/* Wait for all work on the context stream; reports device-side errors
 * (SPH_ETIMEOUT) and out-of-grid deletions are visible through sph_get_num. */
int sph_sync(sph_ctx* ctx);

/* Copy the message of the last error on ctx (or, when ctx is NULL, of the
 * last failed sph_create on the calling thread) into buf. */
int sph_last_error(sph_ctx* ctx, char* buf, int len);

/* ---------------------------------------------------------------------------
 * Differentiable rollout.  No counterpart in the reference.  Reverse-mode
 * gradients of a loss of the final state of an nsteps-step rollout with
 * respect to its initial state and the viscosity coefficient, through
 * adjoints of density, force, wall collision and leapfrog; sorting and
 * hashing are piecewise constant and not differentiated.  The wall and
 * friction tests and the acceleration clamp are taken as the forward run
 * took them (the gradient of the branch the trajectory is on).
 * ------------------------------------------------------------------------- */

/* Run nsteps fused steps from the current state (as sph_step), keeping the
 * state every K steps (checkpoints).  Leaves the final state in the context.
 * Needs a fixed particle set: SPH_EOOB when a particle leaves the grid during
 * the rollout, SPH_ESTATE when a deletion is pending.  Blocking. */
int sph_adjoint_record(sph_ctx* ctx, float dt, int nsteps, int K);

/* Backward pass of the recorded rollout.  Inputs: the loss gradient with
 * respect to the final pos_u / vel_u / veleval_u (NULL: zero); outputs: the
 * gradient with respect to the initial ones (NULL: not wanted) and to
 * SPHParams.viscosity (FP64 sum; NULL: not wanted).  All arrays are DEVICE
 * pointers of num float4 in original particle order (w lanes ignored / 0).
 * Recomputes each K-step segment from its checkpoint (tape memory: K *
 * (132 * max_num + 8 * nb_cells) bytes) and leaves the context's state as
 * the rollout's final state; the sort scratch buffers (SORT_HASHES) hold
 * recomputation leftovers afterwards.  Blocking. */
int sph_adjoint_backward(sph_ctx* ctx, const sph_float4* dL_dpos, const sph_float4* dL_dvel,
                         const sph_float4* dL_dveleval, sph_float4* dL_dpos0, sph_float4* dL_dvel0,
                         sph_float4* dL_dveleval0, double* dL_dvisc);

/* The backward pass for a loss of the final positions only: dL_dvel0 (device,
 * num float4) and *dL_dvisc (host).  nsteps and K must be those recorded. */
int sph_adjoint_rollout(sph_ctx* ctx, int nsteps, int K, const sph_float4* dL_dpos_final,
                        sph_float4* dL_dvel0, float* dL_dvisc);

/* Put the recorded rollout's initial state back into the context (for the
 * next iteration of an optimisation loop).  Blocking. */
int sph_adjoint_rewind(sph_ctx* ctx);

/* Mean squared distance of the current positions to target (device, num
 * float4, original order): *loss = (1/num) sum |x_i - x*_i|^2 (FP64 sum) and
 * dL_dpos (device, num float4) = 2 (x_i - x*_i) / num.  Blocking. */
int sph_loss_mse(sph_ctx* ctx, const sph_float4* target, sph_float4* dL_dpos, double* loss);

/* ---------------------------------------------------------------------------
 * Batches: many independent systems ("scenes", each with its own SPHParams,
 * grid and particle count) stepped together.  No counterpart in the
 * reference, which steps one system per SPH object.  All scenes share one
 * launch sequence per step (captured in one CUDA graph); every scene steps
 * exactly as it would in its own context, deletions included: particles that
 * leave their scene's grid are removed from it as SPH::updateGPU removes
 * them (SPH.cpp:220-250), the scene's count drops (sph_batch_get_num) and
 * the removed particles can be read back (sph_batch_get_deleted).
 * ------------------------------------------------------------------------- */
typedef struct sph_batch sph_batch;

/* nscenes scenes: sphp[s], grids[s] (grids_scaled may be NULL: derived from
 * simulation_scale), capacity max_num[s].  Blocking. */
int sph_batch_create(int nscenes, const SPHParams* sphp, const GridParams* grids,
                     const GridParams* grids_scaled, const int* max_num, sph_batch** out);
int sph_batch_destroy(sph_batch* batch);
int sph_batch_set_stream(sph_batch* batch, void* stream);
int sph_batch_set_exact(sph_batch* batch, int exact);
/* Launch shapes and autotuner of the batched step (sph_launch_config): the
 * same as for one system, keyed per (total particle slots, total cells,
 * arithmetic mode) of the batch. */
int sph_batch_get_launch_config(sph_batch* batch, sph_launch_config* cfg);
int sph_batch_set_launch_config(sph_batch* batch, const sph_launch_config* cfg);
int sph_batch_autotune(sph_batch* batch, float dt, int steps, int flags, sph_launch_config* chosen);

/* Scheduler of the batch's neighbour passes (no counterpart in the
 * reference).  SPH_SCHED_GRID (default): one thread per sorted particle of
 * every scene, one grid per pass, each particle's scene looked up from its
 * key.  SPH_SCHED_QUEUE: as many blocks as fit on the GPU, each taking
 * (scene, tile) items from a device counter; a block's scene parameters sit
 * in shared memory.  The results are the same bits either way. */
#define SPH_SCHED_GRID 0
#define SPH_SCHED_QUEUE 1
int sph_batch_set_scheduler(sph_batch* batch, int scheduler);
int sph_batch_get_scheduler(sph_batch* batch, int* scheduler);
/* Test support for the queue scheduler's bounded waits: with hold set the
 * block that builds the queue's item table never publishes it, so every
 * block's wait for it runs out after spin_limit polls (a poll is about
 * 0.25 us; the default limit is 2^22) and the next sph_batch_sync returns
 * SPH_ETIMEOUT; the batch stays usable.  hold = 0 restores normal steps. */
int sph_batch_queue_test_hold(sph_batch* batch, int hold, unsigned spin_limit);
/* Replace scene `scene`'s particles (veleval NULL: zero).  Blocking. */
int sph_batch_upload(sph_batch* batch, int scene, const sph_float4* pos, const sph_float4* vel,
                     const sph_float4* veleval, int n);
/* nsteps steps of every scene (hash ... force+collision+leapfrog).  Asynchronous. */
int sph_batch_step(sph_batch* batch, float dt, int nsteps);
/* Copy n elements of pos_u, vel_u or veleval_u of one scene.  Blocking. */
int sph_batch_download(sph_batch* batch, int scene, int field, void* host, int n);
/* Number of particles, over all scenes, that the last step removed because
 * they had left their scene's grid.  Blocking. */
int sph_batch_out_of_grid(sph_batch* batch, int* count);
/* Current particle count of one scene (SPH::getNum; it drops after a
 * deletion).  Blocking. */
int sph_batch_get_num(sph_batch* batch, int scene, int* n);
/* The particles removed by the scene's last deletion, in sorted order, as
 * SPH::getDeletedPos / getDeletedVel (SPH.h:83-84): *count = how many; the
 * first min(count, cap) positions and velocities are copied to the host
 * arrays.  Valid until the scene's next upload or deletion.  Blocking. */
int sph_batch_get_deleted(sph_batch* batch, int scene, sph_float4* pos, sph_float4* vel, int cap, int* count);
int sph_batch_sync(sph_batch* batch);
/* The message of the last error on batch (or, when batch is NULL, of the
 * last failed sph_batch_create on the calling thread). */
int sph_batch_last_error(sph_batch* batch, char* buf, int len);
/* Replace scene `scene`'s SPHParams (same simulation_scale; the grid stays).
 * Blocking. */
int sph_batch_set_params(sph_batch* batch, int scene, const SPHParams* sphp);
int sph_batch_get_params(sph_batch* batch, int scene, SPHParams* sphp);
/* Device address of pos_u / vel_u / veleval_u of the whole batch: one float4
 * per particle slot, scene s's particles at slots [offset_s, offset_s + num_s)
 * (sph_batch_slot_offset). */
int sph_batch_get_device_ptr(sph_batch* batch, int field, void** dptr);
int sph_batch_slot_offset(sph_batch* batch, int scene, int* offset);

/* Differentiable rollout of every scene at once (see sph_adjoint_record):
 * one launch sequence per step and per reverse step for all scenes, the
 * viscosity gradient per scene.  Arrays are DEVICE pointers in slot layout
 * (one float4 per particle slot; unused slots are ignored on input and
 * unspecified on output); dL_dvisc is a host array of nscenes doubles.
 * Needs every particle to stay inside its scene's grid (SPH_EOOB).
 * Blocking. */
int sph_batch_adjoint_record(sph_batch* batch, float dt, int nsteps, int K);
int sph_batch_adjoint_backward(sph_batch* batch, const sph_float4* dL_dpos, const sph_float4* dL_dvel,
                               const sph_float4* dL_dveleval, sph_float4* dL_dpos0, sph_float4* dL_dvel0,
                               sph_float4* dL_dveleval0, double* dL_dvisc);
int sph_batch_adjoint_rewind(sph_batch* batch);
/* Per-scene mean squared distance to target (device, slot layout): loss (host,
 * nscenes doubles) and its gradient dL_dpos (device, slot layout; zero in
 * unused slots).  Blocking. */
int sph_batch_loss_mse(sph_batch* batch, const sph_float4* target, sph_float4* dL_dpos, double* loss);

/* Trajectory form (losses on the positions at the checkpoint times 0, K, 2K,
 * ..., nsteps of the recorded rollout; nck = ceil(nsteps / K) + 1 of them).
 * Arrays of positions or gradients over the trajectory are DEVICE pointers of
 * nck * nslots float4, time-major (checkpoint c at offset c * nslots).
 *   sph_batch_trajectory      copy the recorded positions at those times
 *   sph_batch_loss_traj       per scene, the mean over the times 1..nck-1 of
 *                             (1/N_s) sum_i rho(|x_i - x*_i|), and its
 *                             gradient (zero at time 0); rho(d) = d^2 when
 *                             huber = 0, else the Huber function with
 *                             delta = huber * smoothing_distance of the scene
 *                             (quadratic up to delta, linear beyond: a few
 *                             particles far from their targets cannot
 *                             dominate the loss)
 *   sph_batch_adjoint_backward_traj  backward pass with a position-loss
 *                             gradient at every checkpoint time
 * All blocking. */
int sph_batch_trajectory(sph_batch* batch, sph_float4* pos_traj);
int sph_batch_loss_traj(sph_batch* batch, const sph_float4* targets, sph_float4* dL_dpos_traj, float huber,
                        double* loss);
int sph_batch_adjoint_backward_traj(sph_batch* batch, const sph_float4* dL_dpos_traj, sph_float4* dL_dpos0,
                                    sph_float4* dL_dvel0, sph_float4* dL_dveleval0, double* dL_dvisc);

/* Sort n (key, value) pairs held in caller-owned device memory, without
 * allocating any device memory.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: a host application that owns all
 * device memory through its own pool, a real-time frame loop that cannot take
 * the synchronisation an allocation may bring, or code that has no access to
 * the allocator.  Same stable LSD radix sort as sph_stage_sort: ascending keys
 * (the low key_bits bits of each key are the sort key; keys must fit in them),
 * equal keys keep their input order.  keys_in/vals_in are read only;
 * keys_out/vals_out must not overlap them or each other (SPH_EINVAL).
 * Bits of a key above key_bits are ignored by the ordering and kept in the
 * output.  stream is a cudaStream_t (NULL: the legacy default stream).
 *
 * Limit: n <= 1,048,576 (SPH_EINVAL above).  All scratch memory lives in one
 * statically sized device array of the library (about 9 MiB, held by every
 * GPU that loads the library until the process exits).  Calls share the
 * array: calls that overlap on the GPU (other streams, other threads) race and
 * corrupt each other; each call clears the parts of it that must start at
 * zero.  Blocking: every call copies its status word back on the given stream
 * and waits for that stream (and no other) before it returns, so the call
 * cannot be captured into a CUDA graph; make every call outside stream
 * capture.  The address is cached per device for the life of the
 * process: a cudaDeviceReset invalidates it, so do not call this function
 * after resetting a device it was used on. */
int sph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                           uint32_t* vals_out, int n, int key_bits, void* stream);

/* Library identification string (build flags, arch). */
const char* sph_build_info(void);

#ifdef __cplusplus
}
#endif

#endif /* RTPS_SPH_H */
