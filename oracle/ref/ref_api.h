// TEST INFRASTRUCTURE: C entry points of oracle/_ref/librtps_ref.so, the
// reference's own OpenCL kernels compiled for the host (see build_ref.py).
#pragma once
#include <cstdint>
extern "C" {
void ref_hash(int n, const float* pos_u, const void* gp, uint32_t* keys, uint32_t* idx);
void ref_bitonic_sort(int n, uint32_t* keys, uint32_t* idx);
int ref_cellindices(int n, const uint32_t* keys, const uint32_t* idx, uint32_t* start, uint32_t* end, const void* gp);
void ref_permute(int n, const uint32_t* idx, const float* pos_u, const float* vel_u, const float* veleval_u,
                 float* pos_s, float* vel_s, float* veleval_s);
void ref_density(int n, const float* pos_s, float* density, const uint32_t* start, const uint32_t* end,
                 const void* gps, const void* sphp);
void ref_force(int n, const float* pos_s, const float* density, const float* veleval_s, float* force, float* xsph,
               const uint32_t* start, const uint32_t* end, const void* gps, const void* sphp);
void ref_collision_wall(int n, const float* pos_s, const float* vel_s, float* force, const void* gps,
                        const void* sphp);
void ref_leapfrog(int n, float* pos_u, const float* pos_s, float* vel_u, const float* vel_s, float* veleval_u,
                  const float* force, const float* xsph, const uint32_t* idx, const void* sphp, float dt);
void ref_gravity(int n, int nsrc, const float* points, const float* masses, const float* alphas, const float* pos_s,
                 float* force, float scale);
void ref_euler(int n, float* pos_u, const float* pos_s, float* vel_u, const float* vel_s, const float* force,
               const uint32_t* idx, const void* sphp, float dt);
void ref_collision_triangles(int n, const float* pos_s, const float* vel_s, float* force, const float* tris, int ntri,
                             const void* sphp, float dt);
void ref_setup_domain(const float* bnd_min, const float* bnd_max, float cell_size, float sim_scale, void* grid,
                      void* grid_scaled);
}

// SPH::calculate + SPH::updateParams + System::setupDomain over a settings
// map (rtpslib/system/SPHSettings.cpp, RTPSSettings.cpp); returns
// sizeof(SPHParams) of the reference's struct.
extern "C" int ref_params_from_settings(int count, const char* const* keys, const char* const* values, void* sphp,
                                        void* grid, void* grid_scaled, float* spacing);

// Hose (rtpslib/system/common/Hose.cpp): create, spray, update, refill.
extern "C" void* ref_hose_create(float dt, int total_n, const float* center, const float* velocity, float radius,
                                 float spacing);
extern "C" int ref_hose_spray(void* h, float* out, int cap, float* velocity);
extern "C" void ref_hose_update(void* h, const float* center, const float* velocity, float radius, float spacing);
extern "C" void ref_hose_refill(void* h, int n);
extern "C" void ref_hose_destroy(void* h);
extern "C" void ref_srand(unsigned seed);

// Colour field (sph/cl_src/colorfield.cl) and its image tiling.
extern "C" int ref_colorfield_slices(int res);
extern "C" int ref_colorfield(int res, int n, const float* pos_s, const float* density, const unsigned* cell_start,
                              const unsigned* cell_end, const void* grid_scaled, const void* sphp, float* field,
                              float* image);

// Marching cubes (common/cl_src/classifycubes.cl, constructhp.cl, traversehp.cl)
// on a res^3 field in (s + t res + r res^2) order; returns the triangle count.
extern "C" int ref_marching_cubes(int res, const float* field, float isolevel, float* tris, float* normals,
                                  int cap_tri, float* base_level);
