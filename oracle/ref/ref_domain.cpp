// TEST INFRASTRUCTURE: the reference's own Domain::calculateCells
// (rtpslib/domain/Domain.cpp:38-81, compiled from the reference tree) driven
// as System::setupDomain does (rtpslib/system/System.cpp:294-329).
#include <cstring>
#include <vector>
#include "domain/Domain.h"
#include "domain/IV.h"
#include "ref_api.h"

extern "C" void ref_setup_domain(const float* bmin, const float* bmax, float cell_size, float sim_scale, void* grid,
                                 void* grid_scaled) {
    rtps::float4 lo(bmin[0], bmin[1], bmin[2], bmin[3]);
    rtps::float4 hi(bmax[0], bmax[1], bmax[2], bmax[3]);
    rtps::Domain d(lo, hi);
    d.calculateCells(cell_size);
    rtps::GridParams g, s;
    g.grid_min = d.getMin();
    g.grid_max = d.getMax();
    g.bnd_min = d.getBndMin();
    g.bnd_max = d.getBndMax();
    g.grid_res = d.getRes();
    g.grid_size = d.getSize();
    g.grid_delta = d.getDelta();
    g.nb_cells = (int)(g.grid_res.x * g.grid_res.y * g.grid_res.z);
    s.grid_min = g.grid_min * sim_scale;
    s.grid_max = g.grid_max * sim_scale;
    s.bnd_min = g.bnd_min * sim_scale;
    s.bnd_max = g.bnd_max * sim_scale;
    s.grid_res = g.grid_res;
    s.grid_size = g.grid_size * sim_scale;
    s.grid_delta = g.grid_delta / sim_scale;
    s.nb_cells = g.nb_cells;
    static_assert(sizeof(rtps::GridParams) == 128, "GridParams layout");
    std::memcpy(grid, &g, 128);
    std::memcpy(grid_scaled, &s, 128);
}

// The reference's addRect (rtpslib/domain/IV.cpp:165-202, compiled from the
// reference tree): at most num lattice points, written as float4 rows to out;
// returns how many were made.
extern "C" int ref_add_rect(int num, const float* lo, const float* hi, float spacing, float scale, float* out) {
    std::vector<rtps::float4> v = rtps::addRect(num, rtps::float4(lo[0], lo[1], lo[2], lo[3]),
                                                rtps::float4(hi[0], hi[1], hi[2], hi[3]), spacing, scale);
    for (size_t i = 0; i < v.size(); ++i) {
        out[4 * i] = v[i].x;
        out[4 * i + 1] = v[i].y;
        out[4 * i + 2] = v[i].z;
        out[4 * i + 3] = v[i].w;
    }
    return (int)v.size();
}
