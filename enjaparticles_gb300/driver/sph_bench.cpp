// sph_bench.cpp — headless C++ driver of the SPH step through the rtps::SPH
// class (include/rtps_sph.hpp), the way a reference frame loop drives
// rtps::SPH (test/glwidget.cpp:876-916, test/benchmarks/rb_sph_benchmark.cpp:
// 162-198), without a window.
//
// Builds the dam-break scene of n particles (the seeded jittered lattice of
// enjaparticles_gb300/scenes.py, same numbers), steps it, and prints one JSON
// line: particle-updates/s and an FP64 checksum of the final positions.
//
//   sph_bench [--n N] [--steps S] [--warmup W] [--dt DT] [--viscosity MU]
//             [--frames] [--exact] [--mesh] [--post-process RES]
//   --frames: one update()+integrate() pair per step (the reference's frame
//             loop, staged kernels) instead of the fused graph-replayed step.
//   --mesh: load the 524-triangle ramp-and-box mesh (scenes.ramp_and_box_mesh,
//             same vertex bits) with SPH::loadTriangles.
//   --post-process RES: SPH::postProcess with the colour field at RES after
//             the run (every frame with --frames); prints the mesh's triangles.
//   sph_bench --n N --dump-scene FILE: write the scene's positions (N x 4
//             float32) to FILE and exit (no GPU needed).
//   sph_bench --add-rect NUM SPACING SCALE LX LY LZ HX HY HZ FILE: write
//             rtps::addRect(NUM, lo, hi, SPACING, SCALE) (k x 4 float32) to
//             FILE and exit (no GPU needed).
//   sph_bench --settings FILE --box NUM LX LY LZ HX HY HZ [--steps S]
//             [--out-init FILE] [--out FILE]: the reference's construction
//             path: an RTPSSettings filled from FILE (one setting per line,
//             the key then its value), rtps::SPH(&settings), addBox(NUM, lo,
//             hi), then S frames of update()+integrate(); writes the
//             positions after addBox and after the frames (N x 4 float32) and
//             prints the derived parameters and a checksum.
//   sph_bench --n N --add-box NUM SCALE LX LY LZ HX HY HZ FILE: a system with
//             the dam-break parameters of N particles and simulation_scale
//             SCALE, filled by SPH::addBox(NUM, lo, hi, false); writes its
//             positions (getPositions) to FILE and prints getSpacing().
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rtps_sph.hpp"

namespace {

uint64_t splitmix64(uint64_t seed, uint64_t k) {
    uint64_t z = seed + k * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// k-th (from 0) double in [0, 1) of the stream `seed`.
double uniform(uint64_t seed, uint64_t k) {
    return (double)(splitmix64(seed, k + 1) >> 11) * (1.0 / 9007199254740992.0);
}

float lattice_spacing(int n) { return (float)std::pow(0.125 / n, 1.0 / 3.0); }

// Points ((i+1/2)s, (j+1/2)s, (k+1/2)s), z outermost, each coordinate
// jittered by U(-0.01 s, 0.01 s).
std::vector<rtps::float4> dambreak_positions(int n, uint64_t seed) {
    const double s = lattice_spacing(n);
    const long side = (long)std::ceil(0.5 / s - 1e-9), layer = side * side;
    std::vector<rtps::float4> pos((size_t)n);
    for (long k = 0; k < n; ++k) {
        const long iz = k / layer, rem = k % layer, iy = rem / side, ix = rem % side;
        double jit[3];
        for (int a = 0; a < 3; ++a) jit[a] = (2.0 * uniform(seed, 3 * (uint64_t)k + a) - 1.0) * (0.01 * s);
        pos[k] = rtps::make_float4((float)((ix + 0.5) * s + jit[0]), (float)((iy + 0.5) * s + jit[1]),
                                   (float)((iz + 0.5) * s + jit[2]), 1.0f);
    }
    return pos;
}

// scenes.ramp_mesh() + scenes.box_mesh((0.6, 0.3, 0), (0.75, 0.6, 0.3)): the
// vertices from the same double expressions, rounded to float (the stored
// normal is not read by the kernel and is left zero).
std::vector<rtps::Triangle> ramp_and_box_mesh() {
    std::vector<rtps::Triangle> t;
    auto tri = [&](const double* a, const double* b, const double* c) {
        rtps::Triangle x;
        const double* v[3] = {a, b, c};
        for (int k = 0; k < 3; ++k) x.verts[k] = rtps::make_float4((float)v[k][0], (float)v[k][1], (float)v[k][2], 1.f);
        x.normal = rtps::make_float4(0, 0, 0, 0);
        t.push_back(x);
    };
    const int nx = 16, ny = 16;
    const double z0 = 0.12, z1 = 0.22;
    auto z = [&](double x) { return z0 + (z1 - z0) * x; };
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double x0 = i * (1.0 / nx), x1 = (i + 1) * (1.0 / nx), y0 = j * (1.0 / ny), y1 = (j + 1) * (1.0 / ny);
            const double a[3] = {x0, y0, z(x0)}, b[3] = {x1, y0, z(x1)}, c[3] = {x1, y1, z(x1)}, d[3] = {x0, y1, z(x0)};
            tri(a, b, c);
            tri(a, c, d);
        }
    const double lo[3] = {0.6, 0.3, 0.0}, hi[3] = {0.75, 0.6, 0.3};
    double cn[8][3];
    for (int k = 0; k < 8; ++k) {
        static const int sel[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
        for (int a = 0; a < 3; ++a) cn[k][a] = sel[k][a] ? hi[a] : lo[a];
    }
    static const int quads[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {2, 3, 7, 6}, {1, 2, 6, 5}, {3, 0, 4, 7}};
    for (const auto& q : quads) {
        tri(cn[q[0]], cn[q[1]], cn[q[2]]);
        tri(cn[q[0]], cn[q[2]], cn[q[3]]);
    }
    return t;
}

}  // namespace

int main(int argc, char** argv) {
    int n = 262144, steps = 200, warmup = 10, frames = 0, exact = 0, mesh = 0, post_res = 0;
    float dt = 0.001f, mu = 0.01f;
    std::string dump, box_file;
    int box_num = -1, rect_only = 0;
    std::string settings_file, out_init, out_final;
    float box_spacing = 0.f, box_scale = 1.f;
    rtps::float4 box_lo = rtps::make_float4(0, 0, 0, 0), box_hi = box_lo;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() -> const char* {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "missing value for %s\n", a.c_str());
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--n") n = std::atoi(next());
        else if (a == "--steps") steps = std::atoi(next());
        else if (a == "--warmup") warmup = std::atoi(next());
        else if (a == "--dt") dt = (float)std::atof(next());
        else if (a == "--viscosity") mu = (float)std::atof(next());
        else if (a == "--frames") frames = 1;
        else if (a == "--exact") exact = 1;
        else if (a == "--dump-scene") dump = next();
        else if (a == "--mesh") mesh = 1;
        else if (a == "--post-process") post_res = std::atoi(next());
        else if (a == "--settings") settings_file = next();
        else if (a == "--out-init") out_init = next();
        else if (a == "--out") out_final = next();
        else if (a == "--box") {
            box_num = std::atoi(next());
            float v[6];
            for (float& x : v) x = (float)std::atof(next());
            box_lo = rtps::make_float4(v[0], v[1], v[2], 0.f);
            box_hi = rtps::make_float4(v[3], v[4], v[5], 0.f);
        }
        else if (a == "--add-rect" || a == "--add-box") {
            rect_only = a == "--add-rect";
            box_num = std::atoi(next());
            if (rect_only) box_spacing = (float)std::atof(next());
            box_scale = (float)std::atof(next());
            float v[6];
            for (float& x : v) x = (float)std::atof(next());
            box_lo = rtps::make_float4(v[0], v[1], v[2], 0.f);
            box_hi = rtps::make_float4(v[3], v[4], v[5], 0.f);
            box_file = next();
        }
        else {
            std::fprintf(stderr, "unknown argument %s\n", a.c_str());
            return 2;
        }
    }
    if (n <= 0 || steps < 0 || warmup < 0) return 2;
    if (!dump.empty()) {
        const std::vector<rtps::float4> pos = dambreak_positions(n, 20250101ull);
        FILE* f = std::fopen(dump.c_str(), "wb");
        if (!f || std::fwrite(pos.data(), sizeof(rtps::float4), pos.size(), f) != pos.size()) return 1;
        return std::fclose(f) == 0 ? 0 : 1;
    }
    auto write_f4 = [](const std::string& path, const std::vector<rtps::float4>& v) {
        FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) return false;
        const bool ok = v.empty() || std::fwrite(v.data(), sizeof(rtps::float4), v.size(), f) == v.size();
        return std::fclose(f) == 0 && ok;
    };
    if (rect_only) return write_f4(box_file, rtps::addRect(box_num, box_lo, box_hi, box_spacing, box_scale)) ? 0 : 1;
    if (!settings_file.empty()) {
        // the reference's test applications: settings from a file, the
        // system RTPS::generateSystemInstance makes of them, one box of
        // particles, then the frame loop
        rtps::RTPSSettings settings;
        FILE* f = std::fopen(settings_file.c_str(), "r");
        if (!f) return 1;
        char line[1024];
        while (std::fgets(line, sizeof(line), f)) {
            std::string l(line);
            while (!l.empty() && (l.back() == '\n' || l.back() == '\r')) l.pop_back();
            const size_t sp0 = l.find(' ');
            if (l.empty() || sp0 == std::string::npos) continue;
            settings.SetSetting(l.substr(0, sp0), l.substr(sp0 + 1));
        }
        std::fclose(f);
        try {
            rtps::SPH sph(&settings);
            const int added = sph.addBox(box_num, box_lo, box_hi, false);
            if (!out_init.empty() && !write_f4(out_init, sph.getPositions())) return 1;
            for (int s = 0; s < steps; ++s) {
                sph.update();
                sph.integrate();
            }
            const std::vector<rtps::float4> p = sph.getPositions();
            if (!out_final.empty() && !write_f4(out_final, p)) return 1;
            double sum = 0.0;
            for (const rtps::float4& q : p) sum += (double)q.x + 2.0 * q.y + 3.0 * q.z;
            const SPHParams prm = sph.params();
            std::printf("{\"added\": %d, \"num\": %d, \"spacing\": %.9g, \"mass\": %.9g, \"rest_distance\": %.9g, "
                        "\"smoothing_distance\": %.9g, \"simulation_scale\": %.9g, \"max_num\": %d, "
                        "\"checksum\": %.17g}\n",
                        added, sph.getNum(), (double)sph.getSpacing(), (double)prm.mass, (double)prm.rest_distance,
                        (double)prm.smoothing_distance, (double)prm.simulation_scale, prm.max_num, sum);
        } catch (const rtps::SPHError& e) {
            std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
            return 1;
        }
        return 0;
    }
    SPHParams sp;
    GridParams g, gs;
    if (sph_dambreak_params(n, lattice_spacing(n), mu, &sp, &g, &gs) != SPH_OK) {
        std::fprintf(stderr, "sph_dambreak_params failed\n");
        return 1;
    }
    if (!box_file.empty()) {
        try {
            sp.simulation_scale = box_scale;
            rtps::SPH sph(sp, g, n, nullptr, dt);
            const int added = sph.addBox(box_num, box_lo, box_hi, false);
            if (!write_f4(box_file, sph.getPositions())) return 1;
            std::printf("{\"added\": %d, \"num\": %d, \"spacing\": %.9g}\n", added, sph.getNum(),
                        (double)sph.getSpacing());
        } catch (const rtps::SPHError& e) {
            std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
            return 1;
        }
        return 0;
    }
    try {
        rtps::SPH sph(sp, g, n, &gs, dt);
        if (exact) sph_set_exact(sph.handle(), 1);
        if (mesh) {
            std::vector<rtps::Triangle> tris = ramp_and_box_mesh();
            sph.loadTriangles(tris);
        }
        if (post_res > 0) sph.useColorField(true, post_res);
        sph.pushParticles(dambreak_positions(n, 20250101ull), rtps::make_float4(0, 0, 0, 0));
        auto frame = [&](int k) {
            if (frames) {
                for (int s = 0; s < k; ++s) {
                    sph.acquireGLBuffers();
                    sph.update();
                    sph.interact();
                    sph.integrate();
                    sph.postProcess();
                    sph.releaseGLBuffers();
                }
            } else {
                sph.step(k);
            }
        };
        frame(warmup);
        sph.sync();
        const auto t0 = std::chrono::steady_clock::now();
        frame(steps);
        sph.sync();
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        int ntri = -1;
        if (post_res > 0) {
            if (!frames) sph.postProcess();
            ntri = sph.getMesh(nullptr, nullptr);
        }
        const std::vector<rtps::float4> p = sph.getPositions();
        double sum = 0.0;
        for (const rtps::float4& q : p) sum += (double)q.x + 2.0 * q.y + 3.0 * q.z;
        std::printf("{\"metric\": \"particle-updates/s\", \"value\": %.6g, \"n\": %d, \"steps\": %d, \"warmup\": %d, "
                    "\"seconds\": %.6g, \"mode\": \"%s\", \"exact\": %d, \"num_after\": %d, "
                    "\"checksum\": %.17g, \"mesh\": %d, \"triangles\": %d, \"build\": \"%s\"}\n",
                    steps > 0 && el > 0 ? (double)n * steps / el : 0.0, n, steps, warmup, el,
                    frames ? "frames" : "fused", exact, sph.getNum(), sum, mesh, ntri, sph_build_info());
    } catch (const rtps::SPHError& e) {
        std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
        return 1;
    }
    return 0;
}
