// sph_rollout64.cpp — TEST INFRASTRUCTURE, not part of the product.
//
// A whole rollout of the SPH step with every quantity, the particle state
// included, held in double.  It is the reference for the gradients of the
// differentiable rollout, two ways:
//   * oracle_rollout64: the plain FP64 rollout, for central finite
//     differences of a loss (a rollout whose state is rounded to float after
//     every stage is not smooth at the 1e-12 level such differences live at);
//   * oracle_rollout64_jvp: the same rollout on dual numbers, which carries
//     the exact derivative of the FP64 trajectory along one input direction
//     (forward mode), with no step size.
//
// Per step, in the order of SPH::updateGPU / SPH::integrate
// (rtpslib/system/SPH.cpp:149-300, :389-441, collision after gravity):
//   bin      particles by cell of the scaled grid, stable by original index
//            (hash.cl:50-157, cellindices.cl:12-107 with the sort stable)
//   density  rho_i = wpoly6*m * sum_{|r|<=h} (h^2-|r|^2)^3, self included
//            (density.cl:44-126, cl_sph_kernels.h:29-45)
//   force    spiky pressure gradient, viscosity Laplacian, XSPH on veleval
//            (force.cl:43-186, cl_sph_kernels.h:81-127)
//   walls    repulsion and "friction" of the six walls (collision_wall.cl:
//            31-118, cl_sph_collision.h:31-73), bound rest_distance*0.5
//   leapfrog gravity, acceleration clamp, XSPH, veleval (leapfrog.cl:30-121)
// The neighbour set is the same as the kernels' (|r| <= h); the walk order
// and the binning differ from the FP32 path, which changes nothing but
// rounding.
//
// Branch signature: the wall tests (diff > EPSILON), the friction test and
// the acceleration clamp are the step's discontinuities (the first two are
// jumps of the force).  Each rollout returns an order-independent 64-bit
// signature of every (step, particle, branch bits) with a branch taken, and a
// second one of every (step, particle, neighbour count).  Two rollouts whose
// signatures agree took the same branches everywhere.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "sph_oracle.hpp"

namespace {

// Forward-mode dual number: value and derivative along one direction.
struct Dual {
    double v = 0.0, d = 0.0;
    Dual() = default;
    Dual(double x) : v(x), d(0.0) {}
    Dual(double x, double dx) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(Dual a, Dual b) { return Dual(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)); }
inline Dual& operator+=(Dual& a, Dual b) { return a = a + b; }
inline Dual sqrt_(Dual a) {
    const double s = std::sqrt(a.v);
    return Dual(s, s > 0.0 ? a.d / (2.0 * s) : 0.0);
}
inline double sqrt_(double a) { return std::sqrt(a); }
inline double val(double a) { return a; }
inline double val(Dual a) { return a.v; }

template <class T>
struct Vec {
    T x, y, z;
};
template <class T> inline Vec<T> vec(T x, T y, T z) { return Vec<T>{x, y, z}; }
template <class T> inline Vec<T> operator+(Vec<T> a, Vec<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline Vec<T> operator-(Vec<T> a, Vec<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline Vec<T> operator*(T s, Vec<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline T dot3(Vec<T> a, Vec<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

template <class T>
struct Rollout {
    typedef Vec<T> V;
    // parameters (the viscosity may carry a derivative)
    double sc, h, h2, mass, rho0, K, eps, wpoly6, wspiky_d, wvisc_dd, xsph_factor, vlimit, kwall, cwall, bound;
    T visc;
    V gravity;
    double gmin[3], gdelta[3];
    int res[3];
    double bnd_min[3], bnd_max[3];
    int n = 0;
    std::vector<V> pos, vel, veleval;  // original order; pos unscaled
    std::vector<uint32_t> order, cell_of, start, end;
    std::vector<V> ps, vs, es;  // sorted: scaled position, velocity, veleval
    std::vector<T> rho;
    std::vector<V> force, xsph;
    std::vector<uint32_t> nbr;
    std::vector<uint16_t> branches;
    uint64_t sig_branch = 0, sig_nbr = 0;

    // Stable binning by cell of the scaled grid; false if a particle is
    // outside the grid (the reference would delete it).
    bool bin() {
        const int C = res[0] * res[1] * res[2];
        cell_of.assign(n, 0);
        bool ok = true;
        for (int i = 0; i < n; ++i) {
            int c[3];
            const double p[3] = {val(pos[i].x) * sc, val(pos[i].y) * sc, val(pos[i].z) * sc};
            for (int a = 0; a < 3; ++a) {
                const double g = std::floor((p[a] - gmin[a]) * gdelta[a]);
                if (!(g >= 0.0 && g < (double)res[a])) ok = false;
                c[a] = ok ? (int)g : 0;
            }
            cell_of[i] = (uint32_t)((c[2] * res[1] + c[1]) * res[0] + c[0]);
        }
        if (!ok) return false;
        start.assign((size_t)C + 1, 0);
        for (int i = 0; i < n; ++i) start[cell_of[i] + 1]++;
        for (int k = 0; k < C; ++k) start[k + 1] += start[k];
        end.assign(start.begin() + 1, start.end());
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        order.assign(n, 0);
        for (int i = 0; i < n; ++i) order[fill[cell_of[i]]++] = (uint32_t)i;
        return true;
    }

    template <class F>
    void for_each_neighbour(int i, F&& f) const {
        const V pi = ps[i];
        const int cx = (int)std::floor((val(pi.x) - gmin[0]) * gdelta[0]);
        const int cy = (int)std::floor((val(pi.y) - gmin[1]) * gdelta[1]);
        const int cz = (int)std::floor((val(pi.z) - gmin[2]) * gdelta[2]);
        for (int z = cz - 1; z <= cz + 1; ++z) {
            if (z < 0 || z >= res[2]) continue;
            for (int y = cy - 1; y <= cy + 1; ++y) {
                if (y < 0 || y >= res[1]) continue;
                for (int x = cx - 1; x <= cx + 1; ++x) {
                    if (x < 0 || x >= res[0]) continue;
                    const int c = (z * res[1] + y) * res[0] + x;
                    for (uint32_t j = start[c]; j < end[c]; ++j) {
                        const V r = pi - ps[j];
                        const T r2 = dot3(r, r);
                        if (val(r2) <= h2) f((int)j, r, r2);
                    }
                }
            }
        }
    }

    bool step(double dt, int t) {
        if (!bin()) return false;
        ps.resize(n);
        vs.resize(n);
        es.resize(n);
        rho.resize(n);
        force.resize(n);
        xsph.resize(n);
        nbr.resize(n);
        branches.resize(n);
        const T tsc = sc;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            const uint32_t o = order[i];
            ps[i] = tsc * pos[o];
            vs[i] = vel[o];
            es[i] = veleval[o];
        }
        // density (self included)
        const T th2 = h2, dens_coef = wpoly6 * mass;
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            T acc = 0.0;
            uint32_t cnt = 0;
            for_each_neighbour(i, [&](int, const V&, T r2) {
                const T q = th2 - r2;
                acc += q * q * q;
                ++cnt;
            });
            rho[i] = dens_coef * acc;
            nbr[i] = cnt;
        }
        // force
        const T coef_b = -0.5 * wspiky_d, coef_s = visc * T(wvisc_dd), coef_d = 2.0 * mass * wpoly6;
        const T th = h, tK = K, trho0 = rho0, tmass = mass;
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            const T di = rho[i], Pi = tK * (di - trho0);
            V F = vec<T>(0.0, 0.0, 0.0), Vs = F, X = F;
            for_each_neighbour(i, [&](int j, const V& r, T r2) {
                if (j == i) return;
                T rlen = sqrt_(r2);
                if (val(rlen) < eps) rlen = T(eps);
                const T hr = th - rlen;
                const T dj = rho[j], idj = T(1.0) / dj, Pj = tK * (dj - trho0);
                F = F + (hr * hr / rlen * (Pi + Pj) * idj) * r;
                const V dv = es[j] - es[i];
                Vs = Vs + (hr * idj) * dv;
                const T q = th2 - r2;
                X = X + (q * q * q / (di + dj)) * dv;
            });
            force[i] = (tmass / di) * (coef_b * F + coef_s * Vs);
            xsph[i] = coef_d * X;
        }
        // walls + leapfrog
        const T tdt = dt, tk = kwall, tc = cwall, tb = bound, txf = xsph_factor, half = 0.5;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            const V p = ps[i], v = vs[i];
            V f = force[i];
            V rf = vec<T>(0.0, 0.0, 0.0), ff = rf;
            unsigned bits = 0;
            const T diffs[6] = {tb - (p.z - T(bnd_min[2])), tb - (T(bnd_max[2]) - p.z),
                                tb - (p.y - T(bnd_min[1])), tb - (T(bnd_max[1]) - p.y),
                                tb - (p.x - T(bnd_min[0])), tb - (T(bnd_max[0]) - p.x)};
            const V normals[6] = {vec<T>(0.0, 0.0, 1.0), vec<T>(0.0, 0.0, -1.0), vec<T>(0.0, 1.0, 0.0),
                                  vec<T>(0.0, -1.0, 0.0), vec<T>(1.0, 0.0, 0.0), vec<T>(-1.0, 0.0, 0.0)};
            for (int w = 0; w < 6; ++w) {
                if (!(val(diffs[w]) > eps)) continue;
                const V nrm = normals[w];
                const T vn = dot3(nrm, v);
                rf = rf + (tk * diffs[w] - tc * vn) * nrm;
                const V vt = v - vn * v;
                bits |= 1u << w;
                if (val(vt.x + vt.y + vt.z) / 3.0 > 0.0) {
                    ff = ff - vt;
                    bits |= 1u << (6 + w);
                }
            }
            f = f + (rf + ff);
            V g = f + gravity;
            const T speed = sqrt_(dot3(g, g));
            if (val(speed) > vlimit) {
                g = (T(vlimit) / speed) * g;
                bits |= 1u << 12;
            }
            const V vn = v + tdt * g + txf * xsph[i];
            const uint32_t o = order[i];
            const V pn = p + tdt * vn;
            vel[o] = vn;
            veleval[o] = half * (v + vn);
            pos[o] = V{pn.x / tsc, pn.y / tsc, pn.z / tsc};
            branches[i] = (uint16_t)bits;
        }
        uint64_t sb = 0, sn = 0;
        for (int i = 0; i < n; ++i) {
            const uint64_t key = ((uint64_t)t << 40) ^ ((uint64_t)order[i] << 14);
            if (branches[i]) sb ^= mix64(key | branches[i]);
            sn ^= mix64(key ^ ((uint64_t)nbr[i] << 1) ^ 0x5bd1e995ull);
        }
        sig_branch ^= mix64(sb + (uint64_t)t);
        sig_nbr ^= mix64(sn + (uint64_t)t);
        return true;
    }

    bool setup(const SPHParams* sp, const GridParams* gps, T viscosity) {
        sc = sp->simulation_scale;
        h = sp->smoothing_distance;
        h2 = h * h;
        mass = sp->mass;
        rho0 = sp->rest_density;
        K = sp->K;
        eps = sp->EPSILON;
        visc = viscosity;
        wpoly6 = sp->wpoly6_coef;
        wspiky_d = sp->wspiky_d_coef;
        wvisc_dd = sp->wvisc_dd_coef;
        xsph_factor = sp->xsph_factor;
        vlimit = sp->velocity_limit;
        kwall = sp->boundary_stiffness;
        cwall = sp->boundary_dampening;
        bound = (double)sp->rest_distance * 0.5;
        gravity = vec<T>(sp->gravity.x, sp->gravity.y, sp->gravity.z);
        const float* gmin_f = &gps->grid_min.x;
        const float* gdel_f = &gps->grid_delta.x;
        const float* gres_f = &gps->grid_res.x;
        const float* bmin_f = &gps->bnd_min.x;
        const float* bmax_f = &gps->bnd_max.x;
        for (int a = 0; a < 3; ++a) {
            gmin[a] = gmin_f[a];
            gdelta[a] = gdel_f[a];
            res[a] = (int)gres_f[a];
            bnd_min[a] = bmin_f[a];
            bnd_max[a] = bmax_f[a];
            if (res[a] <= 0) return false;
        }
        return true;
    }
};

inline Dual dual(const double* v, const double* dv, size_t k) { return Dual(v[k], dv ? dv[k] : 0.0); }

}  // namespace

extern "C" {

// One FP64 rollout of nsteps steps from (pos, vel, veleval) (n x 3 doubles,
// original order; veleval may be null = 0) with the given viscosity.  Writes
// the final positions (and velocities when vel_out is given) and the branch
// and neighbour signatures.  Returns 0, or -1 when a particle left the grid
// (the reference would have deleted it) or an argument is invalid.
int oracle_rollout64(const SPHParams* sp, const GridParams* gps, double viscosity, double dt, int nsteps, int n,
                     const double* pos, const double* vel, const double* veleval, double* pos_out, double* vel_out,
                     uint64_t* sig_branch, uint64_t* sig_nbr) {
    if (!sp || !gps || !pos || !vel || !pos_out || n <= 0 || nsteps < 0) return -1;
    Rollout<double> R;
    if (!R.setup(sp, gps, viscosity)) return -1;
    R.n = n;
    R.pos.resize(n);
    R.vel.resize(n);
    R.veleval.resize(n);
    for (int i = 0; i < n; ++i) {
        R.pos[i] = vec(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        R.vel[i] = vec(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        R.veleval[i] = veleval ? vec(veleval[3 * i], veleval[3 * i + 1], veleval[3 * i + 2]) : vec(0.0, 0.0, 0.0);
    }
    for (int t = 0; t < nsteps; ++t)
        if (!R.step(dt, t)) return -1;
    for (int i = 0; i < n; ++i) {
        pos_out[3 * i] = R.pos[i].x;
        pos_out[3 * i + 1] = R.pos[i].y;
        pos_out[3 * i + 2] = R.pos[i].z;
        if (vel_out) {
            vel_out[3 * i] = R.vel[i].x;
            vel_out[3 * i + 1] = R.vel[i].y;
            vel_out[3 * i + 2] = R.vel[i].z;
        }
    }
    if (sig_branch) *sig_branch = R.sig_branch;
    if (sig_nbr) *sig_nbr = R.sig_nbr;
    return 0;
}

// The same rollout carrying the derivative along the input direction
// (dpos, dvel, dveleval, dviscosity) (each array nullable = 0): writes the
// final positions and their directional derivative dpos_out (n x 3).
int oracle_rollout64_jvp(const SPHParams* sp, const GridParams* gps, double viscosity, double dviscosity, double dt,
                         int nsteps, int n, const double* pos, const double* vel, const double* veleval,
                         const double* dpos, const double* dvel, const double* dveleval, double* pos_out,
                         double* dpos_out) {
    if (!sp || !gps || !pos || !vel || !pos_out || !dpos_out || n <= 0 || nsteps < 0) return -1;
    Rollout<Dual> R;
    if (!R.setup(sp, gps, Dual(viscosity, dviscosity))) return -1;
    R.n = n;
    R.pos.resize(n);
    R.vel.resize(n);
    R.veleval.resize(n);
    static const double zero3[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < n; ++i) {
        const size_t k = 3 * (size_t)i;
        R.pos[i] = vec(dual(pos, dpos, k), dual(pos, dpos, k + 1), dual(pos, dpos, k + 2));
        R.vel[i] = vec(dual(vel, dvel, k), dual(vel, dvel, k + 1), dual(vel, dvel, k + 2));
        const double* ve = veleval ? veleval + k : zero3;
        const double* dve = dveleval ? dveleval + k : zero3;
        R.veleval[i] = vec(Dual(ve[0], dve[0]), Dual(ve[1], dve[1]), Dual(ve[2], dve[2]));
    }
    for (int t = 0; t < nsteps; ++t)
        if (!R.step(dt, t)) return -1;
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            const Dual& c = a == 0 ? R.pos[i].x : (a == 1 ? R.pos[i].y : R.pos[i].z);
            pos_out[3 * i + a] = c.v;
            dpos_out[3 * i + a] = c.d;
        }
    return 0;
}

}  // extern "C"
