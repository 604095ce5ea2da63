"""Drive the reference's own kernels (oracle/_ref/librtps_ref.so) through one
SPH step in the order of SPH::updateGPU + collision + SPH::integrate.

Test infrastructure.  The device work is the reference's kernel code; the
host logic between the launches follows rtpslib/system/SPH.cpp:149-300,
303-336, 389-441 and System.cpp:145-170, 407-455:

  hash -> bitonic sort (nlpo2 padding, INT_MAX pad keys) -> copy out->in ->
  cellindices (start reset to 0xffffffff, nc = start[C]) -> permute ->
  [0 <= nc <= num: keep the first nc sorted particles, copy sorted ->
   unsorted, hash + sort again] -> density -> force -> (gravity: no sources)
  -> collision_wall -> (collision_triangle, with a mesh loaded) -> leapfrog.

The bitonic sort is not stable.  With canonical=True the sort output is
re-ordered within equal keys by original index, the stable order that the
parity tests are defined in; with canonical=False the raw bitonic
order is kept (results then differ from the stable order only by summation
order within cells).
"""
import ctypes as C

import numpy as np

import oracle_bind as ob

P = ob.ptr


class RefSystem:
    def __init__(self, sphp, grid, grid_scaled, max_num, canonical=True):
        self.lib = ob.ref()
        self.sp = sphp
        self.g = grid
        self.gs = grid_scaled
        self.max_num = max_num
        self.canonical = canonical
        n4 = (max_num, 4)
        self.pos_u = np.zeros(n4, np.float32)
        self.vel_u = np.zeros(n4, np.float32)
        self.veleval_u = np.zeros(n4, np.float32)
        self.pos_s = np.zeros(n4, np.float32)
        self.vel_s = np.zeros(n4, np.float32)
        self.veleval_s = np.zeros(n4, np.float32)
        self.force_s = np.zeros(n4, np.float32)
        self.xsph_s = np.zeros(n4, np.float32)
        self.density_s = np.zeros(max_num, np.float32)
        self.keys = np.full(max_num, 0x7FFFFFFF, np.uint32)
        self.idx = np.full(max_num, 0x7FFFFFFF, np.uint32)
        self.start = np.full(grid.nb_cells + 1, 666, np.uint32)
        self.end = np.full(grid.nb_cells + 1, 666, np.uint32)
        self.num = 0
        self.deleted_pos = np.zeros((0, 4), np.float32)
        self.deleted_vel = np.zeros((0, 4), np.float32)
        self.trace = {}
        # point sources (System.cpp:260-272) and integrator (SPH.cpp:392-436)
        self.grav = None
        self.integrator = "leapfrog"
        # triangle mesh of CollisionTriangle (sph/Collision_triangle.cpp:44-116)
        self.tris = None

    def set_gravity(self, points, masses, alphas):
        self.grav = (np.ascontiguousarray(points, np.float32).reshape(-1, 4),
                     np.ascontiguousarray(masses, np.float32), np.ascontiguousarray(alphas, np.float32))

    def set_triangles(self, tris, dt):
        """(m, 4, 4) float32 triangles; dt is the time_step argument of the
        kernel (passed, not read)."""
        self.tris = (np.ascontiguousarray(tris, np.float32).reshape(-1, 16), float(dt))

    def upload(self, pos, vel):
        n = pos.shape[0]
        self.pos_u[:n] = pos
        self.vel_u[:n] = vel
        self.num = n

    def _params(self):
        self.sp.num = self.num
        return C.addressof(self.sp)

    def hash_and_sort(self):
        n = self.num
        L = self.lib
        L.ref_hash(n, P(self.pos_u), C.addressof(self.g), P(self.keys), P(self.idx))
        self.trace["hash_keys"] = self.keys[:n].copy()
        k = self.keys[:n].copy()
        v = self.idx[:n].copy()
        L.ref_bitonic_sort(n, P(k), P(v))
        if self.canonical:
            order = np.lexsort((v, k))
            k, v = k[order], v[order]
        self.keys[:n] = k
        self.idx[:n] = v

    def update(self, collision=True):
        L = self.lib
        self.hash_and_sort()
        n = self.num
        nc = L.ref_cellindices(n, P(self.keys), P(self.idx), P(self.start), P(self.end), C.addressof(self.g))
        self.trace["nc"] = nc
        L.ref_permute(n, P(self.idx), P(self.pos_u), P(self.vel_u), P(self.veleval_u), P(self.pos_s), P(self.vel_s),
                      P(self.veleval_s))
        if 0 <= nc <= n:
            self.deleted_pos = self.pos_s[nc:n].copy()
            self.deleted_vel = self.vel_s[nc:n].copy()
            self.num = nc
            self.pos_u[:nc] = self.pos_s[:nc]
            self.vel_u[:nc] = self.vel_s[:nc]
            self.veleval_u[:nc] = self.veleval_s[:nc]
            self.hash_and_sort()
        n = self.num
        sp = self._params()
        L.ref_density(n, P(self.pos_s), P(self.density_s), P(self.start), P(self.end), C.addressof(self.gs), sp)
        L.ref_force(n, P(self.pos_s), P(self.density_s), P(self.veleval_s), P(self.force_s), P(self.xsph_s),
                    P(self.start), P(self.end), C.addressof(self.gs), sp)
        self.trace["force_sph"] = self.force_s[:n].copy()
        if self.grav is not None:
            # gravity.execute after force (SPH.cpp:289-296)
            pts, m, a = self.grav
            L.ref_gravity(n, len(m), P(pts), P(m), P(a), P(self.pos_s), P(self.force_s),
                          float(self.sp.simulation_scale))
        self.trace["force_pre_collision"] = self.force_s[:n].copy()
        if collision:
            L.ref_collision_wall(n, P(self.pos_s), P(self.vel_s), P(self.force_s), C.addressof(self.gs), sp)
            if self.tris is not None:
                # SPH::collision: collision_tri after collision_wall (SPH.cpp:303-336)
                self.trace["force_pre_triangles"] = self.force_s[:n].copy()
                t, dt = self.tris
                L.ref_collision_triangles(n, P(self.pos_s), P(self.vel_s), P(self.force_s), P(t), t.shape[0], sp, dt)

    def integrate(self, dt):
        n = self.num
        if self.integrator == "euler":
            self.lib.ref_euler(n, P(self.pos_u), P(self.pos_s), P(self.vel_u), P(self.vel_s), P(self.force_s),
                               P(self.idx), self._params(), float(dt))
            return
        self.lib.ref_leapfrog(n, P(self.pos_u), P(self.pos_s), P(self.vel_u), P(self.vel_s), P(self.veleval_u),
                              P(self.force_s), P(self.xsph_s), P(self.idx), self._params(), float(dt))

    def step(self, dt, nsteps=1):
        for _ in range(nsteps):
            self.update()
            self.integrate(dt)


def params_from_settings(items):
    """The reference's settings path (ref_params_from_settings) for (key,
    value) string pairs: SPHParams bytes (the reference struct's size), both
    GridParams bytes, the spacing and the struct size."""
    lib = ob.ref()
    keys = (C.c_char_p * max(len(items), 1))(*[k.encode() for k, _ in items])
    vals = (C.c_char_p * max(len(items), 1))(*[v.encode() for _, v in items])
    sp = (C.c_uint8 * 256)()
    g = (C.c_uint8 * 128)()
    gs = (C.c_uint8 * 128)()
    spacing = C.c_float()
    size = lib.ref_params_from_settings(len(items), keys, vals, sp, g, gs, C.byref(spacing))
    return bytes(sp)[:size], bytes(g), bytes(gs), spacing.value, size
