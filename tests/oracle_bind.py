"""ctypes bindings of the CPU oracle (oracle/_build/libsph_oracle.so) and of the
reference's own kernels compiled for the host (oracle/_ref/librtps_ref.so).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libsph_oracle.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "librtps_ref.so")

_P = C.c_void_p
_I = C.c_int
_F = C.c_float


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return ORACLE_LIB


_oracle = None
_ref = None


def oracle():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB):
            build_oracle()
        lib = C.CDLL(ORACLE_LIB)
        sig = {
            "oracle_info": (C.c_char_p, []),
            "oracle_threads": (_I, []),
            "oracle_set_threads": (None, [_I]),
            "oracle_hash": (None, [_I, _P, _P, _P, _P]),
            "oracle_sort": (None, [_I, _P, _P]),
            "oracle_sort_std": (None, [_I, _P, _P]),
            "oracle_cellindices": (_I, [_I, _P, _P, _P, _I]),
            "oracle_permute": (None, [_I, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_density": (None, [_I, _I, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_force": (None, [_I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_collision": (None, [_I, _I, _P, _P, _P, _P, _P]),
            "oracle_leapfrog": (None, [_I, _I, _P, _P, _P, _P, _P, _P, _F, _P, _P, _P]),
            "oracle_sim_create": (_P, [_P, _P, _P, _I, _I]),
            "oracle_sim_destroy": (None, [_P]),
            "oracle_sim_set_params": (None, [_P, _P]),
            "oracle_sim_upload": (_I, [_P, _P, _P, _P, _I]),
            "oracle_sim_update": (None, [_P]),
            "oracle_sim_integrate": (None, [_P, _F]),
            "oracle_sim_step": (None, [_P, _F, _I]),
            "oracle_sim_num": (_I, [_P]),
            "oracle_sim_last_nc": (_I, [_P]),
            "oracle_sim_get": (_I, [_P, _I, _P, _I]),
            "oracle_sim_deleted": (_I, [_P, _P, _P, _I]),
            "oracle_gravity": (None, [_I, _I, _I, _P, _P, _P, _P, _P, _F]),
            "oracle_euler": (None, [_I, _I, _P, _P, _P, _P, _P, _F, _P, _P]),
            "oracle_sim_set_gravity": (None, [_P, _I, _P, _P, _P]),
            "oracle_sim_set_integrator": (None, [_P, _I]),
            "oracle_collision_triangles": (None, [_I, _I, _P, _P, _P, _P, _I, _P]),
            "oracle_sim_set_triangles": (None, [_P, _P, _I]),
            "oracle_sim_push": (_I, [_P, _P, _P, _I]),
            "oracle_colorfield": (None, [_I, _I, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_rollout64": (_I, [_P, _P, C.c_double, C.c_double, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_rollout64_jvp": (_I, [_P, _P, C.c_double, C.c_double, C.c_double, _I, _I, _P, _P, _P, _P, _P,
                                          _P, _P, _P]),
            "oracle_dambreak_params": (_I, [_I, _F, _F, _P, _P, _P]),
            "oracle_settings_round": (_F, [_F]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _oracle = lib
    return _oracle


def dambreak_params(n, viscosity=0.01, spacing=None):
    """(SPHParams, GridParams, GridParams scaled) of the dam-break scenes,
    derived by the oracle (oracle/sph_params_oracle.cpp) without loading the
    product library: the structs are the ctypes views of include/rtps_sph.h."""
    from enjaparticles_gb300 import abi, scenes
    sp, g, gs = abi.SPHParams(), abi.GridParams(), abi.GridParams()
    s = scenes.lattice_spacing(n) if spacing is None else spacing
    rc = oracle().oracle_dambreak_params(int(n), float(s), float(viscosity), C.addressof(sp), C.addressof(g),
                                         C.addressof(gs))
    if rc != 0:
        raise ValueError("oracle_dambreak_params: invalid arguments")
    return sp, g, gs


def settings_round(value):
    """A float through the reference's settings map (6 significant digits)."""
    import numpy as np
    return float(oracle().oracle_settings_round(float(np.float32(value))))


def ref_add_rect(num, lo, hi, spacing, scale=1.0):
    """The reference's addRect (rtpslib/domain/IV.cpp:165-202) from oracle/_ref:
    (k, 4) float32 lattice points."""
    lo4 = np.asarray(list(lo) + [0.0] * (4 - len(lo)), np.float32)
    hi4 = np.asarray(list(hi) + [0.0] * (4 - len(hi)), np.float32)
    out = np.zeros((num, 4), np.float32)
    k = ref().ref_add_rect(int(num), ptr(lo4), ptr(hi4), float(spacing), float(scale), ptr(out))
    return out[:k]


def ref_available():
    return os.path.exists(REF_LIB)


def ref():
    """The reference's kernels (built only where the reference tree exists)."""
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_LIB)
        sig = {
            "ref_hash": (None, [_I, _P, _P, _P, _P]),
            "ref_bitonic_sort": (None, [_I, _P, _P]),
            "ref_cellindices": (_I, [_I, _P, _P, _P, _P, _P]),
            "ref_permute": (None, [_I, _P, _P, _P, _P, _P, _P, _P]),
            "ref_density": (None, [_I, _P, _P, _P, _P, _P, _P]),
            "ref_force": (None, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
            "ref_collision_wall": (None, [_I, _P, _P, _P, _P, _P]),
            "ref_leapfrog": (None, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _F]),
            "ref_setup_domain": (None, [_P, _P, _F, _F, _P, _P]),
            "ref_gravity": (None, [_I, _I, _P, _P, _P, _P, _P, _F]),
            "ref_euler": (None, [_I, _P, _P, _P, _P, _P, _P, _P, _F]),
            "ref_collision_triangles": (None, [_I, _P, _P, _P, _P, _I, _P, _F]),
            "ref_hose_create": (_P, [_F, _I, _P, _P, _F, _F]),
            "ref_hose_spray": (_I, [_P, _P, _I, _P]),
            "ref_hose_update": (None, [_P, _P, _P, _F, _F]),
            "ref_hose_refill": (None, [_P, _I]),
            "ref_hose_destroy": (None, [_P]),
            "ref_srand": (None, [C.c_uint]),
            "ref_colorfield_slices": (_I, [_I]),
            "ref_colorfield": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
            "ref_marching_cubes": (_I, [_I, _P, _F, _P, _P, _I, _P]),
            "ref_add_rect": (_I, [_I, _P, _P, _F, _F, _P]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _ref = lib
    return _ref


def ptr(a):
    return None if a is None else a.ctypes.data


FIELD_IDS = {"pos_u": 0, "vel_u": 1, "veleval_u": 2, "pos_s": 3, "vel_s": 4, "veleval_s": 5, "density_s": 6,
             "force_s": 7, "xsph_s": 8, "sort_hashes": 9, "sort_indices": 10, "cell_start": 11, "cell_end": 12,
             "neighbor_count": 13}


class OracleSim:
    """The oracle's whole-system stepper (SPH::updateGPU + collision + integrate)."""

    def __init__(self, sphp, grid, grid_scaled, max_num, f64=False):
        self.lib = oracle()
        self.h = self.lib.oracle_sim_create(C.addressof(sphp), C.addressof(grid), C.addressof(grid_scaled),
                                            int(max_num), 1 if f64 else 0)
        self.nb_cells = grid.nb_cells

    def close(self):
        if self.h:
            self.lib.oracle_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_params(self, sphp):
        self.lib.oracle_sim_set_params(self.h, C.addressof(sphp))

    def set_gravity(self, points, masses, alphas):
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
        m = np.ascontiguousarray(masses, np.float32)
        a = np.ascontiguousarray(alphas, np.float32)
        self._grav = (pts, m, a)
        self.lib.oracle_sim_set_gravity(self.h, len(m), ptr(pts), ptr(m), ptr(a))

    def set_integrator(self, kind):
        """0: leapfrog, 1: euler."""
        self.lib.oracle_sim_set_integrator(self.h, int(kind))

    def push(self, pos, vel):
        """SPH::pushParticles; False when past max_num (dropped)."""
        p = np.ascontiguousarray(pos, np.float32)
        v = np.ascontiguousarray(vel, np.float32)
        return self.lib.oracle_sim_push(self.h, ptr(p), ptr(v), p.shape[0]) == 0

    def set_triangles(self, tris):
        """(m, 4, 4) or (m, 16) float32 triangles; collision_triangle runs after the walls."""
        t = np.ascontiguousarray(tris, np.float32).reshape(-1, 16)
        self._tris = t
        self.lib.oracle_sim_set_triangles(self.h, ptr(t), t.shape[0])

    def upload(self, pos, vel, veleval=None):
        pos = np.ascontiguousarray(pos, np.float32)
        vel = np.ascontiguousarray(vel, np.float32)
        ve = None if veleval is None else np.ascontiguousarray(veleval, np.float32)
        assert self.lib.oracle_sim_upload(self.h, ptr(pos), ptr(vel), ptr(ve), pos.shape[0]) == 0

    def update(self):
        self.lib.oracle_sim_update(self.h)

    def integrate(self, dt):
        self.lib.oracle_sim_integrate(self.h, dt)

    def step(self, dt, n=1):
        self.lib.oracle_sim_step(self.h, dt, n)

    @property
    def num(self):
        return self.lib.oracle_sim_num(self.h)

    def get(self, field, n=None):
        if n is None:
            n = self.nb_cells + 1 if field in ("cell_start", "cell_end") else self.num
        if field in ("density_s",):
            out = np.empty(n, np.float32)
        elif field in ("sort_hashes", "sort_indices", "cell_start", "cell_end", "neighbor_count"):
            out = np.empty(n, np.uint32)
        else:
            out = np.empty((n, 4), np.float32)
        assert self.lib.oracle_sim_get(self.h, FIELD_IDS[field], ptr(out), n) == 0
        return out


def rollout64(sphp, grid_scaled, pos, vel, dt, nsteps, viscosity=None, veleval=None, want_vel=False):
    """FP64 rollout (state in double) from (n,3) or (n,4) arrays.

    Returns (final positions (n,3) float64, final velocities or None,
    branch signature, neighbour signature).  Raises if a particle left the grid.
    """
    lib = oracle()
    p = np.ascontiguousarray(np.asarray(pos, np.float64)[:, :3])
    v = np.ascontiguousarray(np.asarray(vel, np.float64)[:, :3])
    e = None if veleval is None else np.ascontiguousarray(np.asarray(veleval, np.float64)[:, :3])
    n = p.shape[0]
    po = np.empty((n, 3), np.float64)
    vo = np.empty((n, 3), np.float64) if want_vel else None
    sb, sn = C.c_uint64(), C.c_uint64()
    mu = float(sphp.viscosity) if viscosity is None else float(viscosity)
    rc = lib.oracle_rollout64(C.addressof(sphp), C.addressof(grid_scaled), mu, float(dt), int(nsteps), n,
                              ptr(p), ptr(v), ptr(e), ptr(po), ptr(vo), C.addressof(sb), C.addressof(sn))
    if rc != 0:
        raise RuntimeError("oracle_rollout64 failed (a particle left the grid?)")
    return po, vo, sb.value, sn.value


def rollout64_jvp(sphp, grid_scaled, pos, vel, dt, nsteps, dpos=None, dvel=None, dveleval=None, dvisc=0.0,
                  viscosity=None, veleval=None):
    """FP64 rollout on dual numbers: (final positions, their derivative along
    the input direction (dpos, dvel, dveleval, dvisc)), both (n, 3) float64."""
    lib = oracle()
    c3 = lambda a: None if a is None else np.ascontiguousarray(np.asarray(a, np.float64)[:, :3])
    p, v, e = c3(pos), c3(vel), c3(veleval)
    dp, dv, de = c3(dpos), c3(dvel), c3(dveleval)
    n = p.shape[0]
    po = np.empty((n, 3), np.float64)
    dpo = np.empty((n, 3), np.float64)
    mu = float(sphp.viscosity) if viscosity is None else float(viscosity)
    rc = lib.oracle_rollout64_jvp(C.addressof(sphp), C.addressof(grid_scaled), mu, float(dvisc), float(dt),
                                  int(nsteps), n, ptr(p), ptr(v), ptr(e), ptr(dp), ptr(dv), ptr(de), ptr(po),
                                  ptr(dpo))
    if rc != 0:
        raise RuntimeError("oracle_rollout64_jvp failed (a particle left the grid?)")
    return po, dpo
