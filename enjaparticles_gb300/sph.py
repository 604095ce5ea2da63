"""Python mirror of the reference's rtps::SPH system over the C ABI.

Method names follow rtpslib/system/System.h:61-186 and SPH.h:56-155 (update,
integrate, pushParticles, addBox, getNum, ...), with the per-stage entry points
of SPH::updateGPU (SPH.cpp:149-300) exposed for tests.  All compute runs in
librtps_sph.so on the GPU; this class only moves host arrays.
"""
import ctypes as C

import numpy as np

from . import abi


class SPH:
    def __init__(self, sphp, grid, max_num, grid_scaled=None, exact=False, lib=None):
        """lib: a loaded library (abi.load_library(path)), e.g. the
        bounds-checked one; the default library when None."""
        self.lib = lib if lib is not None else abi.load_library()
        self.ctx = C.c_void_p()
        gs = C.byref(grid_scaled) if grid_scaled is not None else None
        abi.check(self.lib, None, self.lib.sph_create(C.byref(sphp), C.byref(grid), gs, int(max_num),
                                                      C.byref(self.ctx)))
        self.max_num = int(max_num)
        self.nb_cells = int(grid.nb_cells)
        if exact:
            self.set_exact(True)

    @classmethod
    def from_settings(cls, settings, exact=False, lib=None):
        """The system the reference builds from a settings map (SPH::SPH,
        SPH.cpp:50-98; System::System, System.cpp:54-62, 260-272): the
        parameter block and grid of SPH::calculate / updateParams /
        System::setupDomain, the "integrator" setting and the point sources
        of gravity_sources / gravity_mass / gravity_alphas.  Returns the
        system and its "time_step"."""
        sp, g, gs, spacing = abi.params_from_settings(settings, lib=lib)
        s = cls(sp, g, sp.max_num, gs, exact=exact, lib=lib)
        s.spacing = spacing
        if str(settings.get("integrator", "")) == "euler":
            s.setIntegrator("euler")
        if "gravity_sources" in settings:
            p = np.array(abi.settings_value(settings["gravity_sources"]).split(), np.float32)
            m = np.array(abi.settings_value(settings.get("gravity_mass", "")).split(), np.float32)
            a = np.array(abi.settings_value(settings.get("gravity_alphas", "")).split(), np.float32)
            ns = len(p) // 4
            if ns > 0:
                mass = np.zeros(ns, np.float32)
                alpha = np.zeros(ns, np.float32)
                mass[:min(ns, len(m))] = m[:ns]
                alpha[:min(ns, len(a))] = a[:ns]
                s.setGravitySources(p[:4 * ns].reshape(ns, 4), mass, alpha)
        dt = float(np.float32(abi.settings_value(settings.get("time_step", "0"))))
        return s, dt

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if self.ctx:
            self.lib.sph_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        return abi.check(self.lib, self.ctx, rc)

    # -- parameters -------------------------------------------------------
    def set_exact(self, on=True):
        self._ck(self.lib.sph_set_exact(self.ctx, 1 if on else 0))

    def updateParams(self, sphp):
        self._ck(self.lib.sph_set_params(self.ctx, C.byref(sphp)))

    def params(self):
        sp, g, gs = abi.SPHParams(), abi.GridParams(), abi.GridParams()
        self._ck(self.lib.sph_get_params(self.ctx, C.byref(sp), C.byref(g), C.byref(gs)))
        return sp, g, gs

    # -- launch shapes ----------------------------------------------------
    def launch_config(self):
        cfg = abi.sph_launch_config()
        self._ck(self.lib.sph_get_launch_config(self.ctx, C.byref(cfg)))
        return cfg.as_tuple()

    def set_launch_config(self, density_threads, force_threads, scan_tile_cells):
        cfg = abi.sph_launch_config(int(density_threads), int(force_threads), int(scan_tile_cells), 0)
        self._ck(self.lib.sph_set_launch_config(self.ctx, C.byref(cfg)))

    def autotune(self, dt=0.001, steps=3, retime=False):
        """Times the candidate launch shapes (state unchanged), keeps the fastest."""
        cfg = abi.sph_launch_config()
        self._ck(self.lib.sph_autotune(self.ctx, float(dt), int(steps), abi.SPH_TUNE_RETIME if retime else 0,
                                       C.byref(cfg)))
        return cfg.as_tuple()

    # -- particles --------------------------------------------------------
    @staticmethod
    def _f4(a, n=None):
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.ndim != 2 or a.shape[1] != 4:
            raise ValueError("expected an (n, 4) float32 array")
        if n is not None and a.shape[0] != n:
            raise ValueError("array length mismatch")
        return a

    def upload(self, pos, vel, veleval=None):
        pos = self._f4(pos)
        n = pos.shape[0]
        vel = self._f4(vel, n)
        ve = None if veleval is None else self._f4(veleval, n)
        self._keep = (pos, vel, ve)  # host memory must outlive the asynchronous copy
        self._ck(self.lib.sph_upload(self.ctx, pos.ctypes.data, vel.ctypes.data,
                                     None if ve is None else ve.ctypes.data, n))
        self.sync()

    def pushParticles(self, pos, vel):
        pos = self._f4(pos)
        vel = self._f4(vel, pos.shape[0])
        self._ck(self.lib.sph_push_particles(self.ctx, pos.ctypes.data, vel.ctypes.data, pos.shape[0]))

    def getNum(self):
        n = C.c_int()
        self._ck(self.lib.sph_get_num(self.ctx, C.byref(n)))
        return n.value

    def get(self, field, n=None):
        """Blocking copy of a field (see abi.FIELDS) to a new numpy array."""
        dt, w = abi.FIELD_DTYPE[field]
        if n is None:
            n = self.nb_cells + 1 if field in ("cell_start", "cell_end") else self.getNum()
        out = np.empty((n, w) if w > 1 else (n,), dtype=dt)
        self._ck(self.lib.sph_download(self.ctx, abi.FIELDS[field], out.ctypes.data, n))
        return out

    def device_ptr(self, field):
        p = C.c_void_p()
        self._ck(self.lib.sph_get_device_ptr(self.ctx, abi.FIELDS[field], C.byref(p)))
        return p.value

    def getDeleted(self):
        cnt = C.c_int()
        self._ck(self.lib.sph_get_deleted(self.ctx, None, None, 0, C.byref(cnt)))
        pos = np.empty((cnt.value, 4), np.float32)
        vel = np.empty((cnt.value, 4), np.float32)
        if cnt.value:
            self._ck(self.lib.sph_get_deleted(self.ctx, pos.ctypes.data, vel.ctypes.data, cnt.value, C.byref(cnt)))
        return pos, vel

    # -- stages (SPH::updateGPU order) -----------------------------------
    def hash(self):
        self._ck(self.lib.sph_stage_hash(self.ctx))

    def sort(self):
        self._ck(self.lib.sph_stage_sort(self.ctx))

    def cellindices(self):
        nc = C.c_int()
        self._ck(self.lib.sph_stage_cellindices(self.ctx, C.byref(nc)))
        return nc.value

    def permute(self):
        self._ck(self.lib.sph_stage_permute(self.ctx))

    def density(self):
        self._ck(self.lib.sph_stage_density(self.ctx))

    def force(self):
        self._ck(self.lib.sph_stage_force(self.ctx))

    def collision(self):
        self._ck(self.lib.sph_stage_collision(self.ctx))

    def leapfrog(self, dt):
        self._ck(self.lib.sph_stage_leapfrog(self.ctx, float(dt)))

    def gravity(self):
        """Gravity::execute: force_s += the point sources' pull."""
        self._ck(self.lib.sph_stage_gravity(self.ctx))

    def euler(self, dt):
        self._ck(self.lib.sph_stage_euler(self.ctx, float(dt)))

    def collision_triangles(self):
        """CollisionTriangle::execute: force_s += the loaded mesh's contacts."""
        self._ck(self.lib.sph_stage_collision_triangles(self.ctx))

    # -- triangle mesh (sph/Collision_triangle.cpp:44-82) ---------------------
    def loadTriangles(self, tris):
        """(m, 4, 4) or (m, 16) float32: three vertices and a normal per
        triangle (scenes.ramp_mesh and box_mesh make them); m = 0 unloads."""
        t = np.ascontiguousarray(tris, np.float32).reshape(-1, 16)
        self._ck(self.lib.sph_load_triangles(self.ctx, t.ctypes.data if t.shape[0] else None, t.shape[0]))

    # -- point sources and integrator (System.cpp:260-272, SPH.cpp:392-436) --
    def setGravitySources(self, points, masses, alphas):
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
        m = np.ascontiguousarray(masses, np.float32)
        a = np.ascontiguousarray(alphas, np.float32)
        self._ck(self.lib.sph_set_gravity_sources(self.ctx, len(m), pts.ctypes.data, m.ctypes.data, a.ctypes.data))

    def setIntegrator(self, name):
        """'leapfrog' or 'euler'."""
        kind = {"leapfrog": abi.SPH_INTEGRATOR_LEAPFROG, "euler": abi.SPH_INTEGRATOR_EULER}[name]
        self._ck(self.lib.sph_set_integrator(self.ctx, kind))

    # -- hoses (SPH.cpp:523-558) ---------------------------------------------
    def addHose(self, total_n, center, velocity, radius, dt):
        """SPH::addHose: radius in particle spacings; returns the hose index."""
        idx = C.c_int()
        self._ck(self.lib.sph_add_hose(self.ctx, int(total_n), abi.vec4(center), abi.vec4(velocity), float(radius),
                                       float(dt), C.byref(idx)))
        return idx.value

    def updateHose(self, index, center, velocity, radius):
        self._ck(self.lib.sph_update_hose(self.ctx, int(index), abi.vec4(center), abi.vec4(velocity), float(radius)))

    def refillHose(self, index, n):
        self._ck(self.lib.sph_refill_hose(self.ctx, int(index), int(n)))

    def sprayHoses(self):
        """SPH::sprayHoses; returns the particles added."""
        k = C.c_int()
        self._ck(self.lib.sph_spray_hoses(self.ctx, C.byref(k)))
        return k.value

    # -- post-process: colour field and surface (SPH.cpp:338-386) -------------
    def colorfield(self, res):
        """The res^3 colour field of the last update, as a numpy array [r, t, s]."""
        self._ck(self.lib.sph_colorfield(self.ctx, int(res)))
        res = max(int(res), 2)
        out = np.empty(res ** 3, np.float32)
        self._ck(self.lib.sph_download_surface(self.ctx, out.ctypes.data, None, None, 0))
        return out.reshape(res, res, res)

    def marchingCubes(self, res, isolevel=0.0001, field_ptr=None):
        """Marching cubes on the context's colour field (or a device field);
        returns (vertices, normals) as (ntri, 3, 3) arrays."""
        n = C.c_int()
        self._ck(self.lib.sph_marching_cubes(self.ctx, field_ptr, int(res), float(isolevel), C.byref(n)))
        return self._mesh(n.value)

    def postProcess(self, res):
        """SPH::postProcess: colour field + marching cubes (isolevel 0.0001)."""
        n = C.c_int()
        self._ck(self.lib.sph_post_process(self.ctx, int(res), C.byref(n)))
        return self._mesh(n.value)

    def _mesh(self, n):
        v = np.empty((n, 3, 3), np.float32)
        nr = np.empty((n, 3, 3), np.float32)
        if n:
            self._ck(self.lib.sph_download_surface(self.ctx, None, v.ctypes.data, nr.ctypes.data, n))
        return v, nr

    # -- whole steps --------------------------------------------------------
    def update(self):
        """SPH::update: hash ... collision."""
        self._ck(self.lib.sph_update(self.ctx))

    def integrate(self, dt):
        """SPH::integrate (leapfrog)."""
        self._ck(self.lib.sph_integrate(self.ctx, float(dt)))

    def step(self, dt, nsteps=1):
        """nsteps fused update+integrate steps, replayed from a CUDA graph."""
        self._ck(self.lib.sph_step(self.ctx, float(dt), int(nsteps)))

    def step_eager(self, dt, nsteps=1):
        self._ck(self.lib.sph_step_eager(self.ctx, float(dt), int(nsteps)))

    def sync(self):
        self._ck(self.lib.sph_sync(self.ctx))

    # -- differentiable rollout ----------------------------------------------
    def adjoint_record(self, dt, nsteps, K):
        """Run nsteps steps keeping a checkpoint every K steps (sph_adjoint_record)."""
        self._ck(self.lib.sph_adjoint_record(self.ctx, float(dt), int(nsteps), int(K)))

    def adjoint_backward(self, dpos=None, dvel=None, dveleval=None, out_pos=None, out_vel=None, out_veleval=None):
        """Backward pass of the recorded rollout (sph_adjoint_backward).

        Arguments are DEVICE addresses (ints, e.g. torch's data_ptr()) of num
        float4 in original particle order, or None.  Returns dL/dviscosity.
        """
        v = C.c_double()
        self._ck(self.lib.sph_adjoint_backward(self.ctx, dpos, dvel, dveleval, out_pos, out_vel, out_veleval,
                                               C.byref(v)))
        return v.value


class Hose:
    """The reference's Hose (common/Hose.cpp) as a host object of the
    library (sph_hose_*): spray() returns the (k, 4) positions one tick
    emits and the velocity they are pushed with."""

    def __init__(self, dt, total_n, center, velocity, radius, spacing):
        self.lib = abi.load_library()
        self.h = C.c_void_p()
        abi.check(self.lib, None, self.lib.sph_hose_create(float(dt), int(total_n), abi.vec4(center),
                                                           abi.vec4(velocity), float(radius), float(spacing),
                                                           C.byref(self.h)))

    def update(self, center, velocity, radius, spacing):
        abi.check(self.lib, None, self.lib.sph_hose_update(self.h, abi.vec4(center), abi.vec4(velocity), float(radius),
                                                           float(spacing)))

    def refill(self, n):
        abi.check(self.lib, None, self.lib.sph_hose_refill(self.h, int(n)))

    def spray(self):
        k = C.c_int()
        abi.check(self.lib, None, self.lib.sph_hose_spray(self.h, C.byref(k)))
        pos = np.zeros((k.value, 4), np.float32)
        v = abi.sph_float4()
        abi.check(self.lib, None, self.lib.sph_hose_particles(self.h, pos.ctypes.data if k.value else None, k.value,
                                                              C.byref(v)))
        return pos, np.array([v.x, v.y, v.z, v.w], np.float32)

    def remaining(self):
        n = C.c_int()
        abi.check(self.lib, None, self.lib.sph_hose_remaining(self.h, C.byref(n)))
        return n.value

    def close(self):
        if self.h:
            self.lib.sph_hose_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dambreak_system(n, viscosity=0.01, max_num=None, exact=False, velocity_sigma=0.0, scene=0):
    """An SPH system holding the dam-break scene of n particles."""
    from .scenes import dambreak
    sp, g, gs = abi.dambreak_params(n, viscosity)
    s = SPH(sp, g, max_num or n, gs, exact=exact)
    pos, vel = dambreak(n, scene=scene, velocity_sigma=velocity_sigma)
    s.upload(pos, vel)
    return s, (sp, g, gs), (pos, vel)
