"""Python view of the batch API (sph_batch_*): many independent scenes stepped
together with one launch sequence per step."""
import ctypes as C

import numpy as np

from . import abi


class Batch:
    def __init__(self, params, max_num, exact=False, lib=None):
        """params: list of (SPHParams, GridParams, GridParams scaled) per scene;
        lib: a loaded library (the default one when None)."""
        self.lib = lib if lib is not None else abi.load_library()
        n = len(params)
        SP = (abi.SPHParams * n)(*[p[0] for p in params])
        G = (abi.GridParams * n)(*[p[1] for p in params])
        GS = (abi.GridParams * n)(*[p[2] for p in params])
        M = (C.c_int * n)(*[int(m) for m in max_num])
        self.h = C.c_void_p()
        rc = self.lib.sph_batch_create(n, C.cast(SP, C.c_void_p), C.cast(G, C.c_void_p), C.cast(GS, C.c_void_p),
                                       C.cast(M, C.c_void_p), C.byref(self.h))
        if rc != abi.SPH_OK:
            buf = C.create_string_buffer(512)
            self.lib.sph_batch_last_error(None, buf, 512)
            raise abi.SPHError(rc, buf.value.decode())
        self.nscenes = n
        self.num = [0] * n
        self.max_num = [int(m) for m in max_num]
        self.nslots = sum(self.max_num)
        if exact:
            self._ck(self.lib.sph_batch_set_exact(self.h, 1))

    def _ck(self, rc):
        if rc != abi.SPH_OK:
            buf = C.create_string_buffer(512)
            self.lib.sph_batch_last_error(self.h, buf, 512)
            raise abi.SPHError(rc, buf.value.decode())

    def close(self):
        if self.h:
            self.lib.sph_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, handle):
        self._ck(self.lib.sph_batch_set_stream(self.h, C.c_void_p(handle)))

    def upload(self, scene, pos, vel, veleval=None):
        pos = np.ascontiguousarray(pos, np.float32)
        vel = np.ascontiguousarray(vel, np.float32)
        ve = None if veleval is None else np.ascontiguousarray(veleval, np.float32)
        self._ck(self.lib.sph_batch_upload(self.h, scene, pos.ctypes.data, vel.ctypes.data,
                                           None if ve is None else ve.ctypes.data, pos.shape[0]))
        self.num[scene] = pos.shape[0]

    def step(self, dt, nsteps=1):
        self._ck(self.lib.sph_batch_step(self.h, float(dt), int(nsteps)))

    def sync(self):
        self._ck(self.lib.sph_batch_sync(self.h))

    def getNum(self, scene):
        """The scene's current particle count (it drops after a deletion)."""
        c = C.c_int()
        self._ck(self.lib.sph_batch_get_num(self.h, int(scene), C.byref(c)))
        self.num[scene] = c.value
        return c.value

    def get(self, scene, field):
        n = self.getNum(scene)
        out = np.empty((n, 4), np.float32)
        self._ck(self.lib.sph_batch_download(self.h, scene, abi.FIELDS[field], out.ctypes.data, n))
        return out

    def getDeleted(self, scene):
        """(pos, vel) of the particles the scene's last deletion removed, sorted order."""
        cnt = C.c_int()
        self._ck(self.lib.sph_batch_get_deleted(self.h, int(scene), None, None, 0, C.byref(cnt)))
        pos = np.empty((cnt.value, 4), np.float32)
        vel = np.empty((cnt.value, 4), np.float32)
        if cnt.value:
            self._ck(self.lib.sph_batch_get_deleted(self.h, int(scene), pos.ctypes.data, vel.ctypes.data, cnt.value,
                                                    C.byref(cnt)))
        return pos, vel

    def launch_config(self):
        cfg = abi.sph_launch_config()
        self._ck(self.lib.sph_batch_get_launch_config(self.h, C.byref(cfg)))
        return cfg.as_tuple()

    def set_launch_config(self, density_threads, force_threads, scan_tile_cells):
        cfg = abi.sph_launch_config(int(density_threads), int(force_threads), int(scan_tile_cells), 0)
        self._ck(self.lib.sph_batch_set_launch_config(self.h, C.byref(cfg)))

    def autotune(self, dt=0.001, steps=3, retime=False):
        cfg = abi.sph_launch_config()
        self._ck(self.lib.sph_batch_autotune(self.h, float(dt), int(steps), abi.SPH_TUNE_RETIME if retime else 0,
                                             C.byref(cfg)))
        return cfg.as_tuple()

    def set_scheduler(self, queue):
        """False: one grid per pass (default); True: persistent blocks over (scene, tile) items."""
        self._ck(self.lib.sph_batch_set_scheduler(self.h, abi.SPH_SCHED_QUEUE if queue else abi.SPH_SCHED_GRID))

    def queue_test_hold(self, hold, spin_limit=1 << 22):
        self._ck(self.lib.sph_batch_queue_test_hold(self.h, 1 if hold else 0, int(spin_limit)))

    def out_of_grid(self):
        """Particles removed by the last step (all scenes)."""
        c = C.c_int()
        self._ck(self.lib.sph_batch_out_of_grid(self.h, C.byref(c)))
        return c.value

    # -- parameters and device views ------------------------------------------
    def params(self, scene):
        sp = abi.SPHParams()
        self._ck(self.lib.sph_batch_get_params(self.h, int(scene), C.byref(sp)))
        return sp

    def set_params(self, scene, sp):
        self._ck(self.lib.sph_batch_set_params(self.h, int(scene), C.byref(sp)))

    def set_viscosity(self, scene, mu):
        sp = self.params(scene)
        sp.viscosity = float(mu)
        self.set_params(scene, sp)

    def device_ptr(self, field):
        p = C.c_void_p()
        self._ck(self.lib.sph_batch_get_device_ptr(self.h, abi.FIELDS[field], C.byref(p)))
        return p.value

    def slot_offsets(self):
        out = []
        for s in range(self.nscenes):
            o = C.c_int()
            self._ck(self.lib.sph_batch_slot_offset(self.h, s, C.byref(o)))
            out.append(o.value)
        return out

    # -- differentiable rollout (device addresses in slot layout) ---------------
    def adjoint_record(self, dt, nsteps, K):
        self._ck(self.lib.sph_batch_adjoint_record(self.h, float(dt), int(nsteps), int(K)))

    def adjoint_backward(self, dpos=None, dvel=None, dveleval=None, out_pos=None, out_vel=None, out_veleval=None):
        """Returns dL/dviscosity per scene (list of floats)."""
        g = (C.c_double * self.nscenes)()
        self._ck(self.lib.sph_batch_adjoint_backward(self.h, dpos, dvel, dveleval, out_pos, out_vel, out_veleval,
                                                     C.cast(g, C.c_void_p)))
        return list(g)

    def adjoint_rewind(self):
        self._ck(self.lib.sph_batch_adjoint_rewind(self.h))

    def trajectory(self, out):
        """Positions at the recorded rollout's checkpoint times into out (device
        address of nck * nslots float4)."""
        self._ck(self.lib.sph_batch_trajectory(self.h, out))

    def loss_traj(self, targets, grads, huber=0.0):
        """Per-scene trajectory loss (sph_batch_loss_traj); huber = 0: mean
        squared distance, else Huber with delta = huber * h."""
        out = (C.c_double * self.nscenes)()
        self._ck(self.lib.sph_batch_loss_traj(self.h, targets, grads, float(huber), C.cast(out, C.c_void_p)))
        return list(out)

    def adjoint_backward_traj(self, grads, out_pos=None, out_vel=None, out_veleval=None):
        g = (C.c_double * self.nscenes)()
        self._ck(self.lib.sph_batch_adjoint_backward_traj(self.h, grads, out_pos, out_vel, out_veleval,
                                                          C.cast(g, C.c_void_p)))
        return list(g)

    def loss_mse(self, target, grad):
        """Per-scene mean squared distance of pos_u to target (device address,
        slot layout); writes its gradient to grad (device address)."""
        out = (C.c_double * self.nscenes)()
        self._ck(self.lib.sph_batch_loss_mse(self.h, target, grad, C.cast(out, C.c_void_p)))
        return list(out)


def dambreak_batch_scenes(nscenes, seed_n=7, seed_mu=None, n_lo=2048, n_hi=32768, mu_lo=0.005, mu_hi=0.05):
    """Scene sizes N_s ~ U{n_lo..n_hi} and viscosities mu_s ~ U[mu_lo, mu_hi]
    from the seeded streams of enjaparticles_gb300.scenes."""
    from .scenes import uniform
    u = uniform(seed_n, nscenes)
    ns = [int(n_lo + min(int(x * (n_hi - n_lo + 1)), n_hi - n_lo)) for x in u]
    mu_u = uniform(seed_n + 1000 if seed_mu is None else seed_mu, nscenes)
    mus = [float(np.float32(mu_lo + x * (mu_hi - mu_lo))) for x in mu_u]
    return ns, mus
