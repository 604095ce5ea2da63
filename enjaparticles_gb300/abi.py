"""ctypes view of include/rtps_sph.h and the loader of librtps_sph.so.

The library is the product: there is no Python or CPU fallback.  If it is
missing, load_library() raises; build it with `python -m enjaparticles_gb300.build_ext`
(or __graft_entry__.build()).
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "librtps_sph.so")
# the same library compiled with every kernel index bounds-checked (SPH_EBOUNDS)
CHECKED_LIB_PATH = os.path.join(PKG, "librtps_sph_checked.so")


class sph_float4(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("w", C.c_float)]


class SPHParams(C.Structure):
    """rtpslib/system/SPHSettings.h:38-136 (144 bytes, 16-byte aligned)."""
    _fields_ = [(name, C.c_float) for name in (
        "rest_density", "mass", "rest_distance", "smoothing_distance", "simulation_scale",
        "boundary_stiffness", "boundary_dampening", "boundary_distance", "K", "viscosity",
        "velocity_limit", "xsph_factor", "friction_coef", "restitution_coef", "shear", "attraction",
        "spring", "EPSILON", "wpoly6_coef", "wpoly6_d_coef", "wpoly6_dd_coef", "wspiky_coef",
        "wspiky_d_coef", "wspiky_dd_coef", "wvisc_coef", "wvisc_d_coef", "wvisc_dd_coef")] + [
        ("num", C.c_int), ("max_num", C.c_int), ("_pad", C.c_int * 3), ("gravity", sph_float4)]


class GridParams(C.Structure):
    """rtpslib/domain/Domain.h:144-158 (128 bytes)."""
    _fields_ = [("grid_size", sph_float4), ("grid_min", sph_float4), ("grid_max", sph_float4),
                ("bnd_min", sph_float4), ("bnd_max", sph_float4), ("grid_res", sph_float4),
                ("grid_delta", sph_float4), ("nb_cells", C.c_int), ("_pad", C.c_int * 3)]


class sph_launch_config(C.Structure):
    """Launch shapes of the step's kernels (include/rtps_sph.h)."""
    _fields_ = [("density_threads", C.c_int), ("force_threads", C.c_int), ("scan_tile_cells", C.c_int),
                ("reserved", C.c_int)]

    def as_tuple(self):
        return (self.density_threads, self.force_threads, self.scan_tile_cells)


LAUNCH_CANDIDATES = [(128, 64, 2048), (256, 128, 4096), (512, 256, 8192)]
SPH_TUNE_RETIME = 1
SPH_SCHED_GRID, SPH_SCHED_QUEUE = 0, 1

assert C.sizeof(SPHParams) == 144 and SPHParams.gravity.offset == 128
assert C.sizeof(GridParams) == 128 and GridParams.nb_cells.offset == 112

SPH_OK, SPH_EINVAL, SPH_ENOMEM, SPH_ECUDA, SPH_EOOB, SPH_ETIMEOUT, SPH_ESTATE, SPH_EBOUNDS = 0, -1, -2, -3, -4, -5, -6, -7
SPH_INTEGRATOR_LEAPFROG, SPH_INTEGRATOR_EULER = 0, 1
SPH_MAX_GRAVITY_SOURCES = 64
SPH_MAX_TRIANGLES = 1 << 20
STATUS_NAMES = {0: "SPH_OK", -1: "SPH_EINVAL", -2: "SPH_ENOMEM", -3: "SPH_ECUDA", -4: "SPH_EOOB",
                -5: "SPH_ETIMEOUT", -6: "SPH_ESTATE", -7: "SPH_EBOUNDS"}
EMPTY_CELL = 0xFFFFFFFF

FIELDS = {
    "pos_u": 0, "vel_u": 1, "veleval_u": 2, "pos_s": 3, "vel_s": 4, "veleval_s": 5, "density_s": 6,
    "force_s": 7, "xsph_s": 8, "sort_hashes": 9, "sort_indices": 10, "cell_start": 11, "cell_end": 12,
    "neighbor_count": 13,
}
FIELD_DTYPE = {name: (np.float32, 4) for name in ("pos_u", "vel_u", "veleval_u", "pos_s", "vel_s", "veleval_s",
                                                  "force_s", "xsph_s")}
FIELD_DTYPE.update({"density_s": (np.float32, 1), "sort_hashes": (np.uint32, 1), "sort_indices": (np.uint32, 1),
                    "cell_start": (np.uint32, 1), "cell_end": (np.uint32, 1), "neighbor_count": (np.uint32, 1)})

_P = C.c_void_p
_I = C.c_int
_F = C.c_float
# name -> (restype, argtypes); every function declared in include/rtps_sph.h
SIGNATURES = {
    "sph_setup_domain": (_I, [C.POINTER(sph_float4), C.POINTER(sph_float4), _F, _F, C.POINTER(GridParams),
                              C.POINTER(GridParams)]),
    "sph_settings_round": (_F, [_F]),
    "sph_kernel_coefficients": (_I, [_F, C.POINTER(SPHParams)]),
    "sph_dambreak_params": (_I, [_I, _F, _F, C.POINTER(SPHParams), C.POINTER(GridParams), C.POINTER(GridParams)]),
    "sph_params_from_settings": (_I, [_I, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.POINTER(SPHParams),
                                      C.POINTER(GridParams), C.POINTER(GridParams), C.POINTER(_F)]),
    "sph_create": (_I, [C.POINTER(SPHParams), C.POINTER(GridParams), C.POINTER(GridParams), _I, C.POINTER(_P)]),
    "sph_destroy": (_I, [_P]),
    "sph_set_params": (_I, [_P, C.POINTER(SPHParams)]),
    "sph_get_params": (_I, [_P, C.POINTER(SPHParams), C.POINTER(GridParams), C.POINTER(GridParams)]),
    "sph_set_stream": (_I, [_P, _P]),
    "sph_upload": (_I, [_P, _P, _P, _P, _I]),
    "sph_push_particles": (_I, [_P, _P, _P, _I]),
    "sph_download": (_I, [_P, _I, _P, _I]),
    "sph_download_async": (_I, [_P, _I, _P, _I]),
    "sph_get_device_ptr": (_I, [_P, _I, C.POINTER(_P)]),
    "sph_get_num": (_I, [_P, C.POINTER(_I)]),
    "sph_set_num": (_I, [_P, _I]),
    "sph_stage_hash": (_I, [_P]),
    "sph_stage_sort": (_I, [_P]),
    "sph_stage_cellindices": (_I, [_P, C.POINTER(_I)]),
    "sph_stage_permute": (_I, [_P]),
    "sph_stage_density": (_I, [_P]),
    "sph_stage_force": (_I, [_P]),
    "sph_stage_collision": (_I, [_P]),
    "sph_stage_leapfrog": (_I, [_P, _F]),
    "sph_update": (_I, [_P]),
    "sph_integrate": (_I, [_P, _F]),
    "sph_step": (_I, [_P, _F, _I]),
    "sph_step_eager": (_I, [_P, _F, _I]),
    "sph_set_exact": (_I, [_P, _I]),
    "sph_get_deleted": (_I, [_P, _P, _P, _I, C.POINTER(_I)]),
    "sph_step_profile": (_I, [_P, _F, _I, C.POINTER(C.c_float), _I, C.POINTER(_I)]),
    "sph_profile_kernel_name": (C.c_char_p, [_P, _I]),
    "sph_sync": (_I, [_P]),
    "sph_last_error": (_I, [_P, C.c_char_p, _I]),
    "sph_adjoint_record": (_I, [_P, _F, _I, _I]),
    "sph_stage_gravity": (_I, [_P]),
    "sph_stage_euler": (_I, [_P, _F]),
    "sph_set_gravity_sources": (_I, [_P, _I, _P, _P, _P]),
    "sph_set_integrator": (_I, [_P, _I]),
    "sph_stage_collision_triangles": (_I, [_P]),
    "sph_load_triangles": (_I, [_P, _P, _I]),
    "sph_hose_create": (_I, [_F, _I, sph_float4, sph_float4, _F, _F, C.POINTER(_P)]),
    "sph_hose_update": (_I, [_P, sph_float4, sph_float4, _F, _F]),
    "sph_hose_refill": (_I, [_P, _I]),
    "sph_hose_spray": (_I, [_P, C.POINTER(_I)]),
    "sph_hose_particles": (_I, [_P, _P, _I, C.POINTER(sph_float4)]),
    "sph_hose_remaining": (_I, [_P, C.POINTER(_I)]),
    "sph_hose_destroy": (None, [_P]),
    "sph_add_hose": (_I, [_P, _I, sph_float4, sph_float4, _F, _F, C.POINTER(_I)]),
    "sph_update_hose": (_I, [_P, _I, sph_float4, sph_float4, _F]),
    "sph_refill_hose": (_I, [_P, _I, _I]),
    "sph_spray_hoses": (_I, [_P, C.POINTER(_I)]),
    "sph_colorfield": (_I, [_P, _I]),
    "sph_marching_cubes": (_I, [_P, _P, _I, _F, C.POINTER(_I)]),
    "sph_post_process": (_I, [_P, _I, C.POINTER(_I)]),
    "sph_get_surface": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(_I), C.POINTER(_I)]),
    "sph_download_surface": (_I, [_P, _P, _P, _P, _I]),
    "sph_mc_case_table": (_I, [_P, _P, C.POINTER(_I)]),
    "sph_adjoint_backward": (_I, [_P, _P, _P, _P, _P, _P, _P, C.POINTER(C.c_double)]),
    "sph_adjoint_rollout": (_I, [_P, _I, _I, _P, _P, C.POINTER(_F)]),
    "sph_batch_create": (_I, [_I, _P, _P, _P, _P, C.POINTER(_P)]),
    "sph_batch_destroy": (_I, [_P]),
    "sph_batch_set_stream": (_I, [_P, _P]),
    "sph_batch_set_exact": (_I, [_P, _I]),
    "sph_batch_upload": (_I, [_P, _I, _P, _P, _P, _I]),
    "sph_batch_step": (_I, [_P, _F, _I]),
    "sph_batch_download": (_I, [_P, _I, _I, _P, _I]),
    "sph_batch_out_of_grid": (_I, [_P, C.POINTER(_I)]),
    "sph_batch_get_num": (_I, [_P, _I, C.POINTER(_I)]),
    "sph_batch_get_deleted": (_I, [_P, _I, _P, _P, _I, C.POINTER(_I)]),
    "sph_batch_sync": (_I, [_P]),
    "sph_batch_last_error": (_I, [_P, C.c_char_p, _I]),
    "sph_batch_set_params": (_I, [_P, _I, _P]),
    "sph_batch_get_params": (_I, [_P, _I, _P]),
    "sph_batch_get_device_ptr": (_I, [_P, _I, C.POINTER(_P)]),
    "sph_batch_slot_offset": (_I, [_P, _I, C.POINTER(_I)]),
    "sph_batch_adjoint_record": (_I, [_P, _F, _I, _I]),
    "sph_batch_adjoint_backward": (_I, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "sph_batch_adjoint_rewind": (_I, [_P]),
    "sph_batch_loss_mse": (_I, [_P, _P, _P, _P]),
    "sph_batch_trajectory": (_I, [_P, _P]),
    "sph_batch_loss_traj": (_I, [_P, _P, _P, _F, _P]),
    "sph_batch_adjoint_backward_traj": (_I, [_P, _P, _P, _P, _P, _P]),
    "sph_adjoint_rewind": (_I, [_P]),
    "sph_loss_mse": (_I, [_P, _P, _P, C.POINTER(C.c_double)]),
    "sph_sort_pairs_noalloc": (_I, [_P, _P, _P, _P, _I, _I, _P]),
    "sph_get_launch_config": (_I, [_P, C.POINTER(sph_launch_config)]),
    "sph_set_launch_config": (_I, [_P, C.POINTER(sph_launch_config)]),
    "sph_autotune": (_I, [_P, _F, _I, _I, C.POINTER(sph_launch_config)]),
    "sph_batch_get_launch_config": (_I, [_P, C.POINTER(sph_launch_config)]),
    "sph_batch_set_launch_config": (_I, [_P, C.POINTER(sph_launch_config)]),
    "sph_batch_autotune": (_I, [_P, _F, _I, _I, C.POINTER(sph_launch_config)]),
    "sph_batch_set_scheduler": (_I, [_P, _I]),
    "sph_batch_get_scheduler": (_I, [_P, C.POINTER(_I)]),
    "sph_batch_queue_test_hold": (_I, [_P, _I, C.c_uint]),
    "sph_build_info": (C.c_char_p, []),
}

_lib = None


def vec4(v):
    """A sph_float4 from a sequence of 3 or 4 numbers (w = 0 when absent)."""
    v = [float(x) for x in v] + [0.0] * (4 - len(v))
    return sph_float4(*v[:4])


def load_library(path=None):
    """Load librtps_sph.so (raises if it is absent: no fallback exists)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("librtps_sph.so not built (%s); run `python -m enjaparticles_gb300.build_ext`" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class SPHError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(code, "?"), code, message))
        self.code = code


def last_error(lib, ctx):
    buf = C.create_string_buffer(512)
    lib.sph_last_error(ctx, buf, 512)
    return buf.value.decode(errors="replace")


def check(lib, ctx, rc):
    if rc != SPH_OK:
        raise SPHError(rc, last_error(lib, ctx))
    return rc


def f4(x, y, z, w=0.0):
    return sph_float4(x, y, z, w)


def dambreak_params(n, viscosity=0.01, spacing=None):
    """(SPHParams, GridParams, GridParams scaled) of the dam-break scenes."""
    from .scenes import lattice_spacing
    lib = load_library()
    sp, g, gs = SPHParams(), GridParams(), GridParams()
    s = lattice_spacing(n) if spacing is None else spacing
    check(lib, None, lib.sph_dambreak_params(n, s, viscosity, C.byref(sp), C.byref(g), C.byref(gs)))
    return sp, g, gs


def settings_value(v):
    """A value as RTPSSettings::SetSetting stores it (`ostringstream << v`):
    strings as they are, numbers with 6 significant digits, float4-like
    sequences as their four lanes separated by spaces."""
    if isinstance(v, str):
        return v
    if isinstance(v, (list, tuple)):
        return " ".join(settings_value(x) for x in v)
    if isinstance(v, (int, np.integer)) and not isinstance(v, bool):
        return str(int(v))
    return "%.6g" % float(v)


def params_from_settings(settings, lib=None):
    """(SPHParams, GridParams, GridParams scaled, spacing) of the SPH system the
    reference builds from this settings map (sph_params_from_settings)."""
    lib = lib if lib is not None else load_library()
    items = [(str(k), settings_value(v)) for k, v in settings.items()]
    keys = (C.c_char_p * max(len(items), 1))(*[k.encode() for k, _ in items])
    vals = (C.c_char_p * max(len(items), 1))(*[v.encode() for _, v in items])
    sp, g, gs, spacing = SPHParams(), GridParams(), GridParams(), C.c_float()
    check(lib, None, lib.sph_params_from_settings(len(items), keys, vals, C.byref(sp), C.byref(g), C.byref(gs),
                                                  C.byref(spacing)))
    return sp, g, gs, spacing.value
