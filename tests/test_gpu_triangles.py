"""Triangle-mesh collision (collision_tri.cl) on the GPU: the staged kernel
alone against the oracle on particles packed around a mesh, and whole steps
against the golden fixture made from the reference's own kernels
(tests/golden/triangles_n2048.npz): bit-exact in exact arithmetic, staged and
fused; within the step tolerances in the default arithmetic (the triangle
stage itself is always exact)."""
import ctypes as C

import numpy as np
import pytest
import torch

import golden_io
import oracle_bind as ob
from enjaparticles_gb300 import abi
from enjaparticles_gb300.scenes import ramp_and_box_mesh, ramp_mesh, uniform
from enjaparticles_gb300.sph import SPH
from mesh_cases import near_mesh_particles

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
STATE = ("pos_u", "vel_u", "veleval_u")


def normwise(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


class _DeviceArray:
    """A float32 (n, 4) view of library device memory for torch."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n, 4), "typestr": "<f4", "data": (ptr, False), "version": 3,
                                         "strides": None}


def _write_field(s, field, arr):
    s.sync()
    dst = torch.as_tensor(_DeviceArray(s.device_ptr(field), arr.shape[0]), device="cuda")
    dst.copy_(torch.from_numpy(np.ascontiguousarray(arr, np.float32)).cuda())
    torch.cuda.synchronize()


def _system(d, sp, g, gs, exact):
    n = d["in_pos"].shape[0]
    s = SPH(sp, g, n, gs, exact=exact)
    s.loadTriangles(d["triangles"])
    s.upload(d["in_pos"], d["in_vel"])
    return s


@pytest.mark.parametrize("scale,mesh", [(1.0, "ramp_and_box"), (0.05, "ramp_and_box"), (1.0, "fine_ramp")])
def test_triangle_stage_equals_oracle(scale, mesh):
    """The stage alone on 20,000 particles around the mesh (every direction of
    motion, zero velocities included): force_s equals the oracle's bit for
    bit.  The fine ramp has 2,312 triangles: eleven 220-triangle chunks over
    ten 256-triangle candidate tiles."""
    n = 20000
    sp, g, gs = abi.dambreak_params(n)
    tris = ramp_and_box_mesh() if mesh == "ramp_and_box" else ramp_mesh(34, 34)
    if scale != 1.0:
        sp.simulation_scale = scale  # the stage reads no grid
        tris = tris.copy()
        tris[:, :3, :3] /= scale
    tris = np.ascontiguousarray(tris.reshape(-1, 16))
    pos, vel = near_mesh_particles(tris, n, sp.boundary_distance, scale, 701)
    f0 = ((uniform(705, 4 * n).reshape(n, 4) - 0.5) * 40).astype(np.float32)
    s = SPH(sp, g, n, gs)
    s.loadTriangles(tris)
    s.upload(pos, vel)
    _write_field(s, "pos_s", pos)
    _write_field(s, "vel_s", vel)
    _write_field(s, "force_s", f0)
    s.collision_triangles()
    got = s.get("force_s", n)
    sp_o = s.params()[0]
    want = f0.copy()
    ob.oracle().oracle_collision_triangles(0, n, ob.ptr(pos), ob.ptr(vel), ob.ptr(want), ob.ptr(tris), tris.shape[0],
                                           C.addressof(sp_o))
    hit = np.abs(want[:, :3] - f0[:, :3]).max(1) > 0
    assert hit.sum() > n // 10
    np.testing.assert_array_equal(got, want)


def test_staged_exact_matches_reference_golden():
    d, sp, g, gs = golden_io.load("triangles_n2048.npz")
    s = _system(d, sp, g, gs, exact=True)
    dt = float(d["dt"])
    s.update()
    np.testing.assert_array_equal(s.get("force_s"), d["s1_force_s"])
    s.integrate(dt)
    for f in STATE:
        np.testing.assert_array_equal(s.get(f), d["s1_" + f], err_msg=f)
    done = 1
    for k in (5, 20):
        for _ in range(k - done):
            s.update()
            s.integrate(dt)
        done = k
        for f in STATE:
            np.testing.assert_array_equal(s.get(f), d["s%d_%s" % (k, f)], err_msg="step %d %s" % (k, f))


def test_fused_exact_matches_reference_golden():
    d, sp, g, gs = golden_io.load("triangles_n2048.npz")
    s = _system(d, sp, g, gs, exact=True)
    dt = float(d["dt"])
    done = 0
    for k in (1, 5, 20):
        s.step(dt, k - done)
        done = k
        for f in STATE:
            np.testing.assert_array_equal(s.get(f), d["s%d_%s" % (k, f)], err_msg="step %d %s" % (k, f))


def test_fused_with_mesh_and_deletion_equals_staged():
    """With a mesh loaded, particles leaving the grid: the graph step (the
    velocity pass's deletion bookkeeping, the triangle kernel's re-indexing)
    equals staged update()+integrate() bit for bit, deleted particles
    included."""
    d, sp, g, gs = golden_io.load("triangles_n2048.npz")
    pos = np.array(d["in_pos"], np.float32)
    vel = np.array(d["in_vel"], np.float32)
    sel = np.arange(0, pos.shape[0], 37)
    pos[sel, 2] = np.float32(5.0)  # far above the grid: deleted by the step
    dt = float(d["dt"])
    out = {}
    for mode in ("staged", "graph"):
        s = SPH(sp, g, pos.shape[0], gs, exact=True)
        s.loadTriangles(d["triangles"])
        s.upload(pos, vel)
        for _ in range(3):
            if mode == "staged":
                s.update()
                s.integrate(dt)
            else:
                s.step(dt, 1)
        out[mode] = [s.getNum()] + [s.get(f) for f in STATE] + list(s.getDeleted())
        s.close()
    assert out["graph"][0] == out["staged"][0] == pos.shape[0] - len(sel)
    for a, b, name in zip(out["graph"][1:], out["staged"][1:], STATE + ("deleted pos", "deleted vel")):
        np.testing.assert_array_equal(a, b, err_msg=name)


def test_fast_within_tolerance_of_reference_golden():
    d, sp, g, gs = golden_io.load("triangles_n2048.npz")
    s = _system(d, sp, g, gs, exact=False)
    s.update()
    assert normwise(s.get("force_s")[:, :3], d["s1_force_s"][:, :3]) <= FORCE_RTOL
    s2 = _system(d, sp, g, gs, exact=False)
    s2.step(float(d["dt"]), 5)
    assert np.abs(s2.get("pos_u") - d["s5_pos_u"]).max() <= 1e-4 * sp.smoothing_distance


def test_unload_restores_the_wall_only_step():
    """Loading a mesh and unloading it again leaves the fused graph step
    equal to a system that never had one."""
    d, sp, g, gs = golden_io.load("triangles_n2048.npz")
    a = _system(d, sp, g, gs, exact=True)
    a.step(float(d["dt"]), 2)
    a.loadTriangles(np.zeros((0, 16), np.float32))
    b = SPH(sp, g, d["in_pos"].shape[0], gs, exact=True)
    b.upload(a.get("pos_u"), a.get("vel_u"), a.get("veleval_u"))
    a.step(float(d["dt"]), 3)
    b.step(float(d["dt"]), 3)
    for f in STATE:
        np.testing.assert_array_equal(a.get(f), b.get(f), err_msg=f)


def test_mesh_errors():
    d, sp, g, gs = golden_io.load("triangles_n2048.npz")
    n = d["in_pos"].shape[0]
    s = SPH(sp, g, n, gs)
    with pytest.raises(abi.SPHError) as e:
        s._ck(s.lib.sph_load_triangles(s.ctx, None, abi.SPH_MAX_TRIANGLES + 1))
    assert e.value.code == abi.SPH_EINVAL
    bad = d["triangles"].copy()
    bad[3, 1, 2] = np.nan
    with pytest.raises(abi.SPHError) as e:
        s.loadTriangles(bad)
    assert e.value.code == abi.SPH_EINVAL
    s.loadTriangles(d["triangles"])
    s.upload(d["in_pos"], d["in_vel"])
    with pytest.raises(abi.SPHError) as e:
        s.adjoint_record(float(d["dt"]), 4, 2)
    assert e.value.code == abi.SPH_ESTATE
    ms = (C.c_float * 32)()
    nk = C.c_int()
    with pytest.raises(abi.SPHError) as e:
        s._ck(s.lib.sph_step_profile(s.ctx, float(d["dt"]), 1, ms, 32, C.byref(nk)))
    assert e.value.code == abi.SPH_ESTATE
    s.loadTriangles(np.zeros((0, 4, 4), np.float32))
    s.adjoint_record(float(d["dt"]), 4, 2)
