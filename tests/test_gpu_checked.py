"""The bounds-checked library (librtps_sph_checked.so, built with
-DSPH_CHECKED) on the paths the GPU tests cover: every gather and scatter
index of the cell sort, the neighbour walk, the density and force passes, the
velocity pass, the integrators and the triangle stage is tested against its
array before the access, and a
failure would end the step with SPH_EBOUNDS.  On every case here the checked
library reports no failure and gives the same bits as the default library:
the fused and staged steps in both arithmetic modes, a crowded cell (more
candidates than the neighbour bitmask holds), particles leaving the grid, a
triangle mesh, point gravity sources with either integrator, a batch of
ragged scenes under both schedulers, and an adjoint rollout."""
import numpy as np
import pytest
import torch

import golden_io
from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.batch import Batch
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu
DT = 0.001
STATE = ("pos_u", "vel_u", "veleval_u")


@pytest.fixture(scope="module")
def libs():
    checked = abi.load_library(abi.CHECKED_LIB_PATH)
    assert "bounds-checked" in checked.sph_build_info().decode()
    return {"default": abi.load_library(), "checked": checked}


def _crowded_layout(n, seed):
    """n particles uniform in [-0.2, 1.2)^3 (some outside the grid, deleted
    by the first step); every 7th one moved onto particle 3, so one cell
    holds n/7 of them."""
    u = scenes.uniform(seed, 3 * n).reshape(n, 3)
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = (u * 1.4 - 0.2).astype(np.float32)
    pos[::7, :3] = pos[3, :3]
    v = scenes.uniform(seed + 1, 3 * n).reshape(n, 3)
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = ((v - 0.5) * 0.2).astype(np.float32)
    return pos, vel


def _run(lib, sp, g, gs, pos, vel, exact, steps, staged=False, triangles=None, gravity=None, integrator=None):
    s = SPH(sp, g, pos.shape[0], gs, exact=exact, lib=lib)
    if triangles is not None:
        s.loadTriangles(triangles)
    if gravity is not None:
        s.setGravitySources(*gravity)
    if integrator is not None:
        s.setIntegrator(integrator)
    s.upload(pos, vel)
    for _ in range(steps):
        if staged:
            s.update()
            s.integrate(DT)
        else:
            s.step(DT, 1)
    s.sync()  # raises SPHError (SPH_EBOUNDS) if a checked index failed
    out = [s.getNum()] + [s.get(f) for f in STATE] + list(s.getDeleted())
    s.close()
    return out


def _same(a, b):
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("exact", [True, False])
def test_dam_break_steps_pass_the_checks(libs, exact):
    n = 16384
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.1)
    got = _run(libs["checked"], sp, g, gs, pos, vel, exact, 20)
    _same(got, _run(libs["default"], sp, g, gs, pos, vel, exact, 20))


@pytest.mark.parametrize("exact,staged", [(True, False), (False, False), (True, True)])
def test_crowded_cell_and_deletion_pass_the_checks(libs, exact, staged):
    n = 60000
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = _crowded_layout(n, 5)
    got = _run(libs["checked"], sp, g, gs, pos, vel, exact, 3, staged=staged)
    assert got[0] < n  # particles outside the grid were deleted
    _same(got, _run(libs["default"], sp, g, gs, pos, vel, exact, 3, staged=staged))


@pytest.mark.parametrize("staged", [False, True])
def test_mesh_step_with_deletion_passes_the_checks(libs, staged):
    d, sp, g, gs = golden_io.load("triangles_n2048.npz")
    pos = np.array(d["in_pos"], np.float32)
    vel = np.array(d["in_vel"], np.float32)
    pos[::37, 2] = np.float32(5.0)
    kw = dict(staged=staged, triangles=d["triangles"])
    got = _run(libs["checked"], sp, g, gs, pos, vel, True, 3, **kw)
    _same(got, _run(libs["default"], sp, g, gs, pos, vel, True, 3, **kw))


@pytest.mark.parametrize("integrator,staged", [("euler", False), ("euler", True), ("leapfrog", True)])
def test_gravity_sources_and_integrators_pass_the_checks(libs, integrator, staged):
    d, sp, g, gs = golden_io.load("gravity_n2048.npz")
    pos = np.array(d["in_pos"], np.float32)
    vel = np.array(d["in_vel"], np.float32)
    kw = dict(staged=staged, gravity=(d["grav_points"], d["grav_masses"], d["grav_alphas"]), integrator=integrator)
    got = _run(libs["checked"], sp, g, gs, pos, vel, True, 3, **kw)
    _same(got, _run(libs["default"], sp, g, gs, pos, vel, True, 3, **kw))


@pytest.mark.parametrize("queue", [False, True])
def test_batch_of_ragged_crowded_scenes_passes_the_checks(libs, queue):
    ns = [4096, 33, 1, 2500, 6001]
    params = [abi.dambreak_params(max(n, 1024), 0.01 + 0.005 * k) for k, n in enumerate(ns)]
    data = []
    for k, n in enumerate(ns):
        pos, vel = scenes.dambreak(max(n, 1024), scene=k, velocity_sigma=0.05)
        pos, vel = pos[:n].copy(), vel[:n].copy()
        if n > 100:
            pos[::5, :3] = pos[3, :3]
        if k == 3:
            pos[::9, 2] = np.float32(5.0)  # deleted from this scene
        data.append((pos, vel))
    out = {}
    for name, lib in libs.items():
        b = Batch(params, [n + 40 for n in ns], exact=True, lib=lib)
        b.set_scheduler(queue)
        for k, (pos, vel) in enumerate(data):
            b.upload(k, pos, vel)
        b.step(DT, 4)
        b.sync()  # raises SPHError (SPH_EBOUNDS) if a checked index failed
        out[name] = [[b.getNum(k)] + [b.get(k, f) for f in STATE] for k in range(len(ns))]
        b.close()
    assert out["checked"][3][0] < ns[3]
    for k in range(len(ns)):
        _same(out["checked"][k], out["default"][k])


def test_adjoint_rollout_passes_the_checks(libs):
    n = 4096
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.1)
    seed = torch.Generator().manual_seed(3)
    dpos = torch.randn((n, 4), generator=seed, dtype=torch.float32)
    dpos[:, 3] = 0
    grads = {}
    for name, lib in libs.items():
        s = SPH(sp, g, n, gs, lib=lib)
        s.upload(pos, vel)
        s.adjoint_record(DT, 20, 5)
        gp = dpos.cuda()
        outs = [torch.zeros((n, 4), dtype=torch.float32, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()
        dmu = s.adjoint_backward(dpos=gp.data_ptr(), out_pos=outs[0].data_ptr(), out_vel=outs[1].data_ptr(),
                                 out_veleval=outs[2].data_ptr())
        s.sync()
        torch.cuda.synchronize()
        grads[name] = [o.cpu().numpy() for o in outs] + [dmu]
        s.close()
    for a, b in zip(grads["checked"][:3], grads["default"][:3]):
        np.testing.assert_array_equal(a, b)
    assert grads["checked"][3] == grads["default"][3]
