"""The 2,097,152-particle dam break of the throughput benchmark against the
oracle directly: exact arithmetic bit for bit, the default arithmetic within
the rollout tolerance (1e-4 h).  The oracle steps this size in well under a
second on the host cores, so no size-independent proxy is needed here."""
import numpy as np
import pytest

import oracle_bind as ob
from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu
DT = 0.001
N = 2097152


@pytest.fixture(scope="module")
def scene():
    sp, g, gs = abi.dambreak_params(N)
    pos, vel = scenes.dambreak(N, velocity_sigma=0.1)
    return sp, g, gs, pos, vel


def test_full_size_exact_steps_equal_oracle(scene):
    sp, g, gs, pos, vel = scene
    s = SPH(sp, g, N, gs, exact=True)
    s.upload(pos, vel)
    s.step(DT, 2)
    sim = ob.OracleSim(sp, g, gs, N)
    sim.upload(pos, vel)
    sim.step(DT, 2)
    assert s.getNum() == sim.num
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(s.get(f), sim.get(f), err_msg=f)
    s.close()


def test_full_size_default_steps_within_tolerance(scene):
    sp, g, gs, pos, vel = scene
    s = SPH(sp, g, N, gs)
    s.upload(pos, vel)
    s.step(DT, 3)
    sim = ob.OracleSim(sp, g, gs, N)
    sim.upload(pos, vel)
    sim.step(DT, 3)
    assert s.getNum() == sim.num
    err = np.abs(s.get("pos_u") - sim.get("pos_u")).max()
    assert err <= 1e-4 * sp.smoothing_distance, err / sp.smoothing_distance
    s.close()


def test_full_size_mesh_step_equals_oracle(scene):
    """The same scene with the 524-triangle ramp-and-box mesh of the mesh
    benchmark: one exact graph step (the triangle kernel after the fused
    passes) bit for bit against the oracle."""
    from enjaparticles_gb300.scenes import ramp_and_box_mesh
    sp, g, gs, pos, vel = scene
    tris = ramp_and_box_mesh()
    s = SPH(sp, g, N, gs, exact=True)
    s.loadTriangles(tris)
    s.upload(pos, vel)
    s.step(DT, 1)
    sim = ob.OracleSim(sp, g, gs, N)
    sim.set_triangles(tris)
    sim.upload(pos, vel)
    sim.step(DT, 1)
    assert s.getNum() == sim.num
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(s.get(f), sim.get(f), err_msg=f)
    s.close()
