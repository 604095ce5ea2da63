"""The step's optional parts together, on the GPU against the oracle, bit for
bit in exact arithmetic: point gravity sources, the triangle mesh after the
walls and a hose emitting particles before every step, over a 30-step
rollout of the graph-replayed step.  The oracle gets the same particles
from a hose driven by hand from the same rand() seed."""
import ctypes as C

import numpy as np
import pytest

import oracle_bind as ob
from enjaparticles_gb300 import abi
from enjaparticles_gb300.scenes import dambreak, ramp_and_box_mesh
from enjaparticles_gb300.sph import SPH, Hose

pytestmark = pytest.mark.gpu

DT = 0.001
SOURCES = (np.array([[0.25, 0.25, 0.9, 1.0], [0.2, 0.3, 0.15, 1.0]], np.float32), np.array([4.0, 0.5], np.float32),
           np.array([2.0, 1.5], np.float32))
HOSE = dict(total_n=400, center=(0.5, 0.5, 0.7, 1.0), velocity=(0.2, 0.0, -1.0, 0.0), radius=4.0)


@pytest.mark.parametrize("integrator", ["leapfrog", "euler"])
def test_gravity_mesh_and_hose_rollout_matches_oracle(integrator):
    n0, extra, steps, seed = 3000, 500, 30, 17
    sp, g, gs = abi.dambreak_params(n0)
    pos, vel = dambreak(n0, velocity_sigma=0.2)
    tris = ramp_and_box_mesh()
    s = SPH(sp, g, n0 + extra, gs, exact=True)
    s.setGravitySources(*SOURCES)
    s.loadTriangles(tris)
    s.setIntegrator(integrator)
    s.upload(pos, vel)
    libc = C.CDLL(None)
    libc.srand(seed)
    s.addHose(HOSE["total_n"], HOSE["center"], HOSE["velocity"], HOSE["radius"], DT)
    s.step(DT, steps)

    sim = ob.OracleSim(sp, g, gs, n0 + extra)
    sim.set_gravity(*SOURCES)
    sim.set_triangles(tris)
    sim.set_integrator(1 if integrator == "euler" else 0)
    sim.upload(pos, vel)
    spacing = s.lib.sph_settings_round(float(np.float32(sp.rest_distance) / np.float32(sp.simulation_scale)))
    libc.srand(seed)
    h = Hose(DT, HOSE["total_n"], HOSE["center"], HOSE["velocity"], HOSE["radius"] * spacing, spacing)
    for _ in range(steps):
        p, v = h.spray()
        if len(p):
            sim.push(p, np.repeat(v[None, :], len(p), axis=0))
        sim.step(DT, 1)
    n = s.getNum()
    assert n == sim.num and n > n0 + 200
    for f in ("pos_u", "vel_u") + (("veleval_u",) if integrator == "leapfrog" else ()):
        np.testing.assert_array_equal(s.get(f), sim.get(f), err_msg=f)
