"""The batched step's counting sort over the cells of all scenes
(sph_batch.cu): scenes with crowded cells, ragged sizes and unused slots
step exactly as they would alone, and particles outside their scene's grid
are frozen, counted and kept out of everyone's neighbourhood."""
import numpy as np
import pytest

from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.batch import Batch
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu
DT = 0.001


def crowded(n, seed, every):
    """A dam break of n particles with every `every`-th one moved onto
    particle 3, so one cell holds n/every of them."""
    pos, vel = scenes.dambreak(max(n, 1024), scene=seed, velocity_sigma=0.05)
    pos, vel = pos[:n].copy(), vel[:n].copy()
    if every:
        pos[::every, :3] = pos[3, :3]
    return pos, vel


def test_crowded_and_ragged_scenes_equal_their_own_contexts():
    ns = [4096, 33, 1, 2500, 6001]
    every = [5, 0, 0, 3, 50]
    params = [abi.dambreak_params(max(n, 1024), 0.01 + 0.005 * k) for k, n in enumerate(ns)]
    data = [crowded(n, k, e) for k, (n, e) in enumerate(zip(ns, every))]
    b = Batch(params, [n + 40 for n in ns], exact=True)  # unused slots after every scene
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.step(DT, 3)
    b.sync()
    for k, ((sp, g, gs), (pos, vel)) in enumerate(zip(params, data)):
        s = SPH(sp, g, ns[k], gs, exact=True)
        s.upload(pos, vel)
        s.step(DT, 3)
        assert s.getNum() == ns[k]
        for f in ("pos_u", "vel_u", "veleval_u"):
            np.testing.assert_array_equal(b.get(k, f), s.get(f), err_msg="scene %d %s" % (k, f))
        s.close()
    b.close()


def test_out_of_grid_particles_are_frozen_and_isolated():
    """Scene 1 has particles far above and below its grid.  They stay where
    they are, are counted every step, and the scene's other particles step
    exactly as a lone context holding only them."""
    ns = [3000, 5000]
    params = [abi.dambreak_params(n, 0.02) for n in ns]
    data = [scenes.dambreak(n, scene=k, velocity_sigma=0.05) for k, n in enumerate(ns)]
    pos1, vel1 = data[1]
    u = scenes.uniform(31, ns[1])
    out = u < 0.2
    pos1[out, 2] = np.where(u[out] < 0.1, np.float32(5.0), np.float32(-5.0))
    b = Batch(params, ns, exact=True)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.step(DT, 4)
    b.sync()
    assert b.out_of_grid() == int(out.sum())
    got_pos, got_vel = b.get(1, "pos_u"), b.get(1, "vel_u")
    np.testing.assert_array_equal(got_pos[out], pos1[out])
    np.testing.assert_array_equal(got_vel[out], vel1[out])
    sp, g, gs = params[1]
    keep = ~out
    s = SPH(sp, g, int(keep.sum()), gs, exact=True)
    s.upload(pos1[keep], vel1[keep])
    s.step(DT, 4)
    assert s.getNum() == int(keep.sum())
    np.testing.assert_array_equal(got_pos[keep], s.get("pos_u"))
    np.testing.assert_array_equal(got_vel[keep], s.get("vel_u"))
    np.testing.assert_array_equal(b.get(1, "veleval_u")[keep], s.get("veleval_u"))
    s.close()
    # scene 0 is untouched by scene 1's frozen particles
    sp, g, gs = params[0]
    s = SPH(sp, g, ns[0], gs, exact=True)
    s.upload(*data[0])
    s.step(DT, 4)
    np.testing.assert_array_equal(b.get(0, "pos_u"), s.get("pos_u"))
    s.close()
    b.close()
