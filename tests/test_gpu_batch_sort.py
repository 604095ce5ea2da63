"""The batched step's counting sort over the cells of all scenes
(sph_batch.cu): scenes with crowded cells, ragged sizes and unused slots
step exactly as they would alone, and particles that leave their scene's
grid are deleted exactly as a lone context deletes them."""
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


def _leaving_scenes():
    """Three scenes: 0 untouched; 1 with 20 % of its particles placed outside
    its grid (deleted by the first step); 2 with 15 % thrown upwards fast
    enough to leave the grid a few steps in (deleted mid-run)."""
    ns = [3000, 5000, 4000]
    params = [abi.dambreak_params(n, 0.02) for n in ns]
    data = [scenes.dambreak(n, scene=k, velocity_sigma=0.05) for k, n in enumerate(ns)]
    pos1 = data[1][0]
    u = scenes.uniform(31, ns[1])
    out = u < 0.2
    pos1[out, 2] = np.where(u[out] < 0.1, np.float32(5.0), np.float32(-5.0))
    vel2 = data[2][1]
    up = scenes.uniform(32, ns[2]) < 0.15
    vel2[up, 2] = np.float32(200.0)
    return ns, params, data


@pytest.mark.parametrize("exact", [True, False])
def test_scenes_that_lose_particles_equal_their_own_contexts(exact):
    """Deletion in a batch is the lone system's deletion (SPH.cpp:220-250):
    after every step each scene has the lone context's particle count, its
    state bit for bit, and the same deleted particles (positions and
    velocities, sorted order); the other scenes are untouched."""
    ns, params, data = _leaving_scenes()
    b = Batch(params, ns, exact=exact)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    lone = []
    for (sp, g, gs), (pos, vel), n in zip(params, data, ns):
        s = SPH(sp, g, n, gs, exact=exact)
        s.upload(pos, vel)
        lone.append(s)
    deleted_total = 0
    for step in range(8):
        b.step(DT, 1)
        b.sync()
        removed = 0
        for k, s in enumerate(lone):
            before = s.getNum()
            s.step(DT, 1)
            n = s.getNum()
            removed += before - n
            assert b.getNum(k) == n, (step, k)
            for f in ("pos_u", "vel_u", "veleval_u"):
                np.testing.assert_array_equal(b.get(k, f), s.get(f), err_msg="step %d scene %d %s" % (step, k, f))
            dp, dv = b.getDeleted(k)
            lp, lv = s.getDeleted()
            if before != n:  # this step's deletion
                np.testing.assert_array_equal(dp, lp)
                np.testing.assert_array_equal(dv, lv)
        assert b.out_of_grid() == removed
        deleted_total += removed
    assert b.getNum(0) == ns[0]
    assert ns[1] - b.getNum(1) == int((scenes.uniform(31, ns[1]) < 0.2).sum())
    assert b.getNum(2) < ns[2]  # some of the thrown particles left mid-run
    assert deleted_total == sum(ns) - sum(b.getNum(k) for k in range(3))
    for s in lone:
        s.close()
    b.close()


def test_upload_after_deletion_restores_the_scene():
    """A scene that lost particles takes a new upload of any size up to its
    capacity; the batch then steps it as a fresh lone context."""
    ns, params, data = _leaving_scenes()
    b = Batch(params, ns, exact=True)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.step(DT, 2)
    assert b.getNum(1) < ns[1]
    pos, vel = scenes.dambreak(ns[1], scene=9, velocity_sigma=0.05)
    b.upload(1, pos, vel)
    assert b.getNum(1) == ns[1]
    b.step(DT, 2)
    sp, g, gs = params[1]
    s = SPH(sp, g, ns[1], gs, exact=True)
    s.upload(pos, vel)
    s.step(DT, 2)
    np.testing.assert_array_equal(b.get(1, "pos_u"), s.get("pos_u"))
    s.close()
    b.close()
