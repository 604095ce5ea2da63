"""The batch's queue scheduler (SPH_SCHED_QUEUE: persistent blocks taking
(scene, tile) items from a device counter) against the grid scheduler: the
same bits in exact and default arithmetic, with every launch shape, with
scenes that delete particles; and its bounded wait, made to run out."""
import numpy as np
import pytest

from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.batch import Batch

pytestmark = pytest.mark.gpu
DT = 0.001
FIELDS = ("pos_u", "vel_u", "veleval_u")


def _scenes():
    ns = [4096, 33, 1, 2500, 6001, 4000]
    params = [abi.dambreak_params(max(n, 1024), 0.01 + 0.004 * k) for k, n in enumerate(ns)]
    data = []
    for k, n in enumerate(ns):
        pos, vel = scenes.dambreak(max(n, 1024), scene=k, velocity_sigma=0.05)
        pos, vel = pos[:n].copy(), vel[:n].copy()
        if k == 5:  # a scene that loses particles mid-run
            vel[scenes.uniform(41, n) < 0.15, 2] = np.float32(200.0)
        data.append((pos, vel))
    return ns, params, data


def _run(queue, exact, shape=None, steps=6):
    ns, params, data = _scenes()
    b = Batch(params, [n + 17 for n in ns], exact=exact)
    b.set_scheduler(queue)
    if shape is not None:
        b.set_launch_config(*shape)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.step(DT, steps)
    b.sync()
    out = [{f: b.get(k, f) for f in FIELDS} for k in range(len(ns))]
    out.append([b.getNum(k) for k in range(len(ns))])
    b.close()
    return out


@pytest.mark.parametrize("exact", [True, False])
def test_queue_equals_grid(exact):
    ref = _run(False, exact)
    assert ref[-1][5] < 4000  # the thrown particles were deleted
    for shape in [None] + abi.LAUNCH_CANDIDATES:
        got = _run(True, exact, shape)
        assert got[-1] == ref[-1]
        for k in range(len(ref) - 1):
            for f in FIELDS:
                np.testing.assert_array_equal(got[k][f], ref[k][f], err_msg="%s scene %d %s" % (shape, k, f))


def test_queue_bounded_wait_runs_out_and_the_batch_recovers():
    ns, params, data = _scenes()
    b = Batch(params, ns, exact=True)
    b.set_scheduler(True)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.queue_test_hold(True, spin_limit=4096)  # the item table is never published
    b.step(DT, 1)
    with pytest.raises(abi.SPHError) as e:
        b.sync()
    assert e.value.code == abi.SPH_ETIMEOUT
    b.queue_test_hold(False)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.step(DT, 6)
    b.sync()
    ref = _run(False, True)
    for k in range(len(ns)):
        np.testing.assert_array_equal(b.get(k, "pos_u"), ref[k]["pos_u"])
    b.close()
