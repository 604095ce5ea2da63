"""Batched scenes: every scene of a batch must step exactly as the same scene
in its own context (sph_step), in both arithmetic modes."""
import numpy as np
import pytest

from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.batch import Batch
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu
DT = 0.001


@pytest.mark.parametrize("exact", [True, False])
def test_batch_scenes_equal_their_own_contexts(exact):
    ns = [2048, 3001, 777, 5000, 4096]
    mus = [0.01, 0.03, 0.005, 0.05, 0.02]
    params = [abi.dambreak_params(n, mu) for n, mu in zip(ns, mus)]
    data = [scenes.dambreak(n, scene=k, velocity_sigma=0.05) for k, n in enumerate(ns)]
    b = Batch(params, [n + 17 for n in ns], exact=exact)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.step(DT, 7)
    b.sync()
    assert b.out_of_grid() == 0
    for k, ((sp, g, gs), (pos, vel)) in enumerate(zip(params, data)):
        s = SPH(sp, g, ns[k], gs, exact=exact)
        s.upload(pos, vel)
        s.step(DT, 7)
        for f in ("pos_u", "vel_u", "veleval_u"):
            np.testing.assert_array_equal(b.get(k, f), s.get(f), err_msg="scene %d %s" % (k, f))
        s.close()
    b.close()


def test_full_batched_configuration_equals_lone_contexts():
    """The batched benchmark's 256 scenes (4.47 M particles, the default
    arithmetic the benchmark times): after three steps every scene equals the
    same scene stepped in its own context, bit for bit."""
    from enjaparticles_gb300.batch import dambreak_batch_scenes
    ns, mus = dambreak_batch_scenes(256)
    params = [abi.dambreak_params(n, mu) for n, mu in zip(ns, mus)]
    data = [scenes.dambreak(n, scene=k) for k, n in enumerate(ns)]
    b = Batch(params, ns)
    for k, (pos, vel) in enumerate(data):
        b.upload(k, pos, vel)
    b.step(DT, 3)
    b.sync()
    for k, ((sp, g, gs), (pos, vel)) in enumerate(zip(params, data)):
        s = SPH(sp, g, ns[k], gs)
        s.upload(pos, vel)
        s.step(DT, 3)
        for f in ("pos_u", "vel_u", "veleval_u"):
            np.testing.assert_array_equal(b.get(k, f), s.get(f), err_msg="scene %d %s" % (k, f))
        s.close()
    b.close()
