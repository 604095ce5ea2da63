"""The autotuner and the launch shapes it chooses among (sph_autotune,
sph_set_launch_config): every candidate shape of the density pass, the
force pass and the cell scan gives the same bits as the default shape, in
exact and default arithmetic, for one system and for a batch; tuning leaves
the state where it was; the choice is remembered per (slots, cells, mode)."""
import itertools

import numpy as np
import pytest

from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.batch import Batch
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu
DT = 0.001
FIELDS = ("pos_u", "vel_u", "veleval_u")
# every candidate, plus shapes that mix them
SHAPES = abi.LAUNCH_CANDIDATES + [(128, 256, 4096), (512, 64, 2048)]


def _run(shape, exact, n=16384, steps=6):
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.1)
    with SPH(sp, g, n, gs, exact=exact) as s:
        if shape is not None:
            s.set_launch_config(*shape)
        s.upload(pos, vel)
        s.step(DT, steps)
        return {f: s.get(f) for f in FIELDS}


@pytest.mark.parametrize("exact", [True, False])
def test_every_shape_gives_the_same_bits(exact):
    ref = _run(None, exact)
    for shape in SHAPES:
        got = _run(shape, exact)
        for f in FIELDS:
            np.testing.assert_array_equal(got[f].view(np.uint32), ref[f].view(np.uint32),
                                          err_msg="%s %s exact=%s" % (shape, f, exact))


def test_autotune_keeps_the_state_and_remembers_its_choice():
    n = 65536
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.1)
    with SPH(sp, g, n, gs) as s:
        s.upload(pos, vel)
        s.step(DT, 3)
        before = {f: s.get(f) for f in FIELDS}
        chosen = s.autotune(DT, steps=2, retime=True)
        assert chosen in [c for c in itertools.product(*zip(*abi.LAUNCH_CANDIDATES))]
        assert s.launch_config() == chosen
        for f in FIELDS:
            np.testing.assert_array_equal(s.get(f), before[f])
        s.step(DT, 2)
        after_tuned = s.get("pos_u")
    with SPH(sp, g, n, gs) as s:
        s.upload(pos, vel)
        s.step(DT, 5)
        np.testing.assert_array_equal(s.get("pos_u"), after_tuned)  # tuning did not advance or perturb
        assert s.autotune(DT, steps=2) == chosen  # remembered for this (slots, cells, mode)


def test_bad_shapes_are_rejected():
    sp, g, gs = abi.dambreak_params(4096)
    with SPH(sp, g, 4096, gs) as s:
        keep = s.launch_config()
        for bad in [(64, 128, 4096), (256, 32, 4096), (256, 128, 1024), (256, 128, 4095)]:
            with pytest.raises(abi.SPHError) as e:
                s.set_launch_config(*bad)
            assert e.value.code == abi.SPH_EINVAL
        assert s.launch_config() == keep
        with pytest.raises(abi.SPHError) as e:
            s.autotune(DT, steps=1)  # no particles
        assert e.value.code == abi.SPH_ESTATE


def test_batch_shapes_and_autotune():
    ns = [3000, 7000, 2048]
    params = [abi.dambreak_params(n, 0.01 + 0.01 * k) for k, n in enumerate(ns)]
    data = [scenes.dambreak(n, scene=k, velocity_sigma=0.05) for k, n in enumerate(ns)]

    def run(shape, tune=False):
        b = Batch(params, ns, exact=True)
        for k, (p, v) in enumerate(data):
            b.upload(k, p, v)
        chosen = None
        if tune:
            chosen = b.autotune(DT, steps=2, retime=True)
        elif shape is not None:
            b.set_launch_config(*shape)
        b.step(DT, 4)
        out = [b.get(k, "pos_u") for k in range(len(ns))]
        b.close()
        return out, chosen

    ref, _ = run(None)
    for shape in SHAPES:
        got, _ = run(shape)
        for k in range(len(ns)):
            np.testing.assert_array_equal(got[k], ref[k], err_msg="%s scene %d" % (shape, k))
    got, chosen = run(None, tune=True)
    assert chosen is not None
    for k in range(len(ns)):
        np.testing.assert_array_equal(got[k], ref[k])
