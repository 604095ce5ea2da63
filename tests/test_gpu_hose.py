"""Hoses owned by a context (SPH::addHose / sprayHoses) on the GPU: stepping
a system with a hose equals spraying a standalone hose by hand and pushing
its particles before every step, as SPH::updateGPU does (SPH.cpp:162-166),
bit for bit; the graph path, the eager path and update() agree."""
import ctypes as C

import numpy as np
import pytest

from enjaparticles_gb300 import abi
from enjaparticles_gb300.scenes import dambreak
from enjaparticles_gb300.sph import SPH, Hose

pytestmark = pytest.mark.gpu

DT = 0.001
STATE = ("pos_u", "vel_u", "veleval_u")
CENTER, VELOCITY, RADIUS = (0.5, 0.5, 0.8, 1.0), (0.3, 0.0, -1.0, 0.0), 4.0


def _libc():
    return C.CDLL(None)


def _system(n0, extra, exact=True):
    sp, g, gs = abi.dambreak_params(n0)
    s = SPH(sp, g, n0 + extra, gs, exact=exact)
    pos, vel = dambreak(n0, velocity_sigma=0.05)
    s.upload(pos, vel)
    return s, sp


def _spacing(s, sp):
    return s.lib.sph_settings_round(float(np.float32(sp.rest_distance) / np.float32(sp.simulation_scale)))


def _by_hand(n0, extra, steps, seed, stepper="step"):
    s, sp = _system(n0, extra)
    sx = _spacing(s, sp)
    _libc().srand(seed)
    h = Hose(DT, 600, CENTER, VELOCITY, RADIUS * sx, sx)
    for _ in range(steps):
        pos, v = h.spray()
        if pos.shape[0] and s.getNum() + pos.shape[0] <= s.max_num:
            s.pushParticles(pos, np.repeat(v[None, :], pos.shape[0], 0))
        if stepper == "step":
            s.step(DT, 1)
        else:
            s.update()
            s.integrate(DT)
    return s


@pytest.mark.parametrize("path", ["graph", "eager", "update"])
def test_hose_steps_equal_spraying_by_hand(path):
    n0, extra, steps, seed = 4096, 700, 30, 5
    want = _by_hand(n0, extra, steps, seed)
    s, _ = _system(n0, extra)
    _libc().srand(seed)
    assert s.addHose(600, CENTER, VELOCITY, RADIUS, DT) == 0
    if path == "graph":
        s.step(DT, steps)
    elif path == "eager":
        s.step_eager(DT, steps)
    else:
        for _ in range(steps):
            s.update()
            s.integrate(DT)
    n = s.getNum()
    assert n == want.getNum() and n > n0 + 300
    for f in STATE:
        np.testing.assert_array_equal(s.get(f), want.get(f), err_msg=f)


def test_hose_refill_update_and_capacity():
    """A refilled and moved hose keeps matching the hand-driven one, and a
    spray that would pass max_num is dropped (SPH.cpp:562-567)."""
    n0, extra, seed = 2048, 120, 9
    s, sp = _system(n0, extra)
    sx = _spacing(s, sp)
    _libc().srand(seed)
    idx = s.addHose(100, CENTER, VELOCITY, RADIUS, DT)
    s.step(DT, 5)
    s.updateHose(idx, (0.3, 0.6, 0.7, 1.0), (0.0, 0.4, -0.6, 0.0), 3.0)
    s.refillHose(idx, 400)
    s.step(DT, 12)
    b, _ = _system(n0, extra)
    _libc().srand(seed)
    h = Hose(DT, 100, CENTER, VELOCITY, RADIUS * sx, sx)
    for k in range(17):
        if k == 5:
            h.update((0.3, 0.6, 0.7, 1.0), (0.0, 0.4, -0.6, 0.0), 3.0 * sx, sx)
            h.refill(400)
        pos, v = h.spray()
        if pos.shape[0] and b.getNum() + pos.shape[0] <= b.max_num:
            b.pushParticles(pos, np.repeat(v[None, :], pos.shape[0], 0))
        b.step(DT, 1)
    assert s.getNum() == b.getNum() <= n0 + extra
    for f in STATE:
        np.testing.assert_array_equal(s.get(f), b.get(f), err_msg=f)


def test_hose_state_errors():
    s, _ = _system(1024, 200)
    with pytest.raises(abi.SPHError) as e:
        s.updateHose(0, CENTER, VELOCITY, 1.0)
    assert e.value.code == abi.SPH_EINVAL
    s.addHose(50, CENTER, VELOCITY, 2.0, DT)
    with pytest.raises(abi.SPHError) as e:
        s.adjoint_record(DT, 4, 2)
    assert e.value.code == abi.SPH_ESTATE
    ms = (C.c_float * 32)()
    nk = C.c_int()
    with pytest.raises(abi.SPHError) as e:
        s._ck(s.lib.sph_step_profile(s.ctx, DT, 1, ms, 32, C.byref(nk)))
    assert e.value.code == abi.SPH_ESTATE
