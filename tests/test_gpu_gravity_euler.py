"""Point-source gravity (gravity.cl) and the Euler integrator (euler.cl) on the
GPU against the golden fixture made from the reference's own kernels
(tests/golden/gravity_n2048.npz): bit-exact in exact arithmetic, staged and
fused; within the step tolerances in the default arithmetic."""
import numpy as np
import pytest

import golden_io
from enjaparticles_gb300 import abi
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5


def normwise(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def _system(d, sp, g, gs, integrator, exact):
    n = d["in_pos"].shape[0]
    s = SPH(sp, g, n, gs, exact=exact)
    s.setGravitySources(d["grav_points"], d["grav_masses"], d["grav_alphas"])
    s.setIntegrator(integrator)
    s.upload(d["in_pos"], d["in_vel"])
    return s


@pytest.mark.parametrize("integrator", ["leapfrog", "euler"])
def test_staged_exact_matches_reference_golden(integrator):
    d, sp, g, gs = golden_io.load("gravity_n2048.npz")
    s = _system(d, sp, g, gs, integrator, exact=True)
    dt = float(d["dt"])
    s.update()
    np.testing.assert_array_equal(s.get("force_s"), d["%s_s1_force_s" % integrator])
    s.integrate(dt)
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(s.get(f), d["%s_s1_%s" % (integrator, f)], err_msg=f)
    for _ in range(4):
        s.update()
        s.integrate(dt)
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(s.get(f), d["%s_s5_%s" % (integrator, f)], err_msg=f)


@pytest.mark.parametrize("integrator", ["leapfrog", "euler"])
def test_fused_exact_matches_reference_golden(integrator):
    d, sp, g, gs = golden_io.load("gravity_n2048.npz")
    s = _system(d, sp, g, gs, integrator, exact=True)
    dt = float(d["dt"])
    s.step(dt, 1)
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(s.get(f), d["%s_s1_%s" % (integrator, f)], err_msg=f)
    s.step(dt, 4)
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(s.get(f), d["%s_s5_%s" % (integrator, f)], err_msg=f)


@pytest.mark.parametrize("integrator", ["leapfrog", "euler"])
def test_fast_within_tolerance_of_reference_golden(integrator):
    d, sp, g, gs = golden_io.load("gravity_n2048.npz")
    s = _system(d, sp, g, gs, integrator, exact=False)
    dt = float(d["dt"])
    s.update()
    assert normwise(s.get("force_s")[:, :3], d["%s_s1_force_s" % integrator][:, :3]) <= FORCE_RTOL
    s2 = _system(d, sp, g, gs, integrator, exact=False)
    s2.step(dt, 5)
    h = sp.smoothing_distance
    assert np.abs(s2.get("pos_u") - d["%s_s5_pos_u" % integrator]).max() <= 1e-4 * h


def test_sources_and_integrator_errors():
    d, sp, g, gs = golden_io.load("gravity_n2048.npz")
    n = d["in_pos"].shape[0]
    s = SPH(sp, g, n, gs)
    too_many = np.zeros((abi.SPH_MAX_GRAVITY_SOURCES + 1, 4), np.float32)
    with pytest.raises(abi.SPHError) as e:
        s.setGravitySources(too_many, np.ones(len(too_many)), np.ones(len(too_many)))
    assert e.value.code == abi.SPH_EINVAL
    with pytest.raises(abi.SPHError) as e:
        s._ck(s.lib.sph_set_integrator(s.ctx, 7))
    assert e.value.code == abi.SPH_EINVAL
    s.setGravitySources(d["grav_points"], d["grav_masses"], d["grav_alphas"])
    s.upload(d["in_pos"], d["in_vel"])
    with pytest.raises(abi.SPHError) as e:
        s.adjoint_record(float(d["dt"]), 4, 2)
    assert e.value.code == abi.SPH_ESTATE
    s.setGravitySources(np.zeros((0, 4)), np.zeros(0), np.zeros(0))  # removed again
    s.adjoint_record(float(d["dt"]), 4, 2)
