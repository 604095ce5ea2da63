"""GPU parity of whole steps through the C ABI: the staged update()+integrate()
path, the fused CUDA-graph step and the eager fused step, against the oracle
and the reference golden rollouts; the out-of-grid deletion path; argument
errors."""
import numpy as np
import pytest

import golden_io
import oracle_bind as ob
from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu
DT = 0.001


def state(s):
    return {f: s.get(f) for f in ("pos_u", "vel_u", "veleval_u")}


def test_fused_exact_equals_staged_exact_equals_reference_golden():
    d, sp, g, gs = golden_io.load("stages_n4096.npz")
    n = d["in_pos"].shape[0]
    a = SPH(sp, g, n, gs, exact=True)
    b = SPH(sp, g, n, gs, exact=True)
    c = SPH(sp, g, n, gs, exact=True)
    for s in (a, b, c):
        s.upload(d["in_pos"], d["in_vel"])
    done = 0
    for k in (1, 2, 10):
        for _ in range(k - done):
            a.update()
            a.integrate(DT)
        b.step(DT, k - done)
        c.step_eager(DT, k - done)
        done = k
        sa, sb, sc = state(a), state(b), state(c)
        for f in sa:
            np.testing.assert_array_equal(sa[f], d["s%d_%s" % (k, f)], err_msg="staged %d %s" % (k, f))
            np.testing.assert_array_equal(sb[f], sa[f], err_msg="graph %d %s" % (k, f))
            np.testing.assert_array_equal(sc[f], sa[f], err_msg="eager %d %s" % (k, f))


def test_cfg0_fast_rollout_within_tolerance_of_reference_golden():
    """16,384-particle dam break, default (fast) arithmetic: after 10 steps the
    maximum position error stays within 1e-4*h of the reference kernels; the
    exact mode reproduces all 100 steps bit for bit."""
    d, sp, g, gs = golden_io.load("cfg0_n16384.npz")
    n = d["in_pos"].shape[0]
    h = sp.smoothing_distance
    fast = SPH(sp, g, n, gs)
    fast.upload(d["in_pos"], d["in_vel"])
    fast.step(DT, 1)
    assert np.abs(fast.get("pos_u") - d["s1_pos_u"]).max() <= 1e-4 * h
    fast.step(DT, 9)
    err10 = np.abs(fast.get("pos_u") - d["s10_pos_u"]).max()
    assert err10 <= 1e-4 * h, err10 / h
    ex = SPH(sp, g, n, gs, exact=True)
    ex.upload(d["in_pos"], d["in_vel"])
    ex.step(DT, 100)
    np.testing.assert_array_equal(ex.get("pos_u"), d["s100_pos_u"])
    np.testing.assert_array_equal(ex.get("vel_u"), d["s100_vel_u"])


def test_out_of_grid_deletion_matches_reference_golden():
    d, sp, g, gs = golden_io.load("outofgrid_n512.npz")
    n = d["in_pos"].shape[0]
    nc = int(d["s1_nc"])
    for mode in ("staged", "graph"):
        s = SPH(sp, g, n, gs, exact=True)
        s.upload(d["in_pos"], d["in_vel"])
        if mode == "staged":
            s.update()
            s.integrate(DT)
        else:
            s.step(DT, 1)
        assert s.getNum() == nc
        dp, dv = s.getDeleted()
        np.testing.assert_array_equal(dp, d["s1_deleted_pos"])
        np.testing.assert_array_equal(dv, d["s1_deleted_vel"])
        np.testing.assert_array_equal(s.get("sort_indices"), d["s1_sort_indices"])
        np.testing.assert_array_equal(s.get("density_s"), d["s1_density_s"])
        for f in ("pos_u", "vel_u", "veleval_u"):
            np.testing.assert_array_equal(s.get(f), d["s1_" + f], err_msg="%s %s" % (mode, f))
        if mode == "staged":
            s.update()
            s.integrate(DT)
        else:
            s.step(DT, 1)
        for f in ("pos_u", "vel_u", "veleval_u"):
            np.testing.assert_array_equal(s.get(f), d["s2_" + f], err_msg="%s step2 %s" % (mode, f))


def test_fast_rollout_random_velocities_against_oracle():
    n = 65536
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.1)
    s = SPH(sp, g, n, gs)
    s.upload(pos, vel)
    s.step(DT, 10)
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(pos, vel)
    sim.step(DT, 10)
    err = np.abs(s.get("pos_u") - sim.get("pos_u")).max()
    assert err <= 1e-4 * sp.smoothing_distance, err / sp.smoothing_distance


def test_push_particles_and_zero_particles():
    n = 2048
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n)
    s = SPH(sp, g, n, gs, exact=True)
    s.upload(pos[:0], vel[:0])
    s.step(DT, 3)  # nothing to do
    assert s.getNum() == 0
    s.pushParticles(pos[:1000], vel[:1000])
    s.pushParticles(pos[1000:], vel[1000:])
    assert s.getNum() == n
    s.step(DT, 2)
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(pos, vel)
    sim.step(DT, 2)
    np.testing.assert_array_equal(s.get("pos_u"), sim.get("pos_u"))
    with pytest.raises(abi.SPHError) as e:
        s.pushParticles(pos[:1], vel[:1])
    assert e.value.code == abi.SPH_EINVAL


def test_argument_errors_are_reported():
    n = 128
    sp, g, gs = abi.dambreak_params(n)
    s = SPH(sp, g, n, gs)
    pos, vel = scenes.dambreak(2 * n)
    with pytest.raises(abi.SPHError) as e:
        s.upload(pos, vel)
    assert e.value.code == abi.SPH_EINVAL
    bad = abi.SPHParams.from_buffer_copy(bytes(sp))
    bad.smoothing_distance = float("nan")
    with pytest.raises(abi.SPHError):
        s.updateParams(bad)
    s.upload(pos[:n], vel[:n])
    s.step(DT, 1)
    s.sync()
    big = abi.GridParams.from_buffer_copy(bytes(g))
    big.nb_cells = 1 << 25
    with pytest.raises(abi.SPHError):
        SPH(sp, big, n, gs)


def test_step_profile_is_the_same_step():
    """sph_step_profile (the fused step launched kernel by kernel, with events
    between the launches) computes the graph step bit for bit, and names its
    eight launches."""
    import ctypes as C
    n = 16384
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.05)
    a = SPH(sp, g, n, gs, exact=True)
    a.upload(pos, vel)
    a.step(DT, 3)
    b = SPH(sp, g, n, gs, exact=True)
    b.upload(pos, vel)
    ms = (C.c_float * 32)()
    nk = C.c_int()
    b._ck(b.lib.sph_step_profile(b.ctx, DT, 3, ms, 32, C.byref(nk)))
    assert nk.value == 8
    names = [b.lib.sph_profile_kernel_name(b.ctx, k).decode() for k in range(nk.value)]
    assert names == ["k_cell_count", "k_cell_totals", "k_cell_scan", "k_cell_place", "k_cell_permute", "k_density",
                     "k_step_velocities", "k_force(fused collision+leapfrog)"]
    assert all(ms[k] > 0.0 for k in range(nk.value))
    sa, sb = state(a), state(b)
    for f in sa:
        np.testing.assert_array_equal(sb[f], sa[f], err_msg=f)
    a.close()
    b.close()
