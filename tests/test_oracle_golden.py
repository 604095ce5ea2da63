"""The CPU oracle against the golden fixtures made from the reference's own
kernels (tests/golden/make_golden.py): every stage and every rollout must be
bit-identical (within-cell order canonicalised by original index)."""
import ctypes as C

import numpy as np
import pytest

import golden_io
import oracle_bind as ob
from mesh_cases import near_mesh_particles

P = ob.ptr


def run_stages(d, sp, g, gs):
    O = ob.oracle()
    n = d["in_pos"].shape[0]
    pos, vel = d["in_pos"], d["in_vel"]
    keys = np.empty(n, np.uint32)
    idx = np.empty(n, np.uint32)
    O.oracle_hash(n, P(pos), C.addressof(g), P(keys), P(idx))
    out = {"hash_keys": keys.copy()}
    O.oracle_sort(n, P(keys), P(idx))
    out["sort_hashes"], out["sort_indices"] = keys, idx
    start = np.full(g.nb_cells + 1, 666, np.uint32)
    end = np.full(g.nb_cells + 1, 666, np.uint32)
    out["nc"] = O.oracle_cellindices(n, P(keys), P(start), P(end), g.nb_cells)
    out["cell_start"], out["cell_end"] = start, end
    ve = np.zeros_like(pos)
    ps, vs, ves = np.empty_like(pos), np.empty_like(pos), np.empty_like(pos)
    O.oracle_permute(n, P(idx), P(pos), P(vel), P(ve), P(ps), P(vs), P(ves))
    out.update(pos_s=ps, vel_s=vs, veleval_s=ves)
    dens = np.empty(n, np.float32)
    O.oracle_density(0, n, P(ps), P(start), P(end), C.addressof(gs), C.addressof(sp), P(dens), None)
    out["density_s"] = dens
    f, x = np.empty_like(pos), np.empty_like(pos)
    O.oracle_force(0, n, P(ps), P(dens), P(ves), P(start), P(end), C.addressof(gs), C.addressof(sp), P(f), P(x))
    out["force_pre"], out["xsph_s"] = f.copy(), x
    O.oracle_collision(0, n, P(ps), P(vs), P(f), C.addressof(gs), C.addressof(sp))
    out["force_s"] = f
    pu, vu, eu = pos.copy(), vel.copy(), ve.copy()
    O.oracle_leapfrog(0, n, P(ps), P(vs), P(f), P(x), P(idx), C.addressof(sp), float(d["dt"]), P(pu), P(vu), P(eu))
    out.update(pos_u=pu, vel_u=vu, veleval_u=eu)
    return out


@pytest.mark.parametrize("name", ["stages_n4096.npz", "ragged_n1000.npz"])
def test_oracle_stages_match_reference_golden(name):
    d, sp, g, gs = golden_io.load(name)
    o = run_stages(d, sp, g, gs)
    for k in ("hash_keys", "sort_hashes", "sort_indices", "cell_start", "cell_end", "pos_s", "vel_s", "veleval_s",
              "density_s", "force_pre", "force_s", "xsph_s", "pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(o[k], d["s1_" + k], err_msg=k)
    assert o["nc"] == int(d["s1_nc"])


@pytest.mark.parametrize("name,steps", [("stages_n4096.npz", (1, 2, 10)), ("ragged_n1000.npz", (1, 3))])
def test_oracle_rollout_matches_reference_golden(name, steps):
    d, sp, g, gs = golden_io.load(name)
    n = d["in_pos"].shape[0]
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(d["in_pos"], d["in_vel"])
    done = 0
    for k in steps:
        sim.step(float(d["dt"]), k - done)
        done = k
        for f in ("pos_u", "vel_u", "veleval_u"):
            np.testing.assert_array_equal(sim.get(f), d["s%d_%s" % (k, f)], err_msg="step %d %s" % (k, f))


def test_oracle_out_of_grid_deletion_matches_reference_golden():
    d, sp, g, gs = golden_io.load("outofgrid_n512.npz")
    n = d["in_pos"].shape[0]
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(d["in_pos"], d["in_vel"])
    sim.update()
    nc = int(d["s1_nc"])
    assert 0 <= nc < n and sim.num == nc
    assert sim.lib.oracle_sim_last_nc(sim.h) == nc
    dp = np.empty((n - nc, 4), np.float32)
    dv = np.empty((n - nc, 4), np.float32)
    assert sim.lib.oracle_sim_deleted(sim.h, P(dp), P(dv), n - nc) == n - nc
    np.testing.assert_array_equal(dp, d["s1_deleted_pos"])
    np.testing.assert_array_equal(dv, d["s1_deleted_vel"])
    np.testing.assert_array_equal(sim.get("sort_indices"), d["s1_sort_indices"])
    np.testing.assert_array_equal(sim.get("density_s"), d["s1_density_s"])
    sim.integrate(float(d["dt"]))
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(sim.get(f), d["s1_" + f])
    sim.step(float(d["dt"]), 1)
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(sim.get(f), d["s2_" + f])


@pytest.mark.slow
def test_oracle_cfg0_rollout_matches_reference_golden():
    d, sp, g, gs = golden_io.load("cfg0_n16384.npz")
    n = d["in_pos"].shape[0]
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(d["in_pos"], d["in_vel"])
    done = 0
    for k in (1, 10, 100):
        sim.step(float(d["dt"]), k - done)
        done = k
        np.testing.assert_array_equal(sim.get("pos_u"), d["s%d_pos_u" % k])
        np.testing.assert_array_equal(sim.get("vel_u"), d["s%d_vel_u" % k])


@pytest.mark.parametrize("integrator", ["leapfrog", "euler"])
def test_oracle_gravity_sources_and_integrators_match_reference_golden(integrator):
    """Point-source gravity (gravity.cl) after force, and both integrators of
    SPH::integrate (leapfrog.cl, euler.cl): step-1 forces and the state after
    1 and 5 steps equal the reference kernels' bit for bit."""
    d, sp, g, gs = golden_io.load("gravity_n2048.npz")
    n = d["in_pos"].shape[0]
    sim = ob.OracleSim(sp, g, gs, n)
    sim.set_gravity(d["grav_points"], d["grav_masses"], d["grav_alphas"])
    sim.set_integrator(1 if integrator == "euler" else 0)
    sim.upload(d["in_pos"], d["in_vel"])
    sim.update()
    np.testing.assert_array_equal(sim.get("force_s"), d["%s_s1_force_s" % integrator])
    sim.integrate(float(d["dt"]))
    for k, done in ((1, 1), (5, 5)):
        if k > 1:
            sim.step(float(d["dt"]), 4)
        for f in ("pos_u", "vel_u", "veleval_u"):
            np.testing.assert_array_equal(sim.get(f), d["%s_s%d_%s" % (integrator, k, f)], err_msg=f)


@pytest.mark.skipif(not ob.ref_available(), reason="reference kernels not built here (needs the reference tree)")
def test_oracle_gravity_and_euler_equal_reference_kernels_on_random_data():
    from enjaparticles_gb300.scenes import uniform
    R = ob.ref()
    O = ob.oracle()
    n, nsrc = 3000, 5
    pos = (uniform(501, 4 * n).reshape(n, 4) * 1.2 - 0.1).astype(np.float32)
    pos[:, 3] = 1.0
    pts = (uniform(502, 4 * nsrc).reshape(nsrc, 4)).astype(np.float32)
    m = (uniform(503, nsrc) * 3).astype(np.float32)
    a = (uniform(504, nsrc) * 2 - 0.5).astype(np.float32)
    f0 = ((uniform(505, 4 * n).reshape(n, 4) - 0.5) * 40).astype(np.float32)
    fr, fo = f0.copy(), f0.copy()
    R.ref_gravity(n, nsrc, P(pts), P(m), P(a), P(pos), P(fr), 1.0)
    O.oracle_gravity(0, n, nsrc, P(pts), P(m), P(a), P(pos), P(fo), 1.0)
    np.testing.assert_array_equal(fo, fr)
    sp, _, _ = __import__("enjaparticles_gb300.abi", fromlist=["abi"]).dambreak_params(n)
    vel = ((uniform(506, 4 * n).reshape(n, 4) - 0.5)).astype(np.float32)
    big = f0 * 30  # some accelerations above the Euler limit of 600
    idx = np.random.default_rng(7).permutation(n).astype(np.uint32)
    pr, vr = np.zeros_like(pos), np.zeros_like(pos)
    po, vo = np.zeros_like(pos), np.zeros_like(pos)
    R.ref_euler(n, P(pr), P(pos), P(vr), P(vel), P(big), P(idx), C.addressof(sp), 0.001)
    O.oracle_euler(0, n, P(pos), P(vel), P(big), P(idx), C.addressof(sp), 0.001, P(po), P(vo))
    np.testing.assert_array_equal(po, pr)
    np.testing.assert_array_equal(vo, vr)


@pytest.mark.skipif(not ob.ref_available(), reason="reference kernels not built here (needs the reference tree)")
@pytest.mark.parametrize("scale", [1.0, 0.05])
def test_oracle_triangle_collision_equals_reference_kernel_on_random_data(scale):
    """collision_triangle (collision_tri.cl:436-520): 524 triangles (three
    shared-memory chunks of 220), particles around every face moving in every
    direction, zero velocities included; simulation_scale 1 and 0.05."""
    from enjaparticles_gb300 import abi
    from enjaparticles_gb300.scenes import ramp_and_box_mesh, uniform
    R, O = ob.ref(), ob.oracle()
    n = 3000
    sp, _, _ = abi.dambreak_params(n)
    tris = ramp_and_box_mesh()
    if scale != 1.0:
        sp.simulation_scale = scale
        tris = tris.copy()
        tris[:, :3, :3] /= scale
    tris = np.ascontiguousarray(tris.reshape(-1, 16))
    pos, vel = near_mesh_particles(tris, n, sp.boundary_distance, scale, 601)
    f0 = ((uniform(605, 4 * n).reshape(n, 4) - 0.5) * 40).astype(np.float32)
    fr, fo = f0.copy(), f0.copy()
    R.ref_collision_triangles(n, P(pos), P(vel), P(fr), P(tris), tris.shape[0], C.addressof(sp), 0.001)
    O.oracle_collision_triangles(0, n, P(pos), P(vel), P(fo), P(tris), tris.shape[0], C.addressof(sp))
    hit = np.abs(fr[:, :3] - f0[:, :3]).max(1) > 0
    assert hit.sum() > n // 5  # a good share of the particles touch the mesh
    np.testing.assert_array_equal(fo, fr)


def test_oracle_triangle_mesh_rollout_matches_reference_golden():
    """SPH::collision with a triangle mesh loaded (collision_wall, then
    collision_triangle; SPH.cpp:303-336): step-1 force and the state after 1,
    5 and 20 steps equal the reference kernels' bit for bit."""
    d, sp, g, gs = golden_io.load("triangles_n2048.npz")
    n = d["in_pos"].shape[0]
    sim = ob.OracleSim(sp, g, gs, n)
    sim.set_triangles(d["triangles"])
    sim.upload(d["in_pos"], d["in_vel"])
    sim.update()
    np.testing.assert_array_equal(sim.get("force_s"), d["s1_force_s"])
    sim.integrate(float(d["dt"]))
    done = 1
    for k in (1, 5, 20):
        sim.step(float(d["dt"]), k - done)
        done = k
        for f in ("pos_u", "vel_u", "veleval_u"):
            np.testing.assert_array_equal(sim.get(f), d["s%d_%s" % (k, f)], err_msg="step %d %s" % (k, f))


def _sorted_state(n=4096, steps=3):
    """pos_s, density_s, cell_start, cell_end of a dam break after `steps`
    oracle steps and one more update."""
    from enjaparticles_gb300 import abi, scenes
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.2)
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(pos, vel)
    sim.step(0.001, steps)
    sim.update()
    return (sp, g, gs, sim.num, sim.get("pos_s"), sim.get("density_s"), sim.get("cell_start", g.nb_cells + 1),
            sim.get("cell_end", g.nb_cells + 1))


@pytest.mark.skipif(not ob.ref_available(), reason="reference kernels not built here (needs the reference tree)")
@pytest.mark.parametrize("res", [2, 7, 16, 32])
def test_oracle_colorfield_equals_reference_kernel(res):
    """colorfield_update (colorfield.cl) at res^3 sample points over the
    scaled grid bounds: the oracle equals the reference's kernel bit for bit."""
    sp, g, gs, n, ps, dens, cs, ce = _sorted_state()
    R, O = ob.ref(), ob.oracle()
    want = np.zeros(res ** 3, np.float32)
    R.ref_colorfield(res, n, P(ps), P(dens), P(cs), P(ce), C.addressof(gs), C.addressof(sp), P(want), None)
    got = np.zeros(res ** 3, np.float32)
    O.oracle_colorfield(0, res, P(ps), P(dens), P(cs), P(ce), C.addressof(gs), C.addressof(sp), P(got))
    assert (want > 0).sum() > res ** 3 // 20
    np.testing.assert_array_equal(got, want)
