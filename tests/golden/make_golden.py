#!/usr/bin/env python3
"""Generate the golden fixtures of tests/golden/ from the reference's own kernels.

Needs oracle/_ref/librtps_ref.so (python oracle/ref/build_ref.py, which reads
the reference tree).  Every array here comes from the reference's OpenCL
kernels compiled for the host and driven in SPH::updateGPU order by
tests/ref_driver.py, with the (unstable) bitonic sort canonicalised within
equal keys by original index.  The inputs are the seeded scenes of
enjaparticles_gb300.scenes and the parameter blocks of sph_dambreak_params;
both are stored too, so the fixtures stand alone.

Fixtures
  stages_n4096.npz   dam-break rule at N=4096, v0 ~ N(0, 0.1^2): every stage
                     output of step 1, and pos/vel/veleval after steps 2 and 10
  ragged_n1000.npz   N=1000 (not a multiple of any block size), 3 steps
  outofgrid_n512.npz N=512 with 37 particles placed outside the grid: the
                     out-of-grid deletion path of SPH.cpp:220-250, 2 steps
  cfg0_n16384.npz    the 16,384-particle dam break: pos/vel after 1, 10, 100 steps
  gravity_n2048.npz  N=2048, v0 ~ N(0, 0.1^2), two point gravity sources
                     (gravity.cl), with the leapfrog and with the Euler
                     integrator (euler.cl): step 1 forces, state after 1 and 5
  triangles_n2048.npz N=2048, v0 ~ N(0, 0.3^2), the 524-triangle ramp and box
                     mesh of scenes.ramp_and_box_mesh (collision_tri.cl after
                     the walls): step 1 forces before and after the triangle
                     stage, state after 1, 5 and 20 steps
  surface_n4096.npz  N=4096, v0 ~ N(0, 0.2^2), after 20 steps: the reference's
                     colour field (colorfield.cl) at res 16 and 32 and its
                     marching-cubes mesh (classifycubes/constructhp/
                     traversehp.cl) at isolevel 0.0001
  hose_sprays.npz    the reference's Hose (common/Hose.cpp, addDiscRandom)
                     through the scripts of tests/hose_cases.py, rand()
                     seeded per script: counts, positions, push velocities
  addrect.npz        the reference's addRect (domain/IV.cpp) for the boxes of
                     tests/addrect_cases.py at the getSpacing() of each
                     system (System::addBox): the spacing and the points
  settings.npz       the reference's settings path (RTPSSettings.cpp,
                     SPHSettings.cpp SPH::calculate / updateParams,
                     Domain::calculateCells as System::setupDomain drives
                     it) for the settings maps of tests/settings_cases.py:
                     the keys and values, the SPHParams and both GridParams
                     bytes and the spacing
Usage: python tests/golden/make_golden.py [--only NAME ...]
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from enjaparticles_gb300 import abi, scenes  # noqa: E402
import ref_driver  # noqa: E402

DT = 0.001


def params_blob(sp, g, gs):
    return {"sphp": np.frombuffer(bytes(sp), np.uint8).copy(), "grid": np.frombuffer(bytes(g), np.uint8).copy(),
            "grid_scaled": np.frombuffer(bytes(gs), np.uint8).copy()}


def state(R, prefix):
    n = R.num
    return {prefix + "pos_u": R.pos_u[:n].copy(), prefix + "vel_u": R.vel_u[:n].copy(),
            prefix + "veleval_u": R.veleval_u[:n].copy(), prefix + "num": np.int32(n)}


def stages_fixture(n, sigma, steps_after=(2, 10)):
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=sigma)
    R = ref_driver.RefSystem(sp, g, gs, n)
    R.upload(pos, vel)
    out = dict(params_blob(sp, g, gs))
    out.update({"in_pos": pos, "in_vel": vel, "dt": np.float32(DT)})
    R.update()
    out.update({"s1_hash_keys": R.trace["hash_keys"], "s1_sort_hashes": R.keys[:n].copy(),
                "s1_sort_indices": R.idx[:n].copy(), "s1_cell_start": R.start.copy(), "s1_cell_end": R.end.copy(),
                "s1_nc": np.int32(R.trace["nc"]), "s1_pos_s": R.pos_s[:n].copy(), "s1_vel_s": R.vel_s[:n].copy(),
                "s1_veleval_s": R.veleval_s[:n].copy(), "s1_density_s": R.density_s[:n].copy(),
                "s1_force_pre": R.trace["force_pre_collision"], "s1_force_s": R.force_s[:n].copy(),
                "s1_xsph_s": R.xsph_s[:n].copy()})
    R.integrate(DT)
    out.update(state(R, "s1_"))
    done = 1
    for k in steps_after:
        R.step(DT, k - done)
        done = k
        out.update(state(R, "s%d_" % k))
    return out


def outofgrid_fixture():
    n = 512
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.05)
    rng_u = scenes.uniform(77, 37 * 3).reshape(37, 3)
    far = np.where(rng_u < 0.5, -0.6 - rng_u, 1.6 + rng_u).astype(np.float32)
    sel = (np.arange(37) * 13 + 5) % n
    pos[sel, :3] = far
    R = ref_driver.RefSystem(sp, g, gs, n)
    R.upload(pos, vel)
    out = dict(params_blob(sp, g, gs))
    out.update({"in_pos": pos, "in_vel": vel, "dt": np.float32(DT)})
    R.update()
    out.update({"s1_nc": np.int32(R.trace["nc"]), "s1_deleted_pos": R.deleted_pos.copy(),
                "s1_deleted_vel": R.deleted_vel.copy(), "s1_sort_indices": R.idx[:R.num].copy(),
                "s1_density_s": R.density_s[:R.num].copy()})
    R.integrate(DT)
    out.update(state(R, "s1_"))
    R.step(DT, 1)
    out.update(state(R, "s2_"))
    return out


def cfg0_fixture():
    n = 16384
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n)
    R = ref_driver.RefSystem(sp, g, gs, n)
    R.upload(pos, vel)
    out = dict(params_blob(sp, g, gs))
    out.update({"in_pos": pos, "in_vel": vel, "dt": np.float32(DT)})
    done = 0
    for k in (1, 10, 100):
        R.step(DT, k - done)
        done = k
        out["s%d_pos_u" % k] = R.pos_u[:n].copy()
        out["s%d_vel_u" % k] = R.vel_u[:n].copy()
    return out


# Two point sources: one above the fluid pulling it up, one inside it, whose
# pull turns into a push within 0.5 * simulation_scale (gravity.cl:26-31).
GRAV_POINTS = np.array([[0.25, 0.25, 0.9, 1.0], [0.2, 0.3, 0.15, 1.0]], np.float32)
GRAV_MASSES = np.array([4.0, 0.5], np.float32)
GRAV_ALPHAS = np.array([2.0, 1.5], np.float32)


def gravity_fixture():
    n = 2048
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.1)
    out = dict(params_blob(sp, g, gs))
    out.update({"in_pos": pos, "in_vel": vel, "dt": np.float32(DT), "grav_points": GRAV_POINTS,
                "grav_masses": GRAV_MASSES, "grav_alphas": GRAV_ALPHAS})
    for integ in ("leapfrog", "euler"):
        R = ref_driver.RefSystem(sp, g, gs, n)
        R.set_gravity(GRAV_POINTS, GRAV_MASSES, GRAV_ALPHAS)
        R.integrator = integ
        R.upload(pos, vel)
        R.update()
        out["%s_s1_force_sph" % integ] = R.trace["force_sph"]
        out["%s_s1_force_pre" % integ] = R.trace["force_pre_collision"]
        out["%s_s1_force_s" % integ] = R.force_s[:n].copy()
        R.integrate(DT)
        out.update(state(R, "%s_s1_" % integ))
        R.step(DT, 4)
        out.update(state(R, "%s_s5_" % integ))
    return out


def triangles_fixture():
    n = 2048
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.3)
    tris = scenes.ramp_and_box_mesh()
    out = dict(params_blob(sp, g, gs))
    out.update({"in_pos": pos, "in_vel": vel, "dt": np.float32(DT), "triangles": tris})
    R = ref_driver.RefSystem(sp, g, gs, n)
    R.set_triangles(tris, DT)
    R.upload(pos, vel)
    R.update()
    out["s1_force_pre_tri"] = R.trace["force_pre_triangles"]
    out["s1_force_s"] = R.force_s[:n].copy()
    out["s1_sort_indices"] = R.idx[:n].copy()
    R.integrate(DT)
    out.update(state(R, "s1_"))
    R.step(DT, 4)
    out.update(state(R, "s5_"))
    R.step(DT, 15)
    out.update(state(R, "s20_"))
    return out


def surface_fixture():
    import ctypes as C
    n, steps = 4096, 20
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.2)
    R = ref_driver.RefSystem(sp, g, gs, n)
    R.upload(pos, vel)
    R.step(DT, steps)
    out = dict(params_blob(sp, g, gs))
    out.update({"in_pos": pos, "in_vel": vel, "dt": np.float32(DT), "steps": np.int32(steps)})
    L = R.lib
    P = lambda a: a.ctypes.data
    spn = R.sp
    spn.num = R.num
    for res in (16, 32):
        field = np.zeros(res ** 3, np.float32)
        L.ref_colorfield(res, R.num, P(R.pos_s), P(R.density_s), P(R.start), P(R.end), C.addressof(gs),
                         C.addressof(spn), P(field), None)
        cap = 200000
        v = np.zeros((cap, 9), np.float32)
        nr = np.zeros((cap, 9), np.float32)
        L.ref_marching_cubes.restype = C.c_int
        L.ref_marching_cubes.argtypes = [C.c_int, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_void_p]
        tot = L.ref_marching_cubes(res, P(field), 0.0001, P(v), P(nr), cap, None)
        out["field%d" % res] = field
        out["mesh%d_vertices" % res] = v[:tot].reshape(-1, 3, 3).copy()
        out["mesh%d_normals" % res] = nr[:tot].reshape(-1, 3, 3).copy()
    return out


def hose_fixture():
    import hose_cases
    out = {}
    for name in hose_cases.SCRIPTS:
        counts, pos, vel = hose_cases.run_script(name, hose_cases.RefHose)
        out.update({name + "_counts": counts, name + "_pos": pos, name + "_vel": vel})
    return out


def settings_fixture():
    import settings_cases
    out = {}
    for name, settings in settings_cases.CASES:
        items = [(k, abi.settings_value(v)) for k, v in settings.items()]
        sp, g, gs, spacing, size = ref_driver.params_from_settings(items)
        out[name + "/keys"] = np.array([k for k, _ in items])
        out[name + "/values"] = np.array([v for _, v in items])
        out[name + "/sphp"] = np.frombuffer(sp, np.uint8).copy()
        out[name + "/grid"] = np.frombuffer(g, np.uint8).copy()
        out[name + "/grid_scaled"] = np.frombuffer(gs, np.uint8).copy()
        out[name + "/spacing"] = np.float32(spacing)
    return out


def addrect_fixture():
    import addrect_cases
    import oracle_bind
    out = {}
    for name, n, scale, num, lo, hi in addrect_cases.CASES:
        sp, _ = addrect_cases.scene_params(n, scale)
        sx = addrect_cases.spacing(sp)
        out[name + "_spacing"] = np.float32(sx)
        out[name + "_points"] = oracle_bind.ref_add_rect(num, lo, hi, sx, 1.0)
    return out


FIXTURES = {
    "stages_n4096.npz": lambda: stages_fixture(4096, 0.1),
    "ragged_n1000.npz": lambda: stages_fixture(1000, 0.1, steps_after=(3,)),
    "outofgrid_n512.npz": outofgrid_fixture,
    "cfg0_n16384.npz": cfg0_fixture,
    "gravity_n2048.npz": gravity_fixture,
    "triangles_n2048.npz": triangles_fixture,
    "hose_sprays.npz": hose_fixture,
    "surface_n4096.npz": surface_fixture,
    "addrect.npz": addrect_fixture,
    "settings.npz": settings_fixture,
}


def main():
    names = sys.argv[sys.argv.index("--only") + 1:] if "--only" in sys.argv else list(FIXTURES)
    for name in names:
        np.savez_compressed(os.path.join(HERE, name), **FIXTURES[name]())
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
