"""The reference's construction path through the C++ class: an RTPSSettings
map -> rtps::SPH(&settings) (the parameters and grid of SPH::calculate,
SPH::updateParams and System::setupDomain) -> addBox -> frames of
update()+integrate() at the "time_step" setting, run by the headless driver.
The same settings through the Python mirror (abi.params_from_settings, the
box's positions as the driver made them) step to the same bits."""
import json
import subprocess

import numpy as np
import pytest

import settings_cases
from enjaparticles_gb300 import abi, build_ext
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,box,steps", [
    ("box5_n16384", (3000, 0.5, 0.5, 0.5, 2.5, 2.5, 2.5), 10),
    ("slab_n100000", (20000, 0.0, 0.0, 0.2, 1.5, 2.0, 1.2), 5),
    ("unit_n4096", (4096, 0.1, 0.1, 0.1, 0.6, 0.6, 0.6), 10),
])
def test_driver_settings_path_equals_python(name, box, steps, tmp_path):
    settings = dict(dict(settings_cases.CASES)[name], time_step=0.001)
    path = tmp_path / "settings.txt"
    path.write_text("".join("%s %s\n" % (k, abi.settings_value(v)) for k, v in settings.items()))
    init, final = tmp_path / "init.bin", tmp_path / "final.bin"
    r = subprocess.run([build_ext.DRIVER, "--settings", str(path), "--box"] + [str(x) for x in box] +
                       ["--steps", str(steps), "--out-init", str(init), "--out", str(final)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    sp, g, gs, spacing = abi.params_from_settings(settings)
    assert np.float32(d["spacing"]) == np.float32(spacing)
    for key, got in (("mass", sp.mass), ("rest_distance", sp.rest_distance),
                     ("smoothing_distance", sp.smoothing_distance), ("simulation_scale", sp.simulation_scale)):
        assert np.float32(d[key]) == np.float32(got), key
    assert d["max_num"] == sp.max_num and d["added"] > 0
    pos0 = np.fromfile(str(init), dtype=np.float32).reshape(-1, 4)
    assert pos0.shape[0] == d["added"]
    s = SPH(sp, g, sp.max_num, gs)
    s.upload(pos0, np.zeros_like(pos0))
    for _ in range(steps):
        s.update()
        s.integrate(0.001)
    got = s.get("pos_u", s.getNum())
    want = np.fromfile(str(final), dtype=np.float32).reshape(-1, 4)
    assert d["num"] == s.getNum()
    np.testing.assert_array_equal(got, want)
    s.close()


def test_driver_settings_with_point_sources_and_euler(tmp_path):
    """The gravity_sources / gravity_mass / gravity_alphas settings and the
    euler integrator setting (System.cpp:260-272, SPH.cpp:89-96) reach the
    system as sph_set_gravity_sources / sph_set_integrator would set them."""
    settings = dict(dict(settings_cases.CASES)["unit_n4096"], time_step=0.001, integrator="euler",
                    gravity_sources="0.3 0.3 0.3 1 0.7 0.5 0.4 1", gravity_mass="0.002 0.001",
                    gravity_alphas="1 0.5")
    path = tmp_path / "settings.txt"
    path.write_text("".join("%s %s\n" % (k, abi.settings_value(v)) for k, v in settings.items()))
    init, final = tmp_path / "init.bin", tmp_path / "final.bin"
    box = (2000, 0.1, 0.1, 0.1, 0.6, 0.6, 0.6)
    r = subprocess.run([build_ext.DRIVER, "--settings", str(path), "--box"] + [str(x) for x in box] +
                       ["--steps", "8", "--out-init", str(init), "--out", str(final)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    pos0 = np.fromfile(str(init), dtype=np.float32).reshape(-1, 4)
    s, dt = SPH.from_settings(settings)
    assert dt == np.float32(0.001)
    s.upload(pos0, np.zeros_like(pos0))
    for _ in range(8):
        s.update()
        s.integrate(dt)
    want = np.fromfile(str(final), dtype=np.float32).reshape(-1, 4)
    np.testing.assert_array_equal(s.get("pos_u", s.getNum()), want)
    s.close()
