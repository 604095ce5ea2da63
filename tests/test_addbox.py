"""System::addBox (System.cpp:331-338): the header's addRect and the
spacing rounding of getSpacing against the reference's own addRect
(rtpslib/domain/IV.cpp:165-202, compiled into oracle/_ref) and its settings
round trip.  No GPU: the driver's --add-rect mode runs the header code only."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import addrect_cases
import oracle_bind
from enjaparticles_gb300 import abi, build_ext

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "addrect.npz"))


def _header_add_rect(num, spacing, scale, lo, hi):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "rect.bin")
        args = [build_ext.DRIVER, "--add-rect", num, repr(float(spacing)), scale] + list(lo[:3]) + list(hi[:3])
        r = subprocess.run([str(a) for a in args] + [out], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr
        return np.fromfile(out, np.float32).reshape(-1, 4)


@pytest.mark.parametrize("case", addrect_cases.CASES, ids=[c[0] for c in addrect_cases.CASES])
def test_header_add_rect_equals_reference(case):
    name, n, scale, num, lo, hi = case
    sp, _ = addrect_cases.scene_params(n, scale)
    sx = addrect_cases.spacing(sp)
    assert np.float32(sx) == GOLD[name + "_spacing"]
    got = _header_add_rect(num, sx, 1.0, lo, hi)
    want = GOLD[name + "_points"]
    assert got.shape == want.shape and np.array_equal(got.view(np.uint32), want.view(np.uint32))
    if oracle_bind.ref_available():
        live = oracle_bind.ref_add_rect(num, lo, hi, sx, 1.0)
        assert np.array_equal(live.view(np.uint32), got.view(np.uint32))


def test_spacing_rounds_through_the_settings_map():
    """getSpacing = the library's sph_settings_round(rest_distance / sc), the
    same float as the reference's ostringstream / istringstream round trip;
    at simulation_scale 0.7 the raw quotient differs from it."""
    lib = abi.load_library()
    differs = 0
    for _, n, scale, _, _, _ in addrect_cases.CASES:
        sp, _ = addrect_cases.scene_params(n, scale)
        q = np.float32(np.float32(sp.rest_distance) / np.float32(sp.simulation_scale))
        assert np.float32(lib.sph_settings_round(float(q))) == np.float32(oracle_bind.settings_round(q))
        differs += int(np.float32(oracle_bind.settings_round(q)) != q)
    assert differs >= 1
