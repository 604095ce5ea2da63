"""The headless C++ driver (rtps::SPH class over the C ABI) steps the same
scene to the same bits as the Python harness, in fused and frame-loop modes."""
import json
import os
import subprocess

import numpy as np
import pytest

import addrect_cases
from enjaparticles_gb300 import abi, build_ext
from enjaparticles_gb300.sph import dambreak_system

pytestmark = pytest.mark.gpu


def _run(*args):
    r = subprocess.run([build_ext.DRIVER] + [str(a) for a in args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_driver_matches_python_exact():
    n, steps, warm = 16384, 20, 3
    fused = _run("--n", n, "--steps", steps, "--warmup", warm, "--exact")
    frames = _run("--n", n, "--steps", steps, "--warmup", warm, "--exact", "--frames")
    s, _, _ = dambreak_system(n, exact=True)
    s.step(0.001, warm + steps)
    p = s.get("pos_u", n).astype(np.float64)
    want = 0.0
    for q in p:  # sph_bench's summation order
        want += q[0] + 2.0 * q[1] + 3.0 * q[2]
    assert fused["checksum"] == want
    assert frames["checksum"] == want
    assert fused["num_after"] == n and fused["value"] > 0


def test_driver_throughput_line():
    d = _run("--n", 262144, "--steps", 100, "--warmup", 5)
    assert d["metric"] == "particle-updates/s" and d["mode"] == "fused" and d["value"] > 1e8


def test_driver_mesh_and_post_process_match_python():
    """--mesh loads the ramp-and-box mesh through rtps::SPH::loadTriangles and
    --post-process runs SPH::postProcess: the same bits and the same surface
    as the Python harness with scenes.ramp_and_box_mesh and postProcess."""
    from enjaparticles_gb300.scenes import ramp_and_box_mesh
    n, steps, warm, res = 16384, 20, 3, 32
    d = _run("--n", n, "--steps", steps, "--warmup", warm, "--exact", "--mesh", "--post-process", res)
    s, _, _ = dambreak_system(n, exact=True)
    s.loadTriangles(ramp_and_box_mesh())
    s.step(0.001, warm + steps)
    p = s.get("pos_u", n).astype(np.float64)
    want = 0.0
    for q in p:
        want += q[0] + 2.0 * q[1] + 3.0 * q[2]
    v, _ = s.postProcess(res)
    assert d["mesh"] == 1 and d["checksum"] == want
    assert d["triangles"] == len(v) > 0


@pytest.mark.parametrize("case", addrect_cases.CASES, ids=[c[0] for c in addrect_cases.CASES])
def test_driver_add_box_equals_reference_add_rect(case, tmp_path):
    """rtps::SPH::addBox through the C++ class: the system's positions are the
    reference's addRect points (golden, from oracle/_ref) at the reference's
    getSpacing, bit for bit, and the class's getSpacing is that spacing."""
    name, n, scale, num, lo, hi = case
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "addrect.npz"))
    out = tmp_path / "box.bin"
    d = _run("--n", n, "--add-box", num, scale, *lo[:3], *hi[:3], out)
    want = gold[name + "_points"]
    got = np.fromfile(out, np.float32).reshape(-1, 4)
    assert d["added"] == d["num"] == len(want)
    assert np.float32(d["spacing"]) == gold[name + "_spacing"]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
