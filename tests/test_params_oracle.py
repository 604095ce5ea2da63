"""The oracle's parameter derivation (oracle/sph_params_oracle.cpp) gives the
same SPHParams / GridParams bytes as the library's sph_dambreak_params, so the
CPU reference arm of bench.py can build its scene without loading the
product library; and that arm indeed maps no library of the product."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle_bind
from enjaparticles_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n", [1000, 4096, 16384, 65536, 2097152, 123457])
@pytest.mark.parametrize("mu", [0.01, 0.005, 0.0371])
def test_oracle_params_equal_library(n, mu):
    a = oracle_bind.dambreak_params(n, mu)
    b = abi.dambreak_params(n, mu)
    for x, y in zip(a, b):
        assert bytes(x) == bytes(y)


def test_oracle_grid_equals_reference_domain():
    if not oracle_bind.ref_available():
        pytest.skip("reference kernels not built (no reference tree)")
    sp, g, gs = oracle_bind.dambreak_params(16384)
    lo = np.array([0, 0, 0, 0], np.float32)
    hi = np.array([1, 1, 1, 0], np.float32)
    rg, rgs = abi.GridParams(), abi.GridParams()
    oracle_bind.ref().ref_setup_domain(lo.ctypes.data, hi.ctypes.data, sp.smoothing_distance, sp.simulation_scale,
                                       oracle_bind.C.addressof(rg), oracle_bind.C.addressof(rgs))
    # the reference's struct leaves its 12 tail bytes after nb_cells unset
    assert bytes(rg)[:116] == bytes(g)[:116] and bytes(rgs)[:116] == bytes(gs)[:116]


def test_reference_arm_loads_no_product_library():
    code = (
        "import sys, runpy\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1', '--n', '4096']\n"
        "try:\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "except SystemExit:\n"
        "    pass\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('MAPPED' if 'librtps_sph' in maps else 'CLEAN')\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "CLEAN"
    assert '"impl": "reference"' in lines[-2]
