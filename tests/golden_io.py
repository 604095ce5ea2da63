"""Load the golden fixtures of tests/golden/ (made by tests/golden/make_golden.py
from the reference's own kernels)."""
import os

import numpy as np

from enjaparticles_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def path(name):
    return os.path.join(GOLDEN, name)


def load(name):
    z = np.load(os.path.join(GOLDEN, name))
    d = {k: z[k] for k in z.files}
    sp = abi.SPHParams.from_buffer_copy(d["sphp"].tobytes())
    g = abi.GridParams.from_buffer_copy(d["grid"].tobytes())
    gs = abi.GridParams.from_buffer_copy(d["grid_scaled"].tobytes())
    return d, sp, g, gs
