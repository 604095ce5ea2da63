"""Hoses on the host: the library's sph_hose (Hose.cpp + addDiscRandom
restated) against the reference's own Hose, through the scripts of
hose_cases.py: the same counts, positions and push velocities, bit for bit,
from the same rand() seed."""
import numpy as np
import pytest

import golden_io
import hose_cases
import oracle_bind as ob
from enjaparticles_gb300 import abi
from enjaparticles_gb300.sph import Hose


@pytest.mark.parametrize("name", sorted(hose_cases.SCRIPTS))
def test_hose_matches_reference_golden(name):
    d = np.load(golden_io.path("hose_sprays.npz"))
    counts, pos, vel = hose_cases.run_script(name, Hose)
    np.testing.assert_array_equal(counts, d[name + "_counts"])
    np.testing.assert_array_equal(pos, d[name + "_pos"])
    np.testing.assert_array_equal(vel, d[name + "_vel"])


@pytest.mark.skipif(not ob.ref_available(), reason="reference kernels not built here (needs the reference tree)")
@pytest.mark.parametrize("name", sorted(hose_cases.SCRIPTS))
def test_hose_equals_reference_hose(name):
    a = hose_cases.run_script(name, hose_cases.RefHose)
    b = hose_cases.run_script(name, Hose)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_hose_argument_errors():
    with pytest.raises(abi.SPHError):
        Hose(0.0, 10, (0, 0, 0, 1), (0, 0, -1, 0), 0.1, 0.01)
    with pytest.raises(abi.SPHError):
        Hose(0.001, -1, (0, 0, 0, 1), (0, 0, -1, 0), 0.1, 0.01)
    with pytest.raises(abi.SPHError):
        Hose(0.001, 10, (0, 0, np.nan, 1), (0, 0, -1, 0), 0.1, 0.01)
    h = Hose(0.001, 10, (0, 0, 0, 1), (0, 0, -1, 0), 0.1, 0.01)
    with pytest.raises(abi.SPHError):
        h.refill(-3)
    assert h.remaining() == 10
