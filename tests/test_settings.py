"""The reference's settings path (a settings map -> SPH::calculate,
SPH::updateParams, System::setupDomain) through sph_params_from_settings:
the parameter block, both grids and the spacing equal the reference's own
code (RTPSSettings.cpp and SPHSettings.cpp compiled from the reference
tree) bit for bit, against the committed fixture and, where the reference
tree is built (oracle/_ref), against it directly.  Host only."""
import ctypes as C
import os

import numpy as np
import pytest

import settings_cases
from enjaparticles_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "librtps_ref.so")

# bytes of SPHParams that hold values (the struct's tail padding holds none):
# rest_density .. max_num, then gravity
SPHP_FIELDS = [(0, 116), (128, 144)]


def _same_params(mine, ref):
    for lo, hi in SPHP_FIELDS:
        assert bytes(mine)[lo:hi] == bytes(ref)[lo:hi], (lo, hi)


def _same_grid(mine, ref):
    assert bytes(mine)[:116] == bytes(ref)[:116]


@pytest.fixture(scope="module")
def fixture():
    return np.load(os.path.join(HERE, "golden", "settings.npz"))


@pytest.mark.parametrize("name", [c[0] for c in settings_cases.CASES])
def test_settings_path_equals_reference_fixture(fixture, name):
    keys = [str(k) for k in fixture[name + "/keys"]]
    values = [str(v) for v in fixture[name + "/values"]]
    sp, g, gs, spacing = abi.params_from_settings(dict(zip(keys, values)))
    _same_params(sp, fixture[name + "/sphp"])
    _same_grid(g, fixture[name + "/grid"])
    _same_grid(gs, fixture[name + "/grid_scaled"])
    assert np.float32(spacing) == fixture[name + "/spacing"]


def test_fixture_cases_are_the_current_cases(fixture):
    for name, settings in settings_cases.CASES:
        items = [(k, abi.settings_value(v)) for k, v in settings.items()]
        assert [str(k) for k in fixture[name + "/keys"]] == [k for k, _ in items]
        assert [str(v) for v in fixture[name + "/values"]] == [v for _, v in items]


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference tree not built here (oracle/_ref)")
def test_settings_path_equals_reference_build():
    import ref_driver
    for name, settings in settings_cases.CASES:
        items = [(k, abi.settings_value(v)) for k, v in settings.items()]
        rsp, rg, rgs, rspacing, size = ref_driver.params_from_settings(items)
        assert size == C.sizeof(abi.SPHParams)
        sp, g, gs, spacing = abi.params_from_settings(dict(items))
        _same_params(sp, rsp)
        _same_grid(g, rg)
        _same_grid(gs, rgs)
        assert spacing == rspacing, name


def test_later_entry_of_a_key_wins_and_missing_keys_read_as_zero():
    lib = abi.load_library()
    base = dict(settings_cases.CASES[0][1])
    items = [(k, abi.settings_value(v)) for k, v in base.items()] + [("viscosity", "0.5")]
    keys = (C.c_char_p * len(items))(*[k.encode() for k, _ in items])
    vals = (C.c_char_p * len(items))(*[v.encode() for _, v in items])
    sp, g, gs, spacing = abi.SPHParams(), abi.GridParams(), abi.GridParams(), C.c_float()
    assert lib.sph_params_from_settings(len(items), keys, vals, C.byref(sp), C.byref(g), C.byref(gs),
                                        C.byref(spacing)) == abi.SPH_OK
    assert sp.viscosity == np.float32(0.5)
    sp2 = abi.params_from_settings(dict(settings_cases.CASES[6][1]))[0]  # no gravity, no gas constant
    assert (sp2.gravity.x, sp2.gravity.y, sp2.gravity.z, sp2.gravity.w) == (0, 0, 0, 0)
    assert sp2.K == 0 and sp2.viscosity == 0


@pytest.mark.parametrize("bad", [
    {"rest_density": 0, "max_num_particles": 1024, "domain_min": "0 0 0 1", "domain_max": "1 1 1 1"},
    {"rest_density": 1000, "max_num_particles": 1, "domain_min": "0 0 0 1", "domain_max": "1 1 1 1"},
    {"rest_density": 1000, "max_num_particles": 1024, "domain_min": "0 0 0 1", "domain_max": "1 0 1 1"},
    {"rest_density": 1000, "max_num_particles": 1024},
])
def test_invalid_settings_are_rejected(bad):
    with pytest.raises(abi.SPHError) as e:
        abi.params_from_settings(bad)
    assert e.value.code == abi.SPH_EINVAL
