"""The C ABI as a library user sees it, without a GPU: every function that
include/rtps_sph.h declares is exported by librtps_sph.so and bound in
enjaparticles_gb300.abi; the host-side parameter helpers work; the C++
rtps::SPH class compiles; the C++ driver builds the same scene as Python."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from enjaparticles_gb300 import abi, build_ext
from enjaparticles_gb300.scenes import dambreak_positions, lattice_spacing

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rtps_sph.h")


@pytest.fixture(scope="module")
def lib():
    if not (os.path.exists(abi.LIB_PATH) and os.path.exists(abi.CHECKED_LIB_PATH) and
            os.path.exists(build_ext.DRIVER)):
        build_ext.build()
    return abi.load_library()


@pytest.fixture(scope="module")
def checked_lib(lib):
    return abi.load_library(abi.CHECKED_LIB_PATH)


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(sph_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("sph_create", "sph_step", "sph_stage_hash", "sph_stage_sort", "sph_stage_cellindices",
                 "sph_stage_permute", "sph_stage_density", "sph_stage_force", "sph_stage_collision",
                 "sph_stage_leapfrog", "sph_download", "sph_get_device_ptr", "sph_batch_step",
                 "sph_adjoint_rollout", "sph_sort_pairs_noalloc"):
        assert must in names


def test_every_declared_function_is_exported_and_bound(lib):
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing
    unbound = [f for f in declared_functions() if f not in abi.SIGNATURES]
    assert not unbound, unbound


def test_bounds_checked_library_exports_the_same_boundary(lib, checked_lib):
    missing = [f for f in declared_functions() if not hasattr(checked_lib, f)]
    assert not missing, missing
    assert "bounds-checked" in checked_lib.sph_build_info().decode()
    assert "bounds-checked" not in lib.sph_build_info().decode()
    assert abi.STATUS_NAMES[abi.SPH_EBOUNDS] == "SPH_EBOUNDS"


def test_parameter_helpers_without_gpu(lib):
    n = 16384
    sp, g, gs = abi.dambreak_params(n)
    s = lattice_spacing(n)
    assert sp.rest_distance == np.float32(lib.sph_settings_round(s))
    assert g.nb_cells == 30 ** 3 and gs.nb_cells == g.nb_cells
    assert abs(sp.smoothing_distance - 2 * s) < 1e-6 and sp.velocity_limit == 600.0
    bad = abi.SPHParams()
    assert lib.sph_dambreak_params(0, s, 0.01, C.byref(bad), C.byref(abi.GridParams()), None) == abi.SPH_EINVAL
    info = lib.sph_build_info().decode()
    assert "sm_103a" in info


def test_create_errors_are_per_thread(lib):
    """A failed sph_create leaves its message for sph_last_error(NULL) on the
    thread that called it; other threads keep their own (argument checks run
    before any CUDA call, so this needs no GPU)."""
    import threading

    sp, g, gs = abi.dambreak_params(4096)
    msgs = {}
    barrier = threading.Barrier(4)

    def worker(k):
        out = C.c_void_p()
        for _ in range(200):
            rc = lib.sph_create(C.byref(sp), C.byref(g), C.byref(gs), -(k + 1), C.byref(out))
            assert rc == abi.SPH_EINVAL
        barrier.wait()  # every thread has failed before any reads its message
        buf = C.create_string_buffer(256)
        assert lib.sph_last_error(None, buf, 256) == abi.SPH_OK
        msgs[k] = buf.value.decode()

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert msgs == {k: "max_num out of range: %d" % -(k + 1) for k in range(4)}


def test_cpp_class_compiles():
    src = ("#include \"rtps_sph.hpp\"\nint main() { SPHParams p; GridParams g; rtps::SPH* s = nullptr;\n"
           "rtps::RTPSSettings set; set.SetSetting(\"rest_density\", 1000.0f);\n"
           "set.SetSetting(\"domain_min\", rtps::make_float4(0, 0, 0, 1));\n"
           "(void)set.GetSettingAs<float>(\"rest_density\"); (void)set.GetSettingAs<rtps::float4>(\"domain_min\");\n"
           "if (s) { rtps::SPH t(&set); (void)t.getSpacing(); }\n"
           "if (s) { s->update(); s->interact(); s->integrate(); s->postProcess(); s->acquireGLBuffers();\n"
           "s->releaseGLBuffers(); s->addBox(10, rtps::make_float4(0,0,0,1), rtps::make_float4(1,1,1,1), false);\n"
           "(void)s->getNum(); (void)s->getDeletedPos(); }\n(void)p; (void)g; return 0; }\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-x", "c++", "-"], input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(["gcc", "-std=c11", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-x", "c", "-"], input="#include \"rtps_sph.h\"\nint main(void) { return 0; }\n",
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_driver_scene_matches_python(lib, tmp_path):
    for n in (1000, 65536):
        f = tmp_path / ("scene_%d.bin" % n)
        subprocess.run([build_ext.DRIVER, "--n", str(n), "--dump-scene", str(f)], check=True)
        got = np.fromfile(str(f), dtype=np.float32).reshape(n, 4)
        np.testing.assert_array_equal(got, dambreak_positions(n))
