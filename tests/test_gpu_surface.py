"""Colour field and marching cubes on the GPU (SPH::postProcess) against the
reference's own kernels (tests/golden/surface_n4096.npz: colorfield.cl and
the histopyramid marching cubes after 20 steps of the reference): the field
and the mesh (triangles, vertices, normals, in order) bit for bit."""
import ctypes as C

import numpy as np
import pytest
import torch

import golden_io
import surface_cases as sc
from enjaparticles_gb300 import abi
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu


def _system(exact=True):
    d, sp, g, gs = golden_io.load("surface_n4096.npz")
    n = d["in_pos"].shape[0]
    s = SPH(sp, g, n, gs, exact=exact)
    s.upload(d["in_pos"], d["in_vel"])
    s.step(float(d["dt"]), int(d["steps"]))
    return s, d


@pytest.mark.parametrize("res", [16, 32])
def test_colorfield_exact_matches_reference_golden(res):
    s, d = _system()
    np.testing.assert_array_equal(s.colorfield(res).ravel(), d["field%d" % res])


def test_colorfield_default_arithmetic_close_to_reference_golden():
    s, d = _system(exact=False)
    f = s.colorfield(32).ravel()
    ref = d["field32"]
    assert np.abs(f - ref).max() <= 1e-3 * np.abs(ref).max()


@pytest.mark.parametrize("res", [16, 32])
def test_surface_matches_reference_golden(res):
    """The mesh of SPH::postProcess equals the reference's triangle list bit
    for bit: the same triangles in the same order, each with its vertices and
    normals in the same order."""
    s, d = _system()
    v, nr = s.postProcess(res)
    rv, rn = d["mesh%d_vertices" % res], d["mesh%d_normals" % res]
    assert v.shape == rv.shape and len(v) > 100
    np.testing.assert_array_equal(v.view(np.uint32), rv.view(np.uint32))
    np.testing.assert_array_equal(nr.view(np.uint32), rn.view(np.uint32))


def _blob_field(res, seed=3):
    rng = np.random.default_rng(seed)
    g = np.linspace(0.0, 1.0, res, dtype=np.float64)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    f = np.zeros_like(x)
    for c in rng.uniform(0.25, 0.75, size=(5, 3)):
        f += np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / 0.02)
    return f.astype(np.float32).ravel()  # index s + t res + r res^2


def _morton(tx, ty):
    key = np.zeros_like(tx, dtype=np.int64)
    for b in range(16):
        key |= ((tx >> b) & 1) << (2 * b)
        key |= ((ty >> b) & 1) << (2 * b + 1)
    return key


def _slices(res):
    s = int(2 ** np.ceil(np.log(np.ceil(np.sqrt(np.float32(res))) / np.log(np.float32(2.0)))))
    while s * s < res:
        s *= 2
    return s


@pytest.mark.parametrize("res", [2, 20, 64, 100])
def test_marching_cubes_on_a_device_field(res):
    """Any resolution (the reference's own image holds res <= 64 and its
    pyramid needs a power of two): the triangle count is the table's sum over
    the cubes, the cubes come in the reference's order (Morton order over the
    slice-tiled image), and every vertex lies on an edge of its cube."""
    lib = abi.load_library()
    tri, cnt, _ = sc.case_table(lib)
    f = _blob_field(res)
    iso = 0.5 if res > 2 else float(np.float32(f.mean()))
    s = SPH(*abi.dambreak_params(1024)[:2], 1024)
    dev = torch.from_numpy(f).cuda()
    torch.cuda.synchronize()
    v, nr = s.marchingCubes(res, iso, field_ptr=dev.data_ptr())
    cases = sc.cube_cases(f, res, iso)
    assert len(v) == int(cnt[cases].sum())
    if res == 2:  # every corner but one is on the last layer, which the pyramid reads as 0
        return
    assert np.isfinite(v).all() and np.isfinite(nr).all()
    # the cubes with triangles, in the reference's emission order, each with
    # its count: the triangle list splits into them (a triangle lying in a
    # face shared by two cubes cannot tell its cube by itself)
    z, y, x = np.nonzero(cnt[cases] > 0)
    sl = _slices(res)
    order = np.argsort(_morton(z % sl * res + x, z // sl * res + y), kind="stable")
    z, y, x = z[order], y[order], x[order]
    per = cnt[cases[z, y, x]].astype(np.int64)
    cubes = np.repeat(np.stack([x, y, z], axis=1), per, axis=0)
    assert len(cubes) == len(v)
    g = v.astype(np.float64) / 10.0 * (res - 1) - cubes[:, None, :]
    assert (g >= -1e-5).all() and (g <= 1 + 1e-5).all()
    on_edge = (np.minimum(np.abs(g), np.abs(g - 1)) < 1e-5).sum(axis=2)
    assert (on_edge >= 2).all()
    np.testing.assert_allclose(np.linalg.norm(nr, axis=2), 1.0, atol=1e-5)


def test_surface_errors():
    s, d = _system()
    with pytest.raises(abi.SPHError) as e:
        s.colorfield(513)
    assert e.value.code == abi.SPH_EINVAL
    s.colorfield(16)
    n = C.c_int()
    with pytest.raises(abi.SPHError) as e:
        s._ck(s.lib.sph_marching_cubes(s.ctx, None, 20, 0.0001, C.byref(n)))
    assert e.value.code == abi.SPH_ESTATE
    empty = SPH(*abi.dambreak_params(1024)[:2], 1024)
    v, nr = empty.postProcess(16)
    assert len(v) == 0
