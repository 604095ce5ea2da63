"""Colour field and marching cubes on the host: the oracle's colour field
against the reference's kernel output (tests/golden/surface_n4096.npz), and
the library's marching-cubes case table on its own and against the
reference's kernels, case by case."""
import ctypes as C

import numpy as np
import pytest

import golden_io
import oracle_bind as ob
import surface_cases as sc
from enjaparticles_gb300 import abi


@pytest.mark.parametrize("res", [16, 32])
def test_oracle_colorfield_matches_reference_golden(res):
    d, sp, g, gs = golden_io.load("surface_n4096.npz")
    n = d["in_pos"].shape[0]
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(d["in_pos"], d["in_vel"])
    sim.step(float(d["dt"]), int(d["steps"]))
    field = np.zeros(res ** 3, np.float32)
    P = ob.ptr
    ps, dens, cs, ce = sim.get("pos_s"), sim.get("density_s"), sim.get("cell_start"), sim.get("cell_end")
    ob.oracle().oracle_colorfield(0, res, P(ps), P(dens), P(cs), P(ce), C.addressof(gs), C.addressof(sp), P(field))
    np.testing.assert_array_equal(field, d["field%d" % res])


def test_case_table_is_a_closed_oriented_surface_per_case():
    """Each case uses exactly its crossed edges; every crossed edge is shared
    by an even number of triangle sides within the cube's polygons (closed
    loops); each triangle's normal points from the corners above the
    isolevel to those below (the side the reference's normals point to)."""
    tri, cnt, mx = sc.case_table(abi.load_library())
    assert mx == 5 and cnt[0] == 0 and cnt[255] == 0
    for cs in range(256):
        inside = [(cs >> k) & 1 for k in range(8)]
        crossed = {e for e, (a, b) in enumerate(sc.EDGE) if inside[a] != inside[b]}
        edges = tri[cs][:3 * cnt[cs]]
        assert (tri[cs][3 * cnt[cs]:] == -1).all()
        assert set(edges.tolist()) == crossed
        mid = lambda e: np.add(sc.CORNER[sc.EDGE[e][0]], sc.CORNER[sc.EDGE[e][1]]) / 2.0
        for t in range(cnt[cs]):
            a, b, c = (mid(e) for e in edges[3 * t:3 * t + 3])
            nrm = np.cross(b - a, c - a)
            assert np.linalg.norm(nrm) > 1e-9
            cen = (a + b + c) / 3
            # outward: towards lower blended corner state
            grad = np.zeros(3)
            for k, p in enumerate(sc.CORNER):
                if not inside[k]:
                    continue
                w = [cen[q] if p[q] else 1 - cen[q] for q in range(3)]
                dd = [1.0 if p[q] else -1.0 for q in range(3)]
                grad += [dd[0] * w[1] * w[2], w[0] * dd[1] * w[2], w[0] * w[1] * dd[2]]
            assert nrm @ grad < 0


@pytest.mark.skipif(not ob.ref_available(), reason="reference kernels not built here (needs the reference tree)")
def test_case_table_against_reference_kernels():
    """Every case as a one-cube field (corners 1 above, 0 below, isolevel
    0.5) through the reference's marching cubes: the library's table gives
    the reference's triangles in all 256 cases, in the same order, with the
    same vertex order in each triangle."""
    tri, cnt, _ = sc.case_table(abi.load_library())
    R = ob.ref()
    res = 4  # the reference's pyramid needs a power-of-two image
    for cs in range(256):
        f = np.zeros(res ** 3, np.float32)
        for k, (x, y, z) in enumerate(sc.CORNER):
            if cs >> k & 1:
                f[x + y * res + z * res * res] = 1.0
        v = np.zeros((64, 9), np.float32)
        nr = np.zeros((64, 9), np.float32)
        tot = R.ref_marching_cubes(res, ob.ptr(f), 0.5, ob.ptr(v), ob.ptr(nr), 64, None)
        g = v[:tot].reshape(-1, 3, 3) / 10.0 * (res - 1)
        g = g[(g.mean(1) < 1).all(1)]  # the triangles of cube (0, 0, 0), in emission order
        mid = lambda e: np.add(sc.CORNER[sc.EDGE[e][0]], sc.CORNER[sc.EDGE[e][1]]) / 2.0
        mine = np.array([[mid(e) for e in tri[cs][3 * t:3 * t + 3]] for t in range(cnt[cs])]).reshape(-1, 3, 3)
        assert len(g) == cnt[cs], cs
        np.testing.assert_allclose(g, mine, atol=1e-6, err_msg="case %d" % cs)
