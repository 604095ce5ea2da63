"""The step's sort (a counting sort on the cell key, sph_cellsort.cu) against
the canonical order: keys ascending, equal keys by ascending particle index,
which is what the staged radix sort (sph_stage_sort) and the oracle give.

Layouts the dam break never produces: one crowded cell holding a seventh of
the particles, particles outside the grid (the out-of-grid key nb_cells, which
the update deletes), and particle counts that leave the last warp, block and
scan tile ragged.  Everything compared here is integer or copied data:
bit-exact."""
import ctypes as C

import numpy as np
import pytest

import oracle_bind as ob
from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu
P = ob.ptr
DT = 0.001
EMPTY = 0xFFFFFFFF


def layout(n, seed, lo, hi, crowd):
    """n particles uniform in [lo, hi)^3; every crowd-th one moved onto
    particle 3 (one crowded cell)."""
    u = scenes.uniform(seed, 3 * n).reshape(n, 3)
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = (u * (hi - lo) + lo).astype(np.float32)
    if crowd and n > 3:
        pos[::crowd, :3] = pos[3, :3]
    v = scenes.uniform(seed + 1, 3 * n).reshape(n, 3)
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = ((v - 0.5) * 0.2).astype(np.float32)
    return pos, vel


def canonical(pos, g):
    """Oracle keys, then the stable order and the cell ranges it implies."""
    n = pos.shape[0]
    kk = np.empty(n, np.uint32)
    ii = np.empty(n, np.uint32)
    ob.oracle().oracle_hash(n, P(pos), C.addressof(g), P(kk), P(ii))
    order = np.lexsort((ii, kk))
    keys = kk[order]
    idx = ii[order]
    cells = g.nb_cells + 1
    start = np.full(cells, EMPTY, np.uint32)
    end = np.zeros(cells, np.uint32)
    occ, first, cnt = np.unique(keys, return_index=True, return_counts=True)
    start[occ] = first
    end[occ] = first + cnt
    return keys, idx, start, end, occ


@pytest.mark.parametrize("n,crowd", [(300000, 7), (4097, 2), (33, 0), (1, 0)])
def test_update_sort_and_cells_equal_canonical(n, crowd):
    """sph_update inside the grid: sorted keys and indices, cell_start over
    every cell, cell_end over the occupied ones, and the permuted pos/vel."""
    sp, g, gs = abi.dambreak_params(max(n, 4096))
    pos, vel = layout(n, 11 + n, 0.05, 0.95, crowd)
    keys, idx, start, end, occ = canonical(pos, g)
    assert keys.max() < g.nb_cells  # nothing leaves the grid here
    s = SPH(sp, g, n, gs, exact=True)
    s.upload(pos, vel)
    s.update()
    np.testing.assert_array_equal(s.get("sort_hashes", n), keys)
    np.testing.assert_array_equal(s.get("sort_indices", n), idx)
    np.testing.assert_array_equal(s.get("cell_start"), start)
    np.testing.assert_array_equal(s.get("cell_end")[occ], end[occ])
    np.testing.assert_array_equal(s.get("pos_s", n), pos[idx])
    np.testing.assert_array_equal(s.get("vel_s", n), vel[idx])
    s.close()


def test_update_equals_staged_radix_sort():
    """The same layout through the staged stages (hash, radix sort,
    cellindices, permute) and through sph_update: identical arrays."""
    n = 100003
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = layout(n, 5, -0.3, 1.3, 11)
    a = SPH(sp, g, n, gs, exact=True)
    a.upload(pos, vel)
    a.hash()
    a.sort()
    a.cellindices()
    a.permute()
    b = SPH(sp, g, n, gs, exact=True)
    b.upload(pos, vel)
    b.update()
    # the update deleted the out-of-grid particles after the sort: its keys
    # and cell ranges are the sort's, its kept indices restart at 0
    keys, idx, start, end, occ = canonical(pos, g)
    kept = int((keys < g.nb_cells).sum())
    assert 0 < kept < n
    for f in ("sort_hashes", "cell_start"):
        np.testing.assert_array_equal(b.get(f, a.get(f).shape[0]), a.get(f), err_msg=f)
    np.testing.assert_array_equal(b.get("cell_end")[occ], a.get("cell_end")[occ])
    np.testing.assert_array_equal(a.get("sort_indices", n), idx)
    np.testing.assert_array_equal(b.get("sort_indices", kept), np.arange(kept, dtype=np.uint32))
    a.close()
    b.close()


@pytest.mark.parametrize("frac_out", [0.3, 0.9])
def test_mass_deletion_keeps_index_order(frac_out):
    """Many particles leave at once: the deleted ones come back in ascending
    index order and the kept ones continue in sorted order."""
    n = 60000
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = layout(n, 21, 0.05, 0.95, 0)
    u = scenes.uniform(77, n)
    out = u < frac_out
    # far above or below the grid in z: the hash leaves [0, nb_cells) (an
    # overflow in x alone only moves the key to another row)
    pos[out, 2] = np.where(u[out] < frac_out / 2, np.float32(5.0), np.float32(-5.0))
    keys, idx, _, _, _ = canonical(pos, g)
    kept = int((keys < g.nb_cells).sum())
    assert kept == n - int(out.sum())
    for mode in ("staged", "graph"):
        s = SPH(sp, g, n, gs, exact=True)
        s.upload(pos, vel)
        if mode == "staged":
            s.update()
            s.integrate(DT)
        else:
            s.step(DT, 1)
        assert s.getNum() == kept, mode
        dp, dv = s.getDeleted()
        np.testing.assert_array_equal(dp, pos[idx[kept:]], err_msg=mode)
        np.testing.assert_array_equal(dv, vel[idx[kept:]], err_msg=mode)
        s.close()


def test_fused_step_crowded_and_outside_equals_oracle():
    """Two exact fused steps (CUDA graph) of a layout with a crowded cell and
    particles outside the grid equal the oracle's update+integrate."""
    n = 20000
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = layout(n, 3, -0.1, 1.1, 40)
    s = SPH(sp, g, n, gs, exact=True)
    s.upload(pos, vel)
    s.step(DT, 2)
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(pos, vel)
    sim.step(DT, 2)
    assert s.getNum() == sim.num
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(s.get(f), sim.get(f), err_msg=f)
    s.close()


def test_large_grid_scans_tile_totals_first():
    """A grid of more than 2048 tiles of 4096 cells, where the scan first
    scans the tile totals in one block: two exact fused steps equal the
    oracle, and the cell ranges equal the stable order's."""
    n = 20000
    spacing = 1.0 / 450  # about 12 M cells: more than 2048 tiles, below the 2^24 - 2 cell limit
    sp, g, gs = abi.dambreak_params(n, 0.01, spacing=spacing)
    assert (g.nb_cells + 1 + 4095) // 4096 > 2048 and g.nb_cells <= (1 << 24) - 2
    pos = scenes.dambreak_positions(n, spacing=spacing)
    vel = np.zeros_like(pos)
    s = SPH(sp, g, n, gs, exact=True)
    s.upload(pos, vel)
    s.step(DT, 2)
    sim = ob.OracleSim(sp, g, gs, n)
    sim.upload(pos, vel)
    sim.step(DT, 2)
    for f in ("pos_u", "vel_u", "veleval_u"):
        np.testing.assert_array_equal(s.get(f), sim.get(f), err_msg=f)
    # the last sort: keys of the positions the second step started from
    start_pos = s.get("pos_s", n)
    keys, _, start, end, occ = canonical(start_pos, g)
    np.testing.assert_array_equal(s.get("sort_hashes", n), keys)
    np.testing.assert_array_equal(s.get("cell_start"), start)
    np.testing.assert_array_equal(s.get("cell_end")[occ], end[occ])
    s.close()
