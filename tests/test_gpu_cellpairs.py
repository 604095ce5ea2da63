"""The density pass of the graph step and of sph_update takes, in the default
arithmetic, two particles of one cell per thread (k_density_cellpairs); the
stage API's density pass takes one (k_density_pairs).  They must give the
same sorted positions, densities and neighbour counts bit for bit, whatever
the cells hold: the dam-break lattice, odd and
even cell counts, cells cut by the pass's 128/256/512-particle block
ranges, a crowded cell (more candidates than the neighbour bitmask holds),
particles outside the grid, and particle counts of 1, 2 and 3.  The neighbour
bitmask the force pass reads is checked through the force pass: a batch
(whose density pass takes one particle per thread) steps the same scenes to
the same bits (tests/test_gpu_batch.py, tests/test_gpu_batch_sort.py)."""
import numpy as np
import pytest

from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu
DT = 0.001


def _layout(n, seed, crowd):
    u = scenes.uniform(seed, 3 * n).reshape(n, 3)
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = (u * 1.2 - 0.1).astype(np.float32)
    if crowd and n > 3:
        pos[::crowd, :3] = pos[3, :3]
    vel = np.zeros((n, 4), np.float32)
    return pos, vel


def _density_by_path(sp, g, gs, pos, vel, threads):
    """(pos_s, density_s, neighbour counts) of the in-grid particles after
    the density pass of: the graph step and sph_update (two particles of a
    cell per thread), and the stage API's passes run one by one (one
    particle per thread)."""
    n = pos.shape[0]
    out = {}
    for path in ("step", "update", "stages"):
        s = SPH(sp, g, n, gs)
        cfg = list(s.launch_config())
        cfg[0] = threads
        s.set_launch_config(*cfg)
        s.upload(pos, vel)
        if path == "step":
            s.step(DT, 1)
        elif path == "update":
            s.update()
        else:
            s.hash()
            s.sort()
            s.cellindices()
            s.permute()
            s.density()
        s.sync()
        out[path] = (s.get("pos_s", n), s.get("density_s", n), s.get("neighbor_count", n))
        s.close()
    return out


def _in_grid(sp, g, gs, pos):
    """Particles whose cell key is inside the grid (the ones the density
    pass walks for)."""
    s = SPH(sp, g, pos.shape[0], gs)
    s.upload(pos, np.zeros_like(pos))
    s.hash()
    keys = s.get("sort_hashes", pos.shape[0])
    s.close()
    return int((keys < g.nb_cells).sum())


def _check(sp, g, gs, pos, vel, threads):
    k = _in_grid(sp, g, gs, pos)
    out = _density_by_path(sp, g, gs, pos, vel, threads)
    ref = out["stages"]
    for path in ("step", "update"):
        for got, want in zip(out[path], ref):
            np.testing.assert_array_equal(got[:k], want[:k], err_msg=path)


@pytest.mark.parametrize("threads", [128, 256, 512])
def test_dam_break_lattice(threads):
    n = 16384
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.1)
    _check(sp, g, gs, pos, vel, threads)


@pytest.mark.parametrize("n,crowd", [(60001, 7), (4097, 0), (3, 0), (2, 0), (1, 0)])
def test_ragged_crowded_and_outside(n, crowd):
    sp, g, gs = abi.dambreak_params(max(n, 4096))
    pos, vel = _layout(n, 100 + n, crowd)
    _check(sp, g, gs, pos, vel, 256)
