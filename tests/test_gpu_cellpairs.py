"""The fused step's density pass in the default arithmetic takes two particles
of one cell per thread (k_density_cellpairs); the staged density pass takes
one (k_density_pairs).  Both must give the same densities and neighbour
counts bit for bit, whatever the cells hold: the dam-break lattice, odd and
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


def _fused_and_staged(sp, g, gs, pos, vel, threads):
    n = pos.shape[0]
    out = []
    for staged in (False, True):
        s = SPH(sp, g, n, gs)
        cfg = list(s.launch_config())
        cfg[0] = threads
        s.set_launch_config(*cfg)
        s.upload(pos, vel)
        if staged:
            s.update()  # hash, sort, cellindices, permute, density (one particle per thread), force
        else:
            s.step(DT, 1)  # the graph step: density with two particles of a cell per thread
        s.sync()
        m = s.getNum() if staged else n
        k = min(m, n)
        out.append((s.get("pos_s", k), s.get("density_s", k), s.get("neighbor_count", k)))
        s.close()
    return out


@pytest.mark.parametrize("threads", [128, 256, 512])
def test_dam_break_lattice(threads):
    n = 16384
    sp, g, gs = abi.dambreak_params(n)
    pos, vel = scenes.dambreak(n, velocity_sigma=0.1)
    (p0, d0, c0), (p1, d1, c1) = _fused_and_staged(sp, g, gs, pos, vel, threads)
    np.testing.assert_array_equal(p0, p1)
    np.testing.assert_array_equal(d0, d1)
    np.testing.assert_array_equal(c0, c1)


@pytest.mark.parametrize("n,crowd", [(60001, 7), (4097, 0), (3, 0), (2, 0), (1, 0)])
def test_ragged_crowded_and_outside(n, crowd):
    sp, g, gs = abi.dambreak_params(max(n, 4096))
    pos, vel = _layout(n, 100 + n, crowd)
    (p0, d0, c0), (p1, d1, c1) = _fused_and_staged(sp, g, gs, pos, vel, 256)
    k = min(len(d0), len(d1))
    np.testing.assert_array_equal(p0[:k], p1[:k])
    np.testing.assert_array_equal(d0[:k], d1[:k])
    np.testing.assert_array_equal(c0[:k], c1[:k])
