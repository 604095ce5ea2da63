"""Seeded scene generators (CPU): reproducible, and shaped as the benchmark
configurations describe."""
import numpy as np

from enjaparticles_gb300 import scenes
from enjaparticles_gb300.batch import dambreak_batch_scenes


def test_splitmix64_known_values():
    # splitmix64 from seed 0: first outputs of the published generator
    z = scenes.splitmix64(0, 3)
    assert [int(v) for v in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_dambreak_lattice_shape_and_jitter():
    n = 16384
    pos, vel = scenes.dambreak(n)
    s = scenes.lattice_spacing(n)
    assert pos.shape == (n, 4) and np.all(pos[:, 3] == 1.0) and np.all(vel == 0)
    side = int(np.ceil(0.5 / s - 1e-9))
    k = np.arange(n)
    iz, rem = np.divmod(k, side * side)
    iy, ix = np.divmod(rem, side)
    lattice = np.stack([(ix + 0.5) * s, (iy + 0.5) * s, (iz + 0.5) * s], 1)
    jit = pos[:, :3] - lattice
    assert np.abs(jit).max() <= 0.0101 * s
    assert np.all(pos[:, :3] > 0) and np.all(pos[:, :2] < side * s)  # i, j < ceil(0.5/s)
    p2, _ = scenes.dambreak(n)
    assert np.array_equal(pos, p2)  # reproducible


def test_full_size_lattice_fills_half_box():
    s = scenes.lattice_spacing(2097152)
    assert s == 2.0 ** -8


def test_batch_scene_sizes_follow_the_seeded_rule():
    ns, mus = dambreak_batch_scenes(256)
    assert len(ns) == 256 and min(ns) >= 2048 and max(ns) <= 32768
    assert 0.005 <= min(mus) and max(mus) <= 0.05
    assert dambreak_batch_scenes(256) == (ns, mus)
