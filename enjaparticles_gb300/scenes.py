"""Seeded synthetic scenes of the SPH benchmarks (dam break on a jittered lattice).

The reference fills boxes with System::addBox -> addRect (rtpslib/domain/IV.cpp:
165-202): a lattice enumerated z, then y, then x, stopping after `num` points.
The benchmark scenes use the same enumeration on a lattice of spacing
s = (0.125/N)^(1/3) at points ((i+1/2)s, (j+1/2)s, (k+1/2)s), i, j < ceil(0.5/s),
each coordinate jittered by U(-0.01 s, +0.01 s).  Random numbers come from a
counter-based splitmix64 stream, so every scene is reproducible on any host.
"""
import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, count, offset=0):
    """The first `count` outputs (after `offset` skipped) of splitmix64(seed)."""
    with np.errstate(over="ignore"):
        k = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed, count, offset=0):
    """Doubles in [0, 1) with 53 random bits."""
    return (splitmix64(seed, count, offset) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed, count, sigma=1.0):
    """Box-Muller normals, two uniforms per value (cosine branch only)."""
    u = uniform(seed, 2 * count).reshape(count, 2)
    u1 = 1.0 - u[:, 0]  # (0, 1]
    return sigma * np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u[:, 1])


def lattice_spacing(n):
    """s = (0.125 / n)^(1/3), the spacing that puts n points in [0, 0.5]^3."""
    return float(np.float32((0.125 / n) ** (1.0 / 3.0)))


def dambreak_positions(n, seed=20250101, spacing=None):
    """float32 (n, 4) positions, w = 1, of the jittered dam-break lattice."""
    s = lattice_spacing(n) if spacing is None else float(spacing)
    side = int(math.ceil(0.5 / s - 1e-9))
    layer = side * side
    k = np.arange(n, dtype=np.int64)
    iz, rem = np.divmod(k, layer)
    iy, ix = np.divmod(rem, side)
    jit = (2.0 * uniform(seed, 3 * n).reshape(n, 3) - 1.0) * (0.01 * s)
    pos = np.empty((n, 4), dtype=np.float32)
    pos[:, 0] = (ix + 0.5) * s + jit[:, 0]
    pos[:, 1] = (iy + 0.5) * s + jit[:, 1]
    pos[:, 2] = (iz + 0.5) * s + jit[:, 2]
    pos[:, 3] = 1.0
    return pos


def dambreak(n, scene=0, velocity_sigma=0.0, velocity_seed=11):
    """(pos, vel) float32 (n, 4) of a dam-break scene; vel ~ N(0, sigma^2) per
    component when velocity_sigma > 0 (w lanes 0), else zero."""
    pos = dambreak_positions(n, seed=20250101 + scene)
    vel = np.zeros((n, 4), dtype=np.float32)
    if velocity_sigma > 0:
        vel[:, :3] = normal(velocity_seed, 3 * n, velocity_sigma).reshape(n, 3).astype(np.float32)
    return pos, vel


def rollout_case(n=65536, velocity_sigma=0.1, target_sigma=0.05, target_viscosity=0.03):
    """The differentiable-rollout scene: the dam-break lattice of n particles
    with initial velocities N(0, velocity_sigma^2) per component (seed 11), and
    the initial velocities of its target run, those plus N(0, target_sigma^2)
    (seed 12), to be rolled out with viscosity target_viscosity.

    Returns (pos, vel0, vel0_target, target_viscosity), float32 (n, 4) arrays.
    """
    pos, vel = dambreak(n, scene=0, velocity_sigma=velocity_sigma, velocity_seed=11)
    vt = vel.copy()
    vt[:, :3] += normal(12, 3 * n, target_sigma).reshape(n, 3).astype(np.float32)
    return pos, vel, vt, float(target_viscosity)


def sample_coordinates(n, count, seed=13, offset=0):
    """`count` distinct (particle, axis) pairs drawn uniformly (seeded)."""
    out, k = [], offset
    seen = set()
    while len(out) < count:
        u = uniform(seed, 1, offset=k)[0]
        k += 1
        c = int(u * 3 * n)
        if c in seen:
            continue
        seen.add(c)
        out.append((c // 3, c % 3))
    return out, k


# --- triangle meshes (rtps Triangle: three vertices and a normal, 16 floats,
#     rtpslib/structs.h:586-590) ------------------------------------------------

def _triangles(verts):
    """(m, 3, 3) vertices -> (m, 4, 4) float32 triangles: vertices with w = 1,
    then the unit normal (b - a) x (c - a) with w = 0."""
    v = np.asarray(verts, np.float64)
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    t = np.zeros((v.shape[0], 4, 4), np.float32)
    t[:, :3, :3] = v
    t[:, :3, 3] = 1.0
    t[:, 3, :3] = n
    return t


def ramp_mesh(nx=16, ny=16, z0=0.12, z1=0.22, lo=(0.0, 0.0), hi=(1.0, 1.0)):
    """A plane z = z0 + (z1 - z0) x over [lo, hi] in x, y, as nx*ny quads of
    two triangles each, normals pointing up."""
    xs = np.linspace(lo[0], hi[0], nx + 1)
    ys = np.linspace(lo[1], hi[1], ny + 1)
    z = lambda x: z0 + (z1 - z0) * x
    tris = []
    for j in range(ny):
        for i in range(nx):
            a = (xs[i], ys[j], z(xs[i]))
            b = (xs[i + 1], ys[j], z(xs[i + 1]))
            c = (xs[i + 1], ys[j + 1], z(xs[i + 1]))
            d = (xs[i], ys[j + 1], z(xs[i]))
            tris.append((a, b, c))
            tris.append((a, c, d))
    return _triangles(tris)


def box_mesh(lo, hi):
    """The surface of an axis-aligned box, 12 triangles, normals outwards."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    c = [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0),
         (x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)]
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (3, 0, 4, 7)]
    tris = []
    for a, b, cc, d in quads:
        tris.append((c[a], c[b], c[cc]))
        tris.append((c[a], c[cc], c[d]))
    return _triangles(tris)


def ramp_and_box_mesh():
    """The triangle-collision scene's mesh: a 16 x 16-quad ramp through the
    dam-break block (512 triangles) and a box obstacle beside it (12)."""
    return np.concatenate([ramp_mesh(), box_mesh((0.6, 0.3, 0.0), (0.75, 0.6, 0.3))])
