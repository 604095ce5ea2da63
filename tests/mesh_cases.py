"""Particle sets for the triangle-collision tests."""
import numpy as np


def near_mesh_particles(tris, n, bound, scale, seed):
    """n particles placed around the mesh: a random point of a random triangle
    moved along its normal by up to 1.5 boundary distances, velocities
    N(0, 1) (every 50th zero, every 7th along the normal)."""
    from enjaparticles_gb300.scenes import normal, uniform
    t = np.asarray(tris, np.float64).reshape(-1, 4, 4)
    pick = (uniform(seed, n) * t.shape[0]).astype(np.int64)
    b = uniform(seed + 1, 2 * n).reshape(n, 2)
    flip = b.sum(1) > 1
    b[flip] = 1 - b[flip]
    a, e1, e2 = t[pick, 0, :3], t[pick, 1, :3] - t[pick, 0, :3], t[pick, 2, :3] - t[pick, 0, :3]
    nrm = t[pick, 3, :3]
    off = (2 * uniform(seed + 2, n) - 1) * 1.5 * bound / scale
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = a + b[:, :1] * e1 + b[:, 1:] * e2 + off[:, None] * nrm
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = normal(seed + 3, 3 * n).reshape(n, 3)
    vel[::7, :3] = -nrm[::7] * (0.5 + uniform(seed + 4, n)[::7, None])
    vel[::50] = 0.0
    return pos, vel
