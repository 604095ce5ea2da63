"""Helpers of the surface tests: the case table, per-cube case indices of a
field, and triangle comparisons."""
import ctypes as C

import numpy as np

# corner k of the case index and the local edges (point0, point1)
CORNER = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]
EDGE = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


def case_table(lib):
    tri = np.zeros((256, 18), np.int8)
    cnt = np.zeros(256, np.uint8)
    mx = C.c_int()
    assert lib.sph_mc_case_table(tri.ctypes.data, cnt.ctypes.data, C.byref(mx)) == 0
    return tri, cnt, mx.value


def cube_cases(field, res, iso):
    """Case index of every cube, array [z, y, x] of shape (res-1)^3."""
    f = np.asarray(field, np.float32).reshape(res, res, res)  # [r, t, s] = [z, y, x]
    m = res - 1
    case = np.zeros((m, m, m), np.int32)
    for k, (x, y, z) in enumerate(CORNER):
        case |= (f[z:z + m, y:y + m, x:x + m] > np.float32(iso)).astype(np.int32) << k
    return case


def triangle_cubes(vertices, res):
    """(x, y, z) of the cube of each triangle from its centroid; -1 rows for
    non-finite triangles."""
    g = vertices.astype(np.float64) / 10.0 * (res - 1)
    cen = g.mean(axis=1)
    out = np.full((len(vertices), 3), -1, np.int64)
    ok = np.isfinite(cen).all(1)
    out[ok] = np.floor(cen[ok]).astype(np.int64)
    return out


def vertex_rows(vertices, normals):
    """Unique (position, normal) rows as bit patterns, NaNs made canonical."""
    a = np.concatenate([vertices.reshape(-1, 3), normals.reshape(-1, 3)], axis=1).astype(np.float32)
    a = np.where(np.isnan(a), np.float32(np.nan), a)
    return np.unique(a.view(np.uint32), axis=0)
