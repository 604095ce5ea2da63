"""sph_upload copies vel/veleval on a side stream that the step joins only
before cells+permute.  A round trip through the C ABI without any sync
between upload and step (the end-to-end loop) must give the same bits as
upload, sync, step: on the graph, eager and staged paths, with new state
every round so that a late copy would show."""
import numpy as np
import pytest

from enjaparticles_gb300 import abi
from enjaparticles_gb300.scenes import dambreak, normal
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu

DT = 0.001


def _round(s, pos, vel, ve, path):
    n = pos.shape[0]
    lib = s.lib
    s._ck(lib.sph_upload(s.ctx, pos.ctypes.data, vel.ctypes.data, ve.ctypes.data, n))
    if path == "graph":
        s._ck(lib.sph_step(s.ctx, DT, 1))
    elif path == "eager":
        s._ck(lib.sph_step_eager(s.ctx, DT, 1))
    else:
        s._ck(lib.sph_update(s.ctx))
        s._ck(lib.sph_integrate(s.ctx, DT))
    out = [np.empty((n, 4), np.float32) for _ in range(3)]
    for f, o in zip(("pos_u", "vel_u", "veleval_u"), out):
        s._ck(lib.sph_download_async(s.ctx, abi.FIELDS[f], o.ctypes.data, n))
    s.sync()
    return out


@pytest.mark.parametrize("path", ["graph", "eager", "staged"])
def test_upload_overlap_round_trips_match_synced_uploads(path):
    # at 2M the side-stream copies (67 MB) outlast hash and sort, so a step
    # that did not wait for them would read the previous round's velocities
    n = 2097152
    sp, g, gs = abi.dambreak_params(n)
    a = SPH(sp, g, n, gs, exact=True)
    b = SPH(sp, g, n, gs, exact=True)
    pos, vel = dambreak(n, velocity_sigma=0.1)
    for r in range(4):
        v = vel.copy()
        v[:, :3] += normal(100 + r, 3 * n, 0.05).reshape(n, 3).astype(np.float32)
        ve = np.zeros_like(v)
        ve[:, :3] = normal(200 + r, 3 * n, 0.05).reshape(n, 3).astype(np.float32)
        got = _round(a, pos, v, ve, path)
        b.upload(pos, v, ve)  # synchronises after the copy
        if path == "graph":
            b.step(DT, 1)
        elif path == "eager":
            b.step_eager(DT, 1)
        else:
            b.update()
            b.integrate(DT)
        for f, x in zip(("pos_u", "vel_u", "veleval_u"), got):
            np.testing.assert_array_equal(x, b.get(f, n), err_msg="round %d %s" % (r, f))
        pos = got[0]
