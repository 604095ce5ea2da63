"""Scripted hose runs shared by the hose tests and the golden fixture.

A script creates a hose, sprays it, moves it, refills it; run_script drives
one through an adapter (the reference's Hose in oracle/_ref, or the
library's sph_hose) after seeding the C library's rand(), and returns every
spray's particles and push velocity."""
import ctypes as C

import numpy as np

# (dt, total_n, center, velocity, radius, spacing), then the calls
SCRIPTS = {
    # y velocity 0 (replaced by 1e-7), a spray every call
    "down": ((0.001, 400, (0.5, 0.5, 0.8, 1.0), (0.3, 0.0, -1.0, 0.0), 0.04, 0.01),
             [("spray", 12), ("update", (0.4, 0.45, 0.7, 1.0), (0.0, 0.2, -0.8, 0.0), 0.05, 0.01), ("spray", 6),
              ("refill", 150), ("spray", 8)]),
    # slow: a spray every 18 calls; total_n below one disc
    "slow": ((0.001, 30, (0.2, 0.3, 0.4, 1.0), (0.0, 0.05, -0.1, 0.0), 0.06, 0.02),
             [("spray", 40), ("refill", 200), ("spray", 60)]),
    # sideways, large disc
    "side": ((0.0005, 2000, (0.1, 0.5, 0.5, 1.0), (2.0, 0.1, 0.05, 0.0), 0.1, 0.0078125),
             [("spray", 5)]),
}
SEEDS = {"down": 11, "slow": 12, "side": 13}


def libc():
    return C.CDLL(None)


def run_script(name, make):
    """make(dt, total_n, center, velocity, radius, spacing) -> adapter with
    spray() -> (pos (k, 4), velocity (4,)), update(c, v, r, s), refill(n)."""
    (dt, n, c, v, r, s), calls = SCRIPTS[name]
    libc().srand(SEEDS[name])
    h = make(dt, n, c, v, r, s)
    counts, pos, vel = [], [], []
    for call in calls:
        if call[0] == "spray":
            for _ in range(call[1]):
                p, pv = h.spray()
                counts.append(p.shape[0])
                pos.append(p)
                vel.append(pv)
        elif call[0] == "update":
            h.update(*call[1:])
        else:
            h.refill(call[1])
    return (np.asarray(counts, np.int32), np.concatenate(pos).reshape(-1, 4).astype(np.float32),
            np.asarray(vel, np.float32))


class RefHose:
    """The reference's Hose (oracle/_ref)."""

    def __init__(self, dt, n, c, v, r, s):
        import oracle_bind as ob
        self.L = ob.ref()
        cc, vv = np.asarray(c, np.float32), np.asarray(v, np.float32)
        self.h = self.L.ref_hose_create(dt, n, cc.ctypes.data, vv.ctypes.data, r, s)
        self.buf = np.zeros((65536, 4), np.float32)

    def spray(self):
        v = np.zeros(4, np.float32)
        k = self.L.ref_hose_spray(self.h, self.buf.ctypes.data, self.buf.shape[0], v.ctypes.data)
        return self.buf[:k].copy(), v

    def update(self, c, v, r, s):
        cc, vv = np.asarray(c, np.float32), np.asarray(v, np.float32)
        self.L.ref_hose_update(self.h, cc.ctypes.data, vv.ctypes.data, r, s)

    def refill(self, n):
        self.L.ref_hose_refill(self.h, n)
