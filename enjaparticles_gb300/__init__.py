"""GB300 (sm_103a) SPH particle step of the RTPS / EnjaParticles particle system.

The compute lives in librtps_sph.so (include/rtps_sph.h); this package holds
its in-tree build (build_ext), a ctypes view of the ABI (abi), the Python mirror
of rtps::SPH (sph) and the seeded benchmark scenes (scenes).
"""
from . import abi, scenes  # noqa: F401

__all__ = ["abi", "scenes", "SPH", "dambreak_system"]


def __getattr__(name):
    if name in ("SPH", "dambreak_system"):
        from . import sph
        return getattr(sph, name)
    raise AttributeError(name)
