"""Boxes filled by rtps::SPH::addBox (System.cpp:331-338 -> addRect,
rtpslib/domain/IV.cpp:165-202) in the tests: (name, scene particle count,
simulation_scale, num, lo, hi).  The spacing is the system's getSpacing():
rest_distance / simulation_scale through the settings map (6 significant
digits, SPHSettings.cpp:94-96), so a simulation_scale other than 1 makes the
rounding matter."""

CASES = [
    ("unit_scale", 4096, 1.0, 500, (0.1, 0.2, 0.05, 0.0), (0.3, 0.45, 0.2, 0.0)),
    ("scaled", 4096, 0.7, 3000, (0.05, 0.05, 0.05, 0.0), (0.5, 0.5, 0.5, 0.0)),
    ("truncated", 16384, 1.3, 257, (0.0, 0.0, 0.0, 0.0), (1.0, 1.0, 1.0, 0.0)),
    ("short_box", 4096, 1.0, 4096, (0.2, 0.2, 0.2, 0.0), (0.25, 0.3, 0.21, 0.0)),
]


def scene_params(n, scale):
    """The dam-break parameter block of n particles with simulation_scale
    replaced (the grids are derived from it by sph_create)."""
    import oracle_bind
    sp, g, _ = oracle_bind.dambreak_params(n)
    sp.simulation_scale = scale
    return sp, g


def spacing(sp):
    import oracle_bind
    return oracle_bind.settings_round(sp.rest_distance / sp.simulation_scale)
