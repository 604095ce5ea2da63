"""Settings maps for the reference's settings path (RTPSSettings ->
SPH::calculate / SPH::updateParams / System::setupDomain), shared by the
fixture generator (tests/golden/make_golden.py) and the tests.  Values are
given as RTPSSettings stores them: strings, or numbers / sequences that
abi.settings_value writes as SetSetting would."""

BASE = {"rest_density": 1000, "gas_constant": 15, "viscosity": 0.01, "velocity_limit": 600, "xsph_factor": 0.15,
        "gravity": (0, 0, -9.8, 0), "boundary_stiffness": 20000, "boundary_dampening": 256}

CASES = [
    ("box5_n16384", dict(BASE, max_num_particles=16384, domain_min=(0, 0, 0, 1), domain_max=(5, 5, 5, 1))),
    ("box5_n2097152", dict(BASE, max_num_particles=2097152, domain_min=(0, 0, 0, 1), domain_max=(5, 5, 5, 1))),
    ("slab_n100000", dict(BASE, max_num_particles=100000, domain_min=(-1, -1, 0, 1), domain_max=(2, 3, 1.5, 1),
                          gas_constant=3.5, viscosity=0.05, friction_kinetic=0.2, restitution=0.1)),
    ("unit_n4096", dict(BASE, max_num_particles=4096, domain_min=(0, 0, 0, 0), domain_max=(1, 1, 1, 0),
                        gravity=(0, -9.8, 0, 0))),
    ("odd_n1000", dict(BASE, max_num_particles=1000, rest_density=998.2, domain_min="0 0 0",
                       domain_max="2.5 1 0.75", viscosity="0.001")),
    ("wide_n65536", dict(BASE, max_num_particles=65536, domain_min=(-10, -10, -10, 1), domain_max=(10, 10, 10, 1),
                         shear=0.5, attraction=0.25, spring=2)),
    ("sparse_keys_n8192", {"rest_density": "1000", "max_num_particles": "8192", "domain_min": "0 0 0 1",
                           "domain_max": "3 3 3 1"}),
    ("n2_tiny", dict(BASE, max_num_particles=2, domain_min=(0, 0, 0, 1), domain_max=(1, 1, 1, 1))),
]
