"""bench.py's byte model: the step's kernels carry exactly the reference's
per-stage algorithmic bytes, 412 N + 24 C (one read of each input and one
write of each output per stage, physics fields only), whatever kernels the
stages were fused into or split across."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_kernel_bytes_sum_to_the_stage_bytes():
    import bench
    for n, c in ((2097152, 2299968), (16384, 27000), (1, 1)):
        ab = bench.algorithmic_bytes(n, c)
        assert sum(ab.values()) == 412.0 * n + 24.0 * c
        assert all(v >= 0 for v in ab.values())
    assert abs(sum(bench.algorithmic_bytes(2097152, 2299968).values()) - 919.225856e6) < 1.0
