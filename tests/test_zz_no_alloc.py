"""sph_sort_pairs_noalloc: the sort for callers that cannot allocate device
memory (their application owns every byte through its own pool, or a frame
loop cannot afford an allocation's synchronisation).  It must give exactly
what a stable sort on the low key_bits bits of the keys gives (numpy's
stable argsort here) and what the context's own sort (sph_stage_sort) gives,
call after call, without touching its inputs.  This file is collected last
on purpose: it runs after every other GPU test, and alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu


def _stable(keys, vals, key_bits):
    mask = np.uint32(0xFFFFFFFF) if key_bits == 32 else np.uint32((1 << key_bits) - 1)
    order = np.argsort(keys & mask, kind="stable")
    return keys[order], vals[order]


def _sort(lib, torch, keys, vals, key_bits):
    """Two calls in a row on the same inputs; both outputs, inputs checked untouched."""
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals.view(np.int32)).cuda()
    outs = []
    for _ in range(2):
        ok = torch.full_like(dk, -1)
        ov = torch.full_like(dv, -1)
        torch.cuda.synchronize()
        rc = lib.sph_sort_pairs_noalloc(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), len(keys),
                                        key_bits, stream)
        assert rc == abi.SPH_OK
        outs.append((ok.cpu().numpy().view(np.uint32), ov.cpu().numpy().view(np.uint32)))
    np.testing.assert_array_equal(dk.cpu().numpy().view(np.uint32), keys)
    np.testing.assert_array_equal(dv.cpu().numpy().view(np.uint32), vals)
    return outs


# key widths 8, 16, 24, 32 bits: 1, 2, 3 and 4 radix passes (the last pass
# lands in the caller's output from either parity of the ping-pong); random
# bits above key_bits must not take part in the ordering.
@pytest.mark.parametrize("key_bits", [8, 12, 16, 24, 32])
@pytest.mark.parametrize("n", [1, 4097, 1 << 20])
def test_noalloc_sort_equals_stable_argsort(n, key_bits):
    torch = pytest.importorskip("torch")  # the test, as the caller, owns the device arrays
    lib = abi.load_library()
    rng = np.random.default_rng(1000 * key_bits + n % 997)
    keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    if n > 64:
        keys[::7] = keys[3]  # runs of equal keys
    vals = np.arange(n, dtype=np.uint32)[::-1].copy()
    want_k, want_v = _stable(keys, vals, key_bits)
    for got_k, got_v in _sort(lib, torch, keys, vals, key_bits):
        np.testing.assert_array_equal(got_k, want_k)
        np.testing.assert_array_equal(got_v, want_v)


def _scene_keys(n, seed):
    """Unsorted (key, index) pairs from the hash stage, and the stage sort's result."""
    sp, g, gs = abi.dambreak_params(n)
    u = scenes.uniform(seed, 3 * n).reshape(n, 3)
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = (u * 1.4 - 0.2).astype(np.float32)  # some particles outside the grid
    pos[::11, :3] = pos[7, :3]                       # many equal keys
    s = SPH(sp, g, n, gs)
    s.upload(pos, np.zeros_like(pos))
    s.hash()
    keys = s.get("sort_hashes", n)
    vals = s.get("sort_indices", n)
    s.sort()
    ref_k = s.get("sort_hashes", n)
    ref_v = s.get("sort_indices", n)
    s.close()
    bits = max(1, int(g.nb_cells).bit_length())
    return keys, vals, ref_k, ref_v, bits


def test_noalloc_sort_matches_stage_sort_on_two_calls():
    torch = pytest.importorskip("torch")
    lib = abi.load_library()
    for n, seed in ((262144, 3), (70001, 4)):
        keys, vals, ref_k, ref_v, bits = _scene_keys(n, seed)
        want_k, want_v = _stable(keys, vals, bits)
        np.testing.assert_array_equal(ref_k, want_k)
        np.testing.assert_array_equal(ref_v, want_v)
        for got_k, got_v in _sort(lib, torch, keys, vals, bits):
            np.testing.assert_array_equal(got_k, ref_k)
            np.testing.assert_array_equal(got_v, ref_v)


def test_noalloc_sort_rejects_bad_requests():
    lib = abi.load_library()
    dummy = C.c_void_p(16)  # never dereferenced: the argument checks come first
    assert lib.sph_sort_pairs_noalloc(dummy, dummy, dummy, dummy, (1 << 20) + 1, 24, None) == abi.SPH_EINVAL
    assert lib.sph_sort_pairs_noalloc(dummy, dummy, dummy, dummy, 1000, 33, None) == abi.SPH_EINVAL
    # outputs overlapping an input or each other
    a, b, c, d = (C.c_void_p(0x10000 + k * 0x10000) for k in range(4))
    assert lib.sph_sort_pairs_noalloc(a, b, C.c_void_p(0x10000 + 400), d, 1000, 16, None) == abi.SPH_EINVAL
    assert lib.sph_sort_pairs_noalloc(a, b, c, C.c_void_p(0x30000 + 3996), 1000, 16, None) == abi.SPH_EINVAL
    assert lib.sph_sort_pairs_noalloc(a, b, c, a, 1000, 16, None) == abi.SPH_EINVAL
