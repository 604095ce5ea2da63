"""sph_sort_pairs_noalloc: the sort for callers that cannot allocate device
memory (their application owns every byte through its own pool, or a frame
loop cannot afford an allocation's synchronisation).  It must give exactly
what the context's own sort (sph_stage_sort) gives, call after call, without
touching its inputs.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from enjaparticles_gb300 import abi, scenes
from enjaparticles_gb300.sph import SPH

pytestmark = pytest.mark.gpu


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
    torch = pytest.importorskip("torch")  # the test, as the caller, owns the device arrays
    lib = abi.load_library()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n, seed in ((262144, 3), (70001, 4)):
        keys, vals, ref_k, ref_v, bits = _scene_keys(n, seed)
        dk = torch.from_numpy(keys.view(np.int32)).cuda()
        dv = torch.from_numpy(vals.view(np.int32)).cuda()
        ok = torch.empty_like(dk)
        ov = torch.empty_like(dv)
        torch.cuda.synchronize()
        rc = lib.sph_sort_pairs_noalloc(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), n, bits, stream)
        assert rc == abi.SPH_OK
        np.testing.assert_array_equal(ok.cpu().numpy().view(np.uint32), ref_k)
        np.testing.assert_array_equal(ov.cpu().numpy().view(np.uint32), ref_v)
        np.testing.assert_array_equal(dk.cpu().numpy().view(np.uint32), keys)  # inputs untouched
        np.testing.assert_array_equal(dv.cpu().numpy().view(np.uint32), vals)


def test_noalloc_sort_rejects_oversize_requests():
    lib = abi.load_library()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert lib.sph_sort_pairs_noalloc(dummy, dummy, dummy, dummy, (1 << 20) + 1, 24, None) == abi.SPH_EINVAL
    assert lib.sph_sort_pairs_noalloc(dummy, dummy, dummy, dummy, 1000, 33, None) == abi.SPH_EINVAL
