"""spl_sort_pairs_no_alloc: the pair sort for callers that cannot allocate device memory.

Some callers of this library cannot call cudaMalloc when they sort: a host that gives all device
memory to its own pool up front, a plug-in that may only touch the buffers it is handed, or a loop
that must not take the device-wide synchronisation an allocation may imply.  The no-allocation entry point serves them with scratch from a
static device array (at most 262,144 pairs per call).  This test calls it through the C ABI and
checks that two calls in a row give exactly the output of the existing entry point, spl_sort_pairs
(integer keys and values: the tolerance is zero), that every key width routes its passes correctly
(8 and 24 bits take an odd number of passes, so the first one writes straight into the outputs), and
that the call's status word reads back clean.  It lives in its own file so that pytest collects it
last.
"""
import ctypes

import numpy as np
import pytest

from splatter_gb300 import Configuration, Renderer
from splatter_gb300 import _lib

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_no_alloc_sort_matches_sort_pairs_on_two_calls(cuda):
    import torch
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    r = Renderer(Configuration(max_splat_count=_lib.NO_ALLOC_MAX_PAIRS))
    cases = [(200_003, 32, 5000), (_lib.NO_ALLOC_MAX_PAIRS, 16, 40)]  # second call: other size, other key width
    for call, (n, bits, distinct) in enumerate(cases):
        rng = np.random.default_rng(1234 + call)
        keys = (rng.integers(0, distinct, n, dtype=np.int64) * 2654435761 % (1 << 32)).astype(np.uint32)
        vals = rng.permutation(n).astype(np.uint32)
        kd = torch.from_numpy(keys.view(np.int32)).cuda()
        vd = torch.from_numpy(vals.view(np.int32)).cuda()
        # existing entry point
        k_ref, v_ref = r.sort_pairs(kd, vd, key_bits=bits)
        # no-allocation entry point, through the C ABI
        k_out = torch.empty_like(kd)
        v_out = torch.empty_like(vd)
        _lib.check(lib.spl_sort_pairs_no_alloc(_ptr(kd), _ptr(vd), _ptr(k_out), _ptr(v_out), n, bits, stream))
        torch.cuda.synchronize()
        assert torch.equal(k_out, k_ref), f"call {call}: keys differ"
        assert torch.equal(v_out, v_ref), f"call {call}: values differ"
        mask = np.uint32((1 << bits) - 1) if bits < 32 else np.uint32(0xFFFFFFFF)
        order = np.argsort(keys & mask, kind="stable")
        assert np.array_equal(v_out.cpu().numpy().view(np.uint32), vals[order])
        err = ctypes.c_uint32(99)
        assert lib.spl_sort_pairs_no_alloc_status(stream, ctypes.byref(err)) == 0
        assert err.value == 0


@pytest.mark.parametrize("n,bits", [(1, 8), (4095, 24), (70_001, 8), (9_000, 24), (4096, 32)])
def test_no_alloc_sort_every_key_width(cuda, n, bits):
    """Odd pass counts (8, 24 bits) write the first pass straight into the outputs; counts below and at
    one 4096-key tile.  Exact against spl_sort_pairs and numpy's stable argsort of the masked keys."""
    import torch
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    r = Renderer(Configuration(max_splat_count=max(n, 16)))
    rng = np.random.default_rng(n + bits)
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    keys[::7] = keys[0]  # ties: stability is visible
    vals = rng.permutation(n).astype(np.uint32)
    kd = torch.from_numpy(keys.view(np.int32)).cuda()
    vd = torch.from_numpy(vals.view(np.int32)).cuda()
    k_ref, v_ref = r.sort_pairs(kd, vd, key_bits=bits)
    k_out = torch.full_like(kd, -1)
    v_out = torch.full_like(vd, -1)
    _lib.check(lib.spl_sort_pairs_no_alloc(_ptr(kd), _ptr(vd), _ptr(k_out), _ptr(v_out), n, bits, stream))
    assert lib.spl_sort_pairs_no_alloc_status(stream, None) == 0
    assert torch.equal(k_out, k_ref) and torch.equal(v_out, v_ref)
    order = np.argsort(keys & np.uint32((1 << bits) - 1 if bits < 32 else 0xFFFFFFFF), kind="stable")
    assert np.array_equal(v_out.cpu().numpy().view(np.uint32), vals[order])
    assert np.array_equal(k_out.cpu().numpy().view(np.uint32), keys[order])


def test_no_alloc_sort_of_nothing_leaves_the_outputs(cuda):
    import torch
    lib = _lib.load()
    kd = torch.arange(8, dtype=torch.int32, device="cuda")
    k_out = torch.full((8,), 7, dtype=torch.int32, device="cuda")
    v_out = torch.full((8,), 9, dtype=torch.int32, device="cuda")
    assert lib.spl_sort_pairs_no_alloc(_ptr(kd), _ptr(kd), _ptr(k_out), _ptr(v_out), 0, 32, None) == 0
    torch.cuda.synchronize()
    assert int(k_out.sum()) == 56 and int(v_out.sum()) == 72


def test_no_alloc_sort_rejects_counts_above_its_maximum(cuda):
    import torch
    lib = _lib.load()
    n = _lib.NO_ALLOC_MAX_PAIRS + 1
    kd = torch.zeros(n, dtype=torch.int32, device="cuda")
    vd = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = lib.spl_sort_pairs_no_alloc(_ptr(kd), _ptr(vd), _ptr(kd), _ptr(vd), n, 32, None)
    assert rc == _lib.SPL_ERR_INVALID
    assert b"at most" in lib.spl_last_error_string()
