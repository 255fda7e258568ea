"""The allocation-free translate entry point, called through the C ABI.

mgr_translate3d_noalloc is for callers that cannot call cudaMalloc: hosts
that give all device memory to their own pool or arena, and latency-bound
callers that cannot afford the implicit device synchronisation of
cudaMalloc/cudaFree.  It keeps its intermediates in a fixed device array
instead of allocating.  On two calls in a row, which reuse (and overwrite)
that array, its result must equal the allocating entry point's
(mgr_level_translate) bit for bit, and the oracle's translate within the
translate tolerance of the parity tests.  The call itself must allocate
nothing: the library's allocation counter does not move, a call made
while the library's next allocation is armed to fail still succeeds, and
the device's free memory is the same before and after the second call
(the first call on a device may set up the array when the runtime loads
the library's device code).  The test owns its buffers (torch allocates
them before the calls).

This file is collected last (pytest runs files in name order), so that a
run stopping at its first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TRANSLATE_RTOL = 1e-5


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_translate_matches_level_translate_and_allocates_nothing():
    import torch

    import mia_gb300 as M
    from mia_gb300 import _lib
    from oracle import oracle as O

    L = _lib.lib()
    size = (48, 40, 36)
    lv = M.Level(size, rate=4.0)
    o = O.Level(size, rate=4.0)
    cs = (ctypes.c_int * 3)(*lv.csize)
    sz = (ctypes.c_int * 3)(*size)
    rng = np.random.default_rng(11)
    grad_d = torch.empty(lv.nparams, dtype=torch.float64, device="cuda")
    force_d = torch.empty(size[::-1] + (3,), dtype=torch.float32, device="cuda")
    for call in range(2):   # two calls in a row share (and overwrite) the scratch array
        force = rng.normal(size=size[::-1] + (3,)).astype(np.float32)
        want = lv.translate(force)
        force_d.copy_(torch.from_numpy(force))
        grad_d.fill_(np.nan)
        torch.cuda.synchronize()
        allocs0 = L.mgr_allocation_count()
        free0 = torch.cuda.mem_get_info()[0]
        _lib.check(L.mgr_debug_fail_allocation(1))   # the library's next allocation would fail
        try:
            st = L.mgr_translate3d_noalloc(sz, cs, ctypes.c_void_p(force_d.data_ptr()),
                                           ctypes.c_void_p(grad_d.data_ptr()), None)
        finally:
            L.mgr_debug_fail_allocation(0)
        _lib.check(st)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert L.mgr_allocation_count() == allocs0, call
        if call == 1:
            assert free1 == free0, (free0, free1)
        got = grad_d.cpu().numpy()
        assert np.all(np.isfinite(got)), call
        assert np.array_equal(got, want), (call, _rel_l2(got, want))
        assert _rel_l2(got, o.translate(force)) < TRANSLATE_RTOL, call
    lv.close()


def test_noalloc_translate_rejects_sizes_beyond_scratch():
    import mia_gb300 as M
    from mia_gb300 import _lib

    sz = (ctypes.c_int * 3)(512, 512, 256)
    cs = (ctypes.c_int * 3)(130, 130, 66)
    st = _lib.lib().mgr_translate3d_noalloc(sz, cs, ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert st == _lib.MGR_ERR_ARG
    assert "scratch" in M.lib().mgr_last_error().decode()
