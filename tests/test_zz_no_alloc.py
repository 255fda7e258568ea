"""The allocation-free translate entry point, called through the C ABI.

mgr_translate3d_noalloc exists for callers that cannot call cudaMalloc
(stream capture, arena-managed hosts, latency-bound callers): it keeps its
intermediates in a fixed device array instead of allocating.  Its result
must equal the allocating entry point's (mgr_level_translate) within the
translate tolerance of the parity tests, on consecutive calls that reuse
the shared array.  The test owns its buffers (torch allocates them); the
entry point under test allocates nothing.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TRANSLATE_RTOL = 1e-5


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_translate_matches_level_translate():
    import torch

    import mia_gb300 as M
    from mia_gb300 import _lib

    size = (48, 40, 36)
    lv = M.Level(size, rate=4.0)
    cs = (ctypes.c_int * 3)(*lv.csize)
    sz = (ctypes.c_int * 3)(*size)
    rng = np.random.default_rng(11)
    grad_d = torch.empty(lv.nparams, dtype=torch.float64, device="cuda")
    for call in range(2):   # two calls in a row share (and overwrite) the scratch array
        force = rng.normal(size=size[::-1] + (3,)).astype(np.float32)
        want = lv.translate(force)
        force_d = torch.from_numpy(force).cuda()
        grad_d.fill_(np.nan)
        torch.cuda.synchronize()
        st = _lib.lib().mgr_translate3d_noalloc(sz, cs, ctypes.c_void_p(force_d.data_ptr()),
                                                 ctypes.c_void_p(grad_d.data_ptr()), None)
        _lib.check(st)
        torch.cuda.synchronize()
        got = grad_d.cpu().numpy()
        assert np.all(np.isfinite(got)), call
        assert _rel_l2(got, want) < TRANSLATE_RTOL, (call, _rel_l2(got, want))


def test_noalloc_translate_rejects_sizes_beyond_scratch():
    import mia_gb300 as M
    from mia_gb300 import _lib

    sz = (ctypes.c_int * 3)(512, 512, 256)
    cs = (ctypes.c_int * 3)(130, 130, 66)
    st = _lib.lib().mgr_translate3d_noalloc(sz, cs, ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert st == _lib.MGR_ERR_ARG
    assert "scratch" in M.lib().mgr_last_error().decode()
