"""Out-of-memory paths without exhausting a device.

mgr_debug_fail_allocation(k) makes the k-th device or page-locked host
allocation of the library fail as an exhausted device would.  For each
entry point below the test fails every one of its allocations in turn
(k = 1, 2, ... until the call makes fewer than k) and checks that the call
returns MGR_ERR_OOM, that nothing else is reported, and that afterwards
the same call without a failure gives the result of a run that never saw
one (the library stays usable; nothing half-made survives).  The failure
is made on the host, before CUDA is asked for memory: no device is driven
out of memory and no kernel runs on a buffer that was not allocated.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenarios():
    import mia_gb300 as M
    from mia_gb300 import registration as R
    from mia_gb300 import synth
    ref3 = synth.blob_phantom((14, 18, 22), 5, sigma=(2.0, 5.0), seed=1)
    mov3 = np.roll(ref3, 1, axis=2)
    ref2 = synth.blob_phantom((40, 48), 6, sigma=(3.0, 8.0), seed=2)
    mov2 = np.roll(ref2, 2, axis=1)
    ref2b = synth.blob_phantom((36, 44), 6, sigma=(3.0, 8.0), seed=3)
    mov2b = np.roll(ref2b, -1, axis=0)
    mz = R.minimizer("gsl", maxiter=4, step=0.1)

    def level3():
        lv = M.Level((22, 18, 14), rate=4.0, cost="ssd", penalty_weight=2.0)
        try:
            lv.set_images(mov3, ref3)
            p = synth.smooth_params(lv.csize, 0.8, seed=4)
            ci, cp, gi, gp, gt = lv.evaluate(p)
            v = lv.value(p)
            w = lv.warp(p)
            _, f = lv.force(p)
            g = lv.translate(f)
            lv.set_path("plain")
            ci2, _, gi2, _, _ = lv.evaluate(p)
            return [ci, cp, gi, gp, v[0], v[1], w, f, g, ci2, gi2]
        finally:
            lv.close()

    def level2():
        lv = M.Level((48, 40), rate=8.0, cost="ncc", penalty_weight=1.0)
        try:
            lv.set_images(mov2, ref2)
            p = synth.smooth_params(lv.csize, 1.0, seed=5)
            ci, cp, gi, gp, gt = lv.evaluate(p)
            return [ci, cp, gi, gp]
        finally:
            lv.close()

    def register():
        r = R.register_pair(mov2, ref2, 8.0, 2, mz, cost="ssd", penalty_weight=1.0)
        return [r[0], r[2]]

    def batch():
        res = R.register_batch([(mov2, ref2), (mov2b, ref2b)], 8.0, 2, mz, cost="ssd", penalty_weight=1.0)
        return [x for r in res for x in (r[0], r[2])]

    def drivers():
        s = R.scale_image(ref2, (20, 24))
        n = R.normalize_pair(mov2, ref2)
        return [s, n[1], n[2]]

    return {"level3d": level3, "level2d": level2, "register": register, "register_batch": batch,
            "scale_normalize": drivers}


def _same(a, b):
    return all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(a, b))


@pytest.mark.parametrize("name", ["level3d", "level2d", "register", "register_batch", "scale_normalize"])
def test_every_allocation_failure_is_reported_and_the_library_stays_usable(name):
    from mia_gb300 import _lib
    L = _lib.lib()
    run = _scenarios()[name]
    want = run()
    failures = 0
    try:
        for k in range(1, 400):
            _lib.check(L.mgr_debug_fail_allocation(k))
            a0 = L.mgr_allocation_count()
            try:
                run()
                ok = True
            except _lib.MgrError as e:
                assert e.status == _lib.MGR_ERR_OOM, (k, e.status, str(e))
                ok = False
                failures += 1
            made = L.mgr_allocation_count() - a0
            _lib.check(L.mgr_debug_fail_allocation(0))
            if ok:
                assert made < k, (k, made)   # a call that saw its k-th allocation fail cannot succeed
                break
            assert _same(run(), want), k
        else:
            pytest.fail("more than 400 allocations")
    finally:
        L.mgr_debug_fail_allocation(0)
    assert failures > 0
    assert _same(run(), want)
