"""The fused 3D SSD path (MGR_PATH_FUSED): one kernel per 30 x 8 x TZ tile
computes the warped image with a one-voxel halo, the force and its adjoint
contraction.  Its cost and gradients must meet the parity tolerances
against the oracle at both precisions (cost 1e-5 relative, gradients 1e-4
relative L2), on sizes that leave partial tiles on every axis, every z
tile, large displacements (taps outside the staged box), the ssd `norm`
and the image boundaries of small volumes; the split path's results are
compared alongside."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return abs(a - b) / abs(b)


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _pair(shape, seed):
    from mia_gb300 import synth
    ref = synth.blob_phantom(shape, 10, sigma=(2.5, 7.0), seed=seed)
    mov = np.roll(ref, 2, axis=2) * 1.05 + 3.0
    return mov.astype(np.float32), ref


CASES = [
    # size (x, y, z), rate, z tile, coefficient amplitude, ssd norm
    ((61, 37, 29), 5.0, 16, 1.5, False),      # partial tiles on every axis
    ((90, 24, 48), 8.0, 32, 2.0, False),      # whole tiles in x and y
    ((30, 8, 16), 4.0, 16, 1.0, True),        # one tile, norm
    ((17, 11, 7), 3.0, 8, 1.0, False),        # smaller than a tile on every axis
    ((64, 40, 33), 6.0, 4, 1.0, False),       # the shallowest z tile
    ((48, 44, 40), 8.0, 16, 9.0, False),      # displacements beyond the staged box
]


@pytest.mark.parametrize("size,rate,tz,amp,norm", CASES)
def test_fused_matches_oracle(size, rate, tz, amp, norm):
    import mia_gb300 as M
    from mia_gb300 import synth
    mov, ref = _pair(size[::-1], seed=sum(size))
    kw = dict(rate=rate, cost="ssd", ssd_norm=norm, penalty_weight=2.0)
    lv = M.Level(size, **kw)
    lv.set_images(mov, ref)
    p = synth.smooth_params(lv.csize, amp, seed=3)
    split = lv.evaluate(p)
    lv.set_path("fused", (0, 0, tz))
    fused = lv.evaluate(p)
    assert lv.tile[2] == tz
    for prec in (O.PREC_REF, O.PREC_F64):
        o = O.Level(size, precision=prec, **kw)
        o.set_images(mov, ref)
        oi, op, ogi, ogp = o.evaluate(p)
        ci, cp, gi, gp, gt = fused
        assert _rel(ci, oi) <= 1e-5 and _rel(cp, op) <= 1e-5, (prec, ci, oi)
        assert _rel_l2(gi, ogi) <= 1e-4 and _rel_l2(gp, ogp) <= 1e-4, (prec, _rel_l2(gi, ogi))
    assert _rel(fused[0], split[0]) <= 1e-5
    assert _rel_l2(fused[2], split[2]) <= 1e-4
    np.testing.assert_array_equal(fused[3], split[3])      # the penalty does not depend on the path
    # repeatable bit for bit; value() (split warp) agrees
    again = lv.evaluate(p)
    for x, y in zip(fused, again):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    assert _rel(lv.value(p)[0], fused[0]) <= 1e-5
    lv.close()


def test_fused_path_is_3d_ssd_only():
    import mia_gb300 as M
    from mia_gb300 import _lib
    lv = M.Level((40, 30, 20), rate=4.0, cost="ncc")
    with pytest.raises(_lib.MgrError) as e:
        lv.set_path("fused")
    assert e.value.status == _lib.MGR_ERR_ARG
    lv2 = M.Level((64, 48), rate=4.0)
    with pytest.raises(_lib.MgrError):
        lv2.set_path("fused")
