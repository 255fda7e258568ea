"""Registration driver on the GPU (scale filter, normalisation, levels,
upscale/refine, minimizers) against the oracle's CPU restatement."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FINAL_COST_RTOL = 1e-4


def _pair2d(seed, shape=(80, 96), rate=16.0):
    from mia_gb300 import synth
    ref = synth.blob_phantom(shape, 8, sigma=(4, 10), seed=seed)
    lv = O.Level(shape[::-1], rate=rate)
    lv.set_images(ref, ref)
    mov = lv.warp(synth.spline_params(lv.nparams // 2, 2, 1.5, 3.0, seed=seed + 1))
    return mov, ref


def _pair3d(seed, shape=(32, 36, 40), rate=8.0, bias=False):
    from mia_gb300 import synth
    ref = synth.blob_phantom(shape, 10, sigma=(3, 8), seed=seed)
    lv = O.Level(shape[::-1], rate=rate)
    lv.set_images(ref, ref)
    mov = lv.warp(synth.spline_params(lv.nparams // 3, 3, 1.5, 3.0, seed=seed + 1))
    if bias:
        mov = (mov * synth.bias_field(shape, 0.1, seed=seed + 2)).astype(np.float32)
    return mov, ref


@pytest.mark.parametrize("shape,out", [((80, 96), (40, 48)), ((56, 44), (14, 11)), ((32, 36, 40), (16, 18, 20)),
                                       ((48, 40, 36), (12, 10, 9)),
                                       # many blocks of lines, one axis copied unchanged
                                       ((40, 150, 200), (40, 75, 100)),
                                       # odd sizes, factor 4 in x and y, about 2 in z
                                       ((33, 70, 130), (17, 18, 33))])
def test_scale_filter_matches_oracle(shape, out):
    from mia_gb300 import registration as R
    from mia_gb300 import synth
    img = synth.blob_phantom(shape, 6, sigma=(3, 8), seed=3)
    g = R.scale_image(img, out)
    o = O.scale_image(img, out)
    assert np.max(np.abs(g - o)) <= 1e-5 * np.max(np.abs(o))


def test_normalize_matches_oracle():
    from mia_gb300 import registration as R
    mov, ref = _pair2d(5)
    ok_g, sg, rg, mg, sgg = R.normalize_pair(mov * 3 + 7, ref * 3 + 7)
    ok_o, so, ro, mo, sgo = O.normalize_pair(mov * 3 + 7, ref * 3 + 7)
    assert ok_g and ok_o
    assert abs(mg - mo) <= 1e-9 * abs(mo) and abs(sgg - sgo) <= 1e-9 * abs(sgo)
    np.testing.assert_allclose(sg, so, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(rg, ro, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("path", ["split", "plain"])
@pytest.mark.parametrize("kind", ["gsl", "gdsq"])
def test_register_2d_matches_oracle(path, kind):
    from mia_gb300 import registration as R
    mov, ref = _pair2d(11)
    mg = R.minimizer(kind, maxiter=12, step=0.1)
    mo = O.minimizer(kind, maxiter=12, step=0.1)
    pg, csg, fg, ng = R.register_pair(mov, ref, 16.0, 2, mg, path=path, cost="ssd", penalty_weight=10.0)
    po, cso, fo, no = O.register(mov, ref, 16.0, 2, mo, cost="ssd", penalty_weight=10.0)
    assert csg == cso
    assert abs(fg - fo) <= FINAL_COST_RTOL * abs(fo), (fg, fo)
    assert np.linalg.norm(pg - po) <= 1e-3 * np.linalg.norm(po)


@pytest.mark.parametrize("cost,kind", [("ssd", "gsl"), ("ncc", "gdsq")])
def test_register_3d_matches_oracle(cost, kind):
    from mia_gb300 import registration as R
    mov, ref = _pair3d(21, bias=cost == "ncc")
    mg = R.minimizer(kind, maxiter=6, step=0.1)
    mo = O.minimizer(kind, maxiter=6, step=0.1)
    pw = 10.0 if cost == "ssd" else 5.0
    pg, csg, fg, ng = R.register_pair(mov, ref, 8.0, 2, mg, cost=cost, penalty_weight=pw)
    po, cso, fo, no = O.register(mov, ref, 8.0, 2, mo, cost=cost, penalty_weight=pw)
    assert csg == cso
    assert abs(fg - fo) <= FINAL_COST_RTOL * abs(fo), (fg, fo)
    assert np.linalg.norm(pg - po) <= 1e-3 * np.linalg.norm(po)


@pytest.mark.parametrize("dim", [2, 3])
def test_registered_transform_saved_loaded_and_applied(tmp_path, dim):
    """the output of a registration program: the transformation written with
    the transformation IO, read back, and the moving image warped with it"""
    from mia_gb300 import registration as R
    mov, ref = _pair2d(7) if dim == 2 else _pair3d(8)
    rate = 16.0 if dim == 2 else 8.0
    mz = R.minimizer("gsl", maxiter=20, step=0.1)
    params, csize, cost, _ = R.register_pair(mov, ref, rate, 1, mz, cost="ssd", penalty_weight=10.0)
    size = mov.shape[::-1]
    f = tmp_path / ("reg.x%ddt" % dim)
    R.save_transform(f, size, csize, params, rate=rate)
    t = R.load_transform(f)
    assert t["csize"] == tuple(csize) and t["creator"] == "spline:rate=%g" % rate
    warped = R.warp_image(mov, t["csize"], t["params"])
    np.testing.assert_array_equal(warped, R.warp_image(mov, csize, params))
    before = float(np.sum((mov.astype(np.float64) - ref) ** 2))
    after = float(np.sum((warped.astype(np.float64) - ref) ** 2))
    assert after < 0.8 * before
