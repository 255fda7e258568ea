"""The reference's 2D known answers through the GPU path (C ABI).

The same cases as the oracle's 2D golden tests (tests/test_oracle_goldens.py):
the spline transformation's shift and translate tests
(mia/2d/transform/test_spline.cc), the field reproduction of the fixture's
transformation, the coefficient grid from a rate, and the divcurl penalty's
analytic values (mia/2d/test_ppmatrix.cc, mia/2d/splinepenalty/
test_divcurl.cc) evaluated by the 2D gather kernel; each GPU result is also
compared with the oracle's at the parity tolerances.
"""
import math
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import golden2d  # noqa: E402

pytestmark = pytest.mark.gpu


def close_pct(a, b, pct):
    d = abs(a - b)
    return a == b or (d <= pct / 100.0 * abs(a) and d <= pct / 100.0 * abs(b))


@pytest.mark.parametrize("path", ["split", "plain"])
def test_golden_shift_2d_through_gpu(goldens, path):
    import mia_gb300 as M
    g = goldens["test_splines_transform_2d"]
    n = g["size"]
    img = np.array(g["src"], np.float32).reshape(n[1], n[0])
    lv = M.Level(tuple(n), csize=tuple(g["coeff_size"]))
    lv.set_path(path)
    lv.set_images(img, img)
    w = lv.warp(np.tile(np.array(g["shift"]), lv.nparams // 2))
    want = np.array(g["ref"], np.float32).reshape(n[1], n[0])
    m = (want > g["compare_if_above"]) | (w > g["compare_if_above"])
    np.testing.assert_allclose(w[m], want[m], rtol=g["tol_pct"] / 100)


def test_golden_translate_2d_through_gpu(goldens):
    import mia_gb300 as M
    g = goldens["test_splines_translate_2d"]
    r = g["range"]
    lv = M.Level(tuple(r), csize=tuple(g["coeff_size"]))
    force = np.ascontiguousarray(np.broadcast_to(np.array(g["force"], np.float32), (r[1], r[0], 2)))
    cs = lv.csize
    scale = np.prod([(r[i] - 1.0) / (cs[i] - 1 - 2) for i in range(2)])
    gr = lv.translate(force).reshape(cs[1], cs[0], 2)
    inner = gr[4:cs[1] - 3, 4:cs[0] - 3].reshape(-1, 2)
    want = np.array(g["expect_scaled"]) * scale
    np.testing.assert_allclose(inner, np.broadcast_to(want, inner.shape), rtol=g["tol_pct"] / 100)
    o = O.Level(tuple(r), csize=tuple(g["coeff_size"]))
    og = o.translate(force)
    assert np.linalg.norm(lv.translate(force) - og) <= 1e-5 * np.linalg.norm(og)


def test_golden_field_reproduction_2d_through_gpu(goldens):
    """x - T(x) = f(x) for the fixture's transformation, read off the GPU
    warp of the coordinate ramps I(x, y) = x and I(x, y) = y at pixels
    far enough from the border that the mirror-prefiltered ramp is linear
    to float precision (12 pixels: the prefilter's pole^12 < 2e-7)"""
    import mia_gb300 as M
    g = goldens["test_splinestransform_prefix_iterator_2d"]
    r = g["range"]
    lv = M.Level(tuple(r), csize=tuple(g["coeff_size"]))
    p = golden2d.fixture_coefficients(g).ravel()
    X, Y = np.meshgrid(np.arange(r[0], dtype=np.float32), np.arange(r[1], dtype=np.float32))
    fx, fy = golden2d.fixture_field(g, X, Y)
    sl = (slice(12, r[1] - 12), slice(12, r[0] - 12))
    for ramp, want in ((X, fx), (Y, fy)):
        lv.set_images(ramp, ramp)
        u = ramp - lv.warp(p)
        assert np.all(np.abs(u[sl] - want[sl]) <= g["tol_pct"] / 100 * np.abs(want[sl]))


def test_golden_c_rate_grid_2d(goldens):
    import mia_gb300 as M
    g = goldens["test_spline_c_rate_create_2d"]
    lv = M.Level(tuple(g["size"]), rate=tuple(g["c_rate"]))
    assert list(lv.csize) == g["coeff_size"]
    img = np.random.default_rng(3).normal(size=tuple(g["size"][::-1])).astype(np.float32)
    lv.set_images(img, img)
    # zero coefficients: the identity; the warp interpolates the image at
    # the pixel centres, equal to it up to the prefilter's float rounding
    w = lv.warp(np.zeros(lv.nparams))
    assert np.max(np.abs(w - img)) <= 1e-5 * np.max(np.abs(img))


def _gpu_penalty(size, csize, coeffs, wd, wr, weight=1.0):
    import mia_gb300 as M
    lv = M.Level(size, csize=csize, penalty_weight=weight, div=wd, curl=wr)
    z = np.zeros(size[::-1], np.float32)
    lv.set_images(z, z)
    return lv.value(coeffs.ravel())[1]


def test_golden_divcurl_matrix_2d_through_gpu(goldens):
    """the analytic values of the 2D matrix tests; the matrix's range is
    the image size of the level (the penalty's range), 2 range here"""
    for name, c in goldens["divcurl_matrix_2d"].items():
        if "checks" not in c:
            continue
        coeffs, fr = golden2d.ppmatrix_coefficients(c)
        size = tuple(int(v) for v in fr)
        csize = (coeffs.shape[1], coeffs.shape[0])
        # the scale of the terms a near-zero value cancels out of: the full
        # divcurl value of the same field (float arithmetic on the GPU)
        scale = abs(O.divcurl_matrix(coeffs, fr, 1.0, 1.0, with_grad=False, as_float=True, mode=1))
        for chk in c["checks"]:
            if chk["wdiv"] == 0.0 and chk["wrot"] == 0.0:
                continue
            # the level's penalty needs a positive weight: a zero div or
            # curl weight is expressed by the div / curl factors
            v = _gpu_penalty(size, csize, coeffs, chk["wdiv"], chk["wrot"])
            o = O.divcurl_matrix(coeffs, fr, chk["wdiv"], chk["wrot"], with_grad=False, as_float=True, mode=1)
            assert abs(v - o) <= 1e-5 * max(abs(o), scale), (name, chk, v, o)
            if chk["expect"] == "zero":
                assert close_pct(1.0 + v, 1.0, chk["tol_pct"]), (name, chk, v)
            else:
                want = {"6*pi": 6 * math.pi, "4*pi": 4 * math.pi}[chk["expect"]]
                assert close_pct(v, want, chk["tol_pct"]), (name, chk, v)


def test_golden_divcurl_penalty_2d_through_gpu(goldens):
    for name, c in goldens["divcurl_penalty_2d"].items():
        coeffs = golden2d.penalty_coefficients(c)
        size = tuple(int(v) for v in c["range"])
        v = _gpu_penalty(size, tuple(c["size"]), coeffs, c["div"], c["curl"], c["weight"])
        assert close_pct(v, c["value_over_pi"] * math.pi, c["tol_pct"]), (name, v)
        o = O.Level(size, csize=tuple(c["size"]), penalty_weight=c["weight"], div=c["div"], curl=c["curl"])
        z = np.zeros(size[::-1], np.float32)
        o.set_images(z, z)
        assert abs(v - o.value(coeffs.ravel())[1]) <= 1e-5 * abs(v), name


@pytest.mark.parametrize("name", ["test_divergence_expm2_bspline3_grad", "test_rotation_expm2_bspline3_grad_noiso"])
def test_golden_divcurl_gradient_2d_through_gpu(goldens, name):
    """the penalty gradient of the GPU gather against the oracle's, whose
    FD agreement the reference's gradient tests pin (reference sign:
    -weight * gradient)"""
    import mia_gb300 as M
    c = goldens["divcurl_matrix_2d"][name]
    coeffs, fr = golden2d.ppmatrix_coefficients(c)
    size = tuple(int(v) for v in fr)
    csize = (coeffs.shape[1], coeffs.shape[0])
    lv = M.Level(size, csize=csize, penalty_weight=1.0, div=c["wdiv"], curl=c["wrot"])
    z = np.zeros(size[::-1], np.float32)
    lv.set_images(z, z)
    _, cp, _, gp, _ = lv.evaluate(coeffs.ravel())
    _, og = O.divcurl_matrix(coeffs, fr, c["wdiv"], c["wrot"], with_grad=True, as_float=True, mode=0)
    og = -og.ravel()
    assert np.linalg.norm(gp - og) <= 1e-4 * np.linalg.norm(og)
