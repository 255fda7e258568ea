"""Pin the CPU oracle to the reference's own known-answer tests.

The inputs and expected values come from tests/golden/reference_goldens.json
(extracted from the reference test sources by extract_goldens.py); the
tolerances are the ones the reference tests use.  Tests whose expected
values are formulas (NCC closed form, analytic divcurl integrals, finite
differences) restate the formula here.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O


def close_pct(a, b, pct):
    """BOOST_CHECK_CLOSE semantics: relative difference in percent against
    both operands."""
    if a == b:
        return True
    d = abs(a - b)
    return d <= pct / 100.0 * abs(a) and d <= pct / 100.0 * abs(b)


# ---- SSD --------------------------------------------------------------
@pytest.mark.parametrize("name", ["test_SSD_3D_norm", "test_SSD_3D"])
def test_ssd_3d_golden(goldens, name):
    g = goldens[name]
    a = np.array(g["src"], np.float32).reshape(3, 3, 3)
    b = np.array(g["ref"], np.float32).reshape(3, 3, 3)
    assert close_pct(O.ssd_value(a, b, g["norm"]), g["value"], g["value_tol_pct"])
    _, f = O.ssd_force(a, b, g["norm"])
    # BOOST_CHECK_EQUAL on float vectors: compare with the float-rounded expectation
    np.testing.assert_array_equal(f[1, 1, 1], np.float32(g["force_111"]))


def test_ssd_2d_golden(goldens):
    g = goldens["test_SSD_2D"]
    a = np.array(g["src"], np.float32).reshape(4, 4)
    b = np.array(g["ref"], np.float32).reshape(4, 4)
    assert close_pct(O.ssd_value(a, b, True), g["value"], g["value_tol_pct"])
    c, f = O.ssd_force(a, b, True)
    assert close_pct(c, g["value"], g["value_tol_pct"])
    assert close_pct(f[1, 1, 0], g["force_11"][0], g["force_tol_pct"])
    assert close_pct(f[1, 1, 1], g["force_11"][1], g["force_tol_pct"])


# ---- NCC (mia/3d/cost/test_ncc.cc:31-94) -------------------------------
def _ncc_images():
    z, y, x = np.meshgrid(np.arange(4), np.arange(4), np.arange(4), indexing="ij")
    a = (x + y + z).astype(np.float32)
    return a, x, y, z


def _ncc_closed_form(a, b, thresh):
    a = a.astype(np.float64).ravel()
    b = b.astype(np.float64).ravel()
    n = a.size
    ma, mb = a.sum() / n, b.sum() / n
    s2a = (a * a).sum() - a.sum() * ma
    s2b = (b * b).sum() - b.sum() * mb
    cab = (a * b).sum() - ma * mb * n
    p = s2a * s2b
    assert p > thresh
    return 1.0 - cab * cab / p, (2 * cab / p, cab / s2a, ma, mb)


def test_ncc_zero():
    a, *_ = _ncc_images()
    b = 2 * a
    assert abs(O.ncc_value(b, b)) < 1e-7
    assert abs(O.ncc_value(a, b)) < 1e-7


def test_ncc_nonzero():
    a, x, y, z = _ncc_images()
    b = (x + y * z).astype(np.float32)
    v, (k1, k2, ma, mb) = _ncc_closed_form(a, b, 1e-5)
    assert close_pct(O.ncc_value(a, b), v, 0.1)
    c, f = O.ncc_force(a, b)
    assert close_pct(c, v, 0.01)
    ga = O.gradient(a)
    scale = (k1 * (k2 * (a.astype(np.float64) - ma) - (b.astype(np.float64) - mb))).astype(np.float32)
    np.testing.assert_allclose(f, ga * scale[..., None], rtol=1e-4, atol=1e-6)


# ---- spline kernel, boundary, gradient ---------------------------------
def test_bspline3_derivative_weights(goldens):
    g = goldens["test_bspline3_derivatives"]
    for c in g["cases"]:
        ix = O.fastfloor(c["x"])
        assert [ix - 1 + k for k in range(4)] == g["index"]
        w = O.bspline3_deriv_weights(c["x"] - ix, c["degree"])
        for got, want in zip(w, c["weights"]):
            assert close_pct(got, want, g["tol_pct"])


def test_bspline3_weight_at_consistency():
    # mia/core/splinekernel/test_bspline.cc:280-340: weights at x equal the
    # kernel evaluated at the tap distances
    for x in (-0.5, 1.75, 0.2, 3.9):
        ix = O.fastfloor(x)
        w = O.bspline3_weights(x - ix)
        dw = O.bspline3_dweights(x - ix)
        for k in range(4):
            t = x - (ix - 1 + k)
            assert abs(w[k] - O.bspline3_at(t, 0)) < 1e-12
            assert abs(dw[k] - O.bspline3_at(t, 1)) < 1e-12
    assert O.bspline3_at(-1.5, 2) == 0.5 and O.bspline3_at(0, 2) == -2.0


def test_fastfloor_fixed_point():
    # 2^-16 rounding: a value just below an integer floors to that integer
    assert O.fastfloor(2.9999999) == 3
    assert O.fastfloor(2.99) == 2
    assert O.fastfloor(-0.5) == -1
    assert O.fastfloor(-1e-7) == 0
    assert O.fastfloor(7.0) == 7


def test_mirror_boundary_golden(goldens):
    for name, g in goldens["mirror_boundary"].items():
        got = [O.mirror_fold(i, g["width"]) for i in g["index"]]
        assert got[: g["ncheck"]] == g["result"][: g["ncheck"]], name


def test_prefilter_interpolates():
    # mia/core/splinebc/test_bc.cc:167-238: the prefiltered coefficients
    # reproduce the samples at the grid points
    rng = np.random.default_rng(5)
    for n in (2, 3, 4, 5, 17):
        f = rng.normal(size=n)
        c = O.filter_line(f)
        rec = []
        for i in range(n):
            w = O.bspline3_weights(0.0)
            rec.append(sum(w[k] * c[O.mirror_fold(i - 1 + k, n)] for k in range(4)))
        np.testing.assert_allclose(rec, f, atol=1e-12)


def test_gradient_golden(goldens):
    g = goldens["check_gradient"]
    img = np.array(g["image"], np.float32).reshape(4, 4, 4)
    want = np.array(g["gradient"], np.float32).reshape(4, 4, 4, 3)
    np.testing.assert_array_equal(O.gradient(img), want)


# ---- spline transformation ----------------------------------------------
@pytest.mark.parametrize("prec", [O.PREC_REF, O.PREC_F64])
def test_splines_transform_shift(goldens, prec):
    g = goldens["test_splines_transform"]
    n = g["size"]
    img = np.zeros(n[::-1], np.float32)
    img[g["src_slice_z"]] = np.array(g["src"], np.float32).reshape(10, 10)
    lvl = O.Level(tuple(n), csize=tuple(g["coeff_size"]), precision=prec)
    lvl.set_images(img, img)
    params = np.tile(np.array(g["shift"]), lvl.nparams // 3)
    w = lvl.warp(params)[g["ref_slice_z"]]
    want = np.array(g["ref"], np.float32).reshape(10, 10)
    for got, exp in zip(w.ravel(), want.ravel()):
        if exp > g["compare_if_above"] or got > g["compare_if_above"]:
            assert close_pct(got, exp, g["tol_pct"])


def test_splines_translate_constant_force(goldens):
    g = goldens["test_splines_translate"]
    r = g["range"]
    lvl = O.Level(tuple(r), csize=tuple(g["coeff_size"]))
    force = np.broadcast_to(np.array(g["force"], np.float32), tuple(r[::-1]) + (3,))
    gr = lvl.translate(force)
    cs = lvl.csize
    scale = np.prod([(cs[i] - 3) / (r[i] - 1.0) for i in range(3)])
    gr = gr.reshape(cs[2], cs[1], cs[0], 3) * scale
    inner = gr[3:cs[2] - 2, 3:cs[1] - 2, 3:cs[0] - 2].reshape(-1, 3)
    for k in range(3):
        assert np.all(np.abs(inner[:, k] - g["expect_scaled"][k]) <= g["tol_pct"] / 100 * abs(g["expect_scaled"][k]))


# ---- divcurl penalty ----------------------------------------------------
def _divcurl_field(dsize, rng_, fz_zero=False):
    scale = rng_ / dsize
    ax = np.arange(-dsize, dsize + 1) * scale
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    e = np.exp(-x * x - y * y - z * z)
    fz = np.zeros_like(x) if fz_zero else z * e
    field = np.stack([x * e, y * e, fz], -1).astype(np.float32).astype(np.float64)
    return O.prefilter_vec(field)


def test_divcurl_analytic_value(goldens):
    g = goldens["test_nocurl_bspline3_7_4"]
    coeffs = _divcurl_field(g["dsize"], g["range"])
    fr = [2 * g["range"]] * 3
    test = 105.0 * math.pi ** 1.5 / (math.sqrt(2.0) * 8.0)
    div = O.divcurl_matrix(coeffs, fr, 1.0, 0.0, with_grad=False, as_float=False, mode=1)
    dc = O.divcurl_matrix(coeffs, fr, 1.0, 1.0, with_grad=False, as_float=False, mode=1)
    rot = O.divcurl_matrix(coeffs, fr, 0.0, 1.0, with_grad=False, as_float=False, mode=1)
    assert close_pct(div, test, g["tol_pct_div"])
    assert close_pct(dc, test, g["tol_pct_divcurl"])
    assert close_pct(1.0 + rot, 1.0, g["tol_pct_rot_plus1"])


def test_divcurl_gradient_fd(goldens):
    g = goldens["test_mix_bspline4_10_4_grad"]
    coeffs = _divcurl_field(g["dsize"], g["range"], fz_zero=True)
    fr = [2 * g["range"]] * 3
    _, grad = O.divcurl_matrix(coeffs, fr, 1.0, 1.0, with_grad=True, as_float=False, mode=0)
    delta = np.float32(g["delta"])
    flat = coeffs.reshape(-1)
    gflat = grad.reshape(-1)
    for i in range(flat.size):
        c = flat.copy()
        c[i] += delta
        vp = O.divcurl_matrix(c.reshape(coeffs.shape), fr, 1.0, 1.0, with_grad=False, as_float=False, mode=1)
        c[i] -= 2.0 * delta
        vm = O.divcurl_matrix(c.reshape(coeffs.shape), fr, 1.0, 1.0, with_grad=False, as_float=False, mode=1)
        fd = (vp - vm) / (2.0 * delta)
        if abs(fd) < g["small"]:
            assert close_pct(gflat[i] + 1e-7, fd + 1e-7, g["tol_pct_small"])
        else:
            assert close_pct(gflat[i], fd, g["tol_pct"])


def test_divcurl_penalty_plugin_sign_and_weight(goldens):
    """Penalty wrapper returns weight*value and -weight*gradient (Q1)."""
    g = goldens["test_divcurl_cost_w2_d1_c1"]
    cs = g["size"]
    rng_ = g["range"]
    size = tuple(int(v) for v in rng_)
    lvl = O.Level(size, csize=tuple(cs), penalty_weight=g["weight"], div=1.0, curl=1.0)
    z = np.zeros(size[::-1], np.float32)
    lvl.set_images(z, z)
    coef = np.zeros((cs[2], cs[1], cs[0], 3))
    _, cp0, _, _ = lvl.evaluate(coef.ravel())
    assert cp0 == 0.0
    coef[tuple(g["node"][::-1])] = g["coef"]
    _, cp, _, gp = lvl.evaluate(coef.ravel())
    mv, mg = O.divcurl_matrix(coef, rng_, 1.0, 1.0)
    assert cp == g["weight"] * mv
    np.testing.assert_allclose(gp, g["grad_factor"] * mg.ravel(), rtol=g["tol_pct"] / 100, atol=1e-300)
    ci, cpv = lvl.value(coef.ravel())
    assert close_pct(cpv, g["weight"] * O.divcurl_matrix(coef, rng_, 1.0, 1.0, with_grad=False, mode=1), 1e-6)


# ---- 2D -----------------------------------------------------------------
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import golden2d  # noqa: E402


@pytest.mark.parametrize("prec", [O.PREC_REF, O.PREC_F64])
def test_splines_transform_shift_2d(goldens, prec):
    g = goldens["test_splines_transform_2d"]
    n = g["size"]
    img = np.array(g["src"], np.float32).reshape(n[1], n[0])
    lvl = O.Level(tuple(n), csize=tuple(g["coeff_size"]), precision=prec)
    lvl.set_images(img, img)
    w = lvl.warp(np.tile(np.array(g["shift"]), lvl.nparams // 2))
    want = np.array(g["ref"], np.float32).reshape(n[1], n[0])
    for got, exp in zip(w.ravel(), want.ravel()):
        if exp > g["compare_if_above"] or got > g["compare_if_above"]:
            assert close_pct(got, exp, g["tol_pct"])


def test_splines_translate_constant_force_2d(goldens):
    g = goldens["test_splines_translate_2d"]
    r = g["range"]
    lvl = O.Level(tuple(r), csize=tuple(g["coeff_size"]))
    force = np.broadcast_to(np.array(g["force"], np.float32), (r[1], r[0], 2))
    cs = lvl.csize
    scale = np.prod([(r[i] - 1.0) / (cs[i] - 1 - 2) for i in range(2)])
    gr = lvl.translate(force).reshape(cs[1], cs[0], 2)
    inner = gr[4:cs[1] - 3, 4:cs[0] - 3].reshape(-1, 2)
    for k in range(2):
        want = g["expect_scaled"][k] * scale
        assert np.all(np.abs(inner[:, k] - want) <= g["tol_pct"] / 100 * abs(want))


def test_splines_prefix_iterator_2d(goldens):
    """the transformation built from the prefiltered fixture field
    reproduces the field at every pixel: x - T(x) = f(x)"""
    g = goldens["test_splinestransform_prefix_iterator_2d"]
    r = g["range"]
    lvl = O.Level(tuple(r), csize=tuple(g["coeff_size"]))
    z = np.zeros((r[1], r[0]), np.float32)
    lvl.set_images(z, z)
    u = lvl.displacement(golden2d.fixture_coefficients(g).ravel())
    X, Y = np.meshgrid(np.arange(r[0]), np.arange(r[1]))
    fx, fy = golden2d.fixture_field(g, X, Y)
    for got, want in ((u[..., 0], fx), (u[..., 1], fy)):
        m = (np.abs(want) > g["check_if_above"]) & (np.abs(got) > g["check_if_above"])
        assert np.all(np.abs(got[m] - want[m]) <= g["tol_pct"] / 100 * np.abs(want[m]))


def test_spline_c_rate_create_2d(goldens):
    g = goldens["test_spline_c_rate_create_2d"]
    lvl = O.Level(tuple(g["size"]), rate=tuple(g["c_rate"]))
    assert list(lvl.csize) == g["coeff_size"]
    z = np.zeros(tuple(g["size"][::-1]), np.float32)
    lvl.set_images(z, z)
    assert not np.any(lvl.displacement(np.zeros(lvl.nparams)))


def _ppm_cases(goldens, with_checks):
    return [(k, v) for k, v in goldens["divcurl_matrix_2d"].items() if ("checks" in v) == with_checks]


def test_divcurl_matrix_2d_values(goldens):
    """analytic values of the 2D divcurl matrix on divergence-only,
    curl-only and exp(-r^2) fields, applied with the cubic kernel of the
    registration path (the cases written for bspline:d=4 keep their field,
    value and tolerance)"""
    for name, c in _ppm_cases(goldens, True):
        coeffs, fr = golden2d.ppmatrix_coefficients(c)
        for chk in c["checks"]:
            v = O.divcurl_matrix(coeffs, fr, chk["wdiv"], chk["wrot"], with_grad=False, as_float=False, mode=1)
            if chk["expect"] == "zero":
                assert close_pct(1.0 + v, 1.0, chk["tol_pct"]), (name, chk, v)
            else:
                want = {"6*pi": 6 * math.pi, "4*pi": 4 * math.pi}[chk["expect"]]
                assert close_pct(v, want, chk["tol_pct"]), (name, chk, v)


@pytest.mark.parametrize("name", ["test_divergence_expm2_bspline3_grad", "test_rotation_expm2_bspline3_grad",
                                  "test_divergence_expm2_bspline3_grad_noiso",
                                  "test_rotation_expm2_bspline3_grad_noiso"])
def test_divcurl_matrix_2d_gradient_fd(goldens, name):
    c = goldens["divcurl_matrix_2d"][name]
    coeffs, fr = golden2d.ppmatrix_coefficients(c)
    _, grad = O.divcurl_matrix(coeffs, fr, c["wdiv"], c["wrot"], with_grad=True, as_float=False, mode=0)
    flat, gflat = coeffs.reshape(-1), grad.reshape(-1)
    d = c["delta"]
    for i in range(flat.size):
        cc = flat.copy()
        cc[i] += d
        vp = O.divcurl_matrix(cc.reshape(coeffs.shape), fr, c["wdiv"], c["wrot"], with_grad=False, as_float=False,
                              mode=1)
        cc[i] -= 2 * d
        vm = O.divcurl_matrix(cc.reshape(coeffs.shape), fr, c["wdiv"], c["wrot"], with_grad=False, as_float=False,
                              mode=1)
        fd = (vp - vm) / (2 * d)
        if abs(fd) > c["check_if_abs_above"]:
            assert close_pct(gflat[i], fd, c["tol_pct"]), (i, gflat[i], fd)


def test_divcurl_penalty_2d_values(goldens):
    """the 2D divcurl penalty plugin: weight * value = 6 pi / 3 pi on the
    divergence-only (curl-only) field with weight, div and curl scaled"""
    for name, c in goldens["divcurl_penalty_2d"].items():
        coeffs = golden2d.penalty_coefficients(c)
        n = c["size"]
        size = tuple(int(v) for v in c["range"])
        lvl = O.Level(size, csize=tuple(n), penalty_weight=c["weight"], div=c["div"], curl=c["curl"])
        z = np.zeros(size[::-1], np.float32)
        lvl.set_images(z, z)
        _, cp = lvl.value(coeffs.ravel())
        assert close_pct(cp, c["value_over_pi"] * math.pi, c["tol_pct"]), (name, cp)
