"""Extract the known-answer vectors of the reference's own unit tests into
``tests/golden/reference_goldens.json``.

Run with ``MIA_REFERENCE`` set to the root of the reference's source tree
(``MIA_REFERENCE=<path to mia> python tests/golden/extract_goldens.py``);
the script stops when it is unset.  The tests read only the committed JSON,
so nothing at test time needs the reference sources.

Each entry records the reference test file and line of the test case, the
input arrays exactly as written there, the expected values (the literal
arithmetic expression of the test evaluated in double) and the tolerance the
reference test uses (BOOST_CHECK_CLOSE percent, or 0 for BOOST_CHECK_EQUAL).
"""
import json
import os
import re
import sys

REF = os.environ.get("MIA_REFERENCE")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")

_NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?f?"


def read(rel):
    if not REF:
        raise SystemExit("set MIA_REFERENCE to the root of the reference's source tree")
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def case_body(text, name):
    """Return (line, body) of the BOOST test case `name`."""
    m = re.search(r"BOOST_(?:AUTO|FIXTURE)_TEST_CASE\(\s*" + re.escape(name) + r"\b", text)
    if not m:
        raise KeyError(name)
    start = m.start()
    nxt = re.search(r"\nBOOST_(?:AUTO|FIXTURE)_TEST_CASE\(", text[m.end():])
    end = m.end() + nxt.start() if nxt else len(text)
    line = text.count("\n", 0, start) + 1
    return line, text[start:end]


def nums(s):
    return [float(x.rstrip("f")) for x in re.findall(_NUM, s)]


def array(body, name):
    m = re.search(r"\b" + re.escape(name) + r"\s*\[[^\]]*\]\s*=\s*\{(.*?)\};", body, re.S)
    if not m:
        raise KeyError(name)
    inner = re.sub(r"/\*.*?\*/", " ", m.group(1), flags=re.S)
    vecs = re.findall(r"C3DFVector\s*\(([^)]*)\)", inner)
    if vecs:
        return [nums(v) for v in vecs]
    return nums(inner)


def index_list(body, name):
    m = re.search(r"\b" + re.escape(name) + r"\s*=\s*\{(.*?)\};", body, re.S)
    return [int(x) for x in re.findall(r"-?\d+", m.group(1))]


def ev(expr):
    expr = expr.replace("f", "")
    if not re.fullmatch(r"[0-9.+\-*/() eE]+", expr):
        raise ValueError(expr)
    return float(eval(expr, {"__builtins__": {}}, {}))


def main():
    g = {"reference_root_at_extraction": "mia (gerddie/mia) test sources", "cases": {}}
    C = g["cases"]

    # SSD 3D (mia/3d/cost/test_ssd.cc)
    t = read("mia/3d/cost/test_ssd.cc")
    for name, norm in (("test_SSD_3D_norm", True), ("test_SSD_3D", False)):
        line, b = case_body(t, name)
        val = re.search(r"BOOST_CHECK_CLOSE\(cost\.value\(\*src\),\s*(.*?),\s*(" + _NUM + r")\)", b)
        frc = re.search(r"force\(1, 1, 1\),\s*C3DFVector\((.*?)\)\s*\)", b)
        C[name] = {
            "source": "mia/3d/cost/test_ssd.cc:%d" % line,
            "size": [3, 3, 3], "norm": norm,
            "src": array(b, "src_data"), "ref": array(b, "ref_data"),
            "value": ev(val.group(1)), "value_tol_pct": float(val.group(2)),
            "force_111": [ev(e) for e in frc.group(1).split(",")], "force_tol_pct": 0.0,
        }

    # SSD 2D (mia/2d/cost/test_ssd.cc)
    t = read("mia/2d/cost/test_ssd.cc")
    line, b = case_body(t, "test_SSD_2D")
    val = re.search(r"BOOST_CHECK_CLOSE\(cost_value,\s*(.*?),\s*(" + _NUM + r")\)", b)
    fx = re.search(r"force\(1, 1\)\.x,\s*(.*?),\s*(" + _NUM + r")\)", b)
    fy = re.search(r"force\(1, 1\)\.y,\s*(.*?),\s*(" + _NUM + r")\)", b)
    C["test_SSD_2D"] = {
        "source": "mia/2d/cost/test_ssd.cc:%d" % line, "size": [4, 4], "norm": True,
        "src": array(b, "src_data"), "ref": array(b, "ref_data"),
        "value": ev(val.group(1)), "value_tol_pct": float(val.group(2)),
        "force_11": [ev(fx.group(1)), ev(fy.group(1))], "force_tol_pct": float(fx.group(2)),
    }

    # spline transform shift (mia/3d/transform/test_spline.cc)
    t = read("mia/3d/transform/test_spline.cc")
    line, b = case_body(t, "test_splines_transform")
    shift = re.search(r"C3DFVector shift\((.*?)\);", b)
    field = re.search(r"C3DFVectorfield field\(C3DBounds\((.*?)\)\);", b)
    C["test_splines_transform"] = {
        "source": "mia/3d/transform/test_spline.cc:%d" % line,
        "size": [10, 10, 10], "coeff_size": [int(v) for v in nums(field.group(1))],
        "shift": nums(shift.group(1)), "src_slice_z": 4, "ref_slice_z": 5,
        "src": array(b, "src_image_init"), "ref": array(b, "ref_image_init"),
        "tol_pct": 0.1, "compare_if_above": 0.001,
    }

    # translate with constant force: fixture sizes
    line, b = case_body(t, "test_splines_translate")
    fill = re.search(r"C3DFVector\((" + _NUM + r"),\s*(" + _NUM + r"),\s*(" + _NUM + r")\)\);", b)
    C["test_splines_translate"] = {
        "source": "mia/3d/transform/test_spline.cc:%d" % line,
        "range": [50, 80, 30], "coeff_size": [42, 67, 27], "force": nums(" ".join(fill.groups())),
        "expect_scaled": [-1.0, -2.0, -3.0], "tol_pct": 1.0,
        "interior": "2 < index < csize-2 on every axis",
    }

    # mirror boundary (mia/core/splinebc/test_bc.cc)
    t = read("mia/core/splinebc/test_bc.cc")
    mir = {}
    for name, width in (("test_mirror_on_boundary_needed", 6), ("test_mirror_on_boundary_needed_large", 10),
                        ("test_mirror_on_boundary_notneeded", 9)):
        line, b = case_body(t, name)
        w = int(re.search(r"CMirrorOnBoundary bc\((\d+)\)", b).group(1))
        assert w == width
        ncheck = re.search(r"for \((?:int|size_t) i = 0; i < (\d+|index\.size\(\))", b).group(1)
        idx = index_list(b, "index")
        mir[name] = {"source": "mia/core/splinebc/test_bc.cc:%d" % line, "width": w, "index": idx,
                     "result": index_list(b, "result"),
                     "ncheck": len(idx) if not ncheck.isdigit() else int(ncheck)}
    C["mirror_boundary"] = mir

    # cubic B-spline derivative weights (mia/core/splinekernel/test_bspline.cc)
    t = read("mia/core/splinekernel/test_bspline.cc")
    line, b = case_body(t, "test_bspline3_derivatives")
    parts = re.split(r"kernel\.derivative\(", b)[1:]
    d = []
    for p in parts:
        x, deg = re.match(r"\s*(" + _NUM + r"),\s*weight,\s*index,\s*(\d+)\)", p).groups()
        ws = {int(k): float(v) for k, v in re.findall(r"weight\[(\d)\],\s*(" + _NUM + r"),", p)}
        d.append({"x": float(x), "degree": int(deg), "weights": [ws[k] for k in range(4)]})
    C["test_bspline3_derivatives"] = {"source": "mia/core/splinekernel/test_bspline.cc:%d" % line,
                                      "cases": d, "tol_pct": 0.1, "index": [-1, 0, 1, 2]}

    # central-difference gradient (mia/3d/test_image.cc)
    t = read("mia/3d/test_image.cc")
    line, b = case_body(t, "check_gradient")
    C["check_gradient"] = {"source": "mia/3d/test_image.cc:%d" % line, "size": [4, 4, 4],
                           "image": array(b, "init_data"), "gradient": array(b, "vf"), "tol_pct": 0.0}

    # divcurl analytic value (mia/3d/test_ppmatrix.cc), cubic kernel only
    t = read("mia/3d/test_ppmatrix.cc")
    line, b = case_body(t, "test_nocurl_bspline3_7_4")
    init = re.search(r"init\((\d+),\s*(\d+),\s*\"(bspline:d=\d)\"\)", b)
    C["test_nocurl_bspline3_7_4"] = {
        "source": "mia/3d/test_ppmatrix.cc:%d" % line, "dsize": int(init.group(1)), "range": float(init.group(2)),
        "kernel": init.group(3), "field": "x*exp(-r2), y*exp(-r2), z*exp(-r2)",
        "value_expr": "105*pi^1.5/(sqrt(2)*8)", "tol_pct_div": 0.8, "tol_pct_divcurl": 0.8, "tol_pct_rot_plus1": 4.0,
    }
    line, b = case_body(t, "test_mix_bspline4_10_4_grad")
    init = re.search(r"init\((\d+),\s*(\d+),\s*\"(bspline:d=\d)\"\)", b)
    C["test_mix_bspline4_10_4_grad"] = {
        "source": "mia/3d/test_ppmatrix.cc:%d" % line, "dsize": int(init.group(1)), "range": float(init.group(2)),
        "kernel": init.group(3), "field": "x*exp(-r2), y*exp(-r2), 0", "delta": 0.001,
        "tol_pct": 0.1, "tol_pct_small": 5.0, "small": 1e-8,
    }

    # penalty plugin scaling and sign (mia/3d/splinepenalty/test_divcurl.cc)
    t = read("mia/3d/splinepenalty/test_divcurl.cc")
    line, b = case_body(t, "test_divcurl_cost_w2_d1_c1")
    C["test_divcurl_cost_w2_d1_c1"] = {
        "source": "mia/3d/splinepenalty/test_divcurl.cc:%d" % line,
        "size": [int(v) for v in nums(re.search(r"C3DBounds size\((.*?)\)", b).group(1))],
        "range": nums(re.search(r"C3DFVector range\((.*?)\)", b).group(1)),
        "weight": float(re.search(r"divcurl:weight=(" + _NUM + ")", b).group(1)),
        "node": [5, 5, 5], "coef": nums(re.search(r"coefficients\(5, 5, 5\) = C3DFVector\((.*?)\)", b).group(1)),
        "grad_factor": -2.0, "tol_pct": 0.1,
    }

    # ---- 2D --------------------------------------------------------------
    # spline transformation (mia/2d/transform/test_spline.cc)
    t = read("mia/2d/transform/test_spline.cc")
    line, b = case_body(t, "test_splines_transform")
    shift = re.search(r"C2DFVector shift\((.*?)\);", b)
    field = re.search(r"C2DFVectorfield field\(C2DBounds\((.*?)\)\);", b)
    size = re.search(r"const C2DBounds size\((.*?)\);", b)
    C["test_splines_transform_2d"] = {
        "source": "mia/2d/transform/test_spline.cc:%d" % line,
        "size": [int(v) for v in nums(size.group(1))], "coeff_size": [int(v) for v in nums(field.group(1))],
        "shift": nums(shift.group(1)), "src": array(b, "src_image_init"), "ref": array(b, "ref_image_init"),
        "tol_pct": float(re.search(r"BOOST_CHECK_CLOSE\(\*ir, \*itest, (" + _NUM + r")\)", b).group(1)),
        "compare_if_above": 0.001,
    }
    # the fixture: image size `range`, coefficient grid range + 2 (the
    # cubic kernel's coeff_shift of 1 on either side), coefficients the
    # prefiltered samples of two Gaussians
    fx_ = re.search(r"TransformSplineFixture::fx\(float x, float y\)\s*\{(.*?)\}", t, re.S).group(1)
    fy_ = re.search(r"TransformSplineFixture::fy\(float x, float y\)\s*\{(.*?)\}", t, re.S).group(1)
    ex = lambda body: re.search(r"exp\s*\(\s*-\s*\((.*?)\)\s*/", body).group(1)
    fixture = re.search(r"size\((\d+), (\d+)\),.*?range\((\d+), (\d+)\)", t, re.S)
    rng2 = [int(fixture.group(3)), int(fixture.group(4))]
    fix = {"range": rng2, "coeff_size": [rng2[0] + 2, rng2[1] + 2],
           "fx": "exp(-(%s) / (range_x * range_y))" % ex(fx_), "fy": "exp(-(%s) / (range_x * range_y))" % ex(fy_),
           "v": "vx = x - range_x / 2, vy = y - range_y / 2"}
    line, b = case_body(t, "test_splines_translate")
    fill = re.search(r"C2DFVector\((" + _NUM + r"),\s*(" + _NUM + r")\)\);", b)
    C["test_splines_translate_2d"] = dict(fix, **{
        "source": "mia/2d/transform/test_spline.cc:%d" % line, "force": nums(" ".join(fill.groups())),
        "expect_scaled": [-v for v in nums(" ".join(fill.groups()))], "tol_pct": 0.1,
        "interior": "3 < index < csize-3 on every axis"})
    line, b = case_body(t, "test_splinestransform_prefix_iterator")
    C["test_splinestransform_prefix_iterator_2d"] = dict(fix, **{
        "source": "mia/2d/transform/test_spline.cc:%d" % line,
        "tol_pct": float(re.search(r"BOOST_CHECK_CLOSE\(fx\(x, y\), x - i->x, (" + _NUM + r")\)", b).group(1)),
        "check_if_above": 1e-8})
    line, b = case_body(t, "test_spline_c_rate_create")
    C["test_spline_c_rate_create_2d"] = {
        "source": "mia/2d/transform/test_spline.cc:%d" % line,
        "size": [int(v) for v in nums(re.search(r"C2DBounds size\((.*?)\);", b).group(1))],
        "c_rate": nums(re.search(r"C2DFVector c_rate\((.*?)\);", b).group(1)),
        "coeff_size": [int(re.search(r"gridsize\.x, (\d+)u", b).group(1)),
                       int(re.search(r"gridsize\.y, (\d+)u", b).group(1))]}

    # divcurl matrix (mia/2d/test_ppmatrix.cc): the field is sampled on a
    # (2 dsize + 1)^2 grid over [-range, range]^2, prefiltered, and the
    # matrix is built for that grid and the range 2 range
    t = read("mia/2d/test_ppmatrix.cc")
    fields = {"TransformSplineFixtureDivOnly": ["x*exp(-x*x-y*y)", "y*exp(-x*x-y*y)"],
              "TransformSplineFixtureCurlOnly": ["y*exp(-x*x-y*y)", "-x*exp(-x*x-y*y)"],
              "TransformSplineFixtureexpm2Field_44": ["exp(-x*x-y*y)", "exp(-x*x-y*y)"]}
    for name in fields:
        body = re.search(re.escape(name.replace("_44", "")) + r"::fx\(float x, float y\)\s*\{(.*?)\}", t, re.S)
        assert body and "exp" in body.group(1), name
    pp = {}
    for name in ("test_nocurl_bspline3", "test_nocurl_bspline3_noniso", "test_nodiv_bspline3"):
        line, b = case_body(t, name)
        fx_name = re.search(r"BOOST_FIXTURE_TEST_CASE\(\s*\w+,\s*(\w+)", b).group(1)
        m = re.search(r"init2d\(T2DVector<int>\((\d+), (\d+)\), (\d+), \"(bspline:d=\d)\"\)", b) or \
            re.search(r"init\((\d+), (\d+), \"(bspline:d=\d)\"\)", b)
        g_ = m.groups()
        dsize = [int(g_[0]), int(g_[1])] if len(g_) == 4 else [int(g_[0])] * 2
        rng_ = float(g_[-2])
        closes = re.findall(r"BOOST_CHECK_CLOSE\(\s*(1\.0 \+ )?(\w+)\s*\*\s*coeffs,\s*(1\.0|testvalue),\s*(" + _NUM +
                            r")\)", b)
        decl = dict(re.findall(r"C2DPPDivcurlMatrix (\w+)\(field\.get_size\(\), field_range, \*ipf->get_kernel\(\), "
                               r"(" + _NUM + r", " + _NUM + r")\)", b))
        checks = [{"wdiv": nums(decl[v])[0], "wrot": nums(decl[v])[1], "expect": "zero" if plus else "6*pi",
                   "tol_pct": float(tol)} for plus, v, _, tol in closes]
        pp[name] = {"source": "mia/2d/test_ppmatrix.cc:%d" % line, "field": fields[fx_name], "dsize": dsize,
                    "range": rng_, "reference_kernel": g_[-1], "checks": checks}
    for name in ("test_divergence_expm2_bspline3_16_8", "test_divergence_expm2_bspline3_8_8"):
        line, b = case_body(t, name)
        m = re.search(r"run\((\d+), (\d+), \"(bspline:d=\d)\"", b)
        run_line, rb = case_body(t, name)
        tol = float(re.search(r"BOOST_CHECK_CLOSE\(spline, manual,\s*(" + _NUM + r")\)", t).group(1))
        pp[name] = {"source": "mia/2d/test_ppmatrix.cc:%d" % line, "field": fields["TransformSplineFixtureexpm2Field_44"],
                    "dsize": [int(m.group(1))] * 2, "range": float(m.group(2)), "reference_kernel": m.group(3),
                    "checks": [{"wdiv": 1.0, "wrot": 0.0, "expect": "4*pi", "tol_pct": tol}]}
    for name in ("test_divergence_expm2_bspline3_grad", "test_rotation_expm2_bspline3_grad",
                 "test_divergence_expm2_bspline3_grad_noiso", "test_rotation_expm2_bspline3_grad_noiso"):
        line, b = case_body(t, name)
        m = re.search(r"init2d\(T2DVector<int>\((\d+), (\d+)\), (\d+), \"(bspline:d=\d)\"\)", b) or \
            re.search(r"init\((\d+), (\d+), \"(bspline:d=\d)\"\)", b)
        g_ = m.groups()
        dsize = [int(g_[0]), int(g_[1])] if len(g_) == 4 else [int(g_[0])] * 2
        w = nums(re.search(r"C2DPPDivcurlMatrix \w+\(field\.get_size\(\), field_range, \*ipf->get_kernel\(\), (.*?)\);",
                           b).group(1))
        pp[name] = {"source": "mia/2d/test_ppmatrix.cc:%d" % line, "field": fields["TransformSplineFixtureexpm2Field_44"],
                    "dsize": dsize, "range": float(g_[-2]), "reference_kernel": g_[-1], "wdiv": w[0], "wrot": w[1],
                    "delta": 0.001, "check_if_abs_above": 0.0001,
                    "tol_pct": float(re.search(r"BOOST_CHECK_CLOSE\(ig\[0\], test_grad, (" + _NUM + r")\)", b).group(1))}
    C["divcurl_matrix_2d"] = pp

    # divcurl penalty plugin (mia/2d/splinepenalty/test_divcurl.cc)
    t = read("mia/2d/splinepenalty/test_divcurl.cc")
    pen = {}
    for name in ("test_divcurl_cost", "test_divcurl_cost_scale_weight", "test_divcurl_cost_scale_div_weight",
                 "test_divcurl_cost_scale_curl_weight"):
        line, b = case_body(t, name)
        args = nums(re.search(r"C2DDivcurlSplinePenalty\s+penalty\((.*?)\);", b).group(1).replace("false", "0"))
        comp = re.search(r"\*ic = C2DFVector\(\s*(.*?)\);", b).group(1)
        want = re.search(r"BOOST_CHECK_CLOSE\(penalty\.value\(coef\),\s*(\d+) \* M_PI,\s*(" + _NUM + r")\)", b)
        pen[name] = {"source": "mia/2d/splinepenalty/test_divcurl.cc:%d" % line,
                     "weight": args[0], "normalize": bool(args[1]), "div": args[2], "curl": args[3],
                     "size": [int(v) for v in nums(re.search(r"C2DBounds size\((.*?)\);", b).group(1))],
                     "range": nums(re.search(r"C2DFVector range\((.*?)\);", b).group(1)),
                     "field": [c.strip() for c in comp.split(",")],
                     "value_over_pi": float(want.group(1)), "tol_pct": float(want.group(2)),
                     "reference_kernel": re.search(r"produce_spline_kernel\(\"(.*?)\"\)", b).group(1)}
    C["divcurl_penalty_2d"] = pen

    with open(OUT, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", OUT, "with", len(C), "cases")


if __name__ == "__main__":
    sys.exit(main())
