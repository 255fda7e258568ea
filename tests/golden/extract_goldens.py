"""Extract the known-answer vectors of the reference's own unit tests into
``tests/golden/reference_goldens.json``.

Run in a container where the reference sources are mounted (default
``/root/reference``, override with ``MIA_REFERENCE``).  The tests read only
the committed JSON, so nothing at test time needs the reference sources.

Each entry records the reference test file and line of the test case, the
input arrays exactly as written there, the expected values (the literal
arithmetic expression of the test evaluated in double) and the tolerance the
reference test uses (BOOST_CHECK_CLOSE percent, or 0 for BOOST_CHECK_EQUAL).
"""
import json
import os
import re
import sys

REF = os.environ.get("MIA_REFERENCE", "/root/reference")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")

_NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?f?"


def read(rel):
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

    with open(OUT, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", OUT, "with", len(C), "cases")


if __name__ == "__main__":
    sys.exit(main())
