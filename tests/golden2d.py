"""Inputs of the reference's 2D known-answer tests, built from the entries
of tests/golden/reference_goldens.json the way the reference's fixtures
build them (mia/2d/test_ppmatrix.cc, mia/2d/splinepenalty/test_divcurl.cc,
mia/2d/transform/test_spline.cc).  Shared by the oracle and GPU tests.
"""
import numpy as np

from oracle import oracle as O


def _eval(expr, **v):
    return eval(expr, {"__builtins__": {}}, dict(exp=np.exp, **v))


def ppmatrix_coefficients(case):
    """C2DPPDivcurlMatrix test fixture (init2d): the field sampled in float
    at (x scale_x, y scale_y) on the (2 dsize + 1) grid, scale = range /
    dsize, then the interpolator's prefilter (mirror boundary) in double.
    Returns coefficients [y, x, 2] and the matrix range (2 range, per axis)."""
    dx, dy = case["dsize"]
    r = np.float32(case["range"])
    sx, sy = r / np.float32(dx), r / np.float32(dy)
    X = (np.arange(-dx, dx + 1, dtype=np.float32) * sx)[None, :]
    Y = (np.arange(-dy, dy + 1, dtype=np.float32) * sy)[:, None]
    X, Y = np.broadcast_arrays(X, Y)
    f = np.stack([_eval(case["field"][k], x=X, y=Y).astype(np.float32) for k in range(2)], -1)
    return O.prefilter_vec(f.astype(np.float64)), (2.0 * float(case["range"]),) * 2


def penalty_coefficients(case):
    """C2DDivcurlSplinePenalty test: the field at (i - mid) * range / (n - 1)
    in double, stored as float, prefiltered in double and rounded to float
    again (the coefficients the penalty sees).  Returns [y, x, 2]."""
    n = case["size"]
    scale = case["range"][0] / (n[0] - 1)
    mid = (n[0] - 1.0) / 2.0
    fy = ((np.arange(n[1], dtype=np.float32).astype(np.float64) - mid) * scale)[:, None]
    fx = ((np.arange(n[0], dtype=np.float32).astype(np.float64) - mid) * scale)[None, :]
    fx, fy = np.broadcast_arrays(fx, fy)
    v = np.exp(-fx * fx - fy * fy)
    f = np.stack([_eval(case["field"][k], fx=fx, fy=fy, v=v) for k in range(2)], -1).astype(np.float32)
    return O.prefilter_vec(f.astype(np.float64)).astype(np.float32).astype(np.float64)


def fixture_field(case, xs, ys):
    """TransformSplineFixture's fx, fy at float coordinates"""
    rx, ry = case["range"]
    x = np.asarray(xs, np.float32)
    y = np.asarray(ys, np.float32)
    vx = x - np.float32(rx / 2.0)
    vy = y - np.float32(ry / 2.0)
    env = dict(vx=vx, vy=vy, range_x=np.float32(rx), range_y=np.float32(ry))
    return (_eval(case["fx"], **env).astype(np.float32), _eval(case["fy"], **env).astype(np.float32))


def fixture_coefficients(case):
    """TransformSplineFixture: coefficient grid range + 2, the fixture field
    sampled at ivscale (i - 1) and prefiltered along y, then x (mirror)."""
    rx, ry = case["range"]
    ncx, ncy = case["coeff_size"]
    ivx = np.float32(rx - 1) / np.float32(ncx - 2 - 1)
    ivy = np.float32(ry - 1) / np.float32(ncy - 2 - 1)
    xs = ivx * (np.arange(ncx, dtype=np.float32) - np.float32(1))
    ys = ivy * (np.arange(ncy, dtype=np.float32) - np.float32(1))
    X, Y = np.broadcast_arrays(xs[None, :], ys[:, None])
    fx, fy = fixture_field(case, X, Y)
    f = np.stack([fx, fy], -1).astype(np.float64)
    return O.prefilter_vec(f).astype(np.float32).astype(np.float64)
