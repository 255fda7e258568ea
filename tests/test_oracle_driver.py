"""The oracle's registration driver: minimizers (pinned to the reference's
gdsq known answer), the scale filter, the joint normalisation, refine and a
full multiresolution registration."""
import numpy as np
import pytest

from oracle import oracle as O


def test_gdsq_reference_problem():
    # mia/core/minimizer/test_gdsq.cc:39-52: CGDSQMinimizer(0.1, 2.0, 1e-4,
    # 1e-4, 0.0, 100, 1e-6) from (5, 7) reaches (1, 2) within 0.1 %
    mz = O.minimizer("gdsq", maxiter=100, step=0.1, scale=2.0, xtol=1e-4, gtol=1e-4, ftolr=0.0, min_step=1e-6)
    f, x, n = O.minimize_test_problem(mz)
    assert abs(x[0] - 1.0) <= 1e-3 and abs(x[1] - 2.0) <= 2e-3
    assert n > 1


def test_gsl_steepest_descent_reference_problem():
    mz = O.minimizer("gsl", maxiter=100, step=0.1, tol=0.1, eps=0.01)
    f, x, n = O.minimize_test_problem(mz)
    assert abs(x[0] - 1.0) <= 1e-3 and abs(x[1] - 2.0) <= 2e-3
    assert abs(f - 30.0) < 1e-4


def test_scale_constant_and_linear():
    img = np.full((40, 48), 3.5, np.float32)
    out = O.scale_image(img, (20, 24))
    np.testing.assert_allclose(out, 3.5, rtol=1e-6)
    z, y, x = np.meshgrid(np.arange(16), np.arange(20), np.arange(24), indexing="ij")
    lin = (0.5 * x + 0.25 * y + z).astype(np.float32)
    out = O.scale_image(lin, (8, 10, 12))
    # interior samples of a linear ramp are reproduced at the resampled positions
    zz, yy, xx = np.meshgrid(np.arange(8) * 15 / 7, np.arange(10) * 19 / 9, np.arange(12) * 23 / 11, indexing="ij")
    want = 0.5 * xx + 0.25 * yy + zz
    np.testing.assert_allclose(out[2:-2, 2:-2, 2:-2], want[2:-2, 2:-2, 2:-2], rtol=1e-4, atol=1e-4)


def test_normalize_pair_formula():
    rng = np.random.default_rng(0)
    a = rng.normal(50, 10, size=(30, 40)).astype(np.float32)
    b = rng.normal(70, 20, size=(30, 40)).astype(np.float32)
    ok, an, bn, mean, sigma = O.normalize_pair(a, b)
    assert ok
    both = np.concatenate([an.ravel(), bn.ravel()]).astype(np.float64)
    assert abs(both.mean()) < 1e-4 and abs(both.std(ddof=1) - 1.0) < 1e-4
    assert abs(mean - np.concatenate([a.ravel(), b.ravel()]).astype(np.float64).mean()) < 1e-9
    c = np.full((4, 4), 2.0, np.float32)
    assert not O.normalize_pair(c, c)[0]


def test_refine_constant_field():
    p = np.tile([0.5, -1.25, 2.0], 6 * 5 * 7)
    out = O.refine(3, (6, 5, 7), (9, 7, 11), p)
    np.testing.assert_allclose(out.reshape(-1, 3), np.broadcast_to([0.5, -1.25, 2.0], (9 * 7 * 11, 3)), atol=1e-6)
    assert O.refine(3, (6, 5, 7), (6, 5, 7), p) is None


@pytest.mark.parametrize("kind", ["gsl", "gdsq"])
def test_registration_reduces_cost(kind):
    from mia_gb300 import synth
    ref = synth.blob_phantom((80, 96), 8, sigma=(4, 10), seed=1)
    lv = O.Level((96, 80), rate=16.0)
    lv.set_images(ref, ref)
    mov = lv.warp(synth.spline_params(lv.nparams // 2, 2, 1.5, 3.0, seed=2))
    mz = O.minimizer(kind, maxiter=15, step=0.1)
    p, cs, fc, ne = O.register(mov, ref, 16.0, 2, mz, cost="ssd", penalty_weight=10.0)
    assert cs == (8, 7) and p.size == 8 * 7 * 2 and ne > 15
    ok, mn, rn, _, _ = O.normalize_pair(mov, ref)
    lv2 = O.Level((96, 80), csize=cs, cost="ssd", penalty_weight=10.0)
    lv2.set_images(mn, rn)
    c0 = sum(lv2.value(np.zeros(p.size)))
    assert fc < c0
