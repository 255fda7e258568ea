"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances: cost 1e-5 relative, coefficient gradients 1e-4 relative L2
(against the oracle's reference-precision evaluation); the error against
the all-double oracle is asserted with the same bounds.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-5
GRAD_RTOL = 1e-4


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def make_pair(shape, seed, ncc=False):
    from mia_gb300 import synth
    ref = synth.blob_phantom(shape, 10, sigma=(2.0, 5.0), seed=seed)
    mov = synth.blob_phantom(shape, 10, sigma=(2.0, 5.0), seed=seed)
    mov = np.roll(mov, 1, axis=-1)
    if ncc:
        mov = (mov * synth.bias_field(shape, 0.1, seed=seed + 1)).astype(np.float32)
    return mov, ref


def both(size_xyz, **kw):
    import mia_gb300 as M
    g = M.Level(size_xyz, **kw)
    o = O.Level(size_xyz, precision=O.PREC_REF, **kw)
    o64 = O.Level(size_xyz, precision=O.PREC_F64, **kw)
    return g, o, o64


def check_eval(g, o, o64, params, path="split", grad_tol=GRAD_RTOL):
    g.set_path(path)
    ci, cp, gi, gp, gt = g.evaluate(params)
    oi, op, ogi, ogp = o.evaluate(params)
    fi, fp, fgi, fgp = o64.evaluate(params)
    assert rel(ci, oi) < COST_RTOL, (ci, oi)
    assert rel(ci, fi) < COST_RTOL, (ci, fi)
    assert rel_l2(gi, ogi) < grad_tol, rel_l2(gi, ogi)
    assert rel_l2(gi, fgi) < grad_tol, rel_l2(gi, fgi)
    if o.desc.has_penalty:
        assert rel(cp, op) < COST_RTOL, (cp, op)
        assert rel_l2(gp, ogp) < grad_tol
        assert rel_l2(gp, fgp) < grad_tol
    np.testing.assert_array_equal(gt, gi + gp)
    return ci, cp, gi, gp


@pytest.mark.parametrize("cost", ["ssd", "ncc"])
@pytest.mark.parametrize("path", ["split", "plain"])
def test_eval_3d(cost, path):
    size = (37, 29, 21)
    g, o, o64 = both(size, rate=5.0, cost=cost, penalty_weight=10.0)
    mov, ref = make_pair(size[::-1], 3, ncc=cost == "ncc")
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    p = synth.smooth_params(g.csize, 1.5, seed=7)
    check_eval(g, o, o64, p, path)


@pytest.mark.parametrize("cost", ["ssd", "ncc"])
@pytest.mark.parametrize("path", ["split", "plain"])
def test_eval_2d(cost, path):
    size = (61, 47)
    g, o, o64 = both(size, rate=8.0, cost=cost, penalty_weight=10.0)
    mov, ref = make_pair(size[::-1], 5, ncc=cost == "ncc")
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    p = synth.smooth_params(g.csize, 1.5, seed=9)
    # the 2D image cost is the float-accumulated force-pass cost in the
    # reference (mia/2d/fullcost/image.cc:100); the GPU sums in double
    check_eval(g, o, o64, p, path)


def test_ssd_norm_and_weight_3d():
    size = (24, 20, 18)
    g, o, o64 = both(size, rate=4.0, cost="ssd", ssd_norm=True, cost_weight=0.7, penalty_weight=3.0,
                     div=0.5, curl=2.0, penalty_norm=True)
    mov, ref = make_pair(size[::-1], 11)
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    check_eval(g, o, o64, synth.smooth_params(g.csize, 2.0, seed=1))


def test_value_matches_oracle():
    size = (33, 27, 19)
    g, o, _ = both(size, rate=6.0, cost="ncc", penalty_weight=5.0, div=1.0, curl=0.3)
    mov, ref = make_pair(size[::-1], 13, ncc=True)
    g.set_images(mov, ref)
    o.set_images(mov, ref)
    from mia_gb300 import synth
    p = synth.smooth_params(g.csize, 1.0, seed=4)
    ci, cp = g.value(p)
    oi, op = o.value(p)
    assert rel(ci, oi) < COST_RTOL and rel(cp, op) < COST_RTOL


def test_warp_and_translate_3d():
    size = (30, 22, 17)
    g, o, _ = both(size, rate=4.0)
    mov, ref = make_pair(size[::-1], 2)
    g.set_images(mov, ref)
    o.set_images(mov, ref)
    from mia_gb300 import synth
    p = synth.smooth_params(g.csize, 2.0, seed=5)
    wg, wo = g.warp(p), o.warp(p)
    assert np.max(np.abs(wg - wo)) <= 1e-5 * np.max(np.abs(wo))
    f = np.random.default_rng(0).normal(size=wo.shape + (3,)).astype(np.float32)
    assert rel_l2(g.translate(f), o.translate(f)) < 1e-5
    _, fg = g.force(p)
    fo = o.force(p)
    assert rel_l2(fg, fo) < 1e-4


def test_golden_shift_through_gpu(goldens):
    import mia_gb300 as M
    gd = goldens["test_splines_transform"]
    n = gd["size"]
    img = np.zeros(n[::-1], np.float32)
    img[gd["src_slice_z"]] = np.array(gd["src"], np.float32).reshape(10, 10)
    lv = M.Level(tuple(n), csize=tuple(gd["coeff_size"]))
    lv.set_images(img, img)
    w = lv.warp(np.tile(np.array(gd["shift"]), lv.nparams // 3))[gd["ref_slice_z"]]
    want = np.array(gd["ref"], np.float32).reshape(10, 10)
    m = (want > gd["compare_if_above"]) | (w > gd["compare_if_above"])
    np.testing.assert_allclose(w[m], want[m], rtol=gd["tol_pct"] / 100)


def test_golden_translate_through_gpu(goldens):
    import mia_gb300 as M
    gd = goldens["test_splines_translate"]
    r = gd["range"]
    lv = M.Level(tuple(r), csize=tuple(gd["coeff_size"]))
    force = np.broadcast_to(np.array(gd["force"], np.float32), tuple(r[::-1]) + (3,))
    gr = lv.translate(force)
    cs = lv.csize
    scale = np.prod([(cs[i] - 3) / (r[i] - 1.0) for i in range(3)])
    gr = gr.reshape(cs[2], cs[1], cs[0], 3) * scale
    inner = gr[3:cs[2] - 2, 3:cs[1] - 2, 3:cs[0] - 2].reshape(-1, 3)
    np.testing.assert_allclose(inner, np.broadcast_to(gd["expect_scaled"], inner.shape), rtol=gd["tol_pct"] / 100)


def test_golden_ssd_force_through_gpu(goldens):
    """identity transform: the warped image reproduces the source, so the
    force equals the reference's SSD golden (mia/3d/cost/test_ssd.cc)."""
    import mia_gb300 as M
    gd = goldens["test_SSD_3D"]
    a = np.array(gd["src"], np.float32).reshape(3, 3, 3)
    b = np.array(gd["ref"], np.float32).reshape(3, 3, 3)
    lv = M.Level((3, 3, 3), csize=(4, 4, 4))
    lv.set_images(a, b)
    c, f = lv.force(np.zeros(lv.nparams))
    np.testing.assert_allclose(f[1, 1, 1], gd["force_111"], rtol=1e-5)
    assert rel(lv.value(np.zeros(lv.nparams))[0], gd["value"]) < gd["value_tol_pct"] / 100


@pytest.mark.parametrize("size,rate", [((5, 4, 4), 1.0), ((65, 9, 7), 2.0), ((31, 33, 35), 16.0)])
def test_edge_sizes(size, rate):
    g, o, o64 = both(size, rate=rate, cost="ssd", penalty_weight=1.0)
    mov, ref = make_pair(size[::-1], 17)
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    check_eval(g, o, o64, synth.smooth_params(g.csize, 0.8, seed=2))


@pytest.mark.parametrize("size,rate", [((5, 4), 1.0), ((130, 9), 2.0), ((33, 31), 16.0)])
def test_edge_sizes_2d(size, rate):
    g, o, o64 = both(size, rate=rate, cost="ssd", penalty_weight=1.0)
    mov, ref = make_pair(size[::-1], 19)
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    check_eval(g, o, o64, synth.smooth_params(g.csize, 0.8, seed=4))


@pytest.mark.parametrize("cost", ["ssd", "ncc"])
@pytest.mark.parametrize("size,rate", [((33, 27, 19), (3.0, 5.0, 7.0)), ((57, 43), (4.0, 9.0))])
def test_anisotropic_rate_with_cost_and_penalty_options(size, rate, cost):
    """a different spline rate per axis, with the image cost's weight and
    norm and the divcurl penalty's div, curl and norm away from their defaults"""
    g, o, o64 = both(size, rate=rate, cost=cost, ssd_norm=cost == "ssd", cost_weight=0.6, penalty_weight=4.0,
                     div=2.0, curl=0.3, penalty_norm=True)
    mov, ref = make_pair(size[::-1], 23, ncc=cost == "ncc")
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    check_eval(g, o, o64, synth.smooth_params(g.csize, 1.2, seed=6))


@pytest.mark.parametrize("size,csize", [((30, 26, 22), (9, 6, 7)), ((44, 38), (5, 11))])
def test_explicit_coefficient_grid(size, csize):
    """a coefficient grid given directly (as after refine), not derived from a rate"""
    g, o, o64 = both(size, csize=csize, cost="ncc", penalty_weight=2.0)
    assert g.csize == tuple(csize)
    mov, ref = make_pair(size[::-1], 29, ncc=True)
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    check_eval(g, o, o64, synth.smooth_params(g.csize, 1.0, seed=8))


def test_tiles_and_determinism():
    size = (70, 41, 23)
    g, o, o64 = both(size, rate=5.0, cost="ncc", penalty_weight=2.0)
    mov, ref = make_pair(size[::-1], 23, ncc=True)
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    p = synth.smooth_params(g.csize, 1.0, seed=3)
    ref_out = None
    for tile in ((32, 8, 32), (32, 8, 24), (32, 8, 20), (32, 8, 16), (32, 8, 12), (32, 8, 8), (32, 8, 4)):
        g.set_path("split", tile)
        out = g.evaluate(p)
        check_eval(g, o, o64, p, "split")
        if ref_out is None:
            ref_out = out
        again = g.evaluate(p)
        np.testing.assert_array_equal(out[4], again[4])   # bit-identical repeat
        assert rel_l2(out[4], ref_out[4]) < 1e-5
    # a z length that is not compiled in is refused and the level keeps its tile
    from mia_gb300 import _lib
    for bad in ((32, 8, 7), (32, 8, 28), (16, 8, 16)):
        with pytest.raises(_lib.MgrError) as e:
            g.set_path("split", bad)
        assert e.value.status == _lib.MGR_ERR_ARG
    assert g.tile == (32, 8, 4)
    check_eval(g, o, o64, p, "split")


@pytest.mark.parametrize("cost", ["ssd", "ncc"])
def test_large_displacement_beyond_padding(cost):
    """Displacements of 20-30 voxels put the tricubic taps outside the
    mirror-padded copy, so the warp folds the indices on the unpadded image
    (mirror boundary, mia/core/splinebc/bc.cc:52-64)."""
    size = (45, 38, 30)
    g, o, o64 = both(size, rate=6.0, cost=cost, penalty_weight=1.0)
    mov, ref = make_pair(size[::-1], 41, ncc=(cost == "ncc"))
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    p = synth.smooth_params(g.csize, 1.0, seed=4)
    p += np.tile(np.array([23.0, -27.0, 21.0]), len(p) // 3)
    check_eval(g, o, o64, p)


def test_image_gradient_vs_fp64_finite_differences():
    """The image term's gradient against central differences of the FP64
    oracle cost (the gradient is the reference's: force from central
    differences of the warped image, so agreement is to the FD accuracy of
    a smooth problem, not exact)."""
    size = (28, 24, 20)
    g, _, o64 = both(size, rate=5.0, cost="ssd")
    from mia_gb300 import synth
    ref = synth.blob_phantom(size[::-1], 6, sigma=(4.0, 7.0), noise=0.0, seed=1)
    mov = synth.blob_phantom(size[::-1], 6, sigma=(4.0, 7.0), noise=0.0, seed=2)
    g.set_images(mov, ref)
    o64.set_images(mov, ref)
    p = synth.smooth_params(g.csize, 0.5, seed=6)
    _, _, gi, _, _ = g.evaluate(p)
    rng = np.random.default_rng(0)
    idx = rng.choice(np.flatnonzero(np.abs(gi) > 1e-3 * np.abs(gi).max()), 24, replace=False)
    h = 1e-3
    fd = []
    for i in idx:
        pp = p.copy(); pp[i] += h
        pm = p.copy(); pm[i] -= h
        fd.append((o64.value(pp)[0] - o64.value(pm)[0]) / (2 * h))
    assert rel_l2(gi[idx], np.array(fd)) < 5e-2


def test_penalty_gradient_is_minus_fd():
    """Q1: the penalty's value_and_gradient returns -weight * gradient."""
    size = (24, 24, 24)
    g, _, o64 = both(size, rate=4.0, cost="ssd", penalty_weight=10.0)
    z = np.zeros(size[::-1], np.float32)
    g.set_images(z, z)
    o64.set_images(z, z)
    from mia_gb300 import synth
    p = synth.smooth_params(g.csize, 1.0, seed=8)
    _, _, _, gp, _ = g.evaluate(p)
    rng = np.random.default_rng(1)
    idx = rng.choice(p.size, 20, replace=False)
    h = 1e-4
    for i in idx:
        pp = p.copy(); pp[i] += h
        pm = p.copy(); pm[i] -= h
        fd = (o64.value(pp)[1] - o64.value(pm)[1]) / (2 * h)
        assert abs(gp[i] + fd) <= 1e-3 * max(1.0, abs(fd))


@pytest.mark.parametrize("where", [0, 17, 48, 49])
@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_non_finite_parameters_are_rejected(where, bad):
    """evaluate and value refuse parameters that are not finite (any slot,
    the last ones included) and the level keeps working"""
    import mia_gb300 as M
    from mia_gb300 import _lib
    lv = M.Level((30, 26), csize=(5, 5), cost="ssd", penalty_weight=1.0)
    a, b = make_pair((26, 30), 3)
    lv.set_images(a, b)
    p = np.zeros(lv.nparams)
    assert lv.nparams == 50
    p[where] = bad
    with pytest.raises(_lib.MgrError) as e:
        lv.evaluate(p)
    assert e.value.status == _lib.MGR_ERR_ARG
    with pytest.raises(_lib.MgrError):
        lv.value(p)
    p[where] = 0.0
    ci, cp, gi, gp, gt = lv.evaluate(p)
    assert np.isfinite(ci) and np.all(np.isfinite(gt))


@pytest.mark.parametrize("size", [(24, 24, 24), (40, 36)])
def test_corrected_penalty_gradient_is_plus_fd(size):
    """pen_corrected: the penalty gradient with the derivative's sign (the
    default keeps the reference's -weight * gradient); nothing else changes"""
    import mia_gb300 as M
    from mia_gb300 import synth
    kw = dict(rate=4.0, cost="ssd", penalty_weight=10.0)
    g = M.Level(size, **kw)
    gc = M.Level(size, penalty_corrected=True, **kw)
    o64 = O.Level(size, precision=O.PREC_F64, **kw)
    a, b = make_pair(size[::-1], 5)
    for lv in (g, gc, o64):
        lv.set_images(a, b)
    p = synth.smooth_params(g.csize, 1.0, seed=9)
    ci, cp, gi, gp, gt = g.evaluate(p)
    cic, cpc, gic, gpc, gtc = gc.evaluate(p)
    assert (ci, cp) == (cic, cpc)
    np.testing.assert_array_equal(gi, gic)
    np.testing.assert_array_equal(gpc, -gp)
    np.testing.assert_array_equal(gtc, gic + gpc)
    rng = np.random.default_rng(2)
    h = 1e-4
    for i in rng.choice(p.size, 12, replace=False):
        pp = p.copy(); pp[i] += h
        pm = p.copy(); pm[i] -= h
        fd = (o64.value(pp)[1] - o64.value(pm)[1]) / (2 * h)
        assert abs(gpc[i] - fd) <= 1e-3 * max(1.0, abs(fd))


def test_levels_evaluated_concurrently_from_host_threads():
    """one level per registration, each on its own stream: levels used from
    several host threads at once give the results of serial use"""
    import threading

    import mia_gb300 as M
    from mia_gb300 import synth
    cases = [((36, 32, 28), "ssd"), ((30, 34, 26), "ncc"), ((64, 48), "ssd"), ((40, 44, 36), "ssd")]
    levels, params = [], []
    for k, (size, cost) in enumerate(cases):
        lv = M.Level(size, rate=5.0, cost=cost, penalty_weight=2.0)
        a, b = make_pair(size[::-1], 30 + k, ncc=cost == "ncc")
        lv.set_images(a, b)
        levels.append(lv)
        params.append(synth.smooth_params(lv.csize, 1.0, seed=40 + k))
    serial = [[lv.evaluate(p) for _ in range(3)] for lv, p in zip(levels, params)]
    out = [None] * len(levels)
    errors = []

    def run(k):
        try:
            out[k] = [levels[k].evaluate(params[k]) for _ in range(3)]
        except Exception as e:   # reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(k,)) for k in range(len(levels))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
    for s, c in zip(serial, out):
        for rs, rc in zip(s, c):
            assert rs[0] == rc[0] and rs[1] == rc[1]
            for a_, b_ in zip(rs[2:], rc[2:]):
                np.testing.assert_array_equal(a_, b_)


def test_large_volume_identity_and_constant_shift():
    """size-independent properties at a large size (110 M voxels, extents
    not multiples of the tiles): zero coefficients reproduce the moving
    image (cost = the SSD of the two images); a constant coefficient field
    shifts it by that amount (the cubic B-splines sum to one)"""
    import mia_gb300 as M
    size = (512, 480, 448)
    z, y, x = np.meshgrid(*[np.arange(n, dtype=np.float32) for n in size[::-1]], indexing="ij", sparse=True)
    src = (np.sin(x * 0.07) * np.cos(y * 0.05) + 0.5 * np.sin(z * 0.03 + 0.3 * x * 0.01)).astype(np.float32) * 100
    ref = (src + 3.0 * np.cos(x * 0.011 + y * 0.013)).astype(np.float32)
    lv = M.Level(size, rate=16.0, cost="ssd")
    lv.set_images(src, ref)
    p = np.zeros(lv.nparams)
    ci, _ = lv.value(p)
    expect = 0.5 * float(np.sum((src.astype(np.float64) - ref) ** 2))
    assert abs(ci - expect) <= 1e-5 * expect, (ci, expect)
    w = lv.warp(p)
    assert float(np.max(np.abs(w - src))) <= 1e-4 * float(np.max(np.abs(src)))
    p[0::3] = 2.0   # every coefficient's x component: u = (2, 0, 0)
    w = lv.warp(p)
    inner = (slice(2, -2), slice(2, -2), slice(4, -2))
    shifted = np.roll(src, 2, axis=2)   # w(x) = src(x - 2)
    assert float(np.max(np.abs(w[inner] - shifted[inner]))) <= 1e-3 * float(np.max(np.abs(src)))
    lv.close()


@pytest.mark.parametrize("cost", ["ssd", "ncc"])
def test_page_locked_host_buffers_give_the_same_results(cost):
    """page-locked host buffers (the bench's end-to-end path) give the values
    of pageable ones, and non-finite parameters are refused with either"""
    import torch

    import mia_gb300 as M
    from mia_gb300 import _lib, synth
    size = (40, 36, 28)
    lv = M.Level(size, rate=5.0, cost=cost, penalty_weight=3.0)
    a, b = make_pair(size[::-1], 12, ncc=cost == "ncc")
    lv.set_images(a, b)
    p = synth.smooth_params(lv.csize, 1.0, seed=13)
    c1, g1 = lv.evaluate_total(p)
    hp = torch.from_numpy(p.copy()).pin_memory().numpy()
    hg = torch.empty(lv.nparams, dtype=torch.float64).pin_memory().numpy()
    for _ in range(2):
        c2, g2 = lv.evaluate_total(hp, hg)
        assert c2 == c1
        np.testing.assert_array_equal(hg, g1)
    ci, cp, gi, gp, gt = lv.evaluate(hp)
    np.testing.assert_array_equal(gt, g1)
    hp[5] = np.nan
    with pytest.raises(_lib.MgrError) as e:
        lv.evaluate_total(hp, hg)
    assert e.value.status == _lib.MGR_ERR_ARG


def test_bounded_wait_gives_up_and_the_device_stays_usable():
    """a wait on a barrier that nothing completes ends by its limit and
    raises the flag (no fault, no hang); an evaluation afterwards still
    matches the oracle"""
    import ctypes
    from mia_gb300 import _lib
    gave_up, us = ctypes.c_int(-1), ctypes.c_double(-1.0)
    _lib.check(_lib.lib().mgr_selftest_bounded_wait(0, ctypes.byref(gave_up), ctypes.byref(us)))
    assert gave_up.value == 1
    assert us.value > 0.0
    print("one failed try of the bounded wait: %.4g us (production limit 2^20 tries: %.3g s)"
          % (us.value, us.value * 2 ** 20 * 1e-6))
    size = (24, 20, 18)
    g, o, o64 = both(size, rate=4.0, cost="ssd", penalty_weight=1.0)
    mov, ref = make_pair(size[::-1], 13)
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    from mia_gb300 import synth
    check_eval(g, o, o64, synth.smooth_params(g.csize, 1.0, seed=5))


def test_bound_evaluate_call_equals_evaluate_total():
    """the bound C-ABI call (pointers prepared once, the buffers' contents
    changed between calls) gives evaluate_total's cost and gradient, refuses
    non-finite parameters, and the level keeps working"""
    import mia_gb300 as M
    from mia_gb300 import _lib
    from mia_gb300 import synth
    size = (33, 29, 21)
    lv = M.Level(size, rate=5.0, cost="ssd", penalty_weight=3.0)
    a, b = make_pair(size[::-1], 5)
    lv.set_images(a, b)
    params = np.zeros(lv.nparams)
    grad = np.zeros(lv.nparams)
    call = lv.bind_evaluate_total(params, grad)
    for seed in (1, 2):
        params[:] = synth.smooth_params(lv.csize, 1.0, seed=seed)
        c = call()
        want_c, want_g = lv.evaluate_total(params.copy())
        assert c == want_c
        assert np.array_equal(grad, want_g)
    params[3] = np.nan
    with pytest.raises(_lib.MgrError) as e:
        call()
    assert e.value.status == _lib.MGR_ERR_ARG
    params[3] = 0.0
    assert np.isfinite(call())


@pytest.mark.parametrize("cost,size", [("ssd", (33, 29, 21)), ("ncc", (70, 41, 37))])
def test_in_place_evaluation_equals_staged_copies(cost, size):
    """evaluate with the caller's host buffers read and written in place by
    the kernels (coherent host access, Grace-based hosts) gives the staged
    copies' costs and gradients bit for bit; non-finite parameters are
    refused without touching the caller's buffers, and the level keeps
    working"""
    import os
    import platform
    import mia_gb300 as M
    from mia_gb300 import _lib
    from mia_gb300 import synth
    kw = dict(rate=5.0, cost=cost, penalty_weight=3.0)
    lv = M.Level(size, **kw)
    os.environ["MGR_HOST_COPY"] = "1"
    try:
        staged = M.Level(size, **kw)
    finally:
        del os.environ["MGR_HOST_COPY"]
    assert not staged.in_place
    if platform.machine() == "aarch64":
        assert lv.in_place      # Grace: the device reads pageable host memory
    a, b = make_pair(size[::-1], 9)
    lv.set_images(a, b)
    staged.set_images(a, b)
    for seed in (3, 4):
        p = synth.smooth_params(lv.csize, 1.5, seed=seed)
        got, want = lv.evaluate(p), staged.evaluate(p)
        for g, w in zip(got, want):
            assert np.array_equal(np.asarray(g), np.asarray(w))
    params = synth.smooth_params(lv.csize, 1.0, seed=5)
    grad = np.full(lv.nparams, 7.0)
    call = lv.bind_evaluate_total(params, grad)
    params[lv.nparams - 1] = np.inf
    with pytest.raises(_lib.MgrError) as e:
        call()
    assert e.value.status == _lib.MGR_ERR_ARG
    assert np.all(grad == 7.0)
    params[lv.nparams - 1] = 0.0
    c = call()
    want_c, want_g = staged.evaluate_total(params.copy())
    assert c == want_c and np.array_equal(grad, want_g)


@pytest.mark.parametrize("cost,size", [("ssd", (70, 41, 37)), ("ncc", (33, 29, 21))])
def test_overlapped_launches_equal_serial_launches(cost, size):
    """programmatic dependent launch of the warp, adjoint and gather kernels
    (each may start while the one before it finishes) gives the results of
    plain stream-ordered launches (MGR_PDL=0) bit for bit, through evaluate,
    value and the per-kernel timing mode (which launches them one after
    another); the whole-evaluation timing mode reports the total only"""
    import os
    import mia_gb300 as M
    from mia_gb300 import _lib
    from mia_gb300 import synth
    kw = dict(rate=5.0, cost=cost, penalty_weight=3.0)
    lv = M.Level(size, **kw)
    os.environ["MGR_PDL"] = "0"
    try:
        serial = M.Level(size, **kw)
    finally:
        del os.environ["MGR_PDL"]
    a, b = make_pair(size[::-1], 11)
    lv.set_images(a, b)
    serial.set_images(a, b)
    for seed in (6, 7):
        p = synth.smooth_params(lv.csize, 1.5, seed=seed)
        want = serial.evaluate(p)
        for mode in (None, "whole", "per_kernel"):
            if mode is not None:
                lv.set_timing(True, whole=(mode == "whole"))
            got = lv.evaluate(p)
            for g, w in zip(got, want):
                assert np.array_equal(np.asarray(g), np.asarray(w))
            if mode == "whole":
                ms = lv.kernel_times()
                assert ms[0] == ms[1] == ms[2] == 0.0 and ms[3] > 0.0
            elif mode == "per_kernel":
                ms = lv.kernel_times()
                assert min(ms) > 0.0
        lv.set_timing(False)
        assert lv.value(p) == serial.value(p)
    with pytest.raises(_lib.MgrError) as e:
        _lib.check(_lib.lib().mgr_level_set_timing(lv.h, 3))
    assert e.value.status == _lib.MGR_ERR_ARG
