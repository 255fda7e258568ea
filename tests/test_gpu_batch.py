"""Batched registration (mgr_register_batch): many pairs of uneven size in
lock step with device-resident minimizers, against the oracle's per-pair
registration and against the per-pair GPU driver."""
import numpy as np
import pytest

from oracle import oracle as O

FINAL_COST_RTOL = 1e-4


def _oracle_with_spread(mov, ref, rate, levels, mo, **kw):
    """The oracle's registration and how far it moves when the moving image
    is perturbed at float rounding level (relative 1e-7).  gdsq's step rule
    divides by a difference of nearly equal numbers, so some trajectories
    amplify rounding differences; agreement is then asserted within that
    spread instead of the fixed tolerance."""
    po, cso, fo, no = O.register(mov, ref, rate, levels, mo, **kw)
    rng = np.random.default_rng(1)
    m2 = (mov * (1 + 1e-7 * rng.standard_normal(mov.shape))).astype(np.float32)
    p2, c2, f2, n2 = O.register(m2, ref, rate, levels, mo, **kw)
    return po, cso, fo, abs(f2 - fo), np.linalg.norm(p2 - po)


def _assert_close(pg, csg, fg, po, cso, fo, fspread, pspread):
    assert csg == cso
    assert abs(fg - fo) <= max(FINAL_COST_RTOL * abs(fo), 3 * fspread), (fg, fo, fspread)
    assert np.linalg.norm(pg - po) <= max(1e-3 * np.linalg.norm(po), 3 * pspread)


def _pair2d(seed, shape, rate=16.0):
    from mia_gb300 import synth
    ref = synth.blob_phantom(shape, 8, sigma=(4, 10), seed=seed)
    lv = O.Level(shape[::-1], rate=rate)
    lv.set_images(ref, ref)
    mov = lv.warp(synth.spline_params(lv.nparams // 2, 2, 1.5, 3.0, seed=seed + 1))
    return mov, ref


def _pair3d(seed, shape, rate=8.0):
    from mia_gb300 import synth
    ref = synth.blob_phantom(shape, 10, sigma=(3, 8), seed=seed)
    lv = O.Level(shape[::-1], rate=rate)
    lv.set_images(ref, ref)
    mov = lv.warp(synth.spline_params(lv.nparams // 3, 3, 1.5, 3.0, seed=seed + 1))
    mov = (mov * synth.bias_field(shape, 0.1, seed=seed + 2)).astype(np.float32)
    return mov, ref


def test_batch_rejects_mixed_dimensions():
    """argument checks run before any device call"""
    from mia_gb300 import _lib
    from mia_gb300 import registration as R
    a = np.zeros((16, 16), np.float32)
    b = np.zeros((8, 8, 8), np.float32)
    with pytest.raises(_lib.MgrError) as e:
        R.register_batch([(a, a), (b, b)], 4.0, 1, R.minimizer("gsl", maxiter=2))
    assert e.value.status == _lib.MGR_ERR_ARG


@pytest.mark.gpu
def test_batch_rejects_a_rate_too_large_for_the_coarsest_level():
    """the coarsest level's grid is checked where the levels are made ahead
    (a worker thread): the error reaches the caller as an argument error"""
    from mia_gb300 import _lib
    from mia_gb300 import registration as R
    pairs = [_pair2d(71, (64, 64)), _pair2d(72, (48, 56))]
    with pytest.raises(_lib.MgrError) as e:
        R.register_batch(pairs, 40.0, 3, R.minimizer("gsl", maxiter=2), cost="ssd", penalty_weight=10.0)
    assert e.value.status == _lib.MGR_ERR_ARG
    assert "coarsest" in str(e.value)
    # the library stays usable after the failed call
    res = R.register_batch(pairs, 16.0, 1, R.minimizer("gsl", maxiter=2), cost="ssd", penalty_weight=10.0)
    assert len(res) == 2


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["gsl", "gdsq"])
def test_batch_2d_matches_oracle(kind):
    from mia_gb300 import registration as R
    shapes = [(80, 96), (64, 72), (96, 96), (72, 88)]
    pairs = [_pair2d(31 + 7 * i, s) for i, s in enumerate(shapes)]
    # a pair of constant images takes the identity shortcut
    pairs.append((np.full((64, 64), 3.0, np.float32), np.full((64, 64), 3.0, np.float32)))
    mg = R.minimizer(kind, maxiter=12, step=0.1)
    res = R.register_batch(pairs, 16.0, 2, mg, cost="ssd", penalty_weight=10.0)
    mo = O.minimizer(kind, maxiter=12, step=0.1)
    for (mov, ref), (pg, csg, fg, ng) in zip(pairs[:-1], res[:-1]):
        po, cso, fo, fs, ps = _oracle_with_spread(mov, ref, 16.0, 2, mo, cost="ssd", penalty_weight=10.0)
        _assert_close(pg, csg, fg, po, cso, fo, fs, ps)
    pg, csg, fg, ng = res[-1]
    assert ng == 0 and fg == 0.0 and not np.any(pg)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["gsl", "gdsq"])
def test_batch_minimizer_vectors_span_many_blocks(kind):
    """fine grids: the minimizer kernels spread each pair's vectors over
    several blocks of 2048 elements, whose partial sums the pair's last
    block adds in block order"""
    from mia_gb300 import registration as R
    shapes = [(160, 144), (128, 176)]
    pairs = [_pair2d(61 + 5 * i, s) for i, s in enumerate(shapes)]
    mg = R.minimizer(kind, maxiter=8, step=0.1)
    res = R.register_batch(pairs, 2.0, 1, mg, cost="ssd", penalty_weight=10.0)
    assert min(r[0].size for r in res) > 4 * 2048
    mo = O.minimizer(kind, maxiter=8, step=0.1)
    for (mov, ref), (pg, csg, fg, ng) in zip(pairs, res):
        po, cso, fo, fs, ps = _oracle_with_spread(mov, ref, 2.0, 1, mo, cost="ssd", penalty_weight=10.0)
        _assert_close(pg, csg, fg, po, cso, fo, fs, ps)


@pytest.mark.gpu
def test_batch_3d_ncc_matches_oracle():
    from mia_gb300 import registration as R
    shapes = [(32, 36, 40), (24, 32, 32), (32, 32, 48)]
    pairs = [_pair3d(41 + 5 * i, s) for i, s in enumerate(shapes)]
    mg = R.minimizer("gdsq", maxiter=6, step=0.1)
    res = R.register_batch(pairs, 8.0, 2, mg, cost="ncc", penalty_weight=5.0)
    mo = O.minimizer("gdsq", maxiter=6, step=0.1)
    for (mov, ref), (pg, csg, fg, ng) in zip(pairs, res):
        po, cso, fo, fs, ps = _oracle_with_spread(mov, ref, 8.0, 2, mo, cost="ncc", penalty_weight=5.0)
        _assert_close(pg, csg, fg, po, cso, fo, fs, ps)


@pytest.mark.gpu
def test_batch_graphs_match_stream_launches_and_per_pair_driver():
    """graph replay and plain stream launches run the same kernels in the
    same order: bit-identical results; the per-pair driver agrees within the
    final-cost tolerance"""
    from mia_gb300 import registration as R
    shapes = [(64, 80), (96, 64), (80, 80)]
    pairs = [_pair2d(51 + 3 * i, s) for i, s in enumerate(shapes)]
    mg = R.minimizer("gsl", maxiter=20, step=0.1)
    a = R.register_batch(pairs, 16.0, 2, mg, use_graphs=True, cost="ssd", penalty_weight=10.0)
    b = R.register_batch(pairs, 16.0, 2, mg, use_graphs=False, cost="ssd", penalty_weight=10.0)
    for (pa, ca, fa, na), (pb, cb, fb, nb) in zip(a, b):
        assert ca == cb and fa == fb and na == nb
        assert np.array_equal(pa, pb)
    for (mov, ref), (pg, csg, fg, ng) in zip(pairs, a):
        pp, csp, fp, npp = R.register_pair(mov, ref, 16.0, 2, mg, cost="ssd", penalty_weight=10.0)
        assert csg == csp
        assert abs(fg - fp) <= FINAL_COST_RTOL * abs(fp), (fg, fp)


@pytest.mark.gpu
def test_batch_of_identity_pairs_only():
    """every pair holds one value per image: no level is made, nothing is
    minimised, the parameters stay zero"""
    from mia_gb300 import registration as R
    pairs = [(np.full((40, 48), 2.0, np.float32), np.full((40, 48), 2.0, np.float32)),
             (np.full((32, 32), -1.0, np.float32), np.full((32, 32), -1.0, np.float32))]
    res = R.register_batch(pairs, 16.0, 2, R.minimizer("gsl", maxiter=5), cost="ssd", penalty_weight=10.0)
    for pg, csg, fg, ng in res:
        assert ng == 0 and fg == 0.0 and not np.any(pg)


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_batch_of_one_pair_equals_the_per_pair_driver(dim):
    """one pair through the batch runs the per-pair driver's kernels in the
    same order: the same final cost and parameters"""
    from mia_gb300 import registration as R
    mov, ref = _pair2d(81, (64, 72)) if dim == 2 else _pair3d(82, (24, 28, 32))
    rate = 16.0 if dim == 2 else 8.0
    mg = R.minimizer("gsl", maxiter=8, step=0.1)
    (pb, cb, fb, nb), = R.register_batch([(mov, ref)], rate, 2, mg, cost="ssd", penalty_weight=10.0)
    pp, cp, fp, npp = R.register_pair(mov, ref, rate, 2, mg, cost="ssd", penalty_weight=10.0)
    assert cb == cp
    assert abs(fb - fp) <= 1e-6 * abs(fp), (fb, fp)
    assert np.linalg.norm(pb - pp) <= 1e-5 * max(np.linalg.norm(pp), 1e-12)


@pytest.mark.gpu
def test_batch_from_device_images_equals_host_images_and_matches_oracle():
    """3D SSD, GSL steepest descent, three levels, pairs of uneven size: the
    batch from CUDA tensors (mgr_register_batch_device) gives bit for bit the
    results of the batch from host arrays, and both agree with the oracle"""
    import torch
    from mia_gb300 import registration as R
    shapes = [(40, 44, 48), (48, 40, 36)]
    pairs = [_pair3d(91 + 7 * i, s) for i, s in enumerate(shapes)]
    mg = R.minimizer("gsl", maxiter=5, step=0.1)
    kw = dict(cost="ssd", penalty_weight=10.0)
    host = R.register_batch(pairs, 8.0, 3, mg, **kw)
    dpairs = [(torch.from_numpy(m).cuda(), torch.from_numpy(r).cuda()) for m, r in pairs]
    torch.cuda.synchronize()
    dev = R.register_batch_device(dpairs, 8.0, 3, mg, **kw)
    for (ph, ch, fh, nh), (pd, cd, fd, nd) in zip(host, dev):
        assert ch == cd and fh == fd and nh == nd
        assert np.array_equal(ph, pd)
    # host arrays read in place by the device (where it can read pageable
    # host memory) and host arrays staged by copies give the same bits
    import os
    os.environ["MGR_HOST_COPY"] = "1"
    try:
        copied = R.register_batch(pairs, 8.0, 3, mg, **kw)
    finally:
        del os.environ["MGR_HOST_COPY"]
    for (ph, ch, fh, nh), (pc, cc, fc, nc) in zip(host, copied):
        assert ch == cc and fh == fc and nh == nc
        assert np.array_equal(ph, pc)
    mo = O.minimizer("gsl", maxiter=5, step=0.1)
    for (mov, ref), (pg, csg, fg, ng) in zip(pairs, host):
        po, cso, fo, fs, ps = _oracle_with_spread(mov, ref, 8.0, 3, mo, **kw)
        _assert_close(pg, csg, fg, po, cso, fo, fs, ps)


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_batch_ncc_without_penalty_matches_oracle(dim):
    """NCC with no spline penalty (the image term alone), GSL steepest descent"""
    from mia_gb300 import registration as R
    from mia_gb300 import synth
    if dim == 2:
        shapes, rate = [(72, 88), (96, 80)], 16.0
        pairs = [_pair2d(101 + 3 * i, s, rate) for i, s in enumerate(shapes)]
        pairs = [((m * synth.bias_field(m.shape, 0.1, seed=7 + i)).astype(np.float32), r)
                 for i, (m, r) in enumerate(pairs)]
    else:
        shapes, rate = [(40, 36, 44), (36, 44, 40)], 8.0
        pairs = [_pair3d(111 + 3 * i, s, rate) for i, s in enumerate(shapes)]
    mg = R.minimizer("gsl", maxiter=8, step=0.1)
    res = R.register_batch(pairs, rate, 2, mg, cost="ncc")
    mo = O.minimizer("gsl", maxiter=8, step=0.1)
    for (mov, ref), (pg, csg, fg, ng) in zip(pairs, res):
        po, cso, fo, fs, ps = _oracle_with_spread(mov, ref, rate, 2, mo, cost="ncc")
        _assert_close(pg, csg, fg, po, cso, fo, fs, ps)


@pytest.mark.gpu
@pytest.mark.parametrize("use_graphs", [True, False])
def test_batch_persistent_launch_equals_one_block_per_item(use_graphs):
    """3D NCC, three levels, pairs of uneven size: the persistent warp and
    adjoint launches (resident blocks drawing (pair, tile) items from a
    device queue) give bit for bit the results of one block per item"""
    from mia_gb300 import registration as R
    shapes = [(40, 44, 48), (48, 40, 36), (40, 36, 44)]
    pairs = [_pair3d(131 + 5 * i, s) for i, s in enumerate(shapes)]
    mg = R.minimizer("gsl", maxiter=6, step=0.1)
    kw = dict(cost="ncc", penalty_weight=5.0)
    base = R.register_batch(pairs, 8.0, 3, mg, use_graphs=use_graphs, **kw)
    pers = R.register_batch(pairs, 8.0, 3, mg, use_graphs=use_graphs, persistent=True, **kw)
    for (pb, cb, fb, nb), (pp, cp, fp, npp) in zip(base, pers):
        assert cb == cp and fb == fp and nb == npp
        assert np.array_equal(pb, pp)


@pytest.mark.gpu
def test_batch_persistent_launch_many_items_per_block():
    """the persistent launches when each resident block draws several
    (pair, tile) items (its shared-memory ring and barriers reused from one
    item to the next): two SSD pairs of about a thousand tiles each against
    the few hundred resident blocks of one GPU, bit for bit the results of
    one block per item"""
    from mia_gb300 import registration as R
    shapes = [(192, 192, 128), (160, 144, 144)]
    pairs = [_pair3d(171 + 7 * i, s) for i, s in enumerate(shapes)]
    mg = R.minimizer("gsl", maxiter=3, step=0.1)
    kw = dict(cost="ssd", penalty_weight=5.0)
    base = R.register_batch(pairs, 8.0, 1, mg, **kw)
    pers = R.register_batch(pairs, 8.0, 1, mg, persistent=True, **kw)
    for (pb, cb, fb, nb), (pp, cp, fp, npp) in zip(base, pers):
        assert cb == cp and fb == fp and nb == npp
        assert np.array_equal(pb, pp)
