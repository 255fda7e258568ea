"""The adjoint through the torch.autograd binding (mia_gb300.autograd):
against FP64 central finite differences of the FP64 oracle cost and
against the oracle's own gradients."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def _levels(size, **kw):
    import mia_gb300 as M
    from mia_gb300 import synth
    g = M.Level(size, **kw)
    o = O.Level(size, precision=O.PREC_REF, **kw)
    o64 = O.Level(size, precision=O.PREC_F64, **kw)
    ref = synth.blob_phantom(size[::-1], 6, sigma=(4.0, 7.0), noise=0.0, seed=21)
    mov = synth.blob_phantom(size[::-1], 6, sigma=(4.0, 7.0), noise=0.0, seed=22)
    for lv in (g, o, o64):
        lv.set_images(mov, ref)
    return g, o, o64


@pytest.mark.parametrize("size,cost", [((28, 24, 20), "ssd"), ((26, 22, 18), "ncc"), ((72, 64), "ssd")])
def test_backward_matches_fp64_finite_differences(size, cost):
    import torch

    from mia_gb300 import synth
    from mia_gb300.autograd import level_costs
    g, _, o64 = _levels(size, rate=5.0, cost=cost, penalty_weight=2.0)
    p0 = synth.smooth_params(g.csize, 0.5, seed=23)
    p = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
    costs = level_costs(p, g)
    (gi,) = torch.autograd.grad(costs[0], p, retain_graph=True)
    (gpen,) = torch.autograd.grad(costs[1], p)
    gi, gpen = gi.cpu().numpy(), gpen.cpu().numpy()
    # the 24 largest entries: the reference's image gradient (force from
    # central differences of the warped image) approximates the derivative;
    # on small entries that approximation dominates (the oracle's own
    # gradient differs from FD by 3-7 % on random entries of these problems,
    # by about 2 % on the largest)
    idx = np.argsort(-np.abs(gi))[:24]
    fd_i, fd_p = [], []
    for i in idx:
        h = 1e-3
        pp, pm = p0.copy(), p0.copy()
        pp[i] += h
        pm[i] -= h
        vp, vm = o64.value(pp), o64.value(pm)
        fd_i.append((vp[0] - vm[0]) / (2 * h))
        fd_p.append((vp[1] - vm[1]) / (2 * h))
    # the image gradient is the reference's (force from central differences
    # of the warped image): agreement to the accuracy of FD on a smooth problem
    assert _rel_l2(gi[idx], fd_i) < 5e-2
    # the penalty is a quadratic form of the coefficients: FD is exact to rounding
    assert _rel_l2(gpen[idx], fd_p) < 1e-4


def test_backward_equals_the_oracle_gradients_and_composes():
    import torch

    from mia_gb300 import synth
    from mia_gb300.autograd import level_costs
    size = (30, 26, 22)
    g, o, _ = _levels(size, rate=5.0, cost="ssd", penalty_weight=3.0)
    p0 = synth.smooth_params(g.csize, 0.7, seed=24)
    p = torch.tensor(p0, dtype=torch.float64, device="cuda", requires_grad=True)
    costs = level_costs(p, g)
    oi, op, ogi, ogp = o.evaluate(p0)
    assert abs(costs[0].item() - oi) <= 1e-5 * abs(oi)
    assert abs(costs[1].item() - op) <= 1e-5 * abs(op)
    loss = 2.0 * costs[0] + 3.0 * costs[1]
    loss.backward()
    expect = 2.0 * ogi - 3.0 * ogp   # the oracle returns the reference's penalty sign
    assert _rel_l2(p.grad.cpu().numpy(), expect) < 1e-4
