"""The refinement of the spline coefficient grid between the two passes of
a registration level (C2D/C3DSplineTransformation::refine): the host
restatement against the oracle, and the device version the batched driver
uses against the host one, value for value."""
import numpy as np
import pytest

from oracle import oracle as O

CASES = [(3, (22, 24, 20), (42, 46, 38)), (3, (9, 7, 11), (15, 12, 19)), (3, (6, 6, 6), (6, 9, 6)),
         (2, (20, 17), (37, 31)), (2, (8, 8), (8, 14))]


def _params(dim, nc, seed, offset=0.0):
    rng = np.random.default_rng(seed)
    p = rng.standard_normal(int(np.prod(nc)) * dim) * 2.0 + offset
    return p.astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("dim,nc_old,nc_new", CASES)
def test_host_refine_matches_oracle(dim, nc_old, nc_new):
    from mia_gb300 import registration as R
    for seed, offset in ((1, 0.0), (2, 5.0)):   # offset 5: every component positive (minimum taken as 0)
        p = _params(dim, nc_old, seed, offset)
        g = R.refine_coefficients(p, nc_old, nc_new)
        o = O.refine(dim, nc_old, nc_new, p)
        assert g is not None and o is not None
        assert np.array_equal(g, o)


def test_host_refine_without_growth_writes_nothing():
    from mia_gb300 import registration as R
    p = _params(3, (9, 9, 9), 3)
    assert R.refine_coefficients(p, (9, 9, 9), (9, 9, 9)) is None
    assert R.refine_coefficients(p, (9, 9, 9), (9, 8, 9)) is None


@pytest.mark.gpu
@pytest.mark.parametrize("dim,nc_old,nc_new", CASES)
def test_device_refine_equals_host(dim, nc_old, nc_new):
    import torch
    from mia_gb300 import registration as R
    for seed, offset in ((4, 0.0), (5, 5.0)):
        p = _params(dim, nc_old, seed, offset)
        host = R.refine_coefficients(p, nc_old, nc_new)
        # unrounded device input: the device rounds to float as the host does
        raw = p + np.random.default_rng(seed).standard_normal(p.size) * 1e-9
        d_in = torch.from_numpy(raw).cuda()
        d_out = torch.full((int(np.prod(nc_new)) * dim,), np.nan, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        assert R.refine_coefficients_device(d_in, d_out, nc_old, nc_new)
        torch.cuda.synchronize()
        dev = d_out.cpu().numpy()
        host_raw = R.refine_coefficients(raw, nc_old, nc_new)
        assert np.array_equal(dev, host_raw)
        assert np.array_equal(R.refine_coefficients(raw.astype(np.float32).astype(np.float64), nc_old, nc_new),
                              host_raw)
        assert host is not None


@pytest.mark.gpu
def test_device_refine_without_growth_writes_nothing():
    import torch
    from mia_gb300 import registration as R
    d_in = torch.zeros(9 * 9 * 9 * 3, dtype=torch.float64, device="cuda")
    d_out = torch.full((9 * 9 * 9 * 3,), 7.0, dtype=torch.float64, device="cuda")
    assert not R.refine_coefficients_device(d_in, d_out, (9, 9, 9), (9, 9, 9))
    torch.cuda.synchronize()
    assert torch.all(d_out == 7.0)


def test_host_refine_rejects_wrong_sizes():
    from mia_gb300 import registration as R
    p = _params(3, (9, 9, 9), 3)
    with pytest.raises(ValueError):
        R.refine_coefficients(p[:-1], (9, 9, 9), (15, 15, 15))   # one value short of the old grid
    with pytest.raises(ValueError):
        R.refine_coefficients(p, (9, 9, 9), (15, 15))
