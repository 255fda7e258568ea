"""Parity at the benchmark configurations' full sizes (C ABI, GPU).

The 3D single pair 192x192x128 (SSD + divcurl 10, spline rate 8) and the
3D NCC pair 256^3 with a bias field (rate 5, divcurl 5), on the very
inputs the benchmark times (mia_gb300/workloads.py, made on the host):
one cost+gradient evaluation of the split and the plain kernels against
the oracle at the reference's precision and in FP64.  Tolerances: cost
1e-5 relative, gradients 1e-4 relative L2 (the parity contract); the
errors against both oracle precisions are printed.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-5
GRAD_RTOL = 1e-4


def _rel(a, b):
    return abs(a - b) / abs(b)


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", ["3d_ssd_192x192x128", "3d_ncc_256x256x256"])
def test_parity_at_configuration_size(name):
    import mia_gb300 as M
    from mia_gb300 import workloads as WL
    w, mov, ref, params = WL.make_workload(name)
    size = w["size"]
    kw = dict(rate=w["rate"], cost=w["cost"], penalty_weight=w["penalty"])
    threads = os.cpu_count() or 1
    oracles = {}
    for prec, label in ((O.PREC_REF, "reference precision"), (O.PREC_F64, "fp64")):
        o = O.Level(size, precision=prec, threads=threads, **kw)
        o.set_images(mov, ref)
        oracles[label] = o.evaluate(params)
        del o
    lv = M.Level(size, **kw)
    lv.set_images(mov, ref)
    for path in ("split", "plain"):
        lv.set_path(path)
        ci, cp, gi, gp, gt = lv.evaluate(params)
        for label, (oi, op, ogi, ogp) in oracles.items():
            errs = (_rel(ci, oi), _rel(cp, op), _rel_l2(gi, ogi), _rel_l2(gp, ogp))
            print("%s %s vs oracle %s: cost %.2e / %.2e, gradient %.2e / %.2e" % ((name, path, label) + errs))
            assert errs[0] <= COST_RTOL and errs[1] <= COST_RTOL, (path, label, errs)
            assert errs[2] <= GRAD_RTOL and errs[3] <= GRAD_RTOL, (path, label, errs)
        np.testing.assert_allclose(gt, gi + gp, rtol=0, atol=1e-12 * np.abs(gt).max())
    lv.close()
