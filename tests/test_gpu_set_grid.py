"""mgr_level_set_grid: a level moved to another coefficient grid evaluates
exactly as a level created for that grid on the same images (2D and 3D,
SSD and NCC, growing and shrinking the grid)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("size,cost,grids", [((40, 36, 28), "ssd", [(8, 7, 6), (11, 10, 8), (6, 6, 5)]),
                                              ((96, 80), "ncc", [(7, 6), (12, 10), (5, 5)])])
def test_set_grid_equals_a_fresh_level(size, cost, grids):
    import mia_gb300 as M
    from mia_gb300 import synth
    shape = size[::-1]
    ref = synth.blob_phantom(shape, 8, sigma=(3.0, 8.0), seed=4)
    mov = np.roll(ref, 2, axis=-1)
    kw = dict(cost=cost, penalty_weight=3.0, div=1.5, curl=0.5)
    lv = M.Level(size, csize=grids[0], **kw)
    lv.set_images(mov, ref)
    for g in grids:
        lv.set_grid(g)
        assert lv.csize == tuple(g)
        fresh = M.Level(size, csize=g, **kw)
        fresh.set_images(mov, ref)
        p = synth.smooth_params(g, 1.2, seed=len(g) + g[0])
        a, b = lv.evaluate(p), fresh.evaluate(p)
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y))
        assert lv.value(p) == fresh.value(p)
        fresh.close()
    lv.close()
