"""The benchmark workloads: their settings and their seeded synthetic
inputs, made on the host only (numpy / scipy), so that every arm of the
benchmark and the tests at configuration size see the same arrays.

Cost+gradient workloads (metric Mvoxel/s): the 3D single pair
192x192x128 (SSD, spline rate 8, divcurl weight 10) and the 3D NCC pair
256^3 with a multiplicative bias field (rate 5, divcurl weight 5).
Registration workloads (metric registered pairs/s): the 2D single pair
128x128 (SSD, rate 16, divcurl 10, one level, 50 iterations), the 60-frame
2D perfusion series (2 levels x 40 iterations) and the 16-pair 3D cohort
(NCC, 3 levels x 30 iterations).  No public dataset is involved.
"""
import numpy as np

from . import synth

WORKLOADS = {
    "3d_ssd_192x192x128": dict(size=(192, 192, 128), nblobs=40, sigma=(4.0, 16.0), rate=8.0, wsigma=2.0,
                               wclip=4.0, cost="ssd", penalty=10.0, bias=None, seed=2000),
    "3d_ncc_256x256x256": dict(size=(256, 256, 256), nblobs=40, sigma=(4.0, 16.0), rate=5.0, wsigma=2.0,
                               wclip=4.0, cost="ncc", penalty=5.0, bias=0.1, seed=3000),
}

BATCH_WORKLOADS = {
    # one 2D pair, 128x128, 1 level, 50 iterations (mia-2dimageregistration)
    "single2d_128": dict(kind="single", npairs=1, rate=16.0, levels=1, cost="ssd", penalty=10.0, minimizer="gsl",
                         maxiter=50, seed=1000),
    # 60-frame 2D perfusion series, frames of uneven size, all to frame 0
    "series2d_60": dict(kind="series", npairs=60, rate=16.0, levels=2, cost="ssd", penalty=10.0, minimizer="gsl",
                        maxiter=40, seed=4000),
    # 16-pair 3D cohort of uneven size with bias fields
    "cohort3d_16": dict(kind="cohort", npairs=16, rate=8.0, levels=3, cost="ncc", penalty=5.0, minimizer="gsl",
                        maxiter=30, seed=5000),
}

L2_NOTE = "inputs above the 126 MB L2 are not assumed: L2 flushed between GPU steps by a 256 MiB write, " \
          "flush outside the timed region"


def joint_normalise(mov, ref):
    """mean 0 / sigma 1 of the two images together, sigma with n - 1
    (FScaleFilterCreator, mia/template/nonrigidregister.cxx:147-184)"""
    a = mov.astype(np.float64).ravel()
    b = ref.astype(np.float64).ravel()
    n = 2 * a.size
    s = a.sum() + b.sum()
    s2 = (a * a).sum() + (b * b).sum()
    mean = s / n
    sig = np.sqrt((s2 - s * s / n) / (n - 1))
    return ((mov - mean) / sig).astype(np.float32), ((ref - mean) / sig).astype(np.float32)


def make_workload(name):
    """(settings, moving, reference, params): the reference a blob phantom,
    the moving image the phantom warped by a random cubic B-spline field
    (and, with `bias`, times a smooth multiplicative bias), both jointly
    normalised as the registration driver does; params half the scale of
    the true field, the fixed point the evaluations are timed at"""
    w = WORKLOADS[name]
    shape = w["size"][::-1]
    ref = synth.blob_phantom(shape, w["nblobs"], sigma=w["sigma"], seed=w["seed"])
    true_c = synth.spline_field_params(shape, w["rate"], w["wsigma"], w["wclip"], seed=w["seed"] + 1)
    mov = synth.spline_warp_host(ref, true_c)
    if w["bias"]:
        mov = (mov * synth.bias_field(shape, w["bias"], seed=w["seed"] + 2)).astype(np.float32)
    mov, ref = joint_normalise(mov, ref)
    params = 0.5 * synth.spline_params(true_c.size // 3, 3, w["wsigma"], w["wclip"], seed=w["seed"] + 3)
    return w, mov, ref, params


def make_pairs(name):
    """(settings, [(moving, reference)]) of a registration workload"""
    w = BATCH_WORKLOADS[name]
    if w["kind"] == "series":
        pairs = synth.perfusion_series(w["npairs"], synth.host_warp_factory(2), rate=w["rate"], seed=w["seed"])
    elif w["kind"] == "cohort":
        pairs = synth.cohort_pairs(w["npairs"], synth.host_warp_factory(3), rate=w["rate"], seed=w["seed"])
    else:
        ref = synth.blob_phantom((128, 128), 12, sigma=(4.0, 12.0), seed=w["seed"])
        pairs = [(synth.host_warp_factory(2)(ref, w["rate"], w["seed"] + 1), ref)]
    return w, pairs


def line_config(name, csize=None):
    """the `config` object of a benchmark line, the same in every arm"""
    if name in WORKLOADS:
        w = WORKLOADS[name]
        c = {"workload": name, "size": list(w["size"]), "rate": w["rate"], "cost": w["cost"],
             "divcurl_weight": w["penalty"], "bias_field": bool(w["bias"]), "l2": L2_NOTE}
        if csize is not None:
            c["coefficients"] = list(csize)
        return c
    w = BATCH_WORKLOADS[name]
    return {"workload": name, "pairs": w["npairs"], "levels": w["levels"], "rate": w["rate"], "cost": w["cost"],
            "divcurl_weight": w["penalty"], "minimizer": "%s maxiter=%d step=0.1" % (w["minimizer"], w["maxiter"])}
