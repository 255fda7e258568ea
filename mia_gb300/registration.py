"""Multiresolution registration of image pairs on the GPU.

``register_pair`` follows TNonrigidRegisterImpl::run
(mia/template/nonrigidregister.cxx:193-296): joint normalisation, levels
built with the `scale` filter, upscale and refine of the spline
transformation, the `gsl:opt=gd` or `gdsq` minimizer per level.
"""
import ctypes
import re

import numpy as np

from . import _lib
from ._lib import check, lib, minimizer  # noqa: F401

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)


def level_desc(size_xyz, rate, cost="ssd", penalty_weight=None, div=1.0, curl=1.0, ssd_norm=False,
               cost_weight=1.0, penalty_norm=False, penalty_corrected=False):
    d = _lib.LevelDesc()
    d.dim = len(size_xyz)
    d.size = (ctypes.c_int * 3)(*(list(size_xyz) + [1] * (3 - d.dim)))
    d.csize = (ctypes.c_int * 3)(0, 0, 0)
    r = rate if hasattr(rate, "__len__") else [rate] * d.dim
    d.rate = (ctypes.c_float * 3)(*(list(r) + [1.0] * (3 - len(r))))
    d.cost = _lib.COST_NCC if cost == "ncc" else _lib.COST_SSD
    d.ssd_norm, d.cost_weight = int(ssd_norm), float(cost_weight)
    d.has_penalty = int(penalty_weight is not None)
    d.pen_weight = float(penalty_weight or 0.0)
    d.pen_div, d.pen_curl, d.pen_norm = float(div), float(curl), int(penalty_norm)
    d.pen_corrected = int(penalty_corrected)
    return d


def register_pair(src, ref, rate, levels, mz, path="split", device=0, **cost_kw):
    """Returns (params, csize, final_cost, evaluations)."""
    s = np.ascontiguousarray(src, dtype=np.float32)
    r = np.ascontiguousarray(ref, dtype=np.float32)
    if s.shape != r.shape:
        raise ValueError("source and reference differ in shape")
    d = level_desc(s.shape[::-1], rate, **cost_kw)
    # refine targets (size + rate - 1) / rate + 2 <= size + 2 coefficients per axis
    maxp = int(np.prod([n + 3 for n in s.shape])) * s.ndim
    out = np.empty(maxp)
    cs = (ctypes.c_int * 3)()
    fc, ne = ctypes.c_double(), ctypes.c_int()
    p = _lib.PATH_PLAIN if path == "plain" else _lib.PATH_SPLIT
    check(lib().mgr_register(ctypes.byref(d), int(levels), ctypes.byref(mz), s.ctypes.data_as(_fp),
                             r.ctypes.data_as(_fp), p, int(device), out.ctypes.data_as(_dp), maxp, cs,
                             ctypes.byref(fc), ctypes.byref(ne)))
    dim = d.dim
    n = int(np.prod(cs[:dim])) * dim
    return out[:n].copy(), tuple(cs[:dim]), fc.value, ne.value


def scale_image(img, out_shape, device=0):
    """the `scale` filter (downscaling) on the GPU; arrays [z, y, x]"""
    a = np.ascontiguousarray(img, dtype=np.float32)
    out = np.empty(tuple(out_shape), np.float32)
    isz = (ctypes.c_int * 3)(*(list(a.shape[::-1]) + [1] * (3 - a.ndim)))
    osz = (ctypes.c_int * 3)(*(list(out.shape[::-1]) + [1] * (3 - out.ndim)))
    check(lib().mgr_scale_image(a.ndim, isz, a.ctypes.data_as(_fp), osz, out.ctypes.data_as(_fp), int(device)))
    return out


def refine_coefficients(params, nc_old, nc_new):
    """the spline grid refinement on the host: params (prod(nc_old) * dim,
    components interleaved, x fastest) onto nc_new; None when no axis grows"""
    dim = len(nc_old)
    if len(nc_new) != dim:
        raise ValueError("nc_old and nc_new differ in dimension")
    p = np.ascontiguousarray(params, dtype=np.float64)
    if p.size != int(np.prod(nc_old)) * dim:
        raise ValueError("params must hold prod(nc_old) * dim values")
    out = np.empty(int(np.prod(nc_new)) * dim)
    o = (ctypes.c_int * 3)(*(list(nc_old) + [1] * (3 - dim)))
    n = (ctypes.c_int * 3)(*(list(nc_new) + [1] * (3 - dim)))
    grown = ctypes.c_int()
    check(lib().mgr_refine_coefficients(dim, o, n, p.ctypes.data_as(_dp), out.ctypes.data_as(_dp), ctypes.byref(grown)))
    return out if grown.value else None


def refine_coefficients_device(d_params, d_out, nc_old, nc_new, stream=0):
    """refine_coefficients on device buffers (objects with .data_ptr());
    queued on `stream` (a CUDA stream handle, 0: the legacy default stream);
    returns whether the grid grew (d_out written)"""
    dim = len(nc_old)
    o = (ctypes.c_int * 3)(*(list(nc_old) + [1] * (3 - dim)))
    n = (ctypes.c_int * 3)(*(list(nc_new) + [1] * (3 - dim)))
    grown = ctypes.c_int()
    check(lib().mgr_refine_coefficients_device(dim, o, n, ctypes.c_void_p(d_params.data_ptr()),
                                               ctypes.c_void_p(d_out.data_ptr()), ctypes.byref(grown),
                                               ctypes.c_void_p(stream)))
    return bool(grown.value)


def save_transform(path, size_xyz, csize, params, rate=None, creator=None, attributes=None):
    """write a spline transformation (mgr_transform_save): image size
    (x, y[, z]), coefficient grid, parameters; the creator string defaults
    to spline:rate=<rate> (the registration's rate; without one, the mean
    knot spacing of the grid)"""
    dim = len(size_xyz)
    p = np.ascontiguousarray(params, dtype=np.float64)
    if creator is None:
        if rate is None:
            rate = np.mean([(n - 1) / max(c - 3, 1) for n, c in zip(size_xyz, csize)])
        creator = "spline:rate=%g" % rate
    attributes = dict(attributes or {})
    names = (ctypes.c_char_p * max(1, len(attributes)))(*[k.encode() for k in attributes])
    values = (ctypes.c_char_p * max(1, len(attributes)))(*[str(v).encode() for v in attributes.values()])
    sz = (ctypes.c_int * 3)(*(list(size_xyz) + [1] * (3 - dim)))
    cs = (ctypes.c_int * 3)(*(list(csize) + [1] * (3 - dim)))
    check(lib().mgr_transform_save(str(path).encode(), dim, sz, cs, creator.encode(), p.ctypes.data_as(_dp), p.size,
                                   names, values, len(attributes)))


def load_transform(path):
    """read what save_transform wrote: dict(dim, size, csize, creator,
    attributes, params)"""
    dim, n = ctypes.c_int(), ctypes.c_size_t()
    sz, cs = (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
    check(lib().mgr_transform_load(str(path).encode(), ctypes.byref(dim), sz, cs, None, 0, None, 0, None, 0,
                                   ctypes.byref(n)))
    params = np.empty(n.value)
    cap = {"creator": 4096, "attribute": 1 << 16}
    for _ in range(3):   # a string too large for its buffer: grow it to the size the error names
        creator = ctypes.create_string_buffer(cap["creator"])
        attrs = ctypes.create_string_buffer(cap["attribute"])
        status = lib().mgr_transform_load(str(path).encode(), ctypes.byref(dim), sz, cs, creator, len(creator),
                                          attrs, len(attrs), params.ctypes.data_as(_dp), params.size,
                                          ctypes.byref(n))
        m = re.match(r".*(creator|attribute) buffer too small: (\d+) bytes needed",
                     lib().mgr_last_error().decode()) if status == _lib.MGR_ERR_ARG else None
        if not m:
            break
        cap[m.group(1)] = int(m.group(2))
    check(status)
    d = dim.value
    attributes = dict(line.split("\t", 1) for line in attrs.value.decode().splitlines() if line)
    return dict(dim=d, size=tuple(sz[:d]), csize=tuple(cs[:d]), creator=creator.value.decode(),
                attributes=attributes, params=params)


def warp_image(img, csize, params, device=0):
    """the image (numpy [z, y, x], full size) transformed by the spline
    transformation with coefficient grid csize: the registration programs'
    output image (bspline:d=3 interpolation, mirror boundary, clamp)"""
    from .level import Level
    a = np.ascontiguousarray(img, dtype=np.float32)
    lv = Level(a.shape[::-1], csize=tuple(csize), device=device)
    try:
        lv.set_images(a, a)
        return lv.warp(params)
    finally:
        lv.close()


def normalize_pair(src, ref, device=0):
    """(applied, src', ref', mean, sigma): the joint mean-0 / sigma-1
    normalisation; when both images hold one value nothing is applied and
    src', ref' are copies of the inputs"""
    s = np.ascontiguousarray(src, dtype=np.float32)
    r = np.ascontiguousarray(ref, dtype=np.float32)
    if s.shape != r.shape:
        raise ValueError("source and reference differ in shape")
    so, ro = np.empty_like(s), np.empty_like(r)
    m, sg, ok = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    check(lib().mgr_normalize_pair(s.ctypes.data_as(_fp), r.ctypes.data_as(_fp), s.size, so.ctypes.data_as(_fp),
                                   ro.ctypes.data_as(_fp), ctypes.byref(m), ctypes.byref(sg), ctypes.byref(ok),
                                   int(device)))
    if not ok.value:
        return False, s.copy(), r.copy(), m.value, sg.value
    return True, so, ro, m.value, sg.value


def _batch(shapes, sptrs, rptrs, on_device, rate, levels, mz, device, use_graphs, cost_kw):
    cost_kw = dict(cost_kw)
    persistent = cost_kw.pop("persistent", False)   # 3D: persistent warp / adjoint launches
    n = len(shapes)
    descs = (_lib.LevelDesc * n)()
    for i, shp in enumerate(shapes):
        descs[i] = level_desc(tuple(shp)[::-1], rate, **cost_kw)
    sp = (ctypes.c_void_p * n)(*sptrs)
    rp = (ctypes.c_void_p * n)(*rptrs)
    # refine targets (size + rate - 1) / rate + 2 <= size + 2 coefficients per axis
    maxp = [int(np.prod([d + 3 for d in shp])) * len(shp) for shp in shapes]
    outs = [np.empty(m) for m in maxp]
    op = (ctypes.POINTER(ctypes.c_double) * n)(*[o.ctypes.data_as(_dp) for o in outs])
    mp = (ctypes.c_size_t * n)(*maxp)
    cs = (ctypes.c_int * (3 * n))()
    fc = (ctypes.c_double * n)()
    ne = (ctypes.c_int * n)()
    fn = lib().mgr_register_batch_device if on_device else lib().mgr_register_batch
    flags = int(bool(use_graphs)) | (2 if persistent else 0)
    check(fn(n, descs, int(levels), ctypes.byref(mz), sp, rp, int(device), flags, op, mp, cs, fc, ne))
    res = []
    for i, shp in enumerate(shapes):
        dim = len(shp)
        c = tuple(cs[3 * i:3 * i + dim])
        k = int(np.prod(c)) * dim
        res.append((outs[i][:k].copy(), c, fc[i], ne[i]))
    return res


def register_batch(pairs, rate, levels, mz, device=0, use_graphs=True, **cost_kw):
    """Register many (src, ref) host array pairs at once (sizes may differ;
    one dimension, cost and penalty for all).  Returns a list of
    (params, csize, final_cost, evaluations), one per pair."""
    srcs = [np.ascontiguousarray(s, dtype=np.float32) for s, _ in pairs]
    refs = [np.ascontiguousarray(r, dtype=np.float32) for _, r in pairs]
    for s, r in zip(srcs, refs):
        if s.shape != r.shape:
            raise ValueError("source and reference of a pair differ in shape")
    return _batch([s.shape for s in srcs], [s.ctypes.data for s in srcs], [r.ctypes.data for r in refs], False,
                  rate, levels, mz, device, use_graphs, cost_kw)


def register_batch_device(pairs, rate, levels, mz, device=0, use_graphs=True, **cost_kw):
    """register_batch for pairs of contiguous float32 CUDA tensors (any
    object with .shape, .data_ptr(), .is_contiguous() and .dtype)."""
    for s, r in pairs:
        if tuple(s.shape) != tuple(r.shape) or not (s.is_contiguous() and r.is_contiguous()):
            raise ValueError("pairs must be contiguous tensors of equal shape")
        if str(s.dtype) != "torch.float32" or str(r.dtype) != "torch.float32":
            raise ValueError("pairs must be float32")
    return _batch([tuple(s.shape) for s, _ in pairs], [s.data_ptr() for s, _ in pairs],
                  [r.data_ptr() for _, r in pairs], True, rate, levels, mz, device, use_graphs, cost_kw)
