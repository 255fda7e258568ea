"""Python front end of one registration level on the GPU.

A ``Level`` owns an ``mgr_level`` of libmgr: the `spline` transformation
(cubic B-spline coefficients), the `image` full cost with the `ssd` or
`ncc` image cost and the optional `divcurl` spline penalty, evaluated as
TNonrigRegGradientProblem::evaluate_fdf does
(mia/template/nonrigidregister.cxx:415-439).  Arrays are numpy, indexed
[z, y, x] (x fastest) like MIA's data fields; parameter vectors are MIA's
interleaved CDoubleVector layout.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _sized(a, n, what):
    """`a` as given, after checking that it holds exactly n values (the C ABI
    reads or writes n elements through the pointer)"""
    if a.size != n:
        raise ValueError(f"{what} must hold {n} values, got {a.size}")
    return a


class Level:
    """One image pair at one resolution level on one GPU.

    size_xyz      image size (x, y[, z])
    rate          spline `rate` (scalar or per axis); ignored with `csize`
    csize         explicit coefficient grid (incl. the 2-coefficient border)
    cost          'ssd' or 'ncc'
    ssd_norm      ssd `norm`
    cost_weight   image full-cost `weight`
    penalty_weight  divcurl `weight` (None: no penalty); div/curl/penalty_norm
    penalty_corrected  the penalty gradient as +weight * gradient instead of
                  the reference's -weight * gradient
    """

    def __init__(self, size_xyz, rate=None, csize=None, cost="ssd", ssd_norm=False, cost_weight=1.0,
                 penalty_weight=None, div=1.0, curl=1.0, penalty_norm=False, penalty_corrected=False, device=0,
                 stream=None):
        d = _lib.LevelDesc()
        d.dim = len(size_xyz)
        d.size = (ctypes.c_int * 3)(*(list(size_xyz) + [1] * (3 - d.dim)))
        d.csize = (ctypes.c_int * 3)(*(list(csize if csize is not None else [0] * d.dim) + [0] * (3 - d.dim)))
        r = rate if rate is not None else 1.0
        if not hasattr(r, "__len__"):
            r = [r] * d.dim
        d.rate = (ctypes.c_float * 3)(*(list(r) + [1.0] * (3 - len(r))))
        d.cost = _lib.COST_NCC if cost == "ncc" else _lib.COST_SSD
        d.ssd_norm = int(ssd_norm)
        d.cost_weight = float(cost_weight)
        d.has_penalty = int(penalty_weight is not None)
        d.pen_weight = float(penalty_weight or 0.0)
        d.pen_div, d.pen_curl, d.pen_norm = float(div), float(curl), int(penalty_norm)
        d.pen_corrected = int(penalty_corrected)
        self.desc = d
        self.dim = d.dim
        self.size = tuple(size_xyz)
        h = ctypes.c_void_p()
        check(lib().mgr_level_create(ctypes.byref(d), int(device), stream, ctypes.byref(h)))
        self.h = h
        cs = (ctypes.c_int * 3)()
        n = ctypes.c_size_t()
        check(lib().mgr_level_csize(self.h, cs, ctypes.byref(n)))
        self.csize = tuple(cs[: self.dim])
        self.nparams = n.value

    def close(self):
        if getattr(self, "h", None):
            lib().mgr_level_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def shape(self):
        return tuple(self.size[::-1])

    def _params(self, params):
        return _sized(_d(params), self.nparams, "params")

    def set_grid(self, csize):
        """a new coefficient grid (x, y[, z]) on the same images"""
        cs = (ctypes.c_int * 3)(*(list(csize) + [1] * (3 - len(csize))))
        check(lib().mgr_level_set_grid(self.h, cs))
        n = ctypes.c_size_t()
        out = (ctypes.c_int * 3)()
        check(lib().mgr_level_csize(self.h, out, ctypes.byref(n)))
        self.csize = tuple(out[: self.dim])
        self.nparams = n.value

    def set_path(self, path="split", tile=(0, 0, 0)):
        p = {"plain": _lib.PATH_PLAIN, "fused": _lib.PATH_FUSED}.get(path, _lib.PATH_SPLIT)
        t = list(tile) + [0] * (3 - len(tile))
        check(lib().mgr_level_set_path(self.h, p, *t))

    @property
    def tile(self):
        """the split path's tile shape (x, y, z)"""
        t = (ctypes.c_int * 3)()
        check(lib().mgr_level_tile(self.h, t))
        return tuple(t)

    @property
    def in_place(self):
        """True when evaluate reads the parameters and writes the gradients
        in the caller's host memory (coherent host access), False when it
        stages them through device buffers"""
        v = ctypes.c_int(0)
        check(lib().mgr_level_host_access(self.h, ctypes.byref(v)))
        return bool(v.value)

    def set_images(self, src, ref):
        s, r = _f(src), _f(ref)
        if s.shape != self.shape or r.shape != self.shape:
            raise ValueError(f"images must have shape {self.shape} ([z, y, x]), got {s.shape} and {r.shape}")
        check(lib().mgr_level_set_images(self.h, s.ctypes.data_as(_fp), r.ctypes.data_as(_fp)))

    def set_images_device(self, src_ptr, ref_ptr):
        check(lib().mgr_level_set_images_device(self.h, ctypes.c_void_p(src_ptr), ctypes.c_void_p(ref_ptr)))

    def evaluate(self, params):
        """(cost_image, cost_penalty, grad_image, grad_penalty, grad_total)"""
        p = self._params(params)
        gt = np.empty(self.nparams)
        gi = np.empty(self.nparams)
        gp = np.empty(self.nparams)
        ci, cp = ctypes.c_double(), ctypes.c_double()
        check(lib().mgr_level_evaluate(self.h, p.ctypes.data_as(_dp), gt.ctypes.data_as(_dp),
                                       gi.ctypes.data_as(_dp), gp.ctypes.data_as(_dp), ctypes.byref(ci),
                                       ctypes.byref(cp)))
        return ci.value, cp.value, gi, gp, gt

    def evaluate_total(self, params, grad_out=None):
        """cost+gradient as evaluate_fdf returns it (total cost, total gradient)."""
        p = self._params(params)
        if grad_out is None:
            g = np.empty(self.nparams)
        else:
            g = grad_out
            if not (isinstance(g, np.ndarray) and g.dtype == np.float64 and g.flags.c_contiguous and g.flags.writeable):
                raise ValueError("grad_out must be a writeable C-contiguous float64 array")
            _sized(g, self.nparams, "grad_out")
        ci, cp = ctypes.c_double(), ctypes.c_double()
        check(lib().mgr_level_evaluate(self.h, p.ctypes.data_as(_dp), g.ctypes.data_as(_dp), None, None,
                                       ctypes.byref(ci), ctypes.byref(cp)))
        return ci.value + cp.value, g

    def bind_evaluate_total(self, params, grad_out):
        """A callable that evaluates at the values `params` holds when it is
        called, writes the total gradient into `grad_out` and returns the
        total cost: one mgr_level_evaluate call with the pointers prepared
        here once (the arrays' contents may change between calls, not the
        arrays), as a C or C++ caller of the ABI makes it."""
        for name, a in (("params", params), ("grad_out", grad_out)):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise ValueError(name + " must be a C-contiguous float64 array")
            _sized(a, self.nparams, name)
        if not grad_out.flags.writeable:
            raise ValueError("grad_out must be writeable")
        fn, h = lib().mgr_level_evaluate, self.h
        pp, gp = params.ctypes.data_as(_dp), grad_out.ctypes.data_as(_dp)
        ci, cp = ctypes.c_double(), ctypes.c_double()
        bci, bcp = ctypes.byref(ci), ctypes.byref(cp)
        keep = (params, grad_out)

        def call():
            st = fn(h, pp, gp, None, None, bci, bcp)
            if st:
                check(st)
            return ci.value + cp.value
        call.keep = keep
        return call

    def evaluate_device(self, params_ptr, grad_ptr, costs_ptr):
        check(lib().mgr_level_evaluate_device(self.h, ctypes.c_void_p(params_ptr), ctypes.c_void_p(grad_ptr),
                                              ctypes.c_void_p(costs_ptr)))

    def value(self, params):
        p = self._params(params)
        ci, cp = ctypes.c_double(), ctypes.c_double()
        check(lib().mgr_level_value(self.h, p.ctypes.data_as(_dp), ctypes.byref(ci), ctypes.byref(cp)))
        return ci.value, cp.value

    def warp(self, params):
        p = self._params(params)
        out = np.empty(self.shape, np.float32)
        check(lib().mgr_level_warp(self.h, p.ctypes.data_as(_dp), out.ctypes.data_as(_fp)))
        return out

    def force(self, params):
        p = self._params(params)
        out = np.empty(self.shape + (self.dim,), np.float32)
        c = ctypes.c_double()
        check(lib().mgr_level_force(self.h, p.ctypes.data_as(_dp), out.ctypes.data_as(_fp), ctypes.byref(c)))
        return c.value, out

    def translate(self, force):
        f = _sized(_f(force), int(np.prod(self.shape)) * self.dim, "force")
        g = np.empty(self.nparams)
        check(lib().mgr_level_translate(self.h, f.ctypes.data_as(_fp), g.ctypes.data_as(_dp)))
        return g

    def set_timing(self, enable=True, whole=False):
        """record CUDA events around every kernel of each evaluation
        (`whole`: around the whole evaluation only, kernels overlapped as
        in untimed runs)"""
        check(lib().mgr_level_set_timing(self.h, (2 if whole else 1) if enable else 0))

    def kernel_times(self):
        """device ms of the last evaluation: (warp, adjoint, gather, total)"""
        ms = (ctypes.c_double * 4)()
        check(lib().mgr_level_kernel_times(self.h, ms))
        return tuple(ms)

    def sync(self):
        check(lib().mgr_level_sync(self.h))
