"""ctypes front end of the CPU oracle (``oracle/liborc.so``).

TEST INFRASTRUCTURE ONLY: the tests use it as the checker of the CUDA path
and ``bench.py`` times it as the CPU baseline.  The product package never
imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liborc.so")

PREC_REF, PREC_F64 = 0, 1
COST_SSD, COST_NCC = 0, 1

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


class LevelDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("size", ctypes.c_int * 3),
        ("csize", ctypes.c_int * 3),
        ("rate", ctypes.c_float * 3),
        ("cost", ctypes.c_int),
        ("ssd_norm", ctypes.c_int),
        ("cost_weight", ctypes.c_double),
        ("has_penalty", ctypes.c_int),
        ("pen_weight", ctypes.c_double),
        ("pen_div", ctypes.c_double),
        ("pen_curl", ctypes.c_double),
        ("pen_norm", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("threads", ctypes.c_int),
    ]


def build(force=False):
    """Compile liborc.so with the committed Makefile (gcc only)."""
    src = os.path.join(_HERE, "mgr_oracle.cc")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        L.orc_fastfloor.restype = ctypes.c_int
        L.orc_fastfloor.argtypes = [ctypes.c_double]
        L.orc_bspline3_weights.argtypes = [ctypes.c_double, _dp]
        L.orc_bspline3_dweights.argtypes = [ctypes.c_double, _dp]
        L.orc_bspline3_deriv_weights.argtypes = [ctypes.c_double, ctypes.c_int, _dp]
        L.orc_bspline3_at.restype = ctypes.c_double
        L.orc_bspline3_at.argtypes = [ctypes.c_double, ctypes.c_int]
        L.orc_mirror_fold.restype = ctypes.c_int
        L.orc_mirror_fold.argtypes = [ctypes.c_int, ctypes.c_int]
        L.orc_filter_line.argtypes = [_dp, ctypes.c_int]
        L.orc_prefilter.argtypes = [_fp, _fp, ctypes.c_int, _ip]
        L.orc_prefilter_vec_d.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int, _ip]
        L.orc_simpson_integrate2.restype = ctypes.c_double
        L.orc_simpson_integrate2.argtypes = [ctypes.c_double] * 2 + [ctypes.c_int] * 2 + [ctypes.c_double] * 2
        L.orc_gradient.argtypes = [_fp, _fp, ctypes.c_int, _ip]
        L.orc_ssd_value.restype = ctypes.c_double
        L.orc_ssd_value.argtypes = [_fp, _fp, ctypes.c_size_t, ctypes.c_int]
        L.orc_ssd_force.restype = ctypes.c_double
        L.orc_ssd_force.argtypes = [_fp, _fp, _fp, ctypes.c_int, _ip, ctypes.c_int]
        L.orc_ncc_value.restype = ctypes.c_double
        L.orc_ncc_value.argtypes = [_fp, _fp, ctypes.c_size_t]
        L.orc_ncc_force.restype = ctypes.c_double
        L.orc_ncc_force.argtypes = [_fp, _fp, _fp, ctypes.c_int, _ip]
        L.orc_ncc_sums.argtypes = [_fp, _fp, ctypes.c_size_t, _dp]
        L.orc_divcurl_matrix.restype = ctypes.c_double
        L.orc_divcurl_matrix.argtypes = [ctypes.c_int, _ip, _fp, ctypes.c_double, ctypes.c_double,
                                         _dp, _dp, ctypes.c_int, ctypes.c_int]
        L.orc_level_create.restype = ctypes.c_void_p
        L.orc_level_create.argtypes = [ctypes.POINTER(LevelDesc)]
        L.orc_level_destroy.argtypes = [ctypes.c_void_p]
        L.orc_level_csize.restype = ctypes.c_int
        L.orc_level_csize.argtypes = [ctypes.c_void_p, _ip]
        L.orc_level_set_images.argtypes = [ctypes.c_void_p, _fp, _fp]
        L.orc_level_evaluate.restype = ctypes.c_double
        L.orc_level_evaluate.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.orc_level_value.restype = ctypes.c_double
        L.orc_level_value.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        for name in ("orc_level_warp", "orc_level_displacement", "orc_level_force"):
            getattr(L, name).argtypes = [ctypes.c_void_p, _dp, _fp]
        L.orc_level_translate.argtypes = [ctypes.c_void_p, _fp, _dp]
        _lib = L
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _size3(shape_xyz):
    s = list(shape_xyz) + [1] * (3 - len(shape_xyz))
    return (ctypes.c_int * 3)(*s)


def fastfloor(x):
    return lib().orc_fastfloor(float(x))


def bspline3_weights(x):
    w = np.zeros(4)
    lib().orc_bspline3_weights(float(x), w.ctypes.data_as(_dp))
    return w


def bspline3_dweights(x):
    w = np.zeros(4)
    lib().orc_bspline3_dweights(float(x), w.ctypes.data_as(_dp))
    return w


def bspline3_deriv_weights(x, degree):
    w = np.zeros(4)
    lib().orc_bspline3_deriv_weights(float(x), int(degree), w.ctypes.data_as(_dp))
    return w


def bspline3_at(x, degree=0):
    return lib().orc_bspline3_at(float(x), int(degree))


def mirror_fold(i, width):
    return lib().orc_mirror_fold(int(i), int(width))


def filter_line(c):
    c = _d(c).copy()
    lib().orc_filter_line(c.ctypes.data_as(_dp), len(c))
    return c


def _xyz(img):
    """numpy arrays are indexed [z, y, x] (x fastest); returns (dim, size3)."""
    dim = img.ndim
    return dim, _size3(img.shape[::-1])


def prefilter(img):
    img = _f(img)
    out = np.empty_like(img)
    dim, s = _xyz(img)
    lib().orc_prefilter(img.ctypes.data_as(_fp), out.ctypes.data_as(_fp), dim, s)
    return out


def prefilter_vec(field):
    """prefilter a vector field [..., ncomp] in double (vector-valued
    interpolator coefficients)."""
    field = _d(field)
    out = np.empty_like(field)
    ncomp = field.shape[-1]
    dim = field.ndim - 1
    s = _size3(field.shape[:-1][::-1])
    lib().orc_prefilter_vec_d(field.ctypes.data_as(_dp), out.ctypes.data_as(_dp), ncomp, dim, s)
    return out


def integrate2(s1, s2, d1, d2, x0, L):
    return lib().orc_simpson_integrate2(s1, s2, d1, d2, x0, L)


def gradient(img):
    img = _f(img)
    dim, s = _xyz(img)
    g = np.empty(img.shape + (dim,), np.float32)
    lib().orc_gradient(img.ctypes.data_as(_fp), g.ctypes.data_as(_fp), dim, s)
    return g


def ssd_value(a, b, norm):
    a, b = _f(a), _f(b)
    return lib().orc_ssd_value(a.ctypes.data_as(_fp), b.ctypes.data_as(_fp), a.size, int(norm))


def ssd_force(a, b, norm):
    a, b = _f(a), _f(b)
    dim, s = _xyz(a)
    f = np.empty(a.shape + (dim,), np.float32)
    c = lib().orc_ssd_force(a.ctypes.data_as(_fp), b.ctypes.data_as(_fp), f.ctypes.data_as(_fp), dim, s, int(norm))
    return c, f


def ncc_value(a, b):
    a, b = _f(a), _f(b)
    return lib().orc_ncc_value(a.ctypes.data_as(_fp), b.ctypes.data_as(_fp), a.size)


def ncc_force(a, b):
    a, b = _f(a), _f(b)
    dim, s = _xyz(a)
    f = np.empty(a.shape + (dim,), np.float32)
    c = lib().orc_ncc_force(a.ctypes.data_as(_fp), b.ctypes.data_as(_fp), f.ctypes.data_as(_fp), dim, s)
    return c, f


def ncc_sums(a, b):
    a, b = _f(a), _f(b)
    s = np.zeros(6)
    lib().orc_ncc_sums(a.ctypes.data_as(_fp), b.ctypes.data_as(_fp), a.size, s.ctypes.data_as(_dp))
    return s


def divcurl_matrix(coeffs, range_xyz, wdiv, wrot, with_grad=True, as_float=True, mode=0):
    """coeffs: array [.., dim] on the coefficient grid ([z,y,x,3] or [y,x,2])."""
    coeffs = _d(coeffs)
    dim = coeffs.shape[-1]
    cs = _size3(coeffs.shape[:-1][::-1])
    rng = (ctypes.c_float * 3)(*(list(range_xyz) + [1.0] * (3 - len(range_xyz))))
    g = np.zeros(coeffs.shape) if with_grad else None
    v = lib().orc_divcurl_matrix(dim, cs, rng, wdiv, wrot, coeffs.ctypes.data_as(_dp),
                                 g.ctypes.data_as(_dp) if g is not None else None, int(as_float), int(mode))
    return (v, g) if with_grad else v


class Level:
    """One registration level: spline transform + image full cost + divcurl
    penalty, as evaluated by TNonrigRegGradientProblem::evaluate_fdf."""

    def __init__(self, size_xyz, rate=None, csize=None, cost="ssd", ssd_norm=False, cost_weight=1.0,
                 penalty_weight=None, div=1.0, curl=1.0, penalty_norm=False, precision=PREC_REF, threads=1):
        d = LevelDesc()
        d.dim = len(size_xyz)
        d.size = _size3(size_xyz)
        d.csize = _size3(csize if csize is not None else [0] * d.dim)
        r = rate if rate is not None else [1.0] * d.dim
        if not hasattr(r, "__len__"):
            r = [r] * d.dim
        d.rate = (ctypes.c_float * 3)(*(list(r) + [1.0] * (3 - len(r))))
        d.cost = COST_NCC if cost == "ncc" else COST_SSD
        d.ssd_norm = int(ssd_norm)
        d.cost_weight = cost_weight
        d.has_penalty = int(penalty_weight is not None)
        d.pen_weight = penalty_weight or 0.0
        d.pen_div, d.pen_curl, d.pen_norm = div, curl, int(penalty_norm)
        d.precision = precision
        d.threads = threads
        self.desc = d
        self.dim = d.dim
        self.size = tuple(size_xyz)
        self.h = lib().orc_level_create(ctypes.byref(d))
        cs = (ctypes.c_int * 3)()
        self.nparams = lib().orc_level_csize(self.h, cs)
        self.csize = tuple(cs[: self.dim])

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_level_destroy(self.h)
            self.h = None

    @property
    def shape(self):
        return tuple(self.size[::-1])

    def set_images(self, src, ref):
        self._src, self._ref = _f(src), _f(ref)
        lib().orc_level_set_images(self.h, self._src.ctypes.data_as(_fp), self._ref.ctypes.data_as(_fp))

    def evaluate(self, params):
        p = _d(params)
        gi = np.zeros(self.nparams)
        gp = np.zeros(self.nparams)
        ci, cp = ctypes.c_double(), ctypes.c_double()
        lib().orc_level_evaluate(self.h, p.ctypes.data_as(_dp), gi.ctypes.data_as(_dp), gp.ctypes.data_as(_dp),
                                 ctypes.byref(ci), ctypes.byref(cp))
        return ci.value, cp.value, gi, gp

    def value(self, params):
        p = _d(params)
        ci, cp = ctypes.c_double(), ctypes.c_double()
        lib().orc_level_value(self.h, p.ctypes.data_as(_dp), ctypes.byref(ci), ctypes.byref(cp))
        return ci.value, cp.value

    def warp(self, params):
        p = _d(params)
        out = np.empty(self.shape, np.float32)
        lib().orc_level_warp(self.h, p.ctypes.data_as(_dp), out.ctypes.data_as(_fp))
        return out

    def displacement(self, params):
        p = _d(params)
        out = np.empty(self.shape + (self.dim,), np.float32)
        lib().orc_level_displacement(self.h, p.ctypes.data_as(_dp), out.ctypes.data_as(_fp))
        return out

    def force(self, params):
        p = _d(params)
        out = np.empty(self.shape + (self.dim,), np.float32)
        lib().orc_level_force(self.h, p.ctypes.data_as(_dp), out.ctypes.data_as(_fp))
        return out

    def translate(self, force):
        f = _f(force)
        g = np.zeros(self.nparams)
        lib().orc_level_translate(self.h, f.ctypes.data_as(_fp), g.ctypes.data_as(_dp))
        return g


# ---- registration driver --------------------------------------------------
MIN_GSL_SD, MIN_GDSQ = 0, 1


class Minimizer(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("maxiter", ctypes.c_int),
        ("step", ctypes.c_double),
        ("tol", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("scale", ctypes.c_double),
        ("xtol", ctypes.c_double),
        ("gtol", ctypes.c_double),
        ("ftolr", ctypes.c_double),
        ("min_step", ctypes.c_double),
    ]


def minimizer(kind="gsl", maxiter=100, step=None, tol=0.1, eps=0.01, scale=2.0, xtol=0.0, gtol=0.0, ftolr=0.0,
              min_step=1e-6):
    m = Minimizer()
    m.kind = MIN_GDSQ if kind == "gdsq" else MIN_GSL_SD
    m.maxiter = int(maxiter)
    m.step = float(step if step is not None else 0.1)
    m.tol, m.eps, m.scale = float(tol), float(eps), float(scale)
    m.xtol, m.gtol, m.ftolr, m.min_step = float(xtol), float(gtol), float(ftolr), float(min_step)
    return m


def _drv():
    L = lib()
    if not getattr(L, "_drv_ready", False):
        L.orc_normalize_pair.restype = ctypes.c_int
        L.orc_normalize_pair.argtypes = [_fp, _fp, ctypes.c_size_t, _fp, _fp, _dp, _dp]
        L.orc_scale_image.argtypes = [_fp, ctypes.c_int, _ip, _fp, _ip]
        L.orc_refine.restype = ctypes.c_int
        L.orc_refine.argtypes = [ctypes.c_int, _ip, _ip, _dp, _dp, ctypes.c_size_t]
        L.orc_register.restype = ctypes.c_int
        L.orc_register.argtypes = [ctypes.POINTER(LevelDesc), ctypes.c_int, ctypes.POINTER(Minimizer), _fp, _fp,
                                   _dp, ctypes.c_int, _ip, _dp, _ip]
        L.orc_minimize_test_problem.restype = ctypes.c_double
        L.orc_minimize_test_problem.argtypes = [ctypes.POINTER(Minimizer), _dp, _ip]
        L._drv_ready = True
    return L


def normalize_pair(src, ref):
    s, r = _f(src), _f(ref)
    so, ro = np.empty_like(s), np.empty_like(r)
    m, sg = ctypes.c_double(), ctypes.c_double()
    ok = _drv().orc_normalize_pair(s.ctypes.data_as(_fp), r.ctypes.data_as(_fp), s.size, so.ctypes.data_as(_fp),
                                   ro.ctypes.data_as(_fp), ctypes.byref(m), ctypes.byref(sg))
    return bool(ok), so, ro, m.value, sg.value


def scale_image(img, out_shape):
    img = _f(img)
    out = np.empty(tuple(out_shape), np.float32)
    _drv().orc_scale_image(img.ctypes.data_as(_fp), img.ndim, _size3(img.shape[::-1]), out.ctypes.data_as(_fp),
                           _size3(out.shape[::-1]))
    return out


def refine(dim, nc_old, nc_new, params):
    p = _d(params)
    out = np.empty(int(np.prod(nc_new)) * dim)
    n = _drv().orc_refine(dim, _size3(nc_old), _size3(nc_new), p.ctypes.data_as(_dp), out.ctypes.data_as(_dp),
                          out.size)
    return None if n == 0 else out


def minimize_test_problem(mz, x0=(5.0, 7.0)):
    x = np.array(x0, dtype=np.float64)
    ne = ctypes.c_int()
    f = _drv().orc_minimize_test_problem(ctypes.byref(mz), x.ctypes.data_as(_dp), ctypes.byref(ne))
    return f, x, ne.value


def register(src, ref, rate, levels, mz, cost="ssd", penalty_weight=None, div=1.0, curl=1.0, ssd_norm=False,
             cost_weight=1.0, penalty_norm=False, threads=1, precision=PREC_REF):
    """TNonrigidRegisterImpl::run: returns (params, csize, final_cost, evaluations);
    `precision` PREC_F64 runs every evaluation in double"""
    s, r = _f(src), _f(ref)
    d = LevelDesc()
    d.dim = s.ndim
    d.size = _size3(s.shape[::-1])
    d.csize = _size3([0] * d.dim)
    rr = rate if hasattr(rate, "__len__") else [rate] * d.dim
    d.rate = (ctypes.c_float * 3)(*(list(rr) + [1.0] * (3 - len(rr))))
    d.cost = COST_NCC if cost == "ncc" else COST_SSD
    d.ssd_norm, d.cost_weight = int(ssd_norm), cost_weight
    d.has_penalty = int(penalty_weight is not None)
    d.pen_weight = penalty_weight or 0.0
    d.pen_div, d.pen_curl, d.pen_norm = div, curl, int(penalty_norm)
    d.precision, d.threads = precision, threads
    maxp = 1 << 24
    out = np.empty(maxp)
    cs = (ctypes.c_int * 3)()
    fc, ne = ctypes.c_double(), ctypes.c_int()
    n = _drv().orc_register(ctypes.byref(d), int(levels), ctypes.byref(mz), s.ctypes.data_as(_fp),
                            r.ctypes.data_as(_fp), out.ctypes.data_as(_dp), maxp, cs, ctypes.byref(fc),
                            ctypes.byref(ne))
    if n < 0:
        raise RuntimeError("orc_register failed")
    return out[:n].copy(), tuple(cs[: d.dim]), fc.value, ne.value
