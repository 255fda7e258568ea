"""ctypes binding of libmgr.so (the C ABI declared in include/mgr.h).

The library is loaded from this package directory; there is no fallback.
If libmgr.so is missing or cannot be loaded, ``lib()`` raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmgr.so")

MGR_OK, MGR_ERR_ARG, MGR_ERR_CUDA, MGR_ERR_OOM, MGR_ERR_TIMEOUT, MGR_ERR_STATE = range(6)
COST_SSD, COST_NCC = 0, 1
PATH_SPLIT, PATH_PLAIN, PATH_FUSED = 0, 1, 2

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

# every exported entry point of include/mgr.h with (restype, argtypes)
SIGNATURES = {
    "mgr_last_error": (ctypes.c_char_p, []),
    "mgr_kernel_launch_count": (ctypes.c_ulonglong, []),
    "mgr_debug_fail_allocation": (ctypes.c_int, [ctypes.c_longlong]),
    "mgr_allocation_count": (ctypes.c_ulonglong, []),
    "mgr_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                                 ctypes.POINTER(ctypes.c_double)]),
    "mgr_level_create": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.POINTER(_vp)]),
    "mgr_level_destroy": (ctypes.c_int, [_vp]),
    "mgr_level_csize": (ctypes.c_int, [_vp, _ip, ctypes.POINTER(ctypes.c_size_t)]),
    "mgr_level_set_grid": (ctypes.c_int, [_vp, _ip]),
    "mgr_level_set_images": (ctypes.c_int, [_vp, _fp, _fp]),
    "mgr_level_set_images_device": (ctypes.c_int, [_vp, _vp, _vp]),
    "mgr_level_evaluate": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "mgr_level_host_access": (ctypes.c_int, [_vp, _ip]),
    "mgr_level_evaluate_device": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "mgr_level_value": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "mgr_level_warp": (ctypes.c_int, [_vp, _dp, _fp]),
    "mgr_level_force": (ctypes.c_int, [_vp, _dp, _fp, _dp]),
    "mgr_level_translate": (ctypes.c_int, [_vp, _fp, _dp]),
    "mgr_level_set_path": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "mgr_level_set_timing": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mgr_level_kernel_times": (ctypes.c_int, [_vp, _dp]),
    "mgr_level_sync": (ctypes.c_int, [_vp]),
    "mgr_translate3d_noalloc": (ctypes.c_int, [_ip, _ip, _vp, _vp, _vp]),
    "mgr_register": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _fp, _fp, ctypes.c_int, ctypes.c_int, _dp,
                                    ctypes.c_size_t, _ip, _dp, _ip]),
    "mgr_register_batch": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int,
                                          ctypes.c_int, _vp, _vp, _ip, _dp, _ip]),
    "mgr_register_batch_device": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_int, _vp, _vp, _vp, ctypes.c_int,
                                                 ctypes.c_int, _vp, _vp, _ip, _dp, _ip]),
    "mgr_scale_image": (ctypes.c_int, [ctypes.c_int, _ip, _fp, _ip, _fp, ctypes.c_int]),
    "mgr_level_tile": (ctypes.c_int, [_vp, _ip]),
    "mgr_transform_save": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _ip, _ip, ctypes.c_char_p, _dp,
                                          ctypes.c_size_t, ctypes.POINTER(ctypes.c_char_p),
                                          ctypes.POINTER(ctypes.c_char_p), ctypes.c_int]),
    "mgr_transform_load": (ctypes.c_int, [ctypes.c_char_p, _ip, _ip, _ip, ctypes.c_char_p, ctypes.c_size_t,
                                          ctypes.c_char_p, ctypes.c_size_t, _dp, ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_size_t)]),
    "mgr_refine_coefficients": (ctypes.c_int, [ctypes.c_int, _ip, _ip, _dp, _dp, _ip]),
    "mgr_refine_coefficients_device": (ctypes.c_int, [ctypes.c_int, _ip, _ip, _vp, _vp, _ip, _vp]),
    "mgr_normalize_pair": (ctypes.c_int, [_fp, _fp, ctypes.c_size_t, _fp, _fp, _dp, _dp, _ip, ctypes.c_int]),
}


class LevelDesc(ctypes.Structure):
    """mgr_level_desc"""
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
        ("pen_corrected", ctypes.c_int),
    ]


MIN_GSL_SD, MIN_GDSQ = 0, 1


class MinimizerDesc(ctypes.Structure):
    """mgr_minimizer_desc"""
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


def minimizer(kind="gsl", maxiter=100, step=None, tol=0.1, eps=0.01, scale=2.0, xtol=0.0, gtol=0.0,
              ftolr=0.0, min_step=1e-6):
    """gsl:opt=gd (defaults as the plugin, step 0.1 as the CLI) or gdsq"""
    m = MinimizerDesc()
    m.kind = MIN_GDSQ if kind == "gdsq" else MIN_GSL_SD
    m.maxiter = int(maxiter)
    m.step = float(step if step is not None else 0.1)
    m.tol, m.eps, m.scale = float(tol), float(eps), float(scale)
    m.xtol, m.gtol, m.ftolr, m.min_step = float(xtol), float(gtol), float(ftolr), float(min_step)
    return m


class MgrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("mgr status %d: %s" % (status, msg))
        self.status = status


_lib = None


def lib():
    """Load libmgr.so (raises if it is missing: there is no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libmgr.so not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != MGR_OK:
        raise MgrError(status, lib().mgr_last_error().decode())
