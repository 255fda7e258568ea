"""Argument checks of the Python front end that run before any device call:
buffers the C ABI would read past are refused with ValueError."""
import numpy as np
import pytest


def test_pair_shapes_must_match():
    from mia_gb300 import registration as R
    a = np.zeros((8, 9, 10), np.float32)
    b = np.zeros((8, 9, 11), np.float32)
    mz = R.minimizer("gsl", maxiter=1, step=0.1)
    with pytest.raises(ValueError):
        R.register_pair(a, b, 4.0, 1, mz)
    with pytest.raises(ValueError):
        R.normalize_pair(a, b)
    with pytest.raises(ValueError):
        R.register_batch([(a, a), (a, b)], 4.0, 1, mz)


def test_sized_helper():
    from mia_gb300.level import _sized
    a = np.zeros(12)
    assert _sized(a, 12, "x") is a
    with pytest.raises(ValueError, match="x must hold 13 values"):
        _sized(a, 13, "x")


def test_scale_image_rejects_non_positive_sizes():
    import ctypes
    from mia_gb300 import _lib
    a = np.zeros(16, np.float32)
    fp = a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    isz = (ctypes.c_int * 3)(4, 4, 1)
    osz = (ctypes.c_int * 3)(2, 0, 1)
    assert _lib.lib().mgr_scale_image(2, isz, fp, osz, fp, 0) == _lib.MGR_ERR_ARG
    assert b"positive" in _lib.lib().mgr_last_error()


def test_registration_rejects_degenerate_sizes():
    """sizes below 2 are refused before any device call"""
    import ctypes
    from mia_gb300 import _lib
    from mia_gb300 import registration as R
    a = np.zeros(4, np.float32)
    fp = a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    mz = R.minimizer("gsl", maxiter=1)
    d = R.level_desc((4, 1), 2.0)
    out = np.empty(64)
    cs = (ctypes.c_int * 3)()
    st = _lib.lib().mgr_register(ctypes.byref(d), 1, ctypes.byref(mz), fp, fp, _lib.PATH_SPLIT, 0,
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size, cs, None, None)
    assert st == _lib.MGR_ERR_ARG
    assert b">= 2" in _lib.lib().mgr_last_error()


def test_level_methods_refuse_wrong_sizes_before_the_device_call():
    """a Level without a device handle: each method raises ValueError on a
    wrong-size buffer before it would reach the C ABI"""
    from mia_gb300.level import Level
    lv = Level.__new__(Level)
    lv.h, lv.dim, lv.size, lv.nparams = None, 3, (5, 4, 3), 24
    short = np.zeros(23)
    for call in (lambda: lv.evaluate(short), lambda: lv.evaluate_total(short), lambda: lv.value(short),
                 lambda: lv.warp(short), lambda: lv.force(short),
                 lambda: lv.evaluate_total(np.zeros(24), grad_out=np.zeros(23)),
                 lambda: lv.evaluate_total(np.zeros(24), grad_out=np.zeros(24, np.float32)),
                 lambda: lv.evaluate_total(np.zeros(24), grad_out=np.zeros(48)[::2]),
                 lambda: lv.translate(np.zeros((3, 4, 5, 2), np.float32)),
                 lambda: lv.set_images(np.zeros((3, 4, 5)), np.zeros((3, 4, 6)))):
        with pytest.raises(ValueError):
            call()
