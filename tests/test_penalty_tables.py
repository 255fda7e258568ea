"""The product's divcurl penalty tables against the oracle's (CPU).

mia_gb300/csrc/tables.cc builds the P tables of the divcurl penalty from the
energy's definition (tensor products of per-axis overlap integrals and a
term list derived from grad(div u) and grad(curl u)); the oracle restates
the reference's C3DPPDivcurlMatrixImpl / C2DPPDivcurlMatrixImpl::reset
(mia/3d/ppmatrix.cc:175-290, mia/2d/ppmatrix.cc:182-243).  Both run in
double; the tables must agree to 1e-12 relative, and the 2D cell lists must
have the same structure (rows, columns, order).
"""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
RTOL = 1e-12

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_fp = ctypes.POINTER(ctypes.c_float)


@pytest.fixture(scope="module")
def shim():
    d = tempfile.mkdtemp(prefix="mgr_pen_")
    so = os.path.join(d, "libpenshim.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared", "-o", so,
                           os.path.join(HERE, "penalty_tables_shim.cc"),
                           os.path.join(ROOT, "mia_gb300", "csrc", "tables.cc")])
    L = ctypes.CDLL(so)
    L.shim_penalty3.argtypes = [_ip, _fp, ctypes.c_double, ctypes.c_double, _dp]
    L.shim_penalty2.restype = ctypes.c_size_t
    L.shim_penalty2.argtypes = [_ip, _fp, ctypes.c_double, ctypes.c_double, _ip, _ip, _dp, ctypes.c_size_t]
    return L


def _oracle_lib():
    L = O.lib()
    L.orc_divcurl_table3.argtypes = [_ip, _fp, ctypes.c_double, ctypes.c_double, _dp]
    L.orc_divcurl_cells2.restype = ctypes.c_size_t
    L.orc_divcurl_cells2.argtypes = [_ip, _fp, ctypes.c_double, ctypes.c_double, _ip, _ip, _dp, ctypes.c_size_t]
    return L


def _p(a, t):
    return a.ctypes.data_as(t)


CASES3 = [
    ((26, 26, 18), (192.0, 192.0, 128.0), 1.0, 1.0),    # 192x192x128 at rate 8
    ((54, 54, 54), (256.0, 256.0, 256.0), 1.0, 1.0),    # 256^3 at rate 5
    ((26, 26, 18), (192.0, 192.0, 128.0), 2.0, 0.5),    # div != curl: cross entries
    ((7, 9, 5), (20.0, 33.0, 9.0), 0.3, 1.7),           # anisotropic spacing
    ((4, 4, 4), (2.0, 3.0, 4.0), 1.0, 0.0),             # smallest grid, div only
]


@pytest.mark.parametrize("csize,rng,wd,wr", CASES3)
def test_penalty3_cells_match_oracle(shim, csize, rng, wd, wr):
    cs = np.array(csize, dtype=np.int32)
    r = np.array(rng, dtype=np.float32)
    got = np.zeros(729 * 6)
    want = np.zeros(729 * 6)
    shim.shim_penalty3(_p(cs, _ip), _p(r, _fp), wd, wr, _p(got, _dp))
    _oracle_lib().orc_divcurl_table3(_p(cs, _ip), _p(r, _fp), wd, wr, _p(want, _dp))
    got = got.reshape(9, 9, 9, 6)
    # the oracle's cell index runs x fastest as (x + 9 (y + 9 z)): the same
    want = want.reshape(9, 9, 9, 6)
    scale = np.abs(want).max()
    assert scale > 0
    assert np.abs(got - want).max() <= RTOL * scale
    big = np.abs(want) > 1e-6 * scale
    assert np.all(np.abs(got - want)[big] <= 1e-11 * np.abs(want)[big])
    # the table is an even function of the offset (reflection symmetry)
    assert np.allclose(got, got[::-1, ::-1, ::-1], rtol=0, atol=1e-13 * scale)


CASES2 = [
    ((10, 10), (128.0, 128.0), 1.0, 1.0),     # 128x128 at rate 16
    ((8, 7), (96.0, 80.0), 1.0, 1.0),         # series frame, coarse level
    ((14, 12), (192.0, 160.0), 1.0, 1.0),     # series frame after refine
    ((4, 4), (4.0, 4.0), 2.0, 0.5),           # smallest grid: every integral clipped
    ((9, 5), (40.0, 17.0), 0.25, 3.0),        # anisotropic, curl dominant
]


@pytest.mark.parametrize("csize,rng,wd,wr", CASES2)
def test_penalty2_cells_match_oracle(shim, csize, rng, wd, wr):
    cs = np.array(csize, dtype=np.int32)
    r = np.array(rng, dtype=np.float32)
    n = csize[0] * csize[1]
    cap = n * 64
    rowptr = np.zeros(n + 1, dtype=np.int32)
    col = np.zeros(cap, dtype=np.int32)
    val = np.zeros(cap * 3)
    m = shim.shim_penalty2(_p(cs, _ip), _p(r, _fp), wd, wr, _p(rowptr, _ip), _p(col, _ip), _p(val, _dp), cap)
    oi = np.zeros(cap, dtype=np.int32)
    oj = np.zeros(cap, dtype=np.int32)
    ov = np.zeros(cap * 3)
    mo = _oracle_lib().orc_divcurl_cells2(_p(cs, _ip), _p(r, _fp), wd, wr, _p(oi, _ip), _p(oj, _ip),
                                          _p(ov, _dp), cap)
    assert m == mo and m > 0
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    assert np.array_equal(rows, oi[:m])
    assert np.array_equal(col[:m], oj[:m])
    got, want = val[:3 * m], ov[:3 * m]
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= RTOL * scale
    big = np.abs(want) > 1e-6 * scale
    assert np.all(np.abs(got - want)[big] <= 1e-11 * np.abs(want)[big])
