"""Save / load of a spline transformation (the reference's transformation IO,
mia/3d/transio/{xml,serialization}: creator, size, attributes, parameters;
its test mia/3d/test_transio.cc checks that a round trip keeps the size, the
creator string, every parameter and a string attribute)."""
import os

import numpy as np
import pytest


@pytest.mark.parametrize("size,csize", [((20, 22, 23), (7, 8, 9)), ((192, 192, 128), (26, 26, 18)),
                                        ((96, 80), (8, 7))])
def test_round_trip_keeps_size_creator_parameters_and_attributes(tmp_path, size, csize):
    from mia_gb300 import registration as R
    dim = len(size)
    n = int(np.prod(csize)) * dim
    rng = np.random.default_rng(n)
    p = rng.standard_normal(n) * 10.0 ** rng.integers(-8, 8, n)   # values across many magnitudes
    p[0], p[1] = -0.0, 1.0 / 3.0
    f = tmp_path / ("t.x%ddt" % dim)
    R.save_transform(f, size, csize, p, rate=8, attributes={"string_attr": "string", "odd&<name>": 'q"\'v'})
    t = R.load_transform(f)
    assert t["dim"] == dim and t["size"] == tuple(size) and t["csize"] == tuple(csize)
    assert t["creator"] == "spline:rate=8"
    assert t["attributes"] == {"string_attr": "string", "odd&<name>": 'q"\'v'}
    assert t["params"].tobytes() == p.tobytes()   # bit for bit, the sign of zero included


def test_archive_layout(tmp_path):
    """the fields in the order and the layout of the reference's archive"""
    from mia_gb300 import registration as R
    f = tmp_path / "t.x3dt"
    R.save_transform(f, (20, 22, 23), (4, 4, 4), np.arange(1, 4 * 4 * 4 * 3 + 1, dtype=float), creator="spline:rate=6")
    text = f.read_text()
    order = [text.index(tag) for tag in ("<boost_serialization", "<creator>", "<size_x>", "<size_y>", "<size_z>",
                                         "<attributes", "<params>", "</boost_serialization>")]
    assert order == sorted(order)
    assert "<creator>spline:rate=6</creator>" in text
    assert "<count>192</count>" in text and "<item>192</item>" in text


def test_load_rejects_what_is_not_an_archive(tmp_path):
    from mia_gb300 import _lib
    from mia_gb300 import registration as R
    bad = tmp_path / "bad.x3dt"
    bad.write_text("not xml at all")
    with pytest.raises(_lib.MgrError) as e:
        R.load_transform(bad)
    assert e.value.status == _lib.MGR_ERR_ARG
    with pytest.raises(_lib.MgrError):
        R.load_transform(tmp_path / "missing.x3dt")


def test_save_rejects_a_parameter_count_that_does_not_match_the_grid(tmp_path):
    from mia_gb300 import _lib
    from mia_gb300 import registration as R
    with pytest.raises(_lib.MgrError) as e:
        R.save_transform(tmp_path / "t.x3dt", (20, 22, 23), (4, 4, 4), np.zeros(10))
    assert e.value.status == _lib.MGR_ERR_ARG
    assert not os.path.exists(tmp_path / "t.x3dt")


def test_load_refuses_string_buffers_too_small(tmp_path):
    """strings are returned whole: a buffer too small is an error naming the size needed"""
    import ctypes
    from mia_gb300 import _lib
    from mia_gb300 import registration as R
    f = tmp_path / "t.x2dt"
    R.save_transform(f, (20, 18), (5, 5), np.zeros(50), rate=6, attributes={"a": "x" * 40})
    dim, n = ctypes.c_int(), ctypes.c_size_t()
    sz, cs = (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
    small = ctypes.create_string_buffer(8)
    st = _lib.lib().mgr_transform_load(str(f).encode(), ctypes.byref(dim), sz, cs, small, len(small), None, 0,
                                       None, 0, ctypes.byref(n))
    assert st == _lib.MGR_ERR_ARG and b"14 bytes needed" in _lib.lib().mgr_last_error()
    st = _lib.lib().mgr_transform_load(str(f).encode(), ctypes.byref(dim), sz, cs, None, 0, small, len(small),
                                       None, 0, ctypes.byref(n))
    assert st == _lib.MGR_ERR_ARG and b"44 bytes needed" in _lib.lib().mgr_last_error()


def test_load_returns_large_attribute_maps(tmp_path):
    from mia_gb300 import registration as R
    f = tmp_path / "t.x3dt"
    attrs = {"k%03d" % i: "v" * 1000 for i in range(100)}   # about 100 KB of attributes
    R.save_transform(f, (20, 18, 16), (5, 5, 5), np.ones(375), creator="spline:rate=" + "9" * 5000,
                     attributes=attrs)
    t = R.load_transform(f)
    assert t["attributes"] == attrs and t["creator"] == "spline:rate=" + "9" * 5000
