"""The C ABI library loads, exports every entry point that include/mgr.h
declares, and refuses to run without a GPU (no CPU fallback)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "mgr.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mgr_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_all_declared_symbols():
    from mia_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding declares the same set
    assert set(syms) == set(_lib.SIGNATURES)


def test_no_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import mia_gb300 as M
    with pytest.raises(M.MgrError) as e:
        M.Level((16, 16, 16), rate=4.0)
    assert e.value.status == 2   # MGR_ERR_CUDA


def test_argument_validation_before_gpu():
    import mia_gb300 as M
    for kw in (dict(size=(16, 16, 16), rate=20.0), dict(size=(1, 16, 16), rate=2.0),
               dict(size=(16, 16), rate=0.5)):
        with pytest.raises(M.MgrError) as e:
            M.Level(kw["size"], rate=kw["rate"])
        assert e.value.status == 1   # MGR_ERR_ARG
