"""The MIA-side adapter of INTEGRATION.md over the registration driver's
level loop, as a C++ program built with g++ against include/mgr.h only
(tests/adapter/level_loop.cc): three 3D levels (NCC) and two 2D levels
(SSD), each with the transformation upscaled on its old grid and refined
within the level.  Every evaluation through the adapter must equal one on
a level created afresh for the transformation's current grid."""
import os
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def program():
    from mia_gb300 import _lib
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = os.path.join(tempfile.mkdtemp(prefix="mgr_adapter_"), "level_loop")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "adapter", "level_loop.cc"), "-L", libdir, "-lmgr",
                           "-Wl,-rpath," + libdir, "-o", exe])
    return exe


@pytest.mark.parametrize("dim", [3, 2])
def test_adapter_follows_the_grid_through_upscale_and_refine(program, dim):
    r = subprocess.run([program, str(dim)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=600)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr
    out = r.stdout.split()
    assert out[0] == "ok"
    fields = dict(f.split("=") for f in out[1:] if "=" in f)
    assert int(fields["refines"]) >= 1 and int(fields["grids"]) >= 3 - (dim == 2)
