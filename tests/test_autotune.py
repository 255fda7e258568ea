"""The committed autotuner table (mia_gb300/tiles.json, written by
`python -m mia_gb300.autotune` on a GB300) and the library's use of it."""
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TILES = os.path.join(ROOT, "mia_gb300", "tiles.json")
COMPILED3 = {(32, 8, 32), (32, 8, 24), (32, 8, 20), (32, 8, 16), (32, 8, 12), (32, 8, 8), (32, 8, 4)}
COMPILED2 = {(32, 8, 1), (32, 16, 1), (64, 8, 1), (64, 16, 1), (32, 32, 1)}


def _doc():
    with open(TILES) as f:
        return json.load(f)


def test_table_entries_are_measured_compiled_shapes():
    doc = _doc()
    assert doc["entries"] and "GB300" in doc["device"]
    for e in doc["entries"]:
        tile = tuple(e["tile"])
        assert tile in (COMPILED3 if e["dim"] == 3 else COMPILED2)
        times = {k: v for k, v in e["times_us"].items() if v is not None}
        # the chosen shape is the fastest one measured
        assert "x".join(map(str, tile[:e["dim"]])) == min(times, key=times.get)
        assert e["voxels"] == int(__import__("numpy").prod(e["size"]))


def test_table_covers_the_benchmark_workloads():
    sizes = {tuple(e["size"]) for e in _doc()["entries"]}
    assert (192, 192, 128) in sizes and (256, 256, 256) in sizes
    assert (160, 176, 144) in sizes and (192, 160) in sizes


def test_build_writes_the_table_for_the_library():
    from mia_gb300 import build as B
    B.write_tile_table()
    text = open(B.TILE_TABLE).read()
    assert len([ln for ln in text.splitlines() if ln.startswith("{")]) == len(_doc()["entries"])


@pytest.mark.gpu
def test_levels_take_the_tuned_tile():
    import mia_gb300 as M
    for e in _doc()["entries"]:
        lv = M.Level(tuple(e["size"]), rate=e["rate"], cost=e["cost"], penalty_weight=5.0)
        assert lv.tile == tuple(e["tile"]), (e["size"], lv.tile, e["tile"])
        lv.close()
