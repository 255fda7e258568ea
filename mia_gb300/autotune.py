"""Tile-shape autotuner for the split evaluation path.

Run on the target GPU (one GB300):

    python -m mia_gb300.autotune            # writes mia_gb300/tiles.json

For each tuning case (an image size, spline rate and cost that the
registration workloads produce) every tile shape compiled into libmgr is
timed: one cost+gradient evaluation (warp, adjoint, gather + penalty) with
the parameters resident on the device, the L2 flushed before each of
`--reps` timed evaluations, CUDA events on the level's stream around the
whole evaluation (its kernels overlapped as in use); the median counts.  The fastest shape of each case goes into tiles.json, which the
build turns into the table the library consults when it picks a level's
tile (the case nearest in coefficient spacing and image size; a shape whose
shared memory does not fit falls back to the fit rule).  The file records
the times of every shape, the device and the date, so a later run can be
compared with it.
"""
import argparse
import datetime
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "tiles.json")

# image size (x, y[, z]), rate, cost: the 3D eval benchmark workloads, the
# levels of the 3D cohort (full, 1/2, 1/4 of ~160x176x144), denser and
# coarser grids, 2D perfusion frames (series sizes) and large slices
CASES = [
    dict(size=(192, 192, 128), rate=8.0, cost="ssd"),
    dict(size=(256, 256, 256), rate=5.0, cost="ncc"),
    dict(size=(256, 256, 256), rate=8.0, cost="ncc"),
    dict(size=(160, 176, 144), rate=8.0, cost="ncc"),
    dict(size=(80, 88, 72), rate=8.0, cost="ncc"),
    dict(size=(40, 44, 36), rate=8.0, cost="ncc"),
    dict(size=(128, 128, 128), rate=4.0, cost="ssd"),
    dict(size=(192, 192, 192), rate=16.0, cost="ssd"),
    dict(size=(192, 160), rate=16.0, cost="ssd"),
    dict(size=(128, 112), rate=16.0, cost="ssd"),
    dict(size=(96, 96), rate=16.0, cost="ssd"),
    dict(size=(512, 512), rate=8.0, cost="ssd"),
    dict(size=(1024, 1024), rate=16.0, cost="ssd"),
]
TILES3 = [(32, 8, 32), (32, 8, 24), (32, 8, 20), (32, 8, 16), (32, 8, 12), (32, 8, 8), (32, 8, 4)]
TILES2 = [(32, 8, 1), (32, 16, 1), (64, 8, 1), (64, 16, 1), (32, 32, 1)]


def spacing(size, csize):
    """mean voxels per coefficient interval (the grid has a 3-coefficient border)"""
    return float(np.mean([(n - 1) / max(c - 3, 1) for n, c in zip(size, csize)]))


def time_case(case, reps, warmup):
    import torch

    import mia_gb300 as M
    from mia_gb300 import synth
    size = case["size"]
    shape = size[::-1]
    ref = synth.blob_phantom(shape, 10, sigma=(3.0, 8.0), seed=11)
    mov = np.roll(ref, 2, axis=len(shape) - 1).astype(np.float32)
    lv = M.Level(size, rate=case["rate"], cost=case["cost"], penalty_weight=5.0)
    lv.set_images(mov, ref)
    dim = len(size)
    p = synth.smooth_params(lv.csize, 1.5, seed=5)
    dev = torch.device("cuda", 0)
    p_d = torch.from_numpy(np.ascontiguousarray(p, dtype=np.float64)).to(dev)
    g_d = torch.empty(lv.nparams, dtype=torch.float64, device=dev)
    c_d = torch.empty(2, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    lv.set_timing(True, whole=True)   # events around the whole evaluation, launches overlapped as in use
    times = {}
    for tile in (TILES3 if dim == 3 else TILES2):
        try:
            lv.set_path("split", tile)
        except Exception as e:   # shared memory of this shape does not fit the spacing
            times["x".join(map(str, tile[:dim]))] = None
            print("  %s: not usable (%s)" % (tile, str(e).splitlines()[0][:60]), flush=True)
            continue
        try:
            for _ in range(warmup):
                lv.evaluate_device(p_d.data_ptr(), g_d.data_ptr(), c_d.data_ptr())
            lv.sync()
            per = []
            for _ in range(reps):
                flush.zero_()
                torch.cuda.synchronize()
                lv.evaluate_device(p_d.data_ptr(), g_d.data_ptr(), c_d.data_ptr())
                lv.sync()
                per.append(float(lv.kernel_times()[3]) * 1e3)
        except Exception as e:   # a launch the shape's shared memory does not allow
            times["x".join(map(str, tile[:dim]))] = None
            print("  %s: launch refused (%s)" % (tile, str(e).splitlines()[0][:60]), flush=True)
            continue
        times["x".join(map(str, tile[:dim]))] = float(np.median(per))
        print("  %s: %.1f us" % (tile, times["x".join(map(str, tile[:dim]))]), flush=True)
    entry = dict(dim=dim, size=list(size), rate=case["rate"], cost=case["cost"], csize=list(lv.csize),
                 spacing=spacing(size, lv.csize), voxels=int(np.prod(size)), times_us=times)
    best = min((k for k, v in times.items() if v is not None), key=lambda k: times[k])
    t = [int(v) for v in best.split("x")]
    entry["tile"] = t + [1] * (3 - len(t))
    lv.close()
    return entry


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=15)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--out", default=OUT)
    args = ap.parse_args()
    import torch
    from mia_gb300 import build as B
    B.build()
    entries = []
    for case in CASES:
        print("case", case, flush=True)
        entries.append(time_case(case, args.reps, args.warmup))
    doc = {
        "generated_by": "python -m mia_gb300.autotune --reps %d --warmup %d" % (args.reps, args.warmup),
        "device": torch.cuda.get_device_name(0),
        "date": datetime.date.today().isoformat(),
        "metric": "median cost+gradient evaluation time (CUDA events around the whole evaluation), L2 flushed, us",
        "entries": entries,
    }
    with open(args.out, "w") as f:
        json.dump(doc, f, indent=1)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
