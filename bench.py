#!/usr/bin/env python
"""Cost+gradient throughput of the B-spline registration path on GB300.

Workload (default): the 3D single-pair configuration — 192x192x128 float32
blob phantoms (40 blobs, sigma U(4,16), amplitude U(50,200), N(0,2) noise),
the moving volume warped by a random cubic B-spline field (knot spacing 8,
coefficients N(0,2) clipped to +-4), joint mean-0/sigma-1 normalisation as
the registration driver applies it, then repeated evaluations of SSD +
divcurl(weight 10) cost and gradient at fixed coefficients (spline rate 8,
bspline:d=3 interpolation).  A "step" is one cost+gradient evaluation.
The inputs are made on the host (mia_gb300/workloads.py), the same arrays
for every arm.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`value` is device-timed Mvoxel/s with inputs resident in HBM (L2 flushed
between steps, flush excluded); `e2e` is the same metric through the C ABI
with host parameter/gradient buffers (pinned), copies included.  The
default line also carries the 256^3 NCC configuration, the 2D single-pair
registration (128x128, 50 iterations), the 60-frame series and the 16-pair
cohort (pairs/s).  The reference arm times the CPU restatement of the
reference algorithm (the oracle; the reference itself cannot be built
here) on all host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from mia_gb300 import workloads as WL  # noqa: E402  (host-only input synthesis)

METRIC = "cost+grad Mvoxel/s (3D SSD/NCC) & batched pairs/s vs plain GPU, grad err ≤1e-4"

WORKLOADS = WL.WORKLOADS
BATCH_WORKLOADS = WL.BATCH_WORKLOADS


def dist_env():
    from mia_gb300 import replicas
    return replicas.env()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel):
    """per-launch DRAM bytes of `kernel` from the committed ncu summary"""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        v = d.get(kernel)
        if v:
            return float(v["bytes_per_launch"])
    return None


def profile_metric(kernel, key):
    """a per-launch figure of `kernel` from the committed ncu summary"""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            v = json.load(f).get(kernel)
        if v and key in v:
            return float(v[key])
    return None


def cpu_baseline(w, mov, ref, params, seconds, threads):
    from oracle import oracle as O
    size = w["size"]
    lv = O.Level(size, rate=w["rate"], cost=w["cost"], penalty_weight=w["penalty"], threads=threads)
    lv.set_images(mov, ref)
    n = 0
    t0 = time.perf_counter()
    res = None
    while True:
        res = lv.evaluate(params)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    N = int(np.prod(size))
    return N * n / dt / 1e6, n, dt, res


def time_evals(lv, p_d, g_d, c_d, flush, steps, warmup=2, per_kernel=False):
    """device ms of one cost+gradient evaluation (the level's own events
    around the whole evaluation, L2 flushed before each), mean over `steps`;
    per_kernel: the mean (warp, adjoint, gather, total) with events around
    every kernel (the kernels then run one after another)"""
    import torch
    lv.set_timing(True, whole=not per_kernel)
    for _ in range(warmup):
        lv.evaluate_device(p_d.data_ptr(), g_d.data_ptr(), c_d.data_ptr())
    lv.sync()
    per = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        lv.evaluate_device(p_d.data_ptr(), g_d.data_ptr(), c_d.data_ptr())
        lv.sync()
        per.append(lv.kernel_times())
    per = np.array(per)
    return tuple(float(v) for v in per.mean(axis=0)) if per_kernel else float(per[:, 3].mean())


def split_vs_plain(lv, p_d, g_d, c_d, flush, steps, N):
    """the split (fused forward + adjoint) kernels against the plain
    separate init_grid / warp / force / translate kernels, same GPU, same
    inputs"""
    t_split = time_evals(lv, p_d, g_d, c_d, flush, steps)
    lv.set_path("plain")
    t_plain = time_evals(lv, p_d, g_d, c_d, flush, steps)
    lv.set_path("split")
    return {"split_ms": t_split, "plain_ms": t_plain, "plain_value": N / t_plain / 1e3, "unit": "Mvoxel/s",
            "speedup_split_vs_plain": t_plain / t_split}


def fused_vs_split(lv, p_d, g_d, c_d, flush, steps, N, params, tz=16):
    """the fused SSD kernel (warp, force and adjoint in one pass per tile,
    MGR_PATH_FUSED) against the split kernels, same GPU, same inputs: device
    ms per evaluation and the fused result's difference from the split one"""
    t_split = time_evals(lv, p_d, g_d, c_d, flush, steps)
    k_split = time_evals(lv, p_d, g_d, c_d, flush, steps, per_kernel=True)
    ref = lv.evaluate(params)
    lv.set_path("fused", (0, 0, tz))
    t_fused = time_evals(lv, p_d, g_d, c_d, flush, steps)
    k_fused = time_evals(lv, p_d, g_d, c_d, flush, steps, per_kernel=True)
    got = lv.evaluate(params)
    lv.set_path("split")
    return {"split_ms": t_split, "fused_ms": t_fused, "speedup_fused_vs_split": t_split / t_fused,
            "fused_value": N / t_fused / 1e3, "unit": "Mvoxel/s", "fused_tile": [30, 8, tz],
            "kernel_ms_split": {"warp": k_split[0], "adjoint": k_split[1], "gather_penalty": k_split[2]},
            "kernel_ms_fused": {"fused": k_fused[0], "gather_penalty": k_fused[2]},
            "fused_vs_split_cost_rel": abs(got[0] - ref[0]) / abs(ref[0]),
            "fused_vs_split_grad_rel_l2": float(np.linalg.norm(got[2] - ref[2]) / np.linalg.norm(ref[2])),
            "kept": "split" if t_split <= t_fused else "fused"}


def fd_check(w, mov, ref, params, lv, ref_grads, threads, ncoef=64, h=1e-3, seed=7):
    """the gradient against FP64 central finite differences of the FP64
    oracle's total cost on `ncoef` random coefficients; the reference's own
    gradient (the oracle at reference precision) against the same
    differences for comparison: the reference's image gradient takes the
    warped image's derivative by central differences, so neither equals FD
    exactly"""
    from oracle import oracle as O
    o64 = O.Level(w["size"], rate=w["rate"], cost=w["cost"], penalty_weight=w["penalty"], precision=O.PREC_F64,
                  threads=threads)
    o64.set_images(mov, ref)
    _, _, gi, gp, _ = lv.evaluate(params)
    d_gpu = gi - gp   # the penalty gradient carries the reference's sign (-weight * gradient)
    ogi, ogp = ref_grads
    d_ref = ogi - ogp
    idx = np.random.default_rng(seed).choice(params.size, ncoef, replace=False)
    fd = np.empty(ncoef)
    t0 = time.perf_counter()
    for k, i in enumerate(idx):
        pp, pm = params.copy(), params.copy()
        pp[i] += h
        pm[i] -= h
        fd[k] = (sum(o64.value(pp)) - sum(o64.value(pm))) / (2 * h)
    del o64
    nrm = float(np.linalg.norm(fd))
    return {"coefficients": ncoef, "h": h, "seed": seed, "seconds": time.perf_counter() - t0,
            "rel_l2_gpu_vs_fd": float(np.linalg.norm(d_gpu[idx] - fd) / nrm),
            "rel_l2_reference_gradient_vs_fd": float(np.linalg.norm(d_ref[idx] - fd) / nrm),
            "rel_l2_gpu_vs_reference_gradient": float(np.linalg.norm(d_gpu[idx] - d_ref[idx]) /
                                                      np.linalg.norm(d_ref[idx]))}


def ncc_256_summary(device, flush, threads):
    """256^3 NCC with bias field: split against plain kernels on this GPU,
    error against the oracle at reference precision"""
    import torch
    import mia_gb300 as M
    from oracle import oracle as O
    name = "3d_ncc_256x256x256"
    w, mov, ref, params = WL.make_workload(name)
    size = w["size"]
    N = int(np.prod(size))
    lv = M.Level(size, rate=w["rate"], cost=w["cost"], penalty_weight=w["penalty"], device=device)
    lv.set_images(mov, ref)
    dev = torch.device("cuda", device)
    p_d = torch.from_numpy(params).to(dev)
    g_d = torch.empty(lv.nparams, dtype=torch.float64, device=dev)
    c_d = torch.empty(2, dtype=torch.float64, device=dev)
    out = {"workload": name, "config": WL.line_config(name, lv.csize), "tile": list(lv.tile)}
    out.update(split_vs_plain(lv, p_d, g_d, c_d, flush, 5, N))
    out["value"] = N / out["split_ms"] / 1e3
    out["unit"] = "Mvoxel/s"
    ci, cp, gi, gp, _ = lv.evaluate(params)
    o = O.Level(size, rate=w["rate"], cost=w["cost"], penalty_weight=w["penalty"], threads=threads)
    o.set_images(mov, ref)
    oi, op, ogi, ogp = o.evaluate(params)
    out["parity"] = {"cost_image_rel": abs(ci - oi) / abs(oi), "cost_penalty_rel": abs(cp - op) / abs(op),
                     "grad_image_rel_l2": float(np.linalg.norm(gi - ogi) / np.linalg.norm(ogi)),
                     "grad_penalty_rel_l2": float(np.linalg.norm(gp - ogp) / np.linalg.norm(ogp)),
                     "against": "oracle, reference precision"}
    lv.close()
    return out


def oracle_pairs_per_s(w, pairs, seconds, threads):
    """the oracle's registration of the pairs, one after the other with
    `threads` threads per evaluation, until `seconds` have passed"""
    from oracle import oracle as O
    mo = O.minimizer(w["minimizer"], maxiter=w["maxiter"], step=0.1)
    n = 0
    t0 = time.perf_counter()
    while n < len(pairs):
        mov, ref = pairs[n]
        O.register(mov, ref, w["rate"], w["levels"], mo, cost=w["cost"], penalty_weight=w["penalty"],
                   threads=threads)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return n / dt, n, dt


def oracle_final_costs(w, pairs, workers):
    """per pair, three registrations by the oracle: at the reference's
    precision; the same with the moving image perturbed at float rounding
    level (relative 1e-7, seeded); and with every evaluation in FP64.  The
    last two measure how sensitive the pair's registration trajectory is:
    the minimizer's accept/reject decisions compare costs, and the
    reference sums the 2D cost in float (its force pass,
    mia/2d/fullcost/image.cc:100), so rounding alone can move the final
    cost.  Pairs run in parallel host threads, one thread per registration."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    mo = O.minimizer(w["minimizer"], maxiter=w["maxiter"], step=0.1)

    def one(k):
        mov, ref = pairs[k]
        kw = dict(cost=w["cost"], penalty_weight=w["penalty"], threads=1)
        f0 = O.register(mov, ref, w["rate"], w["levels"], mo, **kw)[2]
        rng = np.random.default_rng(1 + k)
        m2 = (mov * (1 + 1e-7 * rng.standard_normal(mov.shape))).astype(np.float32)
        f1 = O.register(m2, ref, w["rate"], w["levels"], mo, **kw)[2]
        f64 = O.register(mov, ref, w["rate"], w["levels"], mo, precision=O.PREC_F64, **kw)[2]
        return f0, abs(f1 - f0), f64
    with ThreadPoolExecutor(max(1, workers)) as ex:
        return list(ex.map(one, range(len(pairs))))


def final_cost_report(res, plain_out, oracle):
    """final costs of the batched path against the plain per-pair GPU path
    and, when given, against the oracle: a pair passes when its final cost
    is within 1e-4 relative of the oracle's at the reference's precision,
    or no further from it than the oracle's own FP64 run or 3x the
    oracle's spread under a 1e-7 perturbation of the moving image (the
    trajectory's sensitivity to rounding, measured per pair)"""
    rel = [abs(r[2] - o[2]) / max(abs(o[2]), 1e-300) for r, o in zip(res, plain_out)]
    rep = {"vs_plain_per_pair": {"max": float(max(rel)), "median": float(np.median(rel)),
                                 "pairs_within_1e-4": int(sum(1 for r in rel if r <= 1e-4)), "pairs": len(rel)}}
    if oracle:
        per = []
        ok_b = ok_p = in_b = 0
        for k, ((fo, spread, f64), r, q) in enumerate(zip(oracle, res, plain_out)):
            tol = max(1e-4 * abs(fo), 3 * spread, abs(f64 - fo))
            db, dp = abs(r[2] - fo), abs(q[2] - fo)
            ok_b += db <= tol
            ok_p += dp <= tol
            in_b += db <= 1e-4 * abs(fo) or abs(r[2] - f64) <= 1e-4 * abs(f64)
            per.append({"pair": k, "batched": r[2], "plain": q[2], "oracle": fo, "oracle_f64": f64,
                        "oracle_perturbation_spread": spread, "batched_rel": db / abs(fo),
                        "batched_rel_vs_f64": abs(r[2] - f64) / abs(f64), "plain_rel": dp / abs(fo)})
        rep["vs_oracle"] = {"rule": "|final - oracle| <= max(1e-4 |oracle|, |oracle_f64 - oracle|, 3 x oracle spread "
                                    "under a 1e-7 perturbation of the moving image)",
                            "batched_pairs_passing": int(ok_b), "plain_pairs_passing": int(ok_p), "pairs": len(per),
                            "batched_within_1e-4_of_oracle_or_oracle_f64": int(in_b),
                            "max_batched_rel": float(max(p["batched_rel"] for p in per)),
                            "max_batched_rel_vs_f64": float(max(p["batched_rel_vs_f64"] for p in per)),
                            "per_pair": per}
    return rep


def measure_batch(name, steps, warmup, device, cpu_seconds=0.0, clocks=None, profile_region=False,
                  oracle_check=False):
    """Registered pairs/s of the batched path (device-resident images), end
    to end from host arrays, and the per-pair GPU driver (plain and split
    paths) on the same pairs."""
    import torch
    import mia_gb300 as M
    from mia_gb300 import registration as R
    w, pairs = WL.make_pairs(name)
    npairs = len(pairs)
    mz = R.minimizer(w["minimizer"], maxiter=w["maxiter"], step=0.1)
    kw = dict(cost=w["cost"], penalty_weight=w["penalty"])
    dev = torch.device("cuda", device)
    dpairs = [(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)) for a, b in pairs]
    torch.cuda.synchronize()

    def batch():
        return R.register_batch_device(dpairs, w["rate"], w["levels"], mz, device=device, **kw)

    for _ in range(warmup):
        batch()
    launches0 = M.lib().mgr_kernel_launch_count()
    times = []
    sampler = clocks if clocks is not None else ClockSampler(device)
    with sampler:
        for i in range(steps):
            torch.cuda.synchronize()
            if profile_region and i == 0:   # the capture region of ncu --profile-from-start off
                torch.cuda.cudart().cudaProfilerStart()
            t0 = time.perf_counter()
            res = batch()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            if profile_region and i == 0:
                torch.cuda.cudart().cudaProfilerStop()
    launches = (M.lib().mgr_kernel_launch_count() - launches0) // max(1, steps)
    t_step = float(np.mean(times))
    # end to end from the host arrays: the same untimed warm-up as above,
    # then every timed call reads all images from host memory again
    for _ in range(warmup):
        R.register_batch(pairs, w["rate"], w["levels"], mz, device=device, **kw)
    e2e_t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        res_h = R.register_batch(pairs, w["rate"], w["levels"], mz, device=device, **kw)
        e2e_t.append(time.perf_counter() - t0)
    t_e2e = float(np.mean(e2e_t))
    per = {}
    for path in ("plain", "split"):
        t0 = time.perf_counter()
        out = [R.register_pair(a, b, w["rate"], w["levels"], mz, path=path, device=device, **kw) for a, b in pairs]
        per[path] = (npairs / (time.perf_counter() - t0), out)
    plain_rate, plain_out = per["plain"]
    persistent = None
    if pairs[0][0].ndim == 3:
        # the warp and adjoint kernels as persistent launches drawing (pair,
        # tile) items from a device queue, against one block per item
        def batch_q():
            return R.register_batch_device(dpairs, w["rate"], w["levels"], mz, device=device, persistent=True, **kw)
        batch_q()
        tq = []
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rq = batch_q()
            torch.cuda.synchronize()
            tq.append(time.perf_counter() - t0)
        persistent = {"value": npairs / float(np.mean(tq)), "unit": "pairs/s",
                      "vs_one_block_per_item": t_step / float(np.mean(tq)),
                      "same_results": all(np.array_equal(a[0], b[0]) and a[2] == b[2] for a, b in zip(res, rq))}
    oracle = oracle_final_costs(w, pairs, min(16, os.cpu_count() or 1)) if oracle_check else None
    rel_split = [abs(r[2] - o[2]) / max(abs(o[2]), 1e-300) for r, o in zip(res, per["split"][1])]
    h2d = int(sum(a.nbytes + b.nbytes for a, b in pairs))
    d2h = int(sum(r[0].nbytes for r in res_h))
    out = {
        "value": npairs / t_step, "unit": "pairs/s", "ms_per_step": t_step * 1e3, "npairs": npairs,
        "voxels": int(sum(a.size for a, _ in pairs)), "evaluations": int(sum(r[3] for r in res)),
        "gpu_launches": int(launches),
        "e2e": {"value": npairs / t_e2e, "unit": "pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "plain_per_pair": {"value": plain_rate, "unit": "pairs/s", "path": "plain"},
        "split_per_pair": {"value": per["split"][0], "unit": "pairs/s", "path": "split"},
        "speedup_vs_plain_per_pair": {"device_resident": npairs / t_step / plain_rate,
                                      "e2e": npairs / t_e2e / plain_rate},
        "final_cost": final_cost_report(res, plain_out, oracle),
        "persistent_launch": persistent,
        "final_cost_rel_diff_vs_split_per_pair": {"max": float(max(rel_split)),
                                                  "median": float(np.median(rel_split))},
        "config": WL.line_config(name),
        "sizes": sorted({"x".join(map(str, a.shape[::-1])) for a, _ in pairs}),
    }
    if cpu_seconds > 0:
        threads = os.cpu_count() or 1
        v, n, dt = oracle_pairs_per_s(w, pairs, cpu_seconds, threads)
        out["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": threads, "kind": "port",
                               "sample": "%d of the %d pairs registered in %.1f s" % (n, npairs, dt)}
    return out


def measure_single2d(device, steps, cpu_seconds=0.0):
    """The 2D single-pair registration (128x128, SSD + divcurl 10, rate 16,
    one level, 50 GSL steepest-descent iterations; the
    mia-2dimageregistration workload, src/2dimageregistration.cc:60-95):
    pairs/s of the per-pair GPU driver from host arrays (split and plain
    kernels) and of the batched path with this one pair, the final cost
    against the oracle's registration, and the oracle timed on the host."""
    from mia_gb300 import registration as R
    name = "single2d_128"
    w, pairs = WL.make_pairs(name)
    mov, ref = pairs[0]
    mz = R.minimizer(w["minimizer"], maxiter=w["maxiter"], step=0.1)
    kw = dict(cost=w["cost"], penalty_weight=w["penalty"])
    out = {"config": WL.line_config(name), "unit": "pairs/s"}
    for path in ("split", "plain"):
        R.register_pair(mov, ref, w["rate"], w["levels"], mz, path=path, device=device, **kw)   # warm-up
        t0 = time.perf_counter()
        for _ in range(steps):
            r = R.register_pair(mov, ref, w["rate"], w["levels"], mz, path=path, device=device, **kw)
        out[path + "_per_pair"] = {"value": steps / (time.perf_counter() - t0), "final_cost": r[2],
                                   "evaluations": r[3]}
    R.register_batch([pairs[0]], w["rate"], w["levels"], mz, device=device, **kw)
    t0 = time.perf_counter()
    for _ in range(steps):
        rb = R.register_batch([pairs[0]], w["rate"], w["levels"], mz, device=device, **kw)
    out["batched_one_pair"] = {"value": steps / (time.perf_counter() - t0), "final_cost": rb[0][2]}
    out["value"] = out["split_per_pair"]["value"]
    out["e2e"] = {"value": out["value"], "unit": "pairs/s", "h2d_bytes_per_step": int(mov.nbytes + ref.nbytes),
                  "d2h_bytes_per_step": int(r[0].nbytes)}
    if cpu_seconds > 0:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        mo = O.minimizer(w["minimizer"], maxiter=w["maxiter"], step=0.1)
        n, t0 = 0, time.perf_counter()
        while True:
            po, cso, fo, no = O.register(mov, ref, w["rate"], w["levels"], mo, threads=threads, **kw)
            n += 1
            if time.perf_counter() - t0 >= cpu_seconds:
                break
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "pairs/s", "cores": threads, "kind": "port",
                               "sample": "%d registrations of the pair in %.1f s" % (n, dt)}
        out["final_cost_vs_oracle"] = {
            "oracle": fo, "split_rel": abs(out["split_per_pair"]["final_cost"] - fo) / abs(fo),
            "plain_rel": abs(out["plain_per_pair"]["final_cost"] - fo) / abs(fo),
            "batched_rel": abs(out["batched_one_pair"]["final_cost"] - fo) / abs(fo)}
    return out


def run_batch(args):
    """one JSON line for a registration workload (pairs/s); with N ranks,
    N replicas of the workload, the slowest rank's time counts"""
    from mia_gb300 import replicas
    ws, rank, local = dist_env()
    import torch
    replicas.init()
    torch.cuda.set_device(local)
    name = args.workload
    clk = ClockSampler(local)
    replicas.barrier()
    r = measure_batch(name, args.steps, args.warmup, local,
                      0.0 if (args.no_cpu_baseline or rank != 0) else args.cpu_seconds,
                      profile_region=args.profile_region, clocks=clk,
                      oracle_check=(rank == 0 and name == "series2d_60" and not args.no_cpu_baseline))
    replicas.barrier()
    value, t_max = replicas.whole_job_rate(r["npairs"], r["ms_per_step"] / 1e3, ws,
                                           device=torch.device("cuda", local))
    e2e_v, _ = replicas.whole_job_rate(r["npairs"], r["npairs"] / r["e2e"]["value"], ws,
                                       device=torch.device("cuda", local))
    if rank != 0:
        return 0
    r["e2e"]["value"] = e2e_v
    r["ms_per_step"] = t_max * 1e3
    line = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic"}
    line.update({k: v for k, v in r.items() if k not in ("value", "unit", "ms_per_step")})
    line["timing"] = "wall clock of the whole batched registration, device synchronised on both sides"
    line["clocks"] = clk.summary()
    print(json.dumps(line))
    return 0


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    name = args.workload
    if name in BATCH_WORKLOADS:
        return run_reference_batch(args)
    # the same host inputs as the GPU arm; no GPU code on this path
    from oracle import oracle as O
    w, mov, ref, params = WL.make_workload(name)
    size = w["size"]
    threads = os.cpu_count() or 1
    lv = O.Level(size, rate=w["rate"], cost=w["cost"], penalty_weight=w["penalty"], threads=threads)
    lv.set_images(mov, ref)
    for _ in range(args.warmup):
        lv.evaluate(params)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lv.evaluate(params)
    dt = time.perf_counter() - t0
    N = int(np.prod(size))
    v = N * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Mvoxel/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": WL.line_config(name, lv.csize),
        "cpu_baseline": {"value": v, "unit": "Mvoxel/s", "cores": threads, "kind": "port",
                         "sample": "%d full evaluations of %s" % (args.steps, "x".join(map(str, size)))},
        "e2e": {"value": v, "unit": "Mvoxel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_reference_batch(args):
    """the oracle's registration on the host cores, pairs/s"""
    w, pairs = WL.make_pairs(args.workload)
    threads = os.cpu_count() or 1
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(args.warmup):
        oracle_pairs_per_s(w, pairs[:1], 0.0, threads)
    counts = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, n, _ = oracle_pairs_per_s(w, pairs, per_step, threads)
        counts += n
    dt = time.perf_counter() - t0
    v = counts / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "pairs/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": WL.line_config(args.workload),
            "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": "%d pair registrations, %.1f s per step at most" % (counts, per_step)},
            "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def e2e_seconds(lv, hp, hg, flush, args):
    """mean seconds of one evaluation through the C ABI from the host
    buffers hp (parameters) and hg (gradient), the L2 flushed before each"""
    import torch
    evaluate = lv.bind_evaluate_total(hp, hg)   # one C-ABI call per evaluation, pointers prepared once
    for _ in range(max(1, args.warmup)):
        evaluate()
    t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        evaluate()
        t.append(time.perf_counter() - t0)
    return float(np.mean(t))


def run_gpu(args):
    import torch
    from mia_gb300 import replicas
    ws, rank, local = dist_env()
    replicas.init()
    torch.cuda.set_device(local)
    import mia_gb300 as M
    name = args.workload
    w, mov, ref, params = WL.make_workload(name)
    size = w["size"]
    N = int(np.prod(size))
    lv = M.Level(size, rate=w["rate"], cost=w["cost"], penalty_weight=w["penalty"], device=local)
    lv.set_images(mov, ref)
    nparams = lv.nparams
    dev = torch.device("cuda", local)
    p_d = torch.from_numpy(params).to(dev)
    g_d = torch.empty(nparams, dtype=torch.float64, device=dev)
    c_d = torch.empty(2, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # events around the whole evaluation: its kernels overlap as in an
    # untimed run (programmatic dependent launch)
    lv.set_timing(True, whole=True)
    torch.cuda.synchronize()

    barrier = replicas.barrier

    for _ in range(args.warmup):
        lv.evaluate_device(p_d.data_ptr(), g_d.data_ptr(), c_d.data_ptr())
        lv.sync()
    launches0 = M.lib().mgr_kernel_launch_count()
    per = []
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            lv.evaluate_device(p_d.data_ptr(), g_d.data_ptr(), c_d.data_ptr())
            per.append(lv.kernel_times())
        lv.sync()
        torch.cuda.synchronize()
    barrier()
    launches = M.lib().mgr_kernel_launch_count() - launches0
    per = np.array(per)
    value, t_step = replicas.whole_job_rate(N / 1e6, per[:, 3].mean() / 1e3, ws, device=dev)
    # the kernels' own times, from a second pass with events around each
    # kernel (which then run one after another)
    per_k = np.array(time_evals(lv, p_d, g_d, c_d, flush, args.steps, per_kernel=True))[None, :]

    # end to end through the C ABI: host (pinned) params in, gradient out;
    # on a host whose memory the device reads coherently the kernels move
    # them in place, and a second level with staged copies (MGR_HOST_COPY=1)
    # is timed beside it
    hp = torch.from_numpy(params).pin_memory().numpy()
    hg = torch.empty(nparams, dtype=torch.float64).pin_memory().numpy()
    lv.set_timing(False)
    e2e_step = replicas.max_over_ranks(e2e_seconds(lv, hp, hg, flush, args), device=dev)
    in_place = lv.in_place
    staged_step = None
    if in_place:
        os.environ["MGR_HOST_COPY"] = "1"
        try:
            lv_staged = M.Level(size, rate=w["rate"], cost=w["cost"], penalty_weight=w["penalty"], device=local)
        finally:
            del os.environ["MGR_HOST_COPY"]
        lv_staged.set_images(mov, ref)
        staged_step = replicas.max_over_ranks(e2e_seconds(lv_staged, hp, hg, flush, args), device=dev)
        del lv_staged

    if rank != 0:
        return 0
    D, C = 3, nparams // 3
    # algorithmic bytes of one evaluation: moving coefficients and reference
    # read once (4 B per voxel each), parameters read as float, gradient
    # written as double (4 + 8 B per parameter)
    b_eval = 8.0 * N + 12.0 * D * C
    peak, peak_kind = measured_peaks()
    kms = {"k_warp3": float(per_k[:, 0].mean()), "k_adjoint3": float(per_k[:, 1].mean()),
           "k_gather3": float(per_k[:, 2].mean())}
    top = max(kms, key=kms.get)
    t_top = kms[top] / 1e3
    roof = {"bound": "hbm", "kernel": top, "achieved": b_eval / t_top / 1e9, "peak": peak,
            "unit": "GB/s", "frac": b_eval / t_top / 1e9 / peak, "traffic": profile_traffic(top),
            "peak_kind": peak_kind, "algorithmic_bytes": b_eval,
            "charged": "B_eval = 8 N + 12 d C bytes of the whole evaluation over the dominant kernel's time"}
    eval_roof = {"achieved": b_eval / t_step / 1e9, "frac": b_eval / t_step / 1e9 / peak,
                 "algorithmic_bytes": b_eval, "unit": "GB/s", "traffic": profile_traffic("evaluation")}
    clocks = clk.summary()
    # the bound that limits k_warp3 in practice: its shared-memory data path
    # (one 128-byte wavefront per SM and clock); wavefronts per launch from
    # the committed ncu capture of this workload, time from this run
    wf = profile_metric("k_warp3", "shared_wavefronts") if name == "3d_ssd_192x192x128" else None
    smem_roof = None
    if wf and clocks.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        peak_smem = sms * 128.0 * clocks["sm_mhz"] * 1e6 / 1e12
        ach = wf * 128.0 / (kms["k_warp3"] / 1e3) / 1e12
        smem_roof = {"kernel": "k_warp3", "bound": "shared memory (L1/shared data path)", "achieved": ach,
                     "peak": peak_smem, "unit": "TB/s", "frac": ach / peak_smem,
                     "wavefronts_per_launch": wf, "peak_rule": "SMs x 128 B x median SM clock of this run"}
    line = {
        "metric": METRIC, "value": value, "unit": "Mvoxel/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": WL.line_config(name, lv.csize),
        "setup": {"path": "split", "tile": list(lv.tile), "parallelism": "replicas" if ws > 1 else "single"},
        "e2e": {"value": ws * N / e2e_step / 1e6, "unit": "Mvoxel/s", "h2d_bytes_per_step": nparams * 8,
                "d2h_bytes_per_step": nparams * 8 + 16,
                "transfer": ("in place: the kernels read the parameters and write the gradient and costs in "
                             "host memory over the coherent CPU-GPU link" if in_place else
                             "staged: cudaMemcpyAsync of the parameters in, the gradient and costs out"),
                "staged_value": None if staged_step is None else ws * N / staged_step / 1e6},
        "gpu_launches": int(launches),
        "kernel_ms": {"warp": kms["k_warp3"], "adjoint": kms["k_adjoint3"], "gather_penalty": kms["k_gather3"]},
        "roofline": roof,
        "eval_roofline": eval_roof,
        "shared_memory_roofline": smem_roof,
        "clocks": clocks,
    }
    if ws == 1:
        line["split_vs_plain"] = split_vs_plain(lv, p_d, g_d, c_d, flush, max(3, min(args.steps, 10)), N)
        if w["cost"] == "ssd":
            line["fused_vs_split"] = fused_vs_split(lv, p_d, g_d, c_d, flush, max(3, min(args.steps, 10)), N,
                                                    params)
    if ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, n, dt, res = cpu_baseline(w, mov, ref, params, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": v, "unit": "Mvoxel/s", "cores": threads, "kind": "port",
                                "sample": "%d full %s evaluations in %.1f s" % (n, "x".join(map(str, size)), dt)}
        ci, cp, gi, gp, gt = lv.evaluate(params)
        oi, op, ogi, ogp = res
        line["parity"] = {
            "cost_image_rel": abs(ci - oi) / abs(oi), "cost_penalty_rel": abs(cp - op) / abs(op),
            "grad_image_rel_l2": float(np.linalg.norm(gi - ogi) / np.linalg.norm(ogi)),
            "grad_penalty_rel_l2": float(np.linalg.norm(gp - ogp) / np.linalg.norm(ogp)),
            "against": "oracle, reference precision"}
        line["fd_check"] = fd_check(w, mov, ref, params, lv, (ogi, ogp), threads)
        if name == "3d_ssd_192x192x128" and not args.no_batched:
            # the 3D NCC configuration: split vs plain kernels and parity
            lv.close()
            line["ncc_256"] = ncc_256_summary(local, flush, threads)
    if ws == 1 and not args.no_batched:
        # the registration workloads (pairs/s): the 2D single pair, and the
        # batched path against the per-pair GPU driver on the same pairs
        lv.close()
        line["single2d_128"] = measure_single2d(local, 5, 0.0 if args.no_cpu_baseline else 5.0)
        line["batched"] = {}
        for bname, cpu_s in (("series2d_60", 6.0), ("cohort3d_16", 10.0)):
            bclk = ClockSampler(local)
            r = measure_batch(bname, 3, 2, local, 0.0 if args.no_cpu_baseline else cpu_s, clocks=bclk,
                              oracle_check=(bname == "series2d_60" and not args.no_cpu_baseline))
            r["clocks"] = bclk.summary()
            r["steps"], r["warmup"] = 3, 2
            line["batched"][bname] = r
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="3d_ssd_192x192x128", choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS))
    ap.add_argument("--no-batched", action="store_true", help="skip the registration summaries of the default line")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-region", action="store_true",
                    help="registration workloads: the first timed batched registration is the profiler's "
                         "capture region (for ncu --profile-from-start off)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in BATCH_WORKLOADS:
        return run_batch(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
