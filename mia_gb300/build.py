"""Build libmgr.so in-tree for sm_103a (GB300) with nvcc.

Translation units are compiled in parallel, one -gencode, no cmake.  The
host-only table code is compiled by g++ with -ffp-contract=off so its
float/double expressions round identically on x86-64 and aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libmgr.so")
BUILD = os.path.join(HERE, "_build")

CU_SOURCES = ["api.cu", "eval.cu", "split.cu", "split3.cu", "fused3.cu", "gather.cu", "prefilter.cu", "noalloc.cu", "pyramid.cu", "register.cu", "batch.cu", "refine.cu"]
CXX_SOURCES = ["tables.cc", "driver.cc", "tune.cc", "transio.cc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
TILES_JSON = os.path.join(HERE, "tiles.json")
TILE_TABLE = os.path.join(BUILD, "tile_table.inc")


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def write_tile_table():
    """tiles.json (the autotuner's committed choices) as C initialisers for
    tune.cc; an empty table when the file is absent"""
    import json
    lines = ["// generated from tiles.json by build.py"]
    if os.path.exists(TILES_JSON):
        with open(TILES_JSON) as f:
            doc = json.load(f)
        for e in doc.get("entries", []):
            t = list(e["tile"]) + [1] * (3 - len(e["tile"]))
            lines.append("{%d, %.9g, %.9g, {%d, %d, %d}}," % (e["dim"], e["spacing"], e["voxels"], t[0], t[1], t[2]))
    text = "\n".join(lines) + "\n"
    if not os.path.exists(TILE_TABLE) or open(TILE_TABLE).read() != text:
        with open(TILE_TABLE, "w") as f:
            f.write(text)


def build(force=False, verbose=False, extra_nvcc=()):
    os.makedirs(BUILD, exist_ok=True)
    # objects built on another host architecture are never reused
    import platform
    stamp = os.path.join(BUILD, "ARCH")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch or not os.path.exists(OUT):
        force = True
    with open(stamp, "w") as f:
        f.write(arch)
    write_tile_table()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hh", ".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "mgr.h"))
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "--expt-relaxed-constexpr", *extra_nvcc, "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s, TILE_TABLE] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", BUILD, "-c", s, "-o",
                         o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    if force or jobs or _stale(OUT, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", OUT, *objs, "-lcudart_static", "-ldl", "-lpthread", "-lrt"])
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
