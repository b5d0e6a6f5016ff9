"""Build recipe for the native library (no cmake): nvcc for the CUDA
translation units (sm_103a only), g++ for the host-only ones, linked in-tree
into hybrid_k_nearest_neighbor_self_join_gb300/_build/:

  libknnsj.so            C ABI of include/knnsj.h; KNNJoinPy takes float
  libknnsj_double.so     the same with KNNJoinPy taking double
  libgpuknnselfjoin.so   symlink to libknnsj.so (the name the reference's
                         Python wrapper loads, knnjoingpu.py:173-175)
  main                   the `main FNAME DIM K` command line

Optional fixed-configuration builds mirror the reference's params.h /
Makefile knobs (Makefile:55-76): set KNNSJ_GPUNUMDIM, KNNSJ_NUMINDEXEDDIM,
KNNSJ_BETA_BUILD before building to bake them in; by default the number of
dimensions, NUMINDEXEDDIM and BETA are chosen per call.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp"]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp"]

CU_SOURCES = ["k_prep.cu", "k_eps.cu", "k_grid.cu", "k_search.cu", "k_tile.cu", "k_outlier.cu", "k_radius.cu", "k_mlp.cu", "join.cu"]
HEADERS = ["knnsj_device.cuh", "exact_sqrt.cuh", "mlp_tc.cuh", "ring_policy.h", "knnsj_internal.h", "knnsj_host.h", "radius_model.cuh", "radius_model_weights.inc"]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _knob_defines() -> list[str]:
    defs = os.environ.get("KNNSJ_NVCC_EXTRA", "").split()
    for env, macro in (("KNNSJ_GPUNUMDIM", "GPUNUMDIM"), ("KNNSJ_NUMINDEXEDDIM", "NUMINDEXEDDIM"),
                       ("KNNSJ_BETA_BUILD", "BETA")):
        v = os.environ.get(env)
        if v:
            defs.append(f"-D{macro}={v}")
    return defs


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {' '.join(cmd[:3])} ...")


def build(force: bool = False, verbose: bool = False) -> dict:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "knnsj.h")]
    knobs = _knob_defines()
    jobs = []
    objs = {}
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs[src] = o
        if force or not _newer(o, [s] + hdrs):
            jobs.append([nvcc, *NVCC_FLAGS, *ARCH, *knobs, "-c", s, "-o", o])
    for variant, extra in (("api_f32.o", []), ("api_f64.o", ["-DKNNSJ_BUILD_DTYPE_DOUBLE"])):
        s = os.path.join(CSRC, "api.cu")
        o = os.path.join(OUT, variant)
        objs[variant] = o
        if force or not _newer(o, [s] + hdrs):
            jobs.append([nvcc, *NVCC_FLAGS, *ARCH, *knobs, *extra, "-c", s, "-o", o])
    s = os.path.join(CSRC, "hostio.cpp")
    o = os.path.join(OUT, "hostio.o")
    objs["hostio"] = o
    if force or not _newer(o, [s] + hdrs):
        jobs.append(["g++", *CXX_FLAGS, "-c", s, "-o", o])
    s = os.path.join(CSRC, "cli_main.cpp")
    o = os.path.join(OUT, "cli_main.o")
    objs["cli"] = o
    if force or not _newer(o, [s] + hdrs):
        jobs.append(["g++", *CXX_FLAGS, *knobs, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))

    common = [objs[s] for s in CU_SOURCES] + [objs["hostio"]]
    libs = {}
    for name, api in (("libknnsj.so", "api_f32.o"), ("libknnsj_double.so", "api_f64.o")):
        target = os.path.join(OUT, name)
        deps = common + [objs[api]]
        if force or not _newer(target, deps):
            _run([nvcc, "-shared", *ARCH, "-Xcompiler", "-fopenmp", "-o", target, *deps, "-lgomp"],
                 verbose)
        libs[name] = target
    link = os.path.join(OUT, "libgpuknnselfjoin.so")
    if not os.path.islink(link):
        if os.path.exists(link):
            os.remove(link)
        os.symlink("libknnsj.so", link)
    libs["libgpuknnselfjoin.so"] = link
    exe = os.path.join(OUT, "main")
    if force or not _newer(exe, [objs["cli"], libs["libknnsj.so"]]):
        _run(["g++", "-o", exe, objs["cli"], "-L" + OUT, "-lknnsj", "-Wl,-rpath,$ORIGIN", "-fopenmp"],
             verbose)
    libs["main"] = exe
    return libs


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
