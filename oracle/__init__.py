"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates the reference kNN self-join on the CPU (see
knnsj_oracle.cpp for the file:line map).  Only the tests, the smoke check and
bench.py's CPU-baseline leg import this module; the product library never
does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libknnsj_oracle.so")
_lib = None


class OrcStats(ctypes.Structure):
    _fields_ = [
        ("avg_distance", ctypes.c_double),
        ("bucket_width", ctypes.c_double),
        ("eps0", ctypes.c_double),
        ("eps_final", ctypes.c_double),
        ("total_distance", ctypes.c_double),
        ("pair_count", ctypes.c_uint64),
        ("candidates", ctypes.c_uint64),
        ("bucket", ctypes.c_int32),
        ("iterations", ctypes.c_int32),
        ("reindexes", ctypes.c_int32),
        ("eps_offset", ctypes.c_uint32),
        ("eps_sample_blocks", ctypes.c_uint32),
        ("perm", ctypes.c_uint32 * 64),
        ("seconds_prep", ctypes.c_double),
        ("seconds_regrid", ctypes.c_double),
        ("seconds_search", ctypes.c_double),
    ]


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH):
        subprocess.check_call(["bash", os.path.join(_HERE, "build_oracle.sh")])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
    return _lib


def _sfx(dtype) -> str:
    dt = np.dtype(dtype)
    if dt == np.float32:
        return "f32"
    if dt == np.float64:
        return "f64"
    raise TypeError(f"unsupported dtype {dt}")


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def max_threads() -> int:
    return int(lib().orc_max_threads())


def reorder(data: np.ndarray):
    """Dimension order of ReorderByDimension (main.cu:2521) and variances."""
    data = np.ascontiguousarray(data)
    n, d = data.shape
    perm = np.zeros(d, np.uint32)
    var = np.zeros(d, data.dtype)
    f = getattr(lib(), "orc_reorder_" + _sfx(data.dtype))
    rc = f(_ptr(data), ctypes.c_uint64(n), ctypes.c_uint32(d), _ptr(perm), _ptr(var))
    assert rc == 0
    return perm, var


def estimate_eps(data_reordered: np.ndarray, k: int, beta: float, nthreads: int = 0):
    """Epsilon estimator (GPU.cu:3088) on already-reordered data."""
    x = np.ascontiguousarray(data_reordered)
    n, d = x.shape
    out = np.zeros(6, np.float64)
    hist = np.zeros(10000, np.uint32)
    f = getattr(lib(), "orc_eps_" + _sfx(x.dtype))
    rc = f(_ptr(x), ctypes.c_uint64(n), ctypes.c_uint32(d), ctypes.c_uint32(k),
           ctypes.c_double(beta), _ptr(out), _ptr(hist), ctypes.c_int(nthreads))
    assert rc == 0
    return {
        "avg": out[0], "bucket_width": out[1], "eps0": out[2], "bucket": int(out[3]),
        "pair_count": int(out[4]), "offset": int(out[5]), "hist": hist,
    }


def grid(data_reordered: np.ndarray, di: int, eps: float, nthreads: int = 0):
    """Grid index at cell width eps (GPU.cu:3715 / main.cu:1968)."""
    x = np.ascontiguousarray(data_reordered)
    n, d = x.shape
    T = x.dtype.type
    minArr = np.zeros(di, x.dtype)
    nCells = np.zeros(di, np.uint32)
    total = ctypes.c_uint64(0)
    keys = np.zeros(n, np.uint64)
    imin = np.zeros(n, np.int32)
    imax = np.zeros(n, np.int32)
    lookup = np.zeros(n, np.uint32)
    nne = ctypes.c_uint64(0)
    f = getattr(lib(), "orc_grid_" + _sfx(x.dtype))
    epsc = ctypes.c_float(eps) if x.dtype == np.float32 else ctypes.c_double(eps)
    rc = f(_ptr(x), ctypes.c_uint64(n), ctypes.c_uint32(d), ctypes.c_uint32(di), epsc,
           _ptr(minArr), _ptr(nCells), ctypes.byref(total), _ptr(keys), _ptr(imin),
           _ptr(imax), _ptr(lookup), ctypes.byref(nne), ctypes.c_int(nthreads))
    assert rc == 0
    c = nne.value
    return {
        "minArr": minArr, "nCells": nCells, "totalCells": total.value,
        "cellKeys": keys[:c].copy(), "indexmin": imin[:c].copy(),
        "indexmax": imax[:c].copy(), "lookup": lookup,
    }


def join(data: np.ndarray, k: int, di: int = 0, beta: float = 0.05, reorder: bool = True,
         queries=None, max_iterations: int = 0, nthreads: int = 0):
    """Reference pipeline (main.cu:109-510).  Returns (rc, ids, dists, stats).

    ids / dists are (N, k+1); rows of queries not processed stay -1 / 0.
    """
    x = np.ascontiguousarray(data)
    n, d = x.shape
    K = k + 1
    ids = np.full((n, K), -1, np.int32)
    dists = np.zeros((n, K), x.dtype)
    st = OrcStats()
    if queries is None:
        qp, nq = None, 0
    else:
        q = np.ascontiguousarray(queries, dtype=np.uint32)
        qp, nq = _ptr(q), q.size
    f = getattr(lib(), "orc_join_" + _sfx(x.dtype))
    rc = f(_ptr(x), ctypes.c_uint64(n), ctypes.c_uint32(d), ctypes.c_uint32(k),
           ctypes.c_int32(di), ctypes.c_double(beta), ctypes.c_int32(1 if reorder else 0),
           qp, ctypes.c_uint64(nq), ctypes.c_int32(max_iterations), _ptr(ids), _ptr(dists),
           ctypes.byref(st), ctypes.c_int(nthreads))
    return rc, ids, dists, st


def range_query(data_summation_order: np.ndarray, eps: float, queries, maxper: int = 4096, nthreads: int = 0):
    """Every point within eps of each query by the reference's rule
    (evalPoint, kernel.cu:116-161), in ascending (acc, id) order.  Returns
    (counts, ids, dists) with rows padded to maxper."""
    x = np.ascontiguousarray(data_summation_order)
    n, d = x.shape
    q = np.ascontiguousarray(queries, dtype=np.uint32)
    counts = np.zeros(q.size, np.uint32)
    ids = np.full((q.size, maxper), -1, np.int32)
    dists = np.zeros((q.size, maxper), x.dtype)
    f = getattr(lib(), "orc_range_" + _sfx(x.dtype))
    epsc = ctypes.c_float(eps) if x.dtype == np.float32 else ctypes.c_double(eps)
    rc = f(_ptr(x), ctypes.c_uint64(n), ctypes.c_uint32(d), epsc, _ptr(q), ctypes.c_uint64(q.size),
           ctypes.c_uint32(maxper), _ptr(counts), _ptr(ids), _ptr(dists), ctypes.c_int(nthreads))
    assert rc == 0, "more than maxper points within eps"
    return counts, ids, dists


def bruteforce(data_summation_order: np.ndarray, K: int, queries, nthreads: int = 0):
    """First K points by (acc, id) for each query, over all points."""
    x = np.ascontiguousarray(data_summation_order)
    n, d = x.shape
    q = np.ascontiguousarray(queries, dtype=np.uint32)
    ids = np.zeros((q.size, K), np.int32)
    dists = np.zeros((q.size, K), x.dtype)
    f = getattr(lib(), "orc_bruteforce_" + _sfx(x.dtype))
    rc = f(_ptr(x), ctypes.c_uint64(n), ctypes.c_uint32(d), ctypes.c_uint32(K), _ptr(q),
           ctypes.c_uint64(q.size), _ptr(ids), _ptr(dists), ctypes.c_int(nthreads))
    assert rc == 0
    return ids, dists


_RK_PATH = os.path.join(_HERE, "_build", "libref_kernel_runner.so")
REF_DIR = os.path.join(_HERE, "_ref")


def ref_kernel_cubin(dtype, d: int, di: int) -> str:
    """Path of the reference kernel built by build_ref_kernel.sh for (DTYPE, GPUNUMDIM, NUMINDEXEDDIM)."""
    name = "float" if np.dtype(dtype) == np.float32 else "double"
    return os.path.join(REF_DIR, f"refkernel_{name}_{d}_{di}.cubin")


def ref_kernel_pairs(x_reordered: np.ndarray, di: int, eps: float, queries=None, threads_per_point: int = 8):
    """Runs the reference's own kernelNDGridIndexGlobalkNN (kernel.cu:61-113)
    once at radius eps on the GPU, over the grid index the oracle builds
    (pinned against the reference's host code).  Returns every (query,
    point, distance) the kernel found within eps, unsorted."""
    x = np.ascontiguousarray(x_reordered)
    n, d = x.shape
    cubin = ref_kernel_cubin(x.dtype, d, di)
    if not os.path.exists(cubin):
        raise FileNotFoundError(cubin)
    if not os.path.exists(_RK_PATH):
        build(force=True)
    g = grid(x, di, eps)
    q = np.arange(n, dtype=np.uint32) if queries is None else np.ascontiguousarray(queries, dtype=np.uint32)
    # capacity: the points of the 3^di cells the kernel visits around each
    # query's cell -- its cell coordinate computed in the data type exactly as
    # the kernel does (kernel.cu:93) -- doubled plus a margin, so that the
    # kernel's unchecked appends (kernel.cu:149-153) cannot overflow
    T = x.dtype.type
    cells = np.floor((x[:, :di] - g["minArr"]) / T(eps)).astype(np.int64)
    mult = np.cumprod(np.concatenate([[1], g["nCells"][:-1].astype(np.int64)]))
    counts = (g["indexmax"] - g["indexmin"] + 1).astype(np.int64)
    keys = g["cellKeys"].astype(np.int64)
    cap = 0
    import itertools
    for off in itertools.product(range(-1, 2), repeat=di):
        c = cells[q] + np.array(off)
        ok = np.all((c >= 0) & (c < g["nCells"].astype(np.int64)), axis=1)
        lin = (c * mult).sum(axis=1)
        pos = np.searchsorted(keys, lin)
        pos = np.minimum(pos, keys.size - 1)
        hit = ok & (keys[pos] == lin)
        cap += int(counts[pos][hit].sum())
    cap = 2 * cap + 1_000_000
    out_q = np.empty(cap, np.int32)
    out_p = np.empty(cap, np.int32)
    out_d = np.empty(cap, x.dtype)
    cnt = ctypes.c_uint64(0)
    err = ctypes.create_string_buffer(512)
    rk = ctypes.CDLL(_RK_PATH)
    epsv = np.array([eps], x.dtype)
    rc = rk.refk_run(cubin.encode(), ctypes.c_int(x.dtype.itemsize), _ptr(x), ctypes.c_uint64(n), ctypes.c_uint32(d),
                     _ptr(epsv), _ptr(g["minArr"]), _ptr(g["nCells"]), ctypes.c_uint32(di), _ptr(g["cellKeys"]),
                     _ptr(g["indexmin"]), _ptr(g["indexmax"]), ctypes.c_uint64(g["cellKeys"].size), _ptr(g["lookup"]),
                     _ptr(q), ctypes.c_uint32(q.size), ctypes.c_uint32(threads_per_point), ctypes.c_uint64(cap),
                     _ptr(out_q), _ptr(out_p), _ptr(out_d), ctypes.byref(cnt), err, ctypes.c_int(512))
    if rc != 0:
        raise RuntimeError("reference kernel: " + err.value.decode())
    m = cnt.value
    return out_q[:m].copy(), out_p[:m].copy(), out_d[:m].copy()


def ref_eps_kernels(x_reordered: np.ndarray, di: int, k: int, beta: float):
    """Runs the reference's epsilon-estimator kernels (kernel.cu:343-381 and
    450-523) on the GPU with their launch shapes (GPU.cu:3275, 3434); the
    histogram kernel gets the oracle's mean and bucket width.  Returns
    (oracle estimate, reference histogram[10001], reference distance total,
    reference pair count)."""
    x = np.ascontiguousarray(x_reordered)
    n, d = x.shape
    cubin = ref_kernel_cubin(x.dtype, d, di)
    if not os.path.exists(cubin):
        raise FileNotFoundError(cubin)
    if not os.path.exists(_RK_PATH):
        build(force=True)
    est = estimate_eps(x, k, beta)
    hist = np.zeros(10001, np.uint32)
    total = ctypes.c_double(0.0)
    cnt = ctypes.c_ulonglong(0)
    err = ctypes.create_string_buffer(512)
    rk = ctypes.CDLL(_RK_PATH)
    rc = rk.refk_eps(cubin.encode(), ctypes.c_int(x.dtype.itemsize), _ptr(x), ctypes.c_uint64(n), ctypes.c_uint32(d),
                     ctypes.c_double(est["avg"]), ctypes.c_double(est["bucket_width"]), ctypes.c_uint32(est["offset"]),
                     _ptr(hist), ctypes.byref(total), ctypes.byref(cnt), err, ctypes.c_int(512))
    if rc != 0:
        raise RuntimeError("reference eps kernels: " + err.value.decode())
    return est, hist, total.value, cnt.value
