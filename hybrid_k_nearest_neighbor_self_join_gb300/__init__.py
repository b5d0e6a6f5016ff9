"""GB300-native exact k-nearest-neighbour self-join.

The hot path -- grid index, starting radius from BETA, range search over the
cell ring with the k+1 nearest selected in-kernel, and re-attempts at larger
radii -- runs as hand-written sm_103a CUDA behind the C ABI of
include/knnsj.h.  This module is a thin host-side convenience layer over that
ABI; the reference's own Python interface is mirrored in knnjoingpu.py.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import KnnsjError, Options, Stats

__all__ = ["selfjoin", "selfjoin_device", "selfjoin_batched", "reorder_dims", "grid_dims", "read_csv", "read_binary",
           "write_knn_out", "write_outlier_scores", "version", "KnnsjError", "Options", "Stats"]


def _dtype_code(dt) -> int:
    dt = np.dtype(dt)
    if dt == np.float32:
        return _lib.KNNSJ_F32
    if dt == np.float64:
        return _lib.KNNSJ_F64
    raise TypeError(f"dtype must be float32 or float64, got {dt}")


def version() -> str:
    return _lib.load().knnsj_version().decode()


RADIUS_PLAIN = _lib.KNNSJ_RADIUS_BETA
RADIUS_LEARNED = _lib.KNNSJ_RADIUS_LEARNED


def selfjoin(data: np.ndarray, k: int, *, num_indexed_dims: int = 0, beta: float | None = None,
             reorder: bool = True, radius_mode: int = 0, max_iterations: int = 0, device: int = -1,
             radius_offset: float = 0.0, out_ids: np.ndarray | None = None,
             out_dists: np.ndarray | None = None, return_stats: bool = False, device_table_mb: int = 0):
    """Exact kNN self-join of row-major host data (N x d, float32/float64).

    Returns (ids, dists), each (N, k+1): row q holds the k+1 nearest points of
    point q, itself included, by ascending distance (ties by id).
    radius_mode: RADIUS_PLAIN (the reference's BETA rule) or RADIUS_LEARNED.
    """
    x = np.ascontiguousarray(data)
    if x.ndim != 2:
        raise ValueError("data must be 2-D (N x d)")
    n, d = x.shape
    K = k + 1
    ids = out_ids if out_ids is not None else np.empty((n, K), np.int32)
    dists = out_dists if out_dists is not None else np.empty((n, K), x.dtype)
    opts = Options.make(num_indexed_dims, beta, reorder, radius_mode, max_iterations, device,
                        radius_offset=radius_offset, device_table_mb=device_table_mb)
    st = Stats.make()
    lib = _lib.load()
    rc = lib.knnsj_selfjoin(x.ctypes.data, _dtype_code(x.dtype), n, d, k, ctypes.byref(opts),
                            ids.ctypes.data, dists.ctypes.data, ctypes.byref(st))
    _lib.check(rc, "knnsj_selfjoin")
    return (ids, dists, st.as_dict()) if return_stats else (ids, dists)


def selfjoin_device(data_ptr: int, dtype, n: int, d: int, k: int, ids_ptr: int, dists_ptr: int, *,
                    num_indexed_dims: int = 0, beta: float | None = None, reorder: bool = True,
                    radius_mode: int = 0, max_iterations: int = 0, radius_offset: float = 0.0) -> dict:
    """Self-join on device pointers (e.g. torch.Tensor.data_ptr()); returns stats."""
    opts = Options.make(num_indexed_dims, beta, reorder, radius_mode, max_iterations, -1,
                        radius_offset=radius_offset)
    st = Stats.make()
    rc = _lib.load().knnsj_selfjoin_device(ctypes.c_void_p(data_ptr), _dtype_code(dtype), n, d, k,
                                           ctypes.byref(opts), ctypes.c_void_p(ids_ptr),
                                           ctypes.c_void_p(dists_ptr), ctypes.byref(st))
    _lib.check(rc, "knnsj_selfjoin_device")
    return st.as_dict()


def selfjoin_batched(datasets, ks, *, beta: float | None = None, radius_mode: int = 0):
    """Many independent self-joins in one call; returns [(ids, dists), ...]."""
    datasets = [np.ascontiguousarray(x) for x in datasets]
    if not datasets:
        return []
    dt = datasets[0].dtype
    sets = (_lib.Set * len(datasets))()
    outs = []
    for i, (x, k) in enumerate(zip(datasets, ks)):
        if x.dtype != dt:
            raise TypeError("all datasets must share one dtype")
        n, d = x.shape
        ids = np.empty((n, k + 1), np.int32)
        dists = np.empty((n, k + 1), dt)
        outs.append((ids, dists))
        sets[i].data = x.ctypes.data
        sets[i].n = n
        sets[i].d = d
        sets[i].k = k
        sets[i].out_ids = ids.ctypes.data
        sets[i].out_dists = dists.ctypes.data
    opts = Options.make(0, beta, True, radius_mode)
    st = Stats.make()
    rc = _lib.load().knnsj_selfjoin_batched(len(datasets), sets, _dtype_code(dt), ctypes.byref(opts),
                                            ctypes.byref(st))
    _lib.check(rc, "knnsj_selfjoin_batched")
    return outs


def get_radius_model() -> np.ndarray:
    """The active learned-radius model (5873 floats)."""
    m = np.empty(_lib.RADIUS_MODEL_FLOATS, np.float32)
    _lib.check(_lib.load().knnsj_get_radius_model(m.ctypes.data))
    return m


def set_radius_model(model: np.ndarray | None) -> None:
    """Replaces the active learned-radius model; None restores the built-in one."""
    if model is None:
        _lib.check(_lib.load().knnsj_set_radius_model(None))
        return
    m = np.ascontiguousarray(model, np.float32)
    if m.size != _lib.RADIUS_MODEL_FLOATS:
        raise ValueError("model must have 5873 floats")
    _lib.check(_lib.load().knnsj_set_radius_model(m.ctypes.data))


def reorder_dims(data: np.ndarray):
    """Dimension order of ReorderByDimension and the sorted variances."""
    x = np.ascontiguousarray(data)
    n, d = x.shape
    perm = np.zeros(d, np.uint32)
    var = np.zeros(d, x.dtype)
    _lib.check(_lib.load().knnsj_reorder_dims(x.ctypes.data, _dtype_code(x.dtype), n, d, perm.ctypes.data,
                                              var.ctypes.data))
    return perm, var


def grid_dims(data: np.ndarray, num_indexed_dims: int, eps: float):
    x = np.ascontiguousarray(data)
    n, d = x.shape
    mn = np.zeros(num_indexed_dims, x.dtype)
    mx = np.zeros(num_indexed_dims, x.dtype)
    nc = np.zeros(num_indexed_dims, np.uint32)
    tot = ctypes.c_uint64(0)
    _lib.check(_lib.load().knnsj_grid_dims(x.ctypes.data, _dtype_code(x.dtype), n, d, num_indexed_dims,
                                           float(eps), mn.ctypes.data, mx.ctypes.data, nc.ctypes.data,
                                           ctypes.byref(tot)))
    return mn, mx, nc, tot.value


def read_csv(path: str, d: int, dtype=np.float32) -> np.ndarray:
    lib = _lib.load()
    n = ctypes.c_uint64(0)
    code = _dtype_code(dtype)
    _lib.check(lib.knnsj_read_csv(path.encode(), code, d, None, ctypes.byref(n)), path)
    out = np.empty((n.value, d), dtype)
    _lib.check(lib.knnsj_read_csv(path.encode(), code, d, out.ctypes.data, ctypes.byref(n)), path)
    return out


def read_binary(path: str, d: int, dtype=np.float32) -> np.ndarray:
    """Points from a .npy file or raw little-endian values (knnsj_read_binary)."""
    lib = _lib.load()
    n = ctypes.c_uint64(0)
    code = _dtype_code(dtype)
    _lib.check(lib.knnsj_read_binary(path.encode(), code, d, None, ctypes.byref(n)), path)
    out = np.empty((n.value, d), dtype)
    _lib.check(lib.knnsj_read_binary(path.encode(), code, d, out.ctypes.data, ctypes.byref(n)), path)
    return out


def write_knn_out(directory: str, ids: np.ndarray, dists: np.ndarray) -> None:
    ids = np.ascontiguousarray(ids, np.int32)
    dists = np.ascontiguousarray(dists)
    n, K = ids.shape
    _lib.check(_lib.load().knnsj_write_knn_out(directory.encode(), n, K, ids.ctypes.data,
                                               dists.ctypes.data, _dtype_code(dists.dtype)))


def outlier_scores_device(ids_ptr: int, dists_ptr: int, dtype, n: int, K: int, mean_ptr: int, dist_rank_ptr: int,
                          in_degree_ptr: int, degree_rank_ptr: int) -> None:
    """Outlier scores of a device-resident result table (knnsj_outlier_scores_device);
    all pointers are device pointers (e.g. torch.Tensor.data_ptr())."""
    _lib.check(_lib.load().knnsj_outlier_scores_device(
        ctypes.c_void_p(ids_ptr), ctypes.c_void_p(dists_ptr), _dtype_code(dtype), n, K, ctypes.c_void_p(mean_ptr),
        ctypes.c_void_p(dist_rank_ptr), ctypes.c_void_p(in_degree_ptr), ctypes.c_void_p(degree_rank_ptr)),
        "knnsj_outlier_scores_device")


def write_outlier_scores(directory: str, ids: np.ndarray, dists: np.ndarray) -> None:
    ids = np.ascontiguousarray(ids, np.int32)
    dists = np.ascontiguousarray(dists)
    n, K = ids.shape
    _lib.check(_lib.load().knnsj_write_outlier_scores(directory.encode(), n, K, ids.ctypes.data,
                                                      dists.ctypes.data, _dtype_code(dists.dtype)))
