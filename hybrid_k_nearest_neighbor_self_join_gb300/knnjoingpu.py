"""Drop-in replacement for the reference's Python wrapper knnjoingpu.py.

Same public functions and arguments as the reference (knnjoingpu.py:146-223):

    ids, dists = knnjoin(DATASET, KNN, NDIM, DTYPE, verbose=False)

DATASET is a flat sequence of N*NDIM numbers (row-major), DTYPE is "float"
or "double"; the result is two flat numpy arrays of N*(KNN+1) neighbour ids
(int32) and distances (float32 / float64), row q at offset q*(KNN+1), the
point itself included.  Like the reference, the library is looked up as
libgpuknnselfjoin.so in the current working directory first
(knnjoingpu.py:173-175); this package's own build is used when none is
there.  The C library's console output is hidden unless verbose=True.
"""
from __future__ import annotations

import csv
import ctypes
import os
import sys

import numpy as np
import numpy.ctypeslib as npct

from . import _lib

__all__ = ["knnjoin", "knnjoinmain", "convert_type", "getColumn", "HideOutput"]


def getColumn(filename, column):
    results = csv.reader(open(filename), delimiter=",")
    return [result[column] for result in results]


def convert_type(in_array, new_dtype):
    """Contiguous numpy array of new_dtype (knnjoingpu.py:18-31)."""
    ret = in_array
    if not isinstance(in_array, np.ndarray):
        ret = np.array(in_array, dtype=new_dtype)
    elif in_array.dtype != new_dtype:
        ret = np.array(ret, dtype=new_dtype)
    if not ret.flags["C_CONTIGUOUS"]:
        ret = np.ascontiguousarray(ret)
    return ret


class HideOutput:
    """Silences file descriptor 1 (the C library's stdout) for its scope."""

    def __enter__(self):
        sys.stdout.flush()
        self._saved = os.dup(1)
        devnull = os.open(os.devnull, os.O_WRONLY)
        os.dup2(devnull, 1)
        os.close(devnull)
        return self

    def __exit__(self, exc_type, exc, tb):
        try:
            libc = ctypes.CDLL(None)
            libc.fflush(None)
        except OSError:
            pass
        os.dup2(self._saved, 1)
        os.close(self._saved)
        return False


def _load_for(dtype_name: str):
    want = _lib.KNNSJ_F32 if dtype_name == "float" else _lib.KNNSJ_F64
    cwd_lib = os.path.join(os.getcwd(), "libgpuknnselfjoin.so")
    candidates = []
    if os.path.exists(cwd_lib):
        candidates.append(cwd_lib)
    candidates += [_lib.library_path("libknnsj.so"), _lib.library_path("libknnsj_double.so")]
    for path in candidates:
        if not os.path.exists(path):
            continue
        lib = ctypes.CDLL(path)
        if not hasattr(lib, "knnsj_build_dtype"):
            continue
        lib.knnsj_build_dtype.restype = ctypes.c_int
        if lib.knnsj_build_dtype() == want:
            return lib
    raise RuntimeError("no libgpuknnselfjoin.so / libknnsj*.so built for DTYPE=%s" % dtype_name)


def knnjoin(DATASET, KNN, NDIM, DTYPE, verbose=False):
    if not verbose:
        with HideOutput():
            return knnjoinmain(DATASET, KNN, NDIM, DTYPE)
    return knnjoinmain(DATASET, KNN, NDIM, DTYPE)


def knnjoinmain(DATASET, KNN, NDIM, DTYPE):
    if DTYPE not in ("float", "double"):
        raise ValueError('DTYPE must be "float" or "double"')
    num_points = int(len(DATASET) / NDIM)
    print("[Python] Number of rows in file: %d" % num_points)
    ctype = ctypes.c_float if DTYPE == "float" else ctypes.c_double
    c_dataset = convert_type(np.asarray(DATASET, dtype=np.float64), ctype)
    out_ids = np.zeros(num_points * (KNN + 1), dtype=ctypes.c_int)
    out_dists = np.zeros(num_points * (KNN + 1), dtype=ctype)
    lib = _load_for(DTYPE)
    arr = npct.ndpointer(dtype=ctype, ndim=1, flags="CONTIGUOUS")
    arr_int = npct.ndpointer(dtype=ctypes.c_int, ndim=1, flags="CONTIGUOUS")
    lib.KNNJoinPy.argtypes = [arr, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, arr_int, arr]
    lib.KNNJoinPy.restype = None
    lib.KNNJoinPy(c_dataset, ctypes.c_uint(num_points), ctypes.c_uint(KNN), ctypes.c_uint(NDIM), out_ids,
                  out_dists)
    print("[Python] Sum of distances to all KNN: %f" % float(np.sum(out_dists)))
    return out_ids, out_dists
