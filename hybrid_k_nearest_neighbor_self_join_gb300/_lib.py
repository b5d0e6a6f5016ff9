"""ctypes binding of the native library (include/knnsj.h).

The library is built in-tree by build.py.  Nothing here falls back to a
Python or CPU implementation: if the library is missing, loading fails with
an error that says how to build it.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")

KNNSJ_OK = 0
KNNSJ_F32 = 0
KNNSJ_F64 = 1
KNNSJ_RADIUS_BETA = 0
KNNSJ_RADIUS_LEARNED = 1

STATUS_NAMES = {
    0: "KNNSJ_OK", 1: "KNNSJ_ERR_INVALID_ARGUMENT", 2: "KNNSJ_ERR_DIM_MISMATCH",
    3: "KNNSJ_ERR_K_TOO_LARGE", 4: "KNNSJ_ERR_NONFINITE_INPUT", 5: "KNNSJ_ERR_TOO_MANY_POINTS",
    6: "KNNSJ_ERR_NO_CONVERGENCE", 7: "KNNSJ_ERR_CUDA", 8: "KNNSJ_ERR_OUT_OF_MEMORY",
    9: "KNNSJ_ERR_NO_DEVICE", 10: "KNNSJ_ERR_UNSUPPORTED", 11: "KNNSJ_ERR_IO",
    12: "KNNSJ_ERR_EXCEEDS_FIXED_SCRATCH",
}


class KnnsjError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}{': ' + what if what else ''}")


class Options(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("num_indexed_dims", ctypes.c_int32),
        ("beta", ctypes.c_double),
        ("no_reorder", ctypes.c_int32),
        ("radius_mode", ctypes.c_int32),
        ("max_iterations", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("verbose", ctypes.c_int32),
        ("radius_offset", ctypes.c_double),
        ("device_table_mb", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 7),
    ]

    @classmethod
    def make(cls, num_indexed_dims=0, beta=None, reorder=True, radius_mode=0, max_iterations=0,
             device=-1, verbose=0, radius_offset=0.0, device_table_mb=0):
        o = cls()
        o.struct_size = ctypes.sizeof(cls)
        o.num_indexed_dims = int(num_indexed_dims or 0)
        o.beta = -1.0 if beta is None else float(beta)
        o.no_reorder = 0 if reorder else 1
        o.radius_mode = int(radius_mode)
        o.max_iterations = int(max_iterations)
        o.device = int(device)
        o.verbose = int(verbose)
        o.radius_offset = float(radius_offset)
        o.device_table_mb = int(device_table_mb)
        return o


class TrainOptions(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("epochs", ctypes.c_int32),
        ("batch", ctypes.c_uint32),
        ("lr", ctypes.c_float),
        ("quantile", ctypes.c_float),
        ("seed", ctypes.c_uint64),
    ]


RADIUS_FEATURES = 24
RADIUS_MODEL_FLOATS = 5873


class Stats(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("iterations", ctypes.c_int32),
        ("regrids", ctypes.c_int32),
        ("eps_bucket", ctypes.c_int32),
        ("eps0", ctypes.c_double),
        ("eps_final", ctypes.c_double),
        ("avg_distance", ctypes.c_double),
        ("total_distance", ctypes.c_double),
        ("candidates", ctypes.c_uint64),
        ("queries_run", ctypes.c_uint64),
        ("nonempty_cells", ctypes.c_uint64),
        ("ms_total", ctypes.c_double),
        ("ms_prep", ctypes.c_double),
        ("ms_search", ctypes.c_double),
        ("ms_transfer", ctypes.c_double),
        ("perm", ctypes.c_uint32 * 64),
        ("kernel_launches", ctypes.c_uint64),
        ("ms_search_kernels", ctypes.c_double),
        ("search_alg_bytes", ctypes.c_double),
        ("search_alg_flops", ctypes.c_double),
        ("radius_model_error", ctypes.c_double),
        ("tile_handovers", ctypes.c_double),
        ("reserved", ctypes.c_double * 6),
    ]

    @classmethod
    def make(cls):
        s = cls()
        s.struct_size = ctypes.sizeof(cls)
        return s

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            if name in ("struct_size", "reserved"):
                continue
            v = getattr(self, name)
            out[name] = list(v) if name == "perm" else v
        return out


class Set(ctypes.Structure):
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("n", ctypes.c_uint64),
        ("d", ctypes.c_uint32),
        ("k", ctypes.c_uint32),
        ("out_ids", ctypes.c_void_p),
        ("out_dists", ctypes.c_void_p),
        ("status", ctypes.c_int),
    ]


_LIBS: dict = {}

# (name, restype, argtypes) of every function declared in include/knnsj.h
_SIGNATURES = [
    ("knnsj_version", ctypes.c_char_p, []),
    ("knnsj_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("knnsj_build_dtype", ctypes.c_int, []),
    ("KNNJoinPy", None, [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p,
                         ctypes.c_void_p]),
    ("knnsj_selfjoin", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32,
                                      ctypes.c_uint32, ctypes.POINTER(Options), ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.POINTER(Stats)]),
    ("knnsj_selfjoin_device", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64,
                                             ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(Options),
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Stats)]),
    ("knnsj_selfjoin_device_noalloc", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64,
                                                     ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(Options),
                                                     ctypes.c_void_p, ctypes.c_void_p]),
    ("knnsj_selfjoin_batched", ctypes.c_int, [ctypes.c_uint32, ctypes.POINTER(Set), ctypes.c_int,
                                              ctypes.POINTER(Options), ctypes.POINTER(Stats)]),
    ("knnsj_release", None, []),
    ("knnsj_reorder_dims", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.c_void_p, ctypes.c_void_p]),
    ("knnsj_grid_dims", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    ("knnsj_read_csv", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p,
                                      ctypes.POINTER(ctypes.c_uint64)]),
    ("knnsj_read_binary", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_uint64)]),
    ("knnsj_write_knn_out", ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint64, ctypes.c_uint32,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    ("knnsj_write_outlier_scores", ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint64, ctypes.c_uint32,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    ("knnsj_outlier_scores_device", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64,
                                                   ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p, ctypes.c_void_p]),
    ("knnsj_get_radius_model", ctypes.c_int, [ctypes.c_void_p]),
    ("knnsj_set_radius_model", ctypes.c_int, [ctypes.c_void_p]),
    ("knnsj_radius_features", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32,
                                             ctypes.c_uint32, ctypes.POINTER(Options), ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_double)]),
    ("knnsj_radius_predict", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]),
    ("knnsj_radius_grad", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                         ctypes.c_float, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    ("knnsj_radius_train", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                          ctypes.POINTER(TrainOptions), ctypes.c_void_p, ctypes.c_void_p]),
]


def library_path(name: str = "libknnsj.so") -> str:
    return os.path.join(BUILD_DIR, name)


def load(name: str = "libknnsj.so"):
    """Loads (once) and returns the native library with typed signatures."""
    if name in _LIBS:
        return _LIBS[name]
    path = library_path(name)
    if not os.path.exists(path):
        raise RuntimeError(
            f"native library {path} is not built; run "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python hybrid_k_nearest_neighbor_self_join_gb300/build.py`")
    lib = ctypes.CDLL(path)
    for fname, res, args in _SIGNATURES:
        f = getattr(lib, fname)
        f.restype = res
        f.argtypes = args
    _LIBS[name] = lib
    return lib


def check(status: int, what: str = "") -> None:
    if status != KNNSJ_OK:
        raise KnnsjError(status, what)
