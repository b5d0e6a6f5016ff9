"""The C-ABI library without a GPU: it loads, exports every function declared
in include/knnsj.h, its host-side pieces match the reference's own host code
(golden fixtures), and argument errors are reported before any device work."""
import ctypes
import os
import re
import tempfile

import numpy as np
import pytest

from hybrid_k_nearest_neighbor_self_join_gb300 import _lib
import hybrid_k_nearest_neighbor_self_join_gb300 as kj

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TAGS = ["float_2_2", "double_6_6", "float_5_3"]


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "knnsj.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(",
                           text, flags=re.M))
    names.discard("defined")
    return sorted(names)


@pytest.mark.parametrize("libname", ["libknnsj.so", "libknnsj_double.so", "libgpuknnselfjoin.so"])
def test_exports_every_declared_function(libname):
    names = declared_functions()
    assert "KNNJoinPy" in names and "knnsj_selfjoin" in names and len(names) >= 13
    lib = ctypes.CDLL(_lib.library_path(libname))
    for n in names:
        assert hasattr(lib, n), n


def test_version_and_build_dtype():
    lib = _lib.load()
    assert lib.knnsj_version().decode().startswith("knnsj")
    assert lib.knnsj_build_dtype() == _lib.KNNSJ_F32
    assert _lib.load("libknnsj_double.so").knnsj_build_dtype() == _lib.KNNSJ_F64
    assert lib.knnsj_status_string(3).decode() == "k+1 exceeds the number of points"


@pytest.mark.parametrize("tag", TAGS)
def test_reorder_dims_matches_reference(golden_dir, tag):
    z = np.load(os.path.join(golden_dir, f"prep_{tag}.npz"))
    perm, _ = kj.reorder_dims(z["data"])
    assert np.array_equal(z["data"][:, perm], z["reordered"])


@pytest.mark.parametrize("tag", TAGS)
def test_grid_dims_matches_reference(golden_dir, tag):
    z = np.load(os.path.join(golden_dir, f"prep_{tag}.npz"))
    di = int(z["num_indexed_dims"])
    mn, mx, nc, tot = kj.grid_dims(z["reordered"], di, float(z["eps"]))
    assert np.array_equal(mn, z["minArr"])
    assert np.array_equal(mx, z["maxArr"])
    assert np.array_equal(nc, z["nCells"])
    assert tot == int(z["totalCells"][0])


def test_read_csv_matches_reference(golden_dir):
    pts = kj.read_csv(os.path.join(golden_dir, "csv_input.csv"), 2, np.float32)
    ref = np.load(os.path.join(golden_dir, "csv_float_2_2.npz"))["points"]
    assert pts.shape == ref.shape
    assert np.array_equal(pts, ref)


def test_read_csv_large_parallel_roundtrip():
    x = np.random.default_rng(5).random((200_000, 3)).astype(np.float32)
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "d.csv")
        with open(p, "w") as f:
            for row in x:
                f.write(",".join(repr(float(v)) for v in row) + "\n")
        y = kj.read_csv(p, 3, np.float32)
    assert np.array_equal(x, y)


def test_read_csv_missing_file():
    with pytest.raises(_lib.KnnsjError) as e:
        kj.read_csv("/nonexistent/file.csv", 2)
    assert e.value.status == 11


def test_knn_out_and_outlier_text_match_reference(golden_dir):
    z = np.load(os.path.join(golden_dir, "print_input.npz"))
    with tempfile.TemporaryDirectory() as t:
        kj.write_knn_out(t, z["ids"], z["dists"])
        kj.write_outlier_scores(t, z["ids"], z["dists"])
        for name in ("KNN_out.txt", "KNN_out_distances.txt", "KNN_outlier_scores.txt"):
            got = open(os.path.join(t, name)).read()
            want = open(os.path.join(golden_dir, "print_" + name)).read()
            assert got == want, name


def _call(data, n, d, k, opts=None, dtype=_lib.KNNSJ_F32):
    lib = _lib.load()
    ids = np.zeros(max(1, n * (k + 1)), np.int32)
    dists = np.zeros(max(1, n * (k + 1)), np.float32)
    o = opts or _lib.Options.make()
    st = _lib.Stats.make()
    ptr = data.ctypes.data if data is not None else None
    return lib.knnsj_selfjoin(ptr, dtype, n, d, k, ctypes.byref(o), ids.ctypes.data, dists.ctypes.data,
                              ctypes.byref(st))


def test_argument_errors_without_device():
    x = np.random.default_rng(0).random((100, 2), dtype=np.float32)
    assert _call(x, 100, 2, 100) == 3            # k+1 > N
    assert _call(x, 0, 2, 1) == 1                # empty
    assert _call(None, 100, 2, 4) == 1           # null data
    assert _call(x, 100, 0, 4) == 1              # d == 0
    assert _call(x, 100, 300, 4) == 1            # d > 256
    assert _call(x, 100, 2, 4, _lib.Options.make(beta=1.5)) == 1
    y = np.zeros((100, 9), np.float32)
    assert _call(y, 100, 9, 4, _lib.Options.make(num_indexed_dims=9)) == 10   # NUMINDEXEDDIM > 8
    assert _call(x, 100, 2, 4, dtype=7) == 1


def test_k_cap_by_dtype_without_device():
    # each query's selection lives in one warp's shared-memory buffer: k+1 up
    # to 16352 for float data, 8160 for double (checked before any device
    # work: the tiny output buffers are never touched)
    lib = _lib.load()
    n = 20_000
    x32 = np.zeros((n, 2), np.float32)
    x64 = np.zeros((n, 2), np.float64)
    ids = np.zeros(4, np.int32)
    dd = np.zeros(4, np.float64)

    def call(x, dt, k):
        o = _lib.Options.make()
        st = _lib.Stats.make()
        return lib.knnsj_selfjoin(x.ctypes.data, dt, n, 2, k, ctypes.byref(o), ids.ctypes.data, dd.ctypes.data,
                                  ctypes.byref(st))

    assert call(x32, _lib.KNNSJ_F32, 16352) == 10
    assert call(x64, _lib.KNNSJ_F64, 8160) == 10
    assert call(x64, _lib.KNNSJ_F64, 16351) == 10


def test_no_device_is_reported():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    x = np.random.default_rng(0).random((100, 2), dtype=np.float32)
    assert _call(x, 100, 2, 4) == 9
