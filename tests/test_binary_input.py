"""Binary input (knnsj_read_binary): .npy files of either float type and raw
little-endian values read back exactly, with the CSV reader's rule that a
trailing partial point is dropped.  Host-only: no GPU needed."""
import os

import numpy as np
import pytest

import hybrid_k_nearest_neighbor_self_join_gb300 as kj
from hybrid_k_nearest_neighbor_self_join_gb300 import _lib


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


@pytest.mark.parametrize("src,dst", [(np.float32, np.float32), (np.float64, np.float64),
                                     (np.float64, np.float32), (np.float32, np.float64)])
def test_npy_roundtrip(tmp_path, src, dst):
    x = np.random.default_rng(3).standard_normal((100_003, 3)).astype(src)
    p = os.path.join(tmp_path, "pts.npy")
    np.save(p, x)
    y = kj.read_binary(p, 3, dst)
    assert y.shape == x.shape and y.dtype == dst
    assert np.array_equal(y, x.astype(dst))


def test_raw_and_partial_point(tmp_path):
    x = np.random.default_rng(4).random(3 * 5000 + 2, dtype=np.float64).astype(np.float32)
    p = os.path.join(tmp_path, "pts.bin")
    x.tofile(p)
    y = kj.read_binary(p, 3, np.float32)
    assert y.shape == (5000, 3)
    assert np.array_equal(y.ravel(), x[:15000])


def test_npy_version2_header(tmp_path):
    x = np.arange(12, dtype=np.float64).reshape(4, 3)
    p = os.path.join(tmp_path, "v2.npy")
    with open(p, "wb") as f:
        np.lib.format.write_array(f, x, version=(2, 0))
    assert np.array_equal(kj.read_binary(p, 3, np.float64), x)


def test_rejects_unsupported(tmp_path):
    p = os.path.join(tmp_path, "ints.npy")
    np.save(p, np.arange(10, dtype=np.int32))
    with pytest.raises(_lib.KnnsjError):
        kj.read_binary(p, 2, np.float32)
    p2 = os.path.join(tmp_path, "fortran.npy")
    np.save(p2, np.asfortranarray(np.ones((4, 3), np.float32)))
    with pytest.raises(_lib.KnnsjError):
        kj.read_binary(p2, 3, np.float32)
    with pytest.raises(_lib.KnnsjError):
        kj.read_binary(os.path.join(tmp_path, "missing.npy"), 2, np.float32)
