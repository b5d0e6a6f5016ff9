"""The CPU oracle against fixtures produced by the reference's own host code
(tests/golden/make_golden.py) and against the brute-force definition."""
import os

import numpy as np
import pytest

import oracle

TAGS = ["float_2_2", "double_6_6", "float_5_3"]


@pytest.mark.parametrize("tag", TAGS)
def test_reorder_matches_reference(golden_dir, tag):
    z = np.load(os.path.join(golden_dir, f"prep_{tag}.npz"))
    perm, _ = oracle.reorder(z["data"])
    assert np.array_equal(z["data"][:, perm], z["reordered"])


@pytest.mark.parametrize("tag", TAGS)
def test_grid_matches_reference(golden_dir, tag):
    z = np.load(os.path.join(golden_dir, f"prep_{tag}.npz"))
    di = int(z["num_indexed_dims"])
    g = oracle.grid(z["reordered"], di, float(z["eps"]))
    assert np.array_equal(g["minArr"], z["minArr"])
    assert np.array_equal(g["nCells"], z["nCells"])
    assert g["totalCells"] == int(z["totalCells"][0])
    assert np.array_equal(g["cellKeys"], z["cellKeys"])
    assert np.array_equal(np.arange(len(z["cellKeys"]), dtype=np.uint32), z["cellIdx"])
    assert np.array_equal(g["indexmin"], z["indexmin"])
    assert np.array_equal(g["indexmax"], z["indexmax"])
    assert np.array_equal(g["lookup"], z["lookup"])


def _check_against_bruteforce(x, k, di, beta, stride):
    rc, ids, dists, st = oracle.join(x, k, di=di, beta=beta)
    assert rc == 0
    assert (ids >= 0).all()
    perm = np.array(st.perm[: x.shape[1]])
    q = np.arange(0, x.shape[0], stride, dtype=np.uint32)
    bi, bd = oracle.bruteforce(x[:, perm], k + 1, q)
    assert np.array_equal(ids[q], bi)
    assert np.array_equal(dists[q], bd)
    return st


def test_join_uniform2d_equals_definition():
    x = np.random.default_rng(0).random((20000, 2), dtype=np.float32)
    st = _check_against_bruteforce(x, 8, 2, 0.0, 7)
    assert st.iterations >= 2  # BETA=0 leaves about half the queries short


def test_join_gmm6d_equals_definition(golden_dir):
    z = np.load(os.path.join(golden_dir, "prep_double_6_6.npz"))
    _check_against_bruteforce(z["data"], 16, 6, 0.05, 3)


def test_join_partial_index_equals_definition(golden_dir):
    z = np.load(os.path.join(golden_dir, "prep_float_5_3.npz"))
    _check_against_bruteforce(z["data"], 10, 3, 0.05, 3)


def test_join_duplicates_and_clumps(golden_dir):
    z = np.load(os.path.join(golden_dir, "prep_float_2_2.npz"))
    _check_against_bruteforce(z["data"], 32, 2, 0.025, 1)


def test_join_k_too_large():
    x = np.random.default_rng(1).random((50, 2), dtype=np.float32)
    rc, *_ = oracle.join(x, 50, di=2)
    assert rc == 3


def test_eps_zero_for_tiny_inputs():
    # N <= 1000: the reference's mean-distance sample pairs point 0 with
    # itself only, so the estimate is 0 (its grid would divide by zero).
    x = np.random.default_rng(2).random((900, 2), dtype=np.float32)
    rc, *_ = oracle.join(x, 4, di=2)
    assert rc == 10


def test_eps_offset_rounding():
    # GPU.cu:3400-3412 in double: for N = 25e6 the sample offset truncates
    # to 49999, not 50000; the oracle follows the same double arithmetic.
    assert int(1.0 / ((50000.0 / 25000000) * 0.01)) == 49999
    x = np.random.default_rng(3).random((100000, 2), dtype=np.float32)
    e = oracle.estimate_eps(x, 8, 0.0)
    assert e["offset"] == int(1.0 / ((50000.0 / 100000) * 0.01))
    assert e["hist"].sum() % 8 == 0
