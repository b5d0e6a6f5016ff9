"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

The bar is bit-exact: identical neighbour ids and identical distance bits in
every row (both order ties by point id).  Full-size configurations are
checked through size-independent properties plus a brute-force sample.
"""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
import hybrid_k_nearest_neighbor_self_join_gb300 as kj
from hybrid_k_nearest_neighbor_self_join_gb300 import _lib, datasets

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()
    __graft_entry__.build_oracle()


def assert_same(ids, dists, oids, odists):
    bad = np.nonzero((ids != oids).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} rows differ in ids, first {bad[:5]}: {ids[bad[0]]} vs {oids[bad[0]]}"
    ib = dists.view(np.uint32 if dists.dtype == np.float32 else np.uint64)
    ob = odists.view(np.uint32 if odists.dtype == np.float32 else np.uint64)
    bad = np.nonzero((ib != ob).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} rows differ in distance bits, first {bad[:5]}"


def gpu_vs_oracle(x, k, di, beta, **kw):
    ids, dists, st = kj.selfjoin(x, k, num_indexed_dims=di, beta=beta, return_stats=True, **kw)
    rc, oids, odists, ost = oracle.join(x, k, di=di, beta=beta)
    assert rc == 0
    assert_same(ids, dists, oids, odists)
    assert st["eps0"] == ost.eps0
    assert list(st["perm"][: x.shape[1]]) == list(ost.perm[: x.shape[1]])
    return ids, dists, st


def fp64_check(x, perm, ids, dists, queries):
    """Independent FP64 check: every returned neighbour is at least as close
    (in exact double arithmetic, up to float rounding) as every point left out."""
    xd = x[:, perm].astype(np.float64)
    K = ids.shape[1]
    for q in queries:
        d2 = ((xd - xd[q]) ** 2).sum(axis=1)
        ret = ids[q]
        inside = np.sqrt(d2[ret]).max()
        mask = np.ones(len(x), bool)
        mask[ret] = False
        outside = np.sqrt(d2[mask]).min() if mask.any() else np.inf
        tol = 1e-5 * max(inside, 1e-30) if x.dtype == np.float32 else 1e-12 * max(inside, 1e-300)
        assert inside <= outside + tol, (q, inside, outside)
        assert len(set(ret.tolist())) == K


def test_smoke():
    import __graft_entry__
    __graft_entry__.smoke()


def test_uniform2d_100k_k8_beta0():
    x = datasets.uniform(100_000, 2, 0)
    ids, dists, st = gpu_vs_oracle(x, 8, 2, 0.0)
    assert st["iterations"] >= 2
    fp64_check(x, np.array(st["perm"][:2]), ids, dists, range(0, 100_000, 997))


def test_sky_like_scaled_k64():
    x = datasets.sky_like(300_000, seed=7)
    gpu_vs_oracle(x, 64, 2, 0.025)


def test_gmm6d_double_k16():
    x = datasets.gmm(60_000, 6, 20, 0.1, seed=8, dtype=np.float64)
    ids, dists, st = gpu_vs_oracle(x, 16, 6, 0.05)
    fp64_check(x, np.array(st["perm"][:6]), ids, dists, range(0, 60_000, 2999))


def test_partial_index_d5_di3():
    x = datasets.gmm(50_000, 5, 10, 0.2, seed=9, dtype=np.float32)
    gpu_vs_oracle(x, 10, 3, 0.05)


def test_duplicates_and_clumps(golden_dir):
    x = np.load(os.path.join(golden_dir, "prep_float_2_2.npz"))["data"]
    gpu_vs_oracle(x, 32, 2, 0.025)


def test_k128_4d():
    x = datasets.heldout4d(80_000, seed=10)
    gpu_vs_oracle(x, 128, 4, 0.05)


@pytest.mark.parametrize("dtype,k", [(np.float32, 4095), (np.float32, 16351), (np.float64, 3000),
                                     (np.float64, 8159)])
def test_large_k(dtype, k):
    # k+1 beyond 2048 (the reference has no cap on k): one warp per block
    # with a selection buffer of up to 128 KB, the largest k+1 each type takes
    n = max(12_000, k + 2_000)
    x = datasets.gmm(n, 2, 6, 0.3, seed=k, dtype=dtype)
    gpu_vs_oracle(x, k, 2, 0.0)


def test_generic_dimension_path_d12():
    x = datasets.gmm(20_000, 12, 5, 0.3, seed=11, dtype=np.float32)
    gpu_vs_oracle(x, 8, 4, 0.05)


def test_double_2d():
    x = datasets.uniform(50_000, 2, 12, dtype=np.float64)
    gpu_vs_oracle(x, 20, 2, 0.1)


@pytest.mark.parametrize("offset", [0.0, 3.0e5])
def test_double_float_prefilter_bound(offset):
    # double data far from the origin: rounding the coordinates to float moves
    # distances by more than the distances themselves, so the float prefilter
    # must let every candidate through to the exact double test; near the
    # origin it rejects most of them.  Both must keep the oracle's rows.
    x = datasets.gmm(30_000, 4, 8, 0.2, 22, dtype=np.float64) * 1e-3 + offset
    gpu_vs_oracle(x, 12, 4, 0.05)


def test_dense_and_sparse_cell_lookup_agree(monkeypatch):
    x = datasets.sky_like(100_000, seed=13)
    monkeypatch.setenv("KNNSJ_DENSE", "0")
    a = kj.selfjoin(x, 16, beta=0.025)
    monkeypatch.setenv("KNNSJ_DENSE", "2")
    b = kj.selfjoin(x, 16, beta=0.025)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("mode", [kj.RADIUS_PLAIN, kj.RADIUS_LEARNED])
def test_graph_passes_match_host_passes(monkeypatch, mode):
    # retry passes inside the conditional CUDA graph against host-driven
    # passes: same rows, same pass count, rebuilds and candidates
    x = datasets.gmm(200_000, 4, 30, 0.2, 21, dtype=np.float32)
    out = {}
    for g in ("0", "1"):
        monkeypatch.setenv("KNNSJ_GRAPH", g)
        out[g] = kj.selfjoin(x, 32, beta=0.0, radius_mode=mode, return_stats=True)
    (a_i, a_d, a_s), (b_i, b_d, b_s) = out["0"], out["1"]
    assert np.array_equal(a_i, b_i) and np.array_equal(a_d, b_d)
    assert a_s["iterations"] > 2
    for key in ("iterations", "regrids", "candidates", "queries_run", "eps_final"):
        assert a_s[key] == b_s[key], key


@pytest.mark.parametrize("tail", ["0", "1"])
def test_far_outliers(monkeypatch, tail):
    # a tight 6-D cluster and a few far outliers: the outliers' radii grow
    # far past the cluster's.  Tail "0": the grid is rebuilt for the largest
    # radius (rings stay within the row cap); tail "1": the last few queries
    # are finished by an exact scan over all points.  Rows match brute force.
    monkeypatch.setenv("KNNSJ_TAIL_BRUTE", tail)
    rng = np.random.default_rng(23)
    c = rng.normal(0.0, 0.01, (40_000, 6)).astype(np.float32)
    o = rng.uniform(-1.0, 1.0, (12, 6)).astype(np.float32)
    x = np.concatenate([c, o])
    ids, dists, st = kj.selfjoin(x, 16, beta=0.05, radius_mode=kj.RADIUS_LEARNED, return_stats=True)
    if tail == "0":
        assert st["regrids"] >= 1
    perm, _ = kj.reorder_dims(x)
    q = np.concatenate([np.arange(40_000, 40_012), np.arange(0, 40_000, 997)])
    bi, bd = oracle.bruteforce(x[:, perm], 17, q)
    assert_same(ids[q], dists[q], bi, bd)


@pytest.mark.parametrize("dtype,mode", [(np.float32, kj.RADIUS_PLAIN), (np.float64, kj.RADIUS_LEARNED)])
def test_sparse_tail_matches_ring_search(monkeypatch, dtype, mode):
    # 2-D clumps with a few isolated points: the same rows whether the last
    # queries are finished by the exact scan (forced at the first due
    # rebuild) or by rebuilt grids
    rng = np.random.default_rng(24)
    c = (rng.normal(0.0, 0.002, (60_000, 2)) + rng.integers(0, 4, (60_000, 1)) * 0.01).astype(dtype)
    o = rng.uniform(-1.0, 1.0, (7, 2)).astype(dtype)
    x = np.concatenate([c, o])
    out = {}
    for tail in ("0", "2"):
        monkeypatch.setenv("KNNSJ_TAIL_BRUTE", tail)
        out[tail] = kj.selfjoin(x, 24, beta=0.0, radius_mode=mode)
    assert np.array_equal(out["0"][0], out["2"][0]) and np.array_equal(out["0"][1], out["2"][1])
    perm, _ = kj.reorder_dims(x)
    q = np.arange(60_000, 60_007)
    bi, bd = oracle.bruteforce(x[:, perm], 25, q)
    assert_same(out["2"][0][q], out["2"][1][q], bi, bd)


def test_tiny_input_eps_fallback():
    # N <= 1000: the reference's sampled mean distance is 0 and its grid
    # divides by zero; the GPU path picks a positive width and stays exact.
    x = datasets.uniform(700, 3, 14)
    ids, dists = kj.selfjoin(x, 5)
    perm, _ = kj.reorder_dims(x)
    bi, bd = oracle.bruteforce(x[:, perm], 6, np.arange(700))
    assert_same(ids, dists, bi, bd)


def test_k_equals_n_minus_1():
    x = datasets.uniform(1500, 2, 15)
    ids, dists = kj.selfjoin(x, 1499)
    perm, _ = kj.reorder_dims(x)
    q = np.arange(0, 1500, 37)
    bi, bd = oracle.bruteforce(x[:, perm], 1500, q)
    assert_same(ids[q], dists[q], bi, bd)


def test_nonfinite_input_is_rejected():
    x = datasets.uniform(5000, 2, 16)
    x[123, 1] = np.nan
    with pytest.raises(_lib.KnnsjError) as e:
        kj.selfjoin(x, 4)
    assert e.value.status == 4


def test_device_pointer_api_matches_host_api():
    torch = pytest.importorskip("torch")
    x = datasets.uniform(40_000, 2, 17)
    h_ids, h_d = kj.selfjoin(x, 12, beta=0.05)
    t = torch.from_numpy(x).cuda()
    ids = torch.empty((40_000, 13), dtype=torch.int32, device="cuda")
    d = torch.empty((40_000, 13), dtype=torch.float32, device="cuda")
    kj.selfjoin_device(t.data_ptr(), np.float32, 40_000, 2, 12, ids.data_ptr(), d.data_ptr(), beta=0.05)
    torch.cuda.synchronize()
    assert np.array_equal(ids.cpu().numpy(), h_ids)
    assert np.array_equal(d.cpu().numpy(), h_d)


def test_repeated_calls_reuse_workspace():
    x = datasets.uniform(30_000, 2, 18)
    a = kj.selfjoin(x, 8)
    y = datasets.uniform(90_000, 3, 19)
    kj.selfjoin(y, 4)
    b = kj.selfjoin(x, 8)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_python_dropin_wrapper():
    from hybrid_k_nearest_neighbor_self_join_gb300 import knnjoingpu
    x = datasets.uniform(20_000, 2, 20)
    for dt, npdt in (("float", np.float32), ("double", np.float64)):
        xs = x.astype(npdt)
        ids, dists = knnjoingpu.knnjoin(xs.flatten().tolist(), 5, 2, dt)
        assert ids.shape == (20_000 * 6,) and dists.dtype == npdt
        rc, oids, odists, _ = oracle.join(xs, 5, di=2, beta=0.05)
        assert np.array_equal(ids.reshape(-1, 6), oids)
        assert np.array_equal(dists.reshape(-1, 6), odists)


def test_cli_main_writes_knn_out():
    x = datasets.uniform(5000, 2, 21)
    exe = os.path.join(ROOT, "hybrid_k_nearest_neighbor_self_join_gb300", "_build", "main")
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "in.csv")
        np.savetxt(p, x, delimiter=",", fmt="%.9g")
        xr = kj.read_csv(p, 2, np.float32)
        env = dict(os.environ, KNNSJ_PRINTNEIGHBORTABLE="1")
        r = subprocess.run([exe, p, "2", "6"], cwd=t, env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        assert "[Verification] Total distance (without square root)" in r.stdout
        rc, oids, odists, _ = oracle.join(xr, 6, di=2, beta=0.05)
        ref_dir = os.path.join(t, "ref")
        os.makedirs(ref_dir)
        kj.write_knn_out(ref_dir, oids, odists)
        for name in ("KNN_out.txt", "KNN_out_distances.txt"):
            assert open(os.path.join(t, name)).read() == open(os.path.join(ref_dir, name)).read()


def _row_properties(ids, dists, n):
    assert (ids >= 0).all() and (ids < n).all()
    assert (np.diff(dists, axis=1) >= 0).all()
    s = np.sort(ids, axis=1)
    assert (np.diff(s, axis=1) > 0).all()
    assert (dists[:, 0] == 0).all()


@pytest.mark.parametrize("name", ["sky2d_25m", "gmm6d_10m"])
def test_full_size_properties(name):
    gen, k, beta, di = datasets.CONFIGS[name]
    x = gen()
    n = x.shape[0]
    ids, dists, st = kj.selfjoin(x, k, num_indexed_dims=di, beta=beta, return_stats=True)
    _row_properties(ids, dists, n)
    perm = np.array(st["perm"][: x.shape[1]])
    q = np.random.default_rng(0).choice(n, 48, replace=False).astype(np.uint32)
    bi, bd = oracle.bruteforce(x[:, perm], k + 1, q)
    assert_same(ids[q], dists[q], bi, bd)
