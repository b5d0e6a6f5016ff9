"""The reference's own range-search kernel, run on the GPU, against the oracle.

oracle/build_ref_kernel.sh compiles the reference's kernel.cu
(kernelNDGridIndexGlobalkNN with evaluateCell and evalPoint, kernel.cu:61-225)
from its sources into a cubin wherever the reference is present;
oracle/ref_kernel_runner.cpp launches it with the grid index the oracle
builds (itself pinned against the reference's host code in
test_oracle_golden.py).  Every (query, point, distance) the reference kernel
reports within epsilon must equal, bit for bit, the oracle's brute-force
range query under the same rule -- which pins the oracle's distance
arithmetic (the fma chain over the reordered dimensions), its square root
and its within-epsilon test on the reference kernel itself, and the GPU
parity tests carry that to this library's kernels.
"""
import os

import numpy as np
import pytest

import oracle
from hybrid_k_nearest_neighbor_self_join_gb300 import datasets

pytestmark = pytest.mark.gpu

# (dtype, GPUNUMDIM, NUMINDEXEDDIM, points, k, BETA, generator)
CASES = [
    ("float", 2, 2, 20_000, 8, 0.025, lambda n: datasets.sky_like(n, seed=41)),
    ("float", 4, 4, 16_000, 32, 0.05, lambda n: datasets.gmm(n, 4, 12, 0.2, 42, dtype=np.float32)),
    ("float", 5, 3, 16_000, 16, 0.05, lambda n: datasets.uniform(n, 5, 43)),
    ("double", 6, 6, 12_000, 16, 0.05, lambda n: datasets.gmm(n, 6, 20, 0.1, 44, dtype=np.float64)),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}_{c[1]}_{c[2]}")
def test_reference_kernel_pairs_equal_oracle_range(case):
    dtype, d, di, n, k, beta, gen = case
    np_dtype = np.float32 if dtype == "float" else np.float64
    cubin = oracle.ref_kernel_cubin(np_dtype, d, di)
    if not os.path.exists(cubin):
        pytest.skip("reference kernel cubin not built (the reference sources were absent when build() ran)")
    x = np.ascontiguousarray(gen(n), dtype=np_dtype)
    perm, _ = oracle.reorder(x)
    xr = np.ascontiguousarray(x[:, perm])
    eps = float(np_dtype(oracle.estimate_eps(xr, k, beta)["eps0"]))
    q, p, dist = oracle.ref_kernel_pairs(xr, di, eps)
    assert q.size > n  # every point finds itself, most find more
    ref_counts = np.bincount(q, minlength=n)
    counts, ids, dists = oracle.range_query(xr, eps, np.arange(n), maxper=int(ref_counts.max()) * 2 + 64)
    assert np.array_equal(ref_counts, counts)
    # both sides in (distance, id) order: the reference appends in atomic order
    o = np.lexsort((p, dist, q))
    ref_ids, ref_d = p[o], dist[o]
    rows = np.repeat(np.arange(n), counts)
    cols = np.concatenate([np.arange(c) for c in counts])
    orc_ids, orc_d = ids[rows, cols], dists[rows, cols]
    o2 = np.lexsort((orc_ids, orc_d, rows))
    orc_ids, orc_d = orc_ids[o2], orc_d[o2]
    assert np.array_equal(ref_ids, orc_ids)
    ub = np.uint32 if np_dtype == np.float32 else np.uint64
    assert np.array_equal(ref_d.view(ub), orc_d.view(ub))


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}_{c[1]}_{c[2]}")
def test_reference_eps_kernels_equal_oracle(case):
    # the histogram's integer counts exactly (same mean and bucket width
    # given); the mean's pair count exactly and its double sum to rounding
    # (the reference adds it with atomics in no fixed order)
    dtype, d, di, n, k, beta, gen = case
    np_dtype = np.float32 if dtype == "float" else np.float64
    if not os.path.exists(oracle.ref_kernel_cubin(np_dtype, d, di)):
        pytest.skip("reference kernel cubin not built (the reference sources were absent when build() ran)")
    n = (n // 256) * 256  # whole 256-point strides: the histogram kernel reads no point past N
    x = np.ascontiguousarray(gen(n), dtype=np_dtype)
    perm, _ = oracle.reorder(x)
    xr = np.ascontiguousarray(x[:, perm])
    est, hist, total, cnt = oracle.ref_eps_kernels(xr, di, k, beta)
    assert cnt == est["pair_count"]
    assert abs(total / cnt - est["avg"]) <= 1e-12 * est["avg"]
    assert np.array_equal(hist[:10000], est["hist"])
    assert hist[:10000].sum() > 0
