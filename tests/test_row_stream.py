"""Where the rows of host-pointer joins go, and that they are the same rows.

* pinned output buffers (default): a kernel copies the device result table
  into them through their mapped addresses after the join;
* pinned buffers with KNNSJ_DIRECT_ROWS=1: the search kernels write every
  row straight into them (no device result table, no copy);
* pinned buffers with KNNSJ_DIRECT_ROWS=0: rows in blocks of query ids
  copied out while the join runs, later passes' rows patched in at the end;
* pageable buffers whose result table is larger than the device-table cap
  (opts->device_table_mb, the memory-bounded mode): the buffers are registered
  with the device for the call and written directly.
Each must equal a join into ordinary pageable buffers (a device table copied
out in one piece after the join) bit for bit, and its verification sum to
rounding.
"""
import numpy as np
import pytest

import hybrid_k_nearest_neighbor_self_join_gb300 as kj
from hybrid_k_nearest_neighbor_self_join_gb300 import datasets

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def pinned(shape, np_dtype):
    torch = pytest.importorskip("torch")
    tdt = {np.dtype(np.int32): torch.int32, np.dtype(np.float32): torch.float32,
           np.dtype(np.float64): torch.float64}[np.dtype(np_dtype)]
    t = torch.empty(shape, dtype=tdt).pin_memory()
    return t, t.numpy()


def reference(x, k, mode, monkeypatch):
    # pageable outputs, device table copied out after the join
    ref_i, ref_d, st = kj.selfjoin(x, k, beta=0.025, radius_mode=mode, return_stats=True)
    # another join of the same size leaves other rows in the device tables,
    # so a row a later join failed to deliver cannot match by chance
    y = datasets.uniform(x.shape[0], x.shape[1], 32).astype(x.dtype)
    kj.selfjoin(y, k, beta=0.025, radius_mode=mode)
    return ref_i, ref_d, st["total_distance"]


def close_sum(got, want):
    # the verification sum adds each row's squared distances in float, lane
    # partial sums first: a row finished by another kernel or pass (same
    # values) may round differently in the last bits
    assert abs(got - want) <= 1e-9 * abs(want), (got, want)


def same(ids, dd, ref_i, ref_d):
    assert np.array_equal(ids, ref_i)
    bits = np.uint32 if dd.dtype == np.float32 else np.uint64
    assert np.array_equal(dd.view(bits), ref_d.view(bits))


@pytest.mark.parametrize("mode,dtype", [(kj.RADIUS_LEARNED, np.float32), (kj.RADIUS_PLAIN, np.float32),
                                        (kj.RADIUS_LEARNED, np.float64)])
def test_table_copied_into_pinned_buffers(monkeypatch, mode, dtype):
    n, k = 400_000, 32
    x = datasets.sky_like(n, seed=37).astype(dtype)
    ref_i, ref_d, ref_sum = reference(x, k, mode, monkeypatch)
    monkeypatch.delenv("KNNSJ_DIRECT_ROWS", raising=False)
    t_i, ids = pinned((n, k + 1), np.int32)
    t_d, dd = pinned((n, k + 1), dtype)
    ids[:] = -7
    dd[:] = np.nan
    _, _, st = kj.selfjoin(x, k, beta=0.025, radius_mode=mode, out_ids=ids, out_dists=dd, return_stats=True)
    same(ids, dd, ref_i, ref_d)
    close_sum(st["total_distance"], ref_sum)
    # an odd-sized table (its byte count not a multiple of 16) into buffers
    # offset by 4 bytes: the copy falls back to 4-byte words
    m = 100_003
    y = np.ascontiguousarray(x[:m])
    yi, yd = kj.selfjoin(y, 6, beta=0.025, radius_mode=mode)
    t_i2, ids2 = pinned((m * 7 + 1,), np.int32)
    t_d2, dd2 = pinned((m * 7 + 1,), dtype)
    oi = ids2[1:].reshape(m, 7)
    od = dd2[1:].reshape(m, 7)
    kj.selfjoin(y, 6, beta=0.025, radius_mode=mode, out_ids=oi, out_dists=od)
    same(oi, od, yi, yd)
    # aligned buffers of that odd size: 16-byte copies and a 4-byte tail
    t_i3, ids3 = pinned((m, 7), np.int32)
    t_d3, dd3 = pinned((m, 7), dtype)
    kj.selfjoin(y, 6, beta=0.025, radius_mode=mode, out_ids=ids3, out_dists=dd3)
    same(ids3, dd3, yi, yd)


@pytest.mark.parametrize("mode,dtype,graph", [(kj.RADIUS_LEARNED, np.float32, "1"),
                                              (kj.RADIUS_PLAIN, np.float32, "0"),
                                              (kj.RADIUS_LEARNED, np.float64, "1")])
def test_direct_rows_into_pinned_buffers(monkeypatch, mode, dtype, graph):
    n, k = 400_000, 32
    x = datasets.sky_like(n, seed=31).astype(dtype)
    ref_i, ref_d, ref_sum = reference(x, k, mode, monkeypatch)
    monkeypatch.setenv("KNNSJ_GRAPH", graph)
    monkeypatch.setenv("KNNSJ_DIRECT_ROWS", "1")
    t_i, ids = pinned((n, k + 1), np.int32)
    t_d, dd = pinned((n, k + 1), dtype)
    ids[:] = -7
    dd[:] = np.nan
    _, _, st = kj.selfjoin(x, k, beta=0.025, radius_mode=mode, out_ids=ids, out_dists=dd, return_stats=True)
    assert st["queries_run"] > n  # some rows were finished after the first pass
    same(ids, dd, ref_i, ref_d)
    close_sum(st["total_distance"], ref_sum)


@pytest.mark.parametrize("mode", [kj.RADIUS_LEARNED, kj.RADIUS_PLAIN])
def test_memory_bounded_pageable_outputs(monkeypatch, mode):
    # a 1 MB cap on the device result table: the pageable outputs are
    # registered for the call and receive their rows directly
    n, k = 300_000, 64
    x = datasets.sky_like(n, seed=41)
    ref_i, ref_d, ref_sum = reference(x, k, mode, monkeypatch)
    ids = np.full((n, k + 1), -7, np.int32)
    dd = np.full((n, k + 1), np.nan, np.float32)
    _, _, st = kj.selfjoin(x, k, beta=0.025, radius_mode=mode, out_ids=ids, out_dists=dd, return_stats=True,
                           device_table_mb=1)
    same(ids, dd, ref_i, ref_d)
    close_sum(st["total_distance"], ref_sum)


@pytest.mark.parametrize("mode,chunks,graph", [(kj.RADIUS_LEARNED, "8", "1"), (kj.RADIUS_PLAIN, "3", "0")])
def test_streamed_rows_match_one_copy(monkeypatch, mode, chunks, graph):
    n, k = 400_000, 32
    x = datasets.sky_like(n, seed=31)
    ref_i, ref_d, ref_sum = reference(x, k, mode, monkeypatch)
    monkeypatch.setenv("KNNSJ_DIRECT_ROWS", "0")
    monkeypatch.setenv("KNNSJ_ROW_CHUNKS", chunks)
    monkeypatch.setenv("KNNSJ_GRAPH", graph)
    t_i, ids = pinned((n, k + 1), np.int32)
    t_d, dd = pinned((n, k + 1), np.float32)
    ids[:] = -7
    dd[:] = np.nan
    _, _, st = kj.selfjoin(x, k, beta=0.025, radius_mode=mode, out_ids=ids, out_dists=dd, return_stats=True)
    same(ids, dd, ref_i, ref_d)
    close_sum(st["total_distance"], ref_sum)
