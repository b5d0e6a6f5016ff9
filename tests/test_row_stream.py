"""Host-pointer joins into pinned output buffers stream their rows out while
the join runs: blocks of query ids searched one after another in the first
pass, each block's rows copied out on a second stream, and the rows finished
by later passes written into the host buffers at the end.  The rows must equal
those of a join into ordinary (pageable) buffers, which come back in one copy
after the join."""
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


@pytest.mark.parametrize("mode,chunks,dtype,graph", [(kj.RADIUS_LEARNED, "8", np.float32, "1"),
                                                     (kj.RADIUS_PLAIN, "3", np.float32, "1"),
                                                     (kj.RADIUS_LEARNED, "32", np.float64, "1"),
                                                     (kj.RADIUS_PLAIN, "8", np.float32, "0")])
def test_streamed_rows_match_one_copy(monkeypatch, mode, chunks, dtype, graph):
    # graph "0": the passes after the first are driven from the host
    n, k = 400_000, 32
    x = datasets.sky_like(n, seed=31).astype(dtype)
    ref_i, ref_d = kj.selfjoin(x, k, beta=0.025, radius_mode=mode)
    # another join of the same size leaves other rows in the device tables,
    # so a row the streamed join failed to deliver cannot match by chance
    y = datasets.uniform(n, 2, 32).astype(dtype)
    kj.selfjoin(y, k, beta=0.025, radius_mode=mode)
    monkeypatch.setenv("KNNSJ_ROW_CHUNKS", chunks)
    monkeypatch.setenv("KNNSJ_GRAPH", graph)
    t_i, ids = pinned((n, k + 1), np.int32)
    t_d, dd = pinned((n, k + 1), dtype)
    ids[:] = -7
    dd[:] = np.nan
    _, _, st = kj.selfjoin(x, k, beta=0.025, radius_mode=mode, out_ids=ids, out_dists=dd, return_stats=True)
    assert st["queries_run"] > n  # some rows were finished after the first pass
    assert np.array_equal(ids, ref_i)
    bits = np.uint32 if dtype == np.float32 else np.uint64
    assert np.array_equal(dd.view(bits), ref_d.view(bits))


def test_small_outputs_come_back_in_one_copy():
    # below the streaming size a pinned buffer takes the single copy
    n, k = 50_000, 8
    x = datasets.uniform(n, 3, 33)
    ref_i, ref_d = kj.selfjoin(x, k)
    t_i, ids = pinned((n, k + 1), np.int32)
    t_d, dd = pinned((n, k + 1), np.float32)
    kj.selfjoin(x, k, out_ids=ids, out_dists=dd)
    assert np.array_equal(ids, ref_i) and np.array_equal(dd, ref_d)
