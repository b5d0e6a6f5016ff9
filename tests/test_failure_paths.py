"""Failure paths of the join, made without any GPU fault.

* KNNSJ_ERR_NO_CONVERGENCE: an iteration cap (max_iterations=1) on a join
  that needs several passes, through the host-driven retry loop, the loop in
  a CUDA graph, and pinned outputs (rows written by the kernels, or streamed
  by copies); the call returns the status, no kernel or copy writing into
  the caller's buffers is left in flight, and the library keeps working
  afterwards.
* The tensor-core radius model's bounded mbarrier waits: with the test
  switch KNNSJ_TEST_MLP_TIMEOUT=1 the MLP issues no MMA (nothing is in
  flight) and waits only briefly, so every tile takes the timeout path; the
  learned join must still return the oracle's rows (every query then starts
  at eps0) and report the error in its stats.
"""
import time

import numpy as np
import pytest

import oracle
import hybrid_k_nearest_neighbor_self_join_gb300 as kj
from hybrid_k_nearest_neighbor_self_join_gb300 import _lib, datasets

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()
    __graft_entry__.build_oracle()


def _expect_no_convergence(x, k, **kw):
    with pytest.raises(_lib.KnnsjError) as e:
        kj.selfjoin(x, k, beta=0.0, max_iterations=1, **kw)
    assert e.value.status == 6, e.value  # KNNSJ_ERR_NO_CONVERGENCE


@pytest.mark.parametrize("graph", ["0", "1"])
def test_iteration_cap_reports_no_convergence(monkeypatch, graph):
    monkeypatch.setenv("KNNSJ_GRAPH", graph)
    x = datasets.uniform(50_000, 2, 5)
    # the plain schedule at BETA=0 needs more than one pass on this set
    _, _, st = kj.selfjoin(x, 8, beta=0.0, return_stats=True)
    assert st["iterations"] >= 2
    _expect_no_convergence(x, 8)
    # the library still works after the error
    ids, dists = kj.selfjoin(x, 8, beta=0.0)
    rc, oids, odists, _ = oracle.join(x, 8, di=2, beta=0.0)
    assert rc == 0
    assert np.array_equal(ids, oids)
    assert np.array_equal(dists.view(np.uint32), odists.view(np.uint32))


@pytest.mark.parametrize("direct", ["2", "1", "0"])
def test_iteration_cap_with_pinned_outputs_leaves_nothing_in_flight(monkeypatch, direct):
    # direct "2": a device table copied in by a kernel after the join; "1":
    # rows written by the kernels into the pinned buffers; "0": rows streamed
    # out of a device table by copies
    monkeypatch.setenv("KNNSJ_DIRECT_ROWS", direct)
    torch = pytest.importorskip("torch")
    n, k = 300_000, 8  # >= 2^18 rows: with direct "0" the rows are streamed during the join
    x = datasets.uniform(n, 2, 6)
    ids = torch.full((n, k + 1), -3, dtype=torch.int32).pin_memory().numpy()
    dists = torch.full((n, k + 1), -3.0, dtype=torch.float32).pin_memory().numpy()
    with pytest.raises(_lib.KnnsjError) as e:
        kj.selfjoin(x, k, beta=0.0, max_iterations=1, out_ids=ids, out_dists=dists)
    assert e.value.status == 6
    snap_i, snap_d = ids.copy(), dists.copy()
    time.sleep(0.3)  # a copy still in flight would change the buffers now
    assert np.array_equal(ids, snap_i)
    assert np.array_equal(dists.view(np.uint32), snap_d.view(np.uint32))
    # the same buffers then receive a complete, correct table
    kj.selfjoin(x, k, beta=0.0, out_ids=ids, out_dists=dists)
    rc, oids, odists, _ = oracle.join(x, k, di=2, beta=0.0)
    assert rc == 0
    assert np.array_equal(ids, oids)
    assert np.array_equal(dists.view(np.uint32), odists.view(np.uint32))


def test_radius_model_timeout_falls_back_to_eps0(monkeypatch):
    x = datasets.gmm(60_000, 2, 20, 0.2, 17, dtype=np.float32)
    k, beta = 32, 0.025
    ids0, d0, st0 = kj.selfjoin(x, k, beta=beta, radius_mode=kj.RADIUS_LEARNED, return_stats=True)
    assert st0["radius_model_error"] == 0
    monkeypatch.setenv("KNNSJ_TEST_MLP_TIMEOUT", "1")
    ids, dists, st = kj.selfjoin(x, k, beta=beta, radius_mode=kj.RADIUS_LEARNED, return_stats=True)
    assert st["radius_model_error"] == 1, st["radius_model_error"]
    rc, oids, odists, _ = oracle.join(x, k, di=2, beta=beta)
    assert rc == 0
    assert np.array_equal(ids, oids)
    assert np.array_equal(dists.view(np.uint32), odists.view(np.uint32))
    monkeypatch.delenv("KNNSJ_TEST_MLP_TIMEOUT")
    _, _, st2 = kj.selfjoin(x, k, beta=beta, radius_mode=kj.RADIUS_LEARNED, return_stats=True)
    assert st2["radius_model_error"] == 0
