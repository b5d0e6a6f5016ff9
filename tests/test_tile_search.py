"""The first pass's tile search (k_tile.cu) against the oracle and against
the per-query search it replaces (KNNSJ_TILE=0), bit for bit.

It covers both dimensions it serves (2-D and 3-D float, all indexed), the
three row capacities (k+1 <= 16, 33, 65), 4, 8 and 16 queries per warp, the
plain and learned starting radii, the streamed-rows path (its queries come by
id blocks) and data whose boundary bin cannot be split (exact duplicates),
which the tile hands over to the per-query search.
"""
import numpy as np
import pytest

import oracle
import hybrid_k_nearest_neighbor_self_join_gb300 as kj
from hybrid_k_nearest_neighbor_self_join_gb300 import datasets

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()
    __graft_entry__.build_oracle()


def same(a, b):
    (ia, da), (ib, db) = a, b
    assert np.array_equal(ia, ib), int((ia != ib).any(axis=1).sum())
    assert np.array_equal(da.view(np.uint32), db.view(np.uint32)), int((da != db).any(axis=1).sum())


def join(x, k, beta, mode, tile, monkeypatch, **kw):
    # tile: True = query tiles always (3), False = off (0), or a KNNSJ_TILE value
    monkeypatch.setenv("KNNSJ_TILE", "3" if tile is True else ("0" if tile is False else tile))
    ids, dists, st = kj.selfjoin(x, k, beta=beta, radius_mode=mode, return_stats=True, **kw)
    return (ids, dists), st


@pytest.mark.parametrize("d,k,beta", [(2, 8, 0.0), (2, 32, 0.025), (2, 64, 0.025), (3, 8, 0.05), (3, 32, 0.0),
                                      (3, 64, 0.05)])
def test_tile_matches_oracle_plain(monkeypatch, d, k, beta):
    x = datasets.gmm(120_000, d, 15, 0.25, 100 + d * k, dtype=np.float32)
    got, st = join(x, k, beta, kj.RADIUS_PLAIN, True, monkeypatch)
    rc, oids, odists, _ = oracle.join(x, k, di=d, beta=beta)
    assert rc == 0
    same(got, (oids, odists))


@pytest.mark.parametrize("d,k", [(2, 64), (2, 8), (3, 32)])
def test_tile_learned_equals_per_query_search(monkeypatch, d, k):
    x = datasets.gmm(150_000, d, 25, 0.2, 7 + d + k, dtype=np.float32)
    a, st = join(x, k, 0.025, kj.RADIUS_LEARNED, True, monkeypatch)
    b, _ = join(x, k, 0.025, kj.RADIUS_LEARNED, False, monkeypatch)
    c, _ = join(x, k, 0.025, kj.RADIUS_PLAIN, True, monkeypatch)
    e, _ = join(x, k, 0.025, kj.RADIUS_PLAIN, "2", monkeypatch)  # one warp per query, finer grid
    f, _ = join(x, k, 0.025, kj.RADIUS_LEARNED, "2", monkeypatch)
    same(a, b)
    same(a, c)
    same(a, e)
    same(a, f)


@pytest.mark.parametrize("qpt", ["4", "8", "16"])
@pytest.mark.parametrize("d,k", [(2, 64), (3, 16)])
def test_tile_queries_per_warp(monkeypatch, qpt, d, k):
    # 4 queries per warp is the default; 8 and 16 (KNNSJ_TILE_QPT) share a
    # box among more queries with larger shared-memory lists
    x = datasets.gmm(100_000, d, 20, 0.2, 17 + d + k, dtype=np.float32)
    b, _ = join(x, k, 0.025, kj.RADIUS_LEARNED, False, monkeypatch)
    monkeypatch.setenv("KNNSJ_TILE_QPT", qpt)
    a, st = join(x, k, 0.025, kj.RADIUS_LEARNED, True, monkeypatch)
    same(a, b)


def test_tile_sky_like(monkeypatch):
    x = datasets.sky_like(400_000, seed=11)
    a, st = join(x, 64, 0.025, kj.RADIUS_LEARNED, True, monkeypatch)
    rc, oids, odists, _ = oracle.join(x, 64, di=2, beta=0.025)
    assert rc == 0
    same(a, (oids, odists))


def test_tile_exact_ties_are_handed_over(monkeypatch):
    # every point appears 40 times: the K-th distance is shared by many keys
    base = datasets.uniform(3_000, 2, 9)
    x = np.ascontiguousarray(np.repeat(base, 40, axis=0)[np.random.default_rng(1).permutation(120_000)])
    a, st = join(x, 64, 0.0, kj.RADIUS_PLAIN, True, monkeypatch)
    assert st["tile_handovers"] > 0
    rc, oids, odists, _ = oracle.join(x, 64, di=2, beta=0.0)
    assert rc == 0
    same(a, (oids, odists))


def test_tile_rows_into_pinned_buffers(monkeypatch):
    torch = pytest.importorskip("torch")
    n, k = 300_000, 32
    x = datasets.gmm(n, 2, 30, 0.2, 5, dtype=np.float32)
    ids = torch.empty((n, k + 1), dtype=torch.int32).pin_memory().numpy()
    dists = torch.empty((n, k + 1), dtype=torch.float32).pin_memory().numpy()
    monkeypatch.setenv("KNNSJ_TILE", "3")
    kj.selfjoin(x, k, beta=0.025, radius_mode=kj.RADIUS_LEARNED, out_ids=ids, out_dists=dists)
    b, _ = join(x, k, 0.025, kj.RADIUS_LEARNED, False, monkeypatch)
    same((ids, dists), b)
