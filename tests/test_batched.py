"""knnsj_selfjoin_batched: many independent self-joins in one call.

Every set's rows must equal those of a knnsj_selfjoin call on that set alone,
bit for bit, whatever launch shape the autotuner picked and whichever worker
ran the set; a set that cannot run reports its own status without stopping
the others.
"""
import ctypes

import numpy as np
import pytest

import hybrid_k_nearest_neighbor_self_join_gb300 as kj
from hybrid_k_nearest_neighbor_self_join_gb300 import _lib, datasets

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def _check_same(outs, xs, ks, **kw):
    for (ids, dists), x, k in zip(outs, xs, ks):
        rids, rdists = kj.selfjoin(x, k, **kw)
        assert np.array_equal(ids, rids)
        ub = np.uint32 if x.dtype == np.float32 else np.uint64
        assert np.array_equal(dists.view(ub), rdists.view(ub))


@pytest.mark.parametrize("radius_mode", [kj.RADIUS_PLAIN, kj.RADIUS_LEARNED])
def test_uneven_sets_match_single_calls(radius_mode):
    sets = list(datasets.batched_sets(24, seed=11, n_lo=2000, n_hi=60000))
    xs = [s[0] for s in sets]
    ks = [s[1] for s in sets]
    for _ in range(2):  # the second call reuses the tuned shapes and the workers' workspaces
        outs = kj.selfjoin_batched(xs, ks, radius_mode=radius_mode)
        _check_same(outs, xs, ks, radius_mode=radius_mode)


def test_double_sets():
    xs = [datasets.gmm(n, d, 5, 0.2, 30 + n % 7, dtype=np.float64) for n, d in ((3000, 2), (25000, 3), (9000, 6))]
    ks = [8, 16, 5]
    _check_same(kj.selfjoin_batched(xs, ks), xs, ks)


def test_bad_set_reports_its_own_status():
    lib = _lib.load()
    good = datasets.gmm(5000, 2, 4, 0.2, 3, dtype=np.float32)
    tiny = np.zeros((4, 2), np.float32)
    sets = (_lib.Set * 2)()
    outs = []
    for i, (x, k) in enumerate(((tiny, 8), (good, 8))):
        ids = np.empty((x.shape[0], k + 1), np.int32)
        ds = np.empty((x.shape[0], k + 1), np.float32)
        outs.append((ids, ds))
        sets[i].data, sets[i].n, sets[i].d, sets[i].k = x.ctypes.data, x.shape[0], x.shape[1], k
        sets[i].out_ids, sets[i].out_dists = ids.ctypes.data, ds.ctypes.data
    opts = _lib.Options.make()
    st = _lib.Stats.make()
    rc = lib.knnsj_selfjoin_batched(2, sets, _lib.KNNSJ_F32, ctypes.byref(opts), ctypes.byref(st))
    assert rc == 3 and sets[0].status == 3 and sets[1].status == 0  # KNNSJ_ERR_K_TOO_LARGE
    _check_same(outs[1:], [good], [8])


_TUNE_SCRIPT = r"""
import sys, json
sys.path.insert(0, sys.argv[1])
import numpy as np
import hybrid_k_nearest_neighbor_self_join_gb300 as kj
from hybrid_k_nearest_neighbor_self_join_gb300 import datasets
xs = [datasets.gmm(30_000 + 1000 * i, 3, 6, 0.2, 40 + i, dtype=np.float32) for i in range(3)]
outs = kj.selfjoin_batched(xs, [8, 8, 8])
ok = all(np.array_equal(o[0], kj.selfjoin(x, 8)[0]) for o, x in zip(outs, xs))
print(json.dumps({"ok": ok}))
"""


def test_tune_cache_persists_across_processes(tmp_path):
    # KNNSJ_TUNE_CACHE: the first process tunes the class (float, d=3, k+1=9)
    # and writes it; a second process loads it instead of tuning again (the
    # shape planted in the file survives), and results stay those of single
    # calls whatever the shape
    import json
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cache = tmp_path / "tune.txt"
    script = tmp_path / "tune_run.py"
    script.write_text(_TUNE_SCRIPT)
    env = dict(os.environ, KNNSJ_TUNE_CACHE=str(cache))
    env.pop("KNNSJ_AUTOTUNE", None)

    def run():
        r = subprocess.run([sys.executable, str(script), root], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        assert json.loads(r.stdout.strip().splitlines()[-1])["ok"]

    run()
    lines = [ln.split() for ln in cache.read_text().splitlines() if ln.strip()]
    mine = [ln for ln in lines if ln[1:5] == ["0", "3", "3", "9"]]
    assert len(mine) == 1, lines
    # plant another shape the tuner tries (4 warps per block, one query per
    # fetch) and a line of another device, then run again
    mine[0][5:8] = ["4", "1", "0"]
    planted = " ".join(mine[0])
    other = "Some_Other_GPU 0 3 3 9 8 16 0"
    cache.write_text(planted + "\n" + other + "\n")
    run()
    # no class was tuned in the second process: the file is as planted
    assert cache.read_text() == planted + "\n" + other + "\n"
