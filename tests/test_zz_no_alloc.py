"""knnsj_selfjoin_device_noalloc against knnsj_selfjoin_device.

The fixed-scratch entry point takes all of its scratch from one static device
array instead of cudaMalloc, for callers whose runtime owns device memory or
that size every allocation before they start.  Its results must be bit-identical to the
ordinary device entry point's (the library's parity bar), call after call:
each call carves its buffers from the same array, which still holds the
previous call's contents.  This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from hybrid_k_nearest_neighbor_self_join_gb300 import _lib, datasets

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MAX_POINTS = 65536  # KNNSJ_NOALLOC_MAX_POINTS


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def _join(fn, x, k, radius_mode=0, with_stats=True, beta=None):
    n, d = x.shape
    dev = torch.from_numpy(x).cuda()
    ids = torch.full((n, k + 1), -7, dtype=torch.int32, device="cuda")
    dists = torch.full((n, k + 1), -1.0, dtype=dev.dtype, device="cuda")
    torch.cuda.synchronize()
    opts = _lib.Options.make(radius_mode=radius_mode, beta=beta)
    code = _lib.KNNSJ_F32 if x.dtype == np.float32 else _lib.KNNSJ_F64
    args = [ctypes.c_void_p(dev.data_ptr()), code, n, d, k, ctypes.byref(opts),
            ctypes.c_void_p(ids.data_ptr()), ctypes.c_void_p(dists.data_ptr())]
    if with_stats:
        st = _lib.Stats.make()
        args.append(ctypes.byref(st))
    rc = fn(*args)
    torch.cuda.synchronize()
    return rc, ids.cpu().numpy(), dists.cpu().numpy()


def _both(x, k, radius_mode=0, beta=None):
    lib = _lib.load()
    rc, ids, dists = _join(lib.knnsj_selfjoin_device_noalloc, x, k, radius_mode, with_stats=False, beta=beta)
    assert rc == _lib.KNNSJ_OK, _lib.STATUS_NAMES.get(rc, rc)
    rc, rids, rdists = _join(lib.knnsj_selfjoin_device, x, k, radius_mode, beta=beta)
    assert rc == _lib.KNNSJ_OK, _lib.STATUS_NAMES.get(rc, rc)
    assert np.array_equal(ids, rids)
    ub = np.uint32 if x.dtype == np.float32 else np.uint64
    assert np.array_equal(dists.view(ub), rdists.view(ub))


def test_two_calls_in_a_row_match_device_entry_point():
    # different sizes, dimensions and k on consecutive calls: the second call
    # reuses the array the first one left behind
    a = datasets.sky_like(20000, seed=3).astype(np.float32)
    b = datasets.gmm(50000, 3, 12, 0.2, 5, dtype=np.float32)
    _both(a, 8)
    _both(b, 16)
    _both(a, 8)


def test_double_and_largest_problem():
    x = datasets.gmm(MAX_POINTS, 8, 20, 0.5, 11, dtype=np.float64)
    _both(x, 127)
    _both(x[:30000, :4].copy(), 32)


def test_learned_radius_mode():
    x = datasets.gmm(60000, 2, 30, 0.2, 9, dtype=np.float32)
    _both(x, 32, radius_mode=_lib.KNNSJ_RADIUS_LEARNED)
    _both(x, 32, radius_mode=_lib.KNNSJ_RADIUS_LEARNED)


def test_allocates_nothing():
    # after a first call (which looks up the array's address), a call leaves
    # the device's free memory exactly as it was: nothing was allocated
    lib = _lib.load()
    x = datasets.gmm(40000, 3, 12, 0.2, 21, dtype=np.float32)
    n, d = x.shape
    k = 16
    dev = torch.from_numpy(x).cuda()
    ids = torch.empty((n, k + 1), dtype=torch.int32, device="cuda")
    dists = torch.empty((n, k + 1), dtype=torch.float32, device="cuda")
    opts = _lib.Options.make()
    args = [ctypes.c_void_p(dev.data_ptr()), _lib.KNNSJ_F32, n, d, k, ctypes.byref(opts),
            ctypes.c_void_p(ids.data_ptr()), ctypes.c_void_p(dists.data_ptr())]
    assert lib.knnsj_selfjoin_device_noalloc(*args) == _lib.KNNSJ_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert lib.knnsj_selfjoin_device_noalloc(*args) == _lib.KNNSJ_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_grid_rebuilds_at_the_limits():
    # eight dimensions, the largest n and k: the plain schedule widens the
    # radius until the grid is rebuilt; every rebuilt buffer still fits
    x = datasets.gmm(MAX_POINTS, 8, 6, 0.05, 13, dtype=np.float32)
    st = None
    lib = _lib.load()
    n, d = x.shape
    k = 127
    dev = torch.from_numpy(x).cuda()
    ids = torch.empty((n, k + 1), dtype=torch.int32, device="cuda")
    dists = torch.empty((n, k + 1), dtype=torch.float32, device="cuda")
    opts = _lib.Options.make(beta=0.0)
    st = _lib.Stats.make()
    assert lib.knnsj_selfjoin_device(ctypes.c_void_p(dev.data_ptr()), _lib.KNNSJ_F32, n, d, k, ctypes.byref(opts),
                                     ctypes.c_void_p(ids.data_ptr()), ctypes.c_void_p(dists.data_ptr()),
                                     ctypes.byref(st)) == _lib.KNNSJ_OK
    assert st.regrids >= 1 and st.iterations >= 3, (st.regrids, st.iterations)
    _both(x, k, beta=0.0)


def test_rejects_problems_beyond_the_array():
    lib = _lib.load()
    x = np.zeros((1, 1), np.float32)
    opts = _lib.Options.make()
    big = MAX_POINTS + 1
    for n, d, k in ((big, 2, 8), (1000, 9, 8), (1000, 2, 128)):
        rc = lib.knnsj_selfjoin_device_noalloc(ctypes.c_void_p(x.ctypes.data), _lib.KNNSJ_F32, n, d, k,
                                               ctypes.byref(opts), ctypes.c_void_p(x.ctypes.data),
                                               ctypes.c_void_p(x.ctypes.data))
        assert rc == 12, (n, d, k, rc)
    assert b"fixed scratch" in lib.knnsj_status_string(12)

