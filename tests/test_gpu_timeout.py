"""The bounded device waits and how their expiry is reported.

Every merge kernel that waits for a bulk copy polls its mbarrier a bounded
number of times (origami_set_wait_limit, default 2^20). With the limit at 0 the
first wait of every CTA gives up at once: the CTA drains the copies it issued,
records the expiry in the sort's error word and returns. No GPU fault and no
hang is involved; the copies complete normally, only the kernel stops
early. These tests drive that path and check that
  * every entry point that waits for its sort returns ORIGAMI_ERR_TIMEOUT,
  * the next sort on the same stream, with the default limit, is bit-exact.
"""
import ctypes

import numpy as np
import pytest

import origami_gpu as og

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()
    assert torch.cuda.is_available()


@pytest.fixture
def expire_waits():
    default = og.wait_limit()
    assert default == 1 << 20
    og.set_wait_limit(0)
    try:
        yield
    finally:
        og.set_wait_limit(default)


def _keys(n, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randint(0, 2**31 - 1, (n,), dtype=torch.int64, device="cuda", generator=g).to(torch.int32)


def _sort_device(d, t, n, flags, stream):
    res = ctypes.c_void_p()
    rc = og.lib().origami_sort_device(og.U32, d.data_ptr(), t.data_ptr(), n, 0, 2, flags, ctypes.byref(res),
                                      ctypes.c_void_p(stream))
    return rc, res.value


@pytest.mark.parametrize("kind", [og.U32, og.U64, og.KV64])
def test_device_sort_reports_expired_wait_then_recovers(kind):
    n = 1 << 20
    ib = og.ITEM_BYTES[kind]
    g = torch.Generator(device="cuda").manual_seed(7 + kind)
    src = torch.randint(0, 256, (n * ib,), dtype=torch.uint8, device="cuda", generator=g)
    s = torch.cuda.Stream()
    default = og.wait_limit()
    og.set_wait_limit(0)
    try:
        d, t = src.clone(), torch.empty_like(src)
        res = ctypes.c_void_p()
        with torch.cuda.stream(s):
            rc = og.lib().origami_sort_device(kind, d.data_ptr(), t.data_ptr(), n, 0, 2, og.FLAG_SYNC,
                                              ctypes.byref(res), ctypes.c_void_p(s.cuda_stream))
        assert rc == og.ERR_TIMEOUT
        assert b"wait expired" in og.lib().origami_last_error()
    finally:
        og.set_wait_limit(default)
    # the same stream, the default limit: the sort is exact again
    d, t = src.clone(), torch.empty_like(src)
    res = ctypes.c_void_p()
    with torch.cuda.stream(s):
        og.check(og.lib().origami_sort_device(kind, d.data_ptr(), t.data_ptr(), n, 0, 2, og.FLAG_SYNC,
                                              ctypes.byref(res), ctypes.c_void_p(s.cuda_stream)))
    got = (d if res.value == d.data_ptr() else t).cpu().numpy()
    host = src.cpu().numpy()
    if kind == og.U32:
        assert np.array_equal(got.view(np.uint32), np.sort(host.view(np.uint32)))
    elif kind == og.U64:
        assert np.array_equal(got.view(np.uint64), np.sort(host.view(np.uint64)))
    else:
        a = host.view(og.KV_DTYPE)
        order = np.argsort(a["key"], kind="stable")
        assert np.array_equal(got.view(og.KV_DTYPE), a[order])


def test_host_sort_reports_expired_wait(expire_waits):
    n = 1 << 20
    a = np.random.default_rng(3).integers(0, 2**32, n, dtype=np.uint32)
    t = np.empty_like(a)
    res = ctypes.c_void_p()
    rc = og.lib().origami_sort(og.U32, a.ctypes.data, t.ctypes.data, n, 0, 2, 0, ctypes.byref(res))
    assert rc == og.ERR_TIMEOUT


def test_segmented_sort_reports_expired_wait(expire_waits):
    lens = [1 << 16, 3 << 15, 1 << 17]
    n = sum(lens)
    off = torch.tensor(np.concatenate([[0], np.cumsum(lens)]).astype(np.int64), device="cuda")
    d = _keys(n, 5)
    t = torch.empty_like(d)
    rc = og.lib().origami_sort_segmented_device(og.U32, d.data_ptr(), t.data_ptr(), off.data_ptr(), len(lens), n,
                                                og.FLAG_SYNC, None)
    assert rc == og.ERR_TIMEOUT


def test_noalloc_sort_reports_expired_wait(expire_waits):
    n = 1 << 20
    d = _keys(n, 9)
    t = torch.empty_like(d)
    res = ctypes.c_void_p()
    rc = og.lib().origami_sort_noalloc_device(og.U32, d.data_ptr(), t.data_ptr(), n, 0, og.FLAG_SYNC,
                                              ctypes.byref(res), None)
    assert rc == og.ERR_TIMEOUT


def test_wait_limit_round_trip():
    default = og.wait_limit()
    og.set_wait_limit(12345)
    assert og.wait_limit() == 12345
    og.set_wait_limit(default)
    assert og.wait_limit() == default
