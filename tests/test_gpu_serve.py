"""GPU tests of the serving loop (origami_server_*).

Correctness bar: every request's result equals an independent stable sort of
that request alone (exact equality: integer keys, no tolerance), whether it was
served alone or coalesced with other requests of mixed kinds, sizes and
memory types. Host faults are exercised with real requests: budget admission,
oversized requests, queue overflow, cancellation, bad arguments."""
import numpy as np
import pytest

import oracle as orc
import origami_gpu as og

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()
    assert torch.cuda.is_available()


def make(kind, n, rng, zipf=False, pinned=False):
    a = og.empty_host(kind, n, pinned=pinned)
    if zipf:
        ranks = np.minimum(rng.zipf(1.5, n), 1 << 20).astype(np.uint64)
        k = ranks * np.uint64(0x9E3779B97F4A7C15)
    else:
        k = rng.integers(0, 2**64, n, dtype=np.uint64)
    if kind == og.U32:
        a[:] = (k >> np.uint64(32)).astype(np.uint32)
    elif kind == og.U64:
        a[:] = k
    elif kind == og.I64:
        a[:] = k.view(np.int64)
    elif kind == og.KV64:
        a["key"] = k.view(np.int64)
        a["value"] = np.arange(n)
    else:
        a["key"] = k
        a["value"] = np.arange(n, dtype=np.uint64)
    return a


def expected(a):
    return a[np.argsort(orc.keys_of(a), kind="stable")]


def request_mix(seed, count, lo=10, hi=21):
    """(kind, n, zipf) triples: kinds 50% u32 / 30% u64 / 20% kvu64, lengths
    log-uniform on [2^lo, 2^hi], uniform or Zipf keys 50/50."""
    rng = np.random.default_rng(seed)
    kinds = rng.choice([og.U32, og.U64, og.KVU64], size=count, p=[0.5, 0.3, 0.2])
    lens = np.floor(np.exp2(rng.uniform(lo, hi, count))).astype(np.int64)
    zipf = rng.random(count) < 0.5
    return [(int(k), int(n), bool(z)) for k, n, z in zip(kinds, lens, zipf)]


def test_alone_equals_in_mix():
    rng = np.random.default_rng(7)
    mix = request_mix(1, 48)
    inputs = [make(k, n, rng, z, pinned=(i % 3 == 0)) for i, (k, n, z) in enumerate(mix)]
    alone = []
    with og.Server(max_inflight=1) as s:
        for a in inputs:
            x = a.copy()
            s.wait(s.submit(x))
            alone.append(x)
    with og.Server() as s:
        bufs = [a.copy() if i % 3 else og.empty_host(mix[i][0], len(a), pinned=True) for i, a in enumerate(inputs)]
        for i, a in enumerate(inputs):
            bufs[i][:] = a
        ids = [s.submit(b) for b in bufs]
        for r in ids:
            s.wait(r)
        st = s.stats()
    assert st["completed"] == len(inputs)
    assert st["batches"] < len(inputs)  # requests were coalesced
    for a, x, y in zip(inputs, alone, bufs):
        assert np.array_equal(x, y)
        assert np.array_equal(y, expected(a))


def test_device_tensors_and_empty_requests():
    rng = np.random.default_rng(9)
    host = [make(og.U32, n, rng) for n in (0, 1, 31, 4096, 100_000, 1 << 20)]
    dev = [torch.from_numpy(a.view(np.int32).copy()).cuda() for a in host]
    with og.Server() as s:
        ids = [s.submit(t, kind=og.U32) for t in dev]
        for r in ids:
            s.wait(r)
    torch.cuda.synchronize()
    for a, t in zip(host, dev):
        got = t.cpu().numpy().view(np.uint32)  # int32 storage of u32 keys
        assert np.array_equal(got, np.sort(a))


def test_budget_admission_serializes():
    # each request needs ~2 x 16 MiB + scratch; the budget admits one at a time
    rng = np.random.default_rng(3)
    n = 1 << 22
    inputs = [make(og.U32, n, rng) for _ in range(4)]
    budget = 48 << 20
    with og.Server(hbm_budget_bytes=budget) as s:
        bufs = [a.copy() for a in inputs]
        ids = [s.submit(b) for b in bufs]
        for r in ids:
            s.wait(r)
        st = s.stats()
    assert st["peak_bytes_reserved"] <= budget
    assert st["batches"] == 4
    assert st["max_concurrent_batches"] == 1
    for a, b in zip(inputs, bufs):
        assert np.array_equal(b, np.sort(a))


def test_oversized_and_bad_arguments():
    with og.Server(hbm_budget_bytes=8 << 20) as s:
        big = np.zeros(4 << 20, np.uint32)  # needs > 32 MiB
        with pytest.raises(og.OrigamiError) as e:
            s.submit(big)
        assert e.value.code == og.ERR_OOM
        L = og.lib()
        import ctypes
        rid = ctypes.c_uint64()
        assert L.origami_serve_submit(s._h, 0, None, None, 10, ctypes.byref(rid)) == og.ERR_INVALID
        assert L.origami_serve_submit(s._h, 9, big.ctypes.data, None, 10, ctypes.byref(rid)) == og.ERR_DTYPE
        # overlapping input and output that are not the same buffer
        assert L.origami_serve_submit(s._h, 0, big.ctypes.data, big.ctypes.data + 4, 10,
                                       ctypes.byref(rid)) == og.ERR_INVALID
        assert L.origami_serve_wait(s._h, 12345, 0) == og.ERR_INVALID
        assert L.origami_serve_cancel(s._h, 12345) == og.ERR_INVALID
        # the server still works after rejected calls
        a = make(og.U32, 1000, np.random.default_rng(1))
        x = a.copy()
        s.wait(s.submit(x))
        assert np.array_equal(x, np.sort(a))


def test_queue_overflow_and_cancel():
    rng = np.random.default_rng(5)
    big = make(og.U32, 1 << 26, rng)  # keeps the single slot busy for a while
    big_in = big.copy()
    small = [make(og.U32, 5000, rng) for _ in range(64)]
    with og.Server(max_inflight=1, max_queue=4) as s:
        bufs = [a.copy() for a in small]
        first = s.submit(big)
        ids, busy = [], False
        for b in bufs:
            try:
                ids.append((s.submit(b), b))
            except og.OrigamiError as e:
                assert e.code == og.ERR_BUSY
                busy = True
                break
        assert busy, "the queue never filled"
        # cancel the last accepted request: OK while it is pending
        rid, b = ids[-1]
        before = b.copy()
        try:
            s.cancel(rid)
            cancelled = True
        except og.OrigamiError as e:
            assert e.code == og.ERR_BUSY  # already admitted
            cancelled = False
        s.wait(first)
        for r, buf in ids[:-1]:
            s.wait(r)
        if cancelled:
            with pytest.raises(og.OrigamiError) as e:
                s.wait(rid)
            assert e.value.code == og.ERR_CANCELLED
            assert np.array_equal(b, before)
        else:
            s.wait(rid)
        st = s.stats()
    assert np.array_equal(big, np.sort(big_in))
    for (r, buf), a in zip(ids[:-1], small):
        assert np.array_equal(buf, np.sort(a))
    assert st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]


def test_wait_timeout_then_result():
    rng = np.random.default_rng(8)
    a = make(og.KVU64, 1 << 24, rng)
    x = a.copy()
    with og.Server() as s:
        rid = s.submit(x)
        try:
            s.wait(rid, timeout_ms=0)
            done = True
        except og.OrigamiError as e:
            assert e.code == og.ERR_TIMEOUT
            done = False
        if not done:
            s.wait(rid)
    assert np.array_equal(x, expected(a))


def test_large_requests_take_the_pipelined_sort():
    # requests of 2^24 items and more run on the server's helper threads as the
    # pipelined single-array sort (copies overlapping the sort), beside
    # segmented batches of smaller ones; every result equals the stable sort
    rng = np.random.default_rng(21)
    specs = [(og.U32, (1 << 24) + 333, True), (og.KVU64, 1 << 22, False), (og.U64, (1 << 24) + 5, False),
             (og.U32, 5000, False), (og.KVU64, 70_000, True), (og.U32, 1 << 22, False)]
    inputs = [make(k, n, rng, zipf=(i % 2 == 0), pinned=p) for i, (k, n, p) in enumerate(specs)]
    outs = [og.empty_host(k, n, pinned=p) for (k, n, p) in specs]
    dev_in = torch.from_numpy(make(og.U64, 1 << 23, rng).view(np.uint8).copy()).cuda()
    dev_keep = dev_in.clone()
    with og.Server() as s:
        ids = [s.submit(a, out=o) for a, o in zip(inputs, outs)]
        ids.append(s.submit(dev_in, kind=og.U64))
        for r in ids:
            s.wait(r)
        st = s.stats()
    assert st["completed"] == len(ids) and st["failed"] == 0
    assert st["pipe_batches"] >= 2 and st["arena_bytes"] > 0
    for a, o in zip(inputs, outs):
        assert np.array_equal(o, expected(a))
    torch.cuda.synchronize()
    got = dev_in.cpu().numpy().view(np.uint64)
    assert np.array_equal(got, np.sort(dev_keep.cpu().numpy().view(np.uint64)))
