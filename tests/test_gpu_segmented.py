"""GPU parity tests of the batched segmented sort (a device-planned tile phase,
then one partition and one persistent merge kernel per merge level over all
segments at once; the plan form replays that sequence as a CUDA graph).

Every segment must equal an independent stable sort of that segment: numpy for
key-value items; for keys-only items also the oracle, which restates the
reference's chunked sort."""
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


def make_items(kind, n, seed, dist="uniform"):
    rng = np.random.default_rng(seed)
    a = orc.empty(kind, n)
    if dist == "uniform":
        k = rng.integers(0, 2**64, n, dtype=np.uint64)
    elif dist == "few":
        k = rng.integers(0, 8, n).astype(np.uint64) << np.uint64(40)
    else:  # equal
        k = np.full(n, 0x1234_5678_9ABC_DEF0, np.uint64)
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


def expected(a, off):
    keys = orc.keys_of(a)
    seg = np.repeat(np.arange(len(off) - 1), np.diff(np.asarray(off, dtype=np.int64)))
    return a[np.lexsort((keys, seg))]  # stable within each segment


def run_device(a, off, kind):
    d = torch.from_numpy(a.view(np.uint8).copy()).cuda()
    o = torch.from_numpy(np.asarray(off, dtype=np.int64)).cuda()
    og.sort_segmented(d, o, kind=kind)
    torch.cuda.synchronize()
    return d.cpu().numpy().view(a.dtype)


def lengths(kind_tile, rng, nseg):
    # log-uniform over [1, 2^17] plus the class edges
    edges = [0, 1, 2, 31, 32, 33, 511, 512, 513, 1023, 1024, 1025, 2047, 2048, 2049, 4095, 4096,
             4097, 8191, 8192, 8193, 16385, 3 * 8192 + 5]
    ln = np.floor(np.exp(rng.uniform(0, np.log(2**17), nseg))).astype(np.int64)
    return np.concatenate([np.array(edges, np.int64), ln])


@pytest.mark.parametrize("kind", [og.U32, og.U64, og.I64, og.KV64, og.KVU64])
@pytest.mark.parametrize("dist", ["uniform", "few", "equal"])
def test_segmented_mixed_sizes(kind, dist):
    rng = np.random.default_rng(100 + kind)
    lens = lengths(kind, rng, 300)
    rng.shuffle(lens)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    a = make_items(kind, int(off[-1]), seed=kind * 7 + 1, dist=dist)
    got = run_device(a, off, kind)
    assert np.array_equal(got, expected(a, off))
    if kind in (og.U32, og.U64, og.I64):
        # the oracle's chunked sort on each segment (reference semantics)
        for s in range(0, len(lens), 37):
            seg = a[off[s]:off[s + 1]]
            ora, _ = orc.sort_single_thread(kind, seg)
            assert np.array_equal(got[off[s]:off[s + 1]], ora)


@pytest.mark.parametrize("kind", [og.U32, og.KV64])
def test_segmented_host_api(kind):
    rng = np.random.default_rng(5)
    lens = rng.integers(0, 20000, 200)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    a = make_items(kind, int(off[-1]), seed=3)
    d = a.copy()
    og.sort_segmented(d, off)
    assert np.array_equal(d, expected(a, off))


def test_segmented_many_small():
    rng = np.random.default_rng(11)
    lens = rng.integers(0, 300, 20000)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    a = make_items(og.U32, int(off[-1]), seed=12)
    assert np.array_equal(run_device(a, off, og.U32), expected(a, off))


def test_segmented_one_large_and_empty():
    off = np.array([0, 0, (1 << 21) + 333, (1 << 21) + 333], np.uint64)
    a = make_items(og.U32, int(off[-1]), seed=21)
    assert np.array_equal(run_device(a, off, og.U32), expected(a, off))


def test_segmented_rejects_decreasing_offsets():
    off = np.array([0, 100, 50, 200], np.uint64)
    a = make_items(og.U32, 200, seed=1)
    with pytest.raises(og.OrigamiError) as e:
        og.sort_segmented(a.copy(), off)
    assert e.value.code == og.ERR_INVALID
    # device form: detected on the device and reported on sync
    d = torch.from_numpy(a.view(np.uint8).copy()).cuda()
    o = torch.tensor([0, 100, 50, 200], dtype=torch.int64, device="cuda")
    with pytest.raises(og.OrigamiError) as e:
        og.sort_segmented(d, o, kind=og.U32)
    assert e.value.code == og.ERR_INVALID


@pytest.mark.parametrize("kind", [og.U32, og.I64, og.KV64])
def test_segmented_graph_plan(kind):
    rng = np.random.default_rng(40 + kind)
    lens = lengths(kind, rng, 200)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    a = make_items(kind, int(off[-1]), seed=kind + 50)
    d = torch.from_numpy(a.view(np.uint8).copy()).cuda()
    tmp = torch.empty_like(d)
    o = torch.from_numpy(off.astype(np.int64)).cuda()
    src = d.clone()
    plan = og.SegmentedPlan(d, o, tmp, kind=kind)
    assert plan.kernels >= 4  # plan, scan, fill, tile phase, then two kernels per merge level
    s = torch.cuda.current_stream().cuda_stream
    want = expected(a, off)
    for _ in range(3):  # replays over refilled input
        d.copy_(src)
        plan.launch(s)
        plan.status(s)
        assert np.array_equal(d.cpu().numpy().view(a.dtype), want)
    plan.close()


@pytest.mark.parametrize("kind", [og.U32, og.U64, og.I64, og.KV64, og.KVU64])
@pytest.mark.parametrize("shape", [0, 1])
def test_segmented_merge_shapes(kind, shape):
    # both merge shapes of the level merges give the exact per-segment sort
    rng = np.random.default_rng(300 + kind)
    lens = lengths(kind, rng, 120)
    rng.shuffle(lens)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    n, nseg = int(off[-1]), len(lens)
    a = make_items(kind, n, seed=kind + 90, dist="few" if shape else "uniform")
    before = og.seg_tuning_get(kind, n, nseg)
    og.seg_tuning_set(kind, n, nseg, shape)
    try:
        assert og.seg_tuning_get(kind, n, nseg) == shape
        got = run_device(a, off, kind)
    finally:
        og.seg_tuning_set(kind, n, nseg, before)
    assert np.array_equal(got, expected(a, off))


@pytest.mark.parametrize("kind", [og.U32, og.KV64])
def test_segmented_autotune(kind):
    rng = np.random.default_rng(17)
    lens = rng.integers(1 << 12, 1 << 16, 64)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    a = make_items(kind, int(off[-1]), seed=18)
    d = torch.from_numpy(a.view(np.uint8).copy()).cuda()
    tmp = torch.empty_like(d)
    o = torch.from_numpy(off.astype(np.int64)).cuda()
    r = og.autotune_segmented(d, tmp, o, kind)
    assert r["shape"] in (0, 1)
    assert r["report"].count("shape=") == 3  # two timings and the choice
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy().view(a.dtype), a)  # the input is left in d
    og.sort_segmented(d, o, kind=kind)
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy().view(a.dtype), expected(a, off))
