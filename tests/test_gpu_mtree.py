"""GPU parity of the merge tree (MergeTree::merge over pointer-bounded streams,
merge_tree.h:2792) and the partitioner (Partition_Ptrs, Partition.h:118).

Merges are compared item for item with the oracle's stable winner-tree k-way
merge (ties taken from the lower stream, which the GPU merge also does), so
key-value results must match exactly, values included. Splits are compared
with the rank rule (the r smallest items under (key, stream, position) order)
and, on distinct keys, with the oracle's restatement of Partition_Ptrs."""
import numpy as np
import pytest

import oracle as orc
import origami_gpu as og

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KINDS = [og.U32, og.U64, og.I64, og.KV64, og.KVU64]


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()
    assert torch.cuda.is_available()


def sorted_stream(kind, n, rng, dist):
    a = orc.empty(kind, n)
    if dist == "uniform":
        k = rng.integers(0, 2**64, n, dtype=np.uint64)
    elif dist == "few":
        k = rng.integers(0, 5, n).astype(np.uint64) << np.uint64(61)
    else:  # equal
        k = np.full(n, 0x8000_0000_0000_0001, np.uint64)
    if kind == og.U32:
        a[:] = (k >> np.uint64(32)).astype(np.uint32)
    elif kind == og.U64:
        a[:] = k
    elif kind == og.I64:
        a[:] = k.view(np.int64)
    elif kind == og.KV64:
        a["key"] = k.view(np.int64)
        a["value"] = rng.integers(0, 2**62, n)
    else:
        a["key"] = k
        a["value"] = rng.integers(0, 2**62, n).astype(np.uint64)
    return a[np.argsort(orc.keys_of(a), kind="stable")]


def to_dev(a):
    return torch.from_numpy(a.view(np.uint8).copy()).cuda()


def make_streams(kind, lens, seed, dist):
    rng = np.random.default_rng(seed)
    host = [sorted_stream(kind, int(n), rng, dist) for n in lens]
    return host, [to_dev(h) for h in host]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("way", [1, 2, 3, 4, 7, 16, 17, 40, 300])
@pytest.mark.parametrize("dist", ["uniform", "few"])
def test_merge_tree_matches_oracle(kind, way, dist):
    rng = np.random.default_rng(way * 10 + kind)
    lens = rng.integers(0, 3000, way)
    if way > 2:
        lens[1] = 0  # an empty stream in the middle
    host, dev = make_streams(kind, lens, seed=way + 7 * kind, dist=dist)
    total = int(sum(lens))
    out = torch.empty(total * og.ITEM_BYTES[kind], dtype=torch.uint8, device="cuda")
    og.merge_tree(dev, out, kind=kind)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(host[0].dtype)
    want = orc.kway_merge(kind, host)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("kind", [og.U32, og.I64, og.KV64])
def test_merge_tree_large_ranges(kind):
    # several k-way ranges per pass, and a two-level tree (way > 16)
    for way, n in ((8, 1 << 19), (24, 1 << 17)):
        lens = [n + (i * 977) % 5000 for i in range(way)]
        host, dev = make_streams(kind, lens, seed=way, dist="uniform")
        out = torch.empty(sum(lens) * og.ITEM_BYTES[kind], dtype=torch.uint8, device="cuda")
        og.merge_tree(dev, out, kind=kind)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().view(host[0].dtype), orc.kway_merge(kind, host))


def test_merge_tree_equal_keys_keep_stream_order():
    host, dev = make_streams(og.KV64, [1000, 2000, 1500, 10], seed=3, dist="equal")
    out = torch.empty(4510 * 16, dtype=torch.uint8, device="cuda")
    og.merge_tree(dev, out, kind=og.KV64)
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(host[0].dtype)
    assert np.array_equal(got, np.concatenate(host))


def rank_splits(kind, host, r):
    keys = np.concatenate([orc.keys_of(h) for h in host])
    sid = np.concatenate([np.full(len(h), i) for i, h in enumerate(host)])
    order = np.argsort(keys, kind="stable")  # (key, stream, position)
    return np.bincount(sid[order[:r]], minlength=len(host))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("K", [1, 5, 16, 100, 256])
@pytest.mark.parametrize("dist", ["uniform", "few", "equal"])
def test_partition_rank_rule(kind, K, dist):
    rng = np.random.default_rng(K + kind)
    lens = rng.integers(0, 700, K)
    host, dev = make_streams(kind, lens, seed=K * 3 + kind, dist=dist)
    total = int(sum(lens))
    ranks = np.unique(np.concatenate([[0, total, max(total - 1, 0), 1], rng.integers(0, total + 1, 20)]))
    got = og.partition(dev, ranks, kind=kind)
    for j, r in enumerate(ranks):
        assert np.array_equal(got[j], rank_splits(kind, host, int(r))), (int(r), total)
        assert int(got[j].sum()) == min(int(r), total)


@pytest.mark.parametrize("kind", [og.U32, og.U64, og.I64, og.KVU64])
def test_partition_ptrs_matches_oracle(kind):
    # distinct keys: the reference's pointer walk and the rank split agree
    rng = np.random.default_rng(kind)
    K = 12
    lens = rng.integers(100, 5000, K)
    host, dev = make_streams(kind, lens, seed=kind + 1, dist="uniform")
    total = int(sum(lens))
    keys = np.concatenate([orc.keys_of(h) for h in host])
    distinct = len(np.unique(keys)) == total
    for target in (1, total // 3, total // 2, total - 1):
        guesses = [int(n * target // total) for n in lens]
        for k in range(K):  # hand the remainder to streams with room: L <= S <= R
            guesses[k] += min(target - sum(guesses), int(lens[k]) - guesses[k])
        got = og.partition_ptrs(dev, guesses, kind=kind)
        assert got == [int(x) for x in rank_splits(kind, host, target)]
        if distinct:
            assert got == orc.partition_ptrs(kind, host, guesses)


def test_partition_and_merge_tree_reject_bad_arguments():
    a = to_dev(sorted_stream(og.U32, 100, np.random.default_rng(0), "uniform"))
    with pytest.raises(og.OrigamiError) as e:
        og.merge_tree([a, a[4:]], a, kind=og.U32)  # output overlaps an input
    assert e.value.code == og.ERR_INVALID
    kv = to_dev(sorted_stream(og.KV64, 10, np.random.default_rng(0), "uniform"))
    out = torch.empty(160, dtype=torch.uint8, device="cuda")
    with pytest.raises(og.OrigamiError) as e:
        og.merge_tree([kv[8:]], out, kind=og.KV64)  # key-value stream not 16-byte aligned
    assert e.value.code == og.ERR_ALIGN
    with pytest.raises(og.OrigamiError) as e:
        og.partition([a] * 1025, [1], kind=og.U32)
    assert e.value.code == og.ERR_INVALID
