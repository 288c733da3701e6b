"""GPU parity tests of the plain sort through the C ABI.

Every result is compared bit for bit with the oracle (oracle/origami_oracle.c,
pinned to the reference) on the same seeded input; key-value results are also
compared with numpy's stable sort, since the GPU sort is stable. At larger
sizes the checks are torch.sort on the device plus size-independent
properties (sortedness, key checksum, multiset)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as orc
import origami_gpu as og

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KINDS = [og.U32, og.U64, og.I64, og.KV64, og.KVU64]
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_digests.json")


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()
    assert torch.cuda.is_available()


def h(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()


def to_host(t, dt):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(dt)


def make(kind, n, dist, seed=0):
    rng = np.random.default_rng(seed * 1000 + n + 7 * kind)
    a = orc.empty(kind, n)
    if dist == "uniform":
        k = rng.integers(0, 2**64, n, dtype=np.uint64)
    elif dist == "equal":
        k = np.full(n, rng.integers(0, 2**64, dtype=np.uint64), np.uint64)
    elif dist == "sorted":
        k = np.sort(rng.integers(0, 2**64, n, dtype=np.uint64))
    elif dist == "reverse":
        k = np.sort(rng.integers(0, 2**64, n, dtype=np.uint64))[::-1].copy()
    elif dist == "few":
        k = rng.integers(0, 16, n).astype(np.uint64)
    elif dist == "zipf":
        k = np.minimum(rng.zipf(1.2, n), 1 << 20).astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    elif dist == "runs8":
        k = np.empty(n, np.uint64)
        for r in range(8):
            m = len(k[r::8])
            k[r::8] = np.sort(rng.integers(0, 2**64, m, dtype=np.uint64))
    else:
        raise ValueError(dist)
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


def expected(a, sort_n=0):
    """Stable chunk sort (numpy) - equal to the GPU output bit for bit."""
    n = len(a)
    step = n if sort_n == 0 or sort_n >= n else sort_n
    keys = orc.keys_of(a)
    chunk = np.arange(n, dtype=np.int64) // max(step, 1)
    return a[np.lexsort((keys, chunk))]  # lexsort is stable


def gpu_sort_device(a, kind, sort_n=0, result_in_tmp=False, min_k=0):
    d = to_dev(a)
    t = torch.empty_like(d)
    r = og.sort(d, t, sort_n=sort_n, min_k=min_k, kind=kind, result_in_tmp=result_in_tmp)
    assert (r is t) == result_in_tmp or len(a) == 0
    return to_host(r, a.dtype)


def check_against_oracle(kind, a, got, sort_n=0):
    ora, _ = orc.sort_single_thread(kind, a, sort_n)
    assert np.array_equal(orc.keys_of(got), orc.keys_of(ora))
    if a.dtype.names:
        assert np.array_equal(orc.pairs_sorted(got), orc.pairs_sorted(ora))
    assert np.array_equal(got, expected(a, sort_n))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("n", [1, 2, 3, 31, 1000, 2047, 2048, 2049, 4096, 8191, 8192, 8193,
                               65541, 300007])
@pytest.mark.parametrize("min_k", [2, 4, 0])
def test_sizes(kind, n, min_k):
    a = make(kind, n, "uniform")
    check_against_oracle(kind, a, gpu_sort_device(a, kind, min_k=min_k))


DISTS = ["uniform", "equal", "sorted", "reverse", "few", "zipf", "runs8"]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("dist", DISTS)
@pytest.mark.parametrize("min_k", [2, 16])
def test_distributions(kind, dist, min_k):
    a = make(kind, (1 << 18) + 3, dist, seed=1)
    check_against_oracle(kind, a, gpu_sort_device(a, kind, min_k=min_k))


# sizes at which a k-way pass splits its groups into exact ranges (K4)
RANGED = {og.U32: 3 * (1 << 20) + 7, og.U64: 3 * (1 << 19) + 5, og.I64: 3 * (1 << 19) + 5,
          og.KV64: 600_001, og.KVU64: 600_001}


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("dist", DISTS)
@pytest.mark.parametrize("min_k", [4, 8, 16])
def test_kway_ranges(kind, dist, min_k):
    a = make(kind, RANGED[kind], dist, seed=7)
    check_against_oracle(kind, a, gpu_sort_device(a, kind, min_k=min_k))


@pytest.mark.parametrize("kind", [og.U32, og.I64, og.KV64])
@pytest.mark.parametrize("sort_n", [2, 8, 64, 1024, 2048, 4096, 8192, 65536, 1 << 20])
@pytest.mark.parametrize("min_k", [2, 0])
def test_chunked(kind, sort_n, min_k):
    a = make(kind, (1 << 21) + 1000, "uniform", seed=2)
    check_against_oracle(kind, a, gpu_sort_device(a, kind, sort_n, min_k=min_k), sort_n)


@pytest.mark.parametrize("kind", KINDS)
def test_result_in_tmp(kind):
    a = make(kind, 100_003, "few", seed=3)
    check_against_oracle(kind, a, gpu_sort_device(a, kind, result_in_tmp=True))


@pytest.mark.parametrize("kind", KINDS)
def test_host_buffers(kind):
    a = make(kind, 123_457, "uniform", seed=4)
    d = a.copy()
    t = np.zeros_like(a)
    r = og.sort_single_thread(d, t)
    assert r is d
    check_against_oracle(kind, a, r)
    d2 = a.copy()
    r2 = og.sort(d2, t, result_in_tmp=True)
    assert r2 is t
    assert np.array_equal(r2, expected(a))


def test_pinned_host_buffers():
    a = make(og.U32, 1 << 20, "uniform", seed=5)
    d = og.empty_host("u32", len(a), pinned=True)
    d[:] = a
    t = og.empty_host("u32", len(a), pinned=True)
    r = og.sort_multi_thread(d, t, n_threads=8, n_cores=8, min_k=16)
    assert np.array_equal(r, np.sort(a))


@pytest.mark.parametrize("kind,n,pinned,sort_n", [
    (og.U32, (1 << 24) + 12345, False, 0),
    (og.U32, 1 << 25, True, 0),
    (og.I64, (1 << 24) + 7, True, 0),
    (og.KV64, (1 << 24) + 3, False, 0),
    (og.U64, 1 << 24, True, 1 << 23),
    (og.KVU64, 1 << 24, True, 1 << 23),
    # 16 chunks merged by one 16-way pass: into pinned output by slices, and
    # into pageable output directly
    (og.U32, 1 << 26, True, 0),
    (og.U64, 1 << 26, False, 0),
])
def test_host_chunked_pipeline(kind, n, pinned, sort_n):
    """Large host sorts: chunks sorted while the next ones arrive, then merged,
    the last pass writing the host buffer (pinned and pageable memory)."""
    a = make(kind, n, "uniform", seed=11)
    d = og.empty_host(kind, n, pinned=pinned) if pinned else orc.empty(kind, n)
    d[:] = a
    t = og.empty_host(kind, n, pinned=pinned) if pinned else orc.empty(kind, n)
    r = og.sort(d, t, sort_n=sort_n)
    assert r is d
    assert np.array_equal(d, expected(a, sort_n))


@pytest.mark.parametrize("kind,n", [(og.U32, (1 << 25) + 99), (og.KV64, (1 << 24) + 3)])
@pytest.mark.parametrize("min_k", [2, 4, 8])
def test_host_chunked_pipeline_fan(kind, n, min_k):
    """Pinned host sorts whose chunks use binary passes (min_k = 2: the first
    chunk arrives whole) or k-way passes (min_k = 4, 8: the first chunk
    arrives in four pieces, merged by one pass)."""
    a = make(kind, n, "uniform", seed=13)
    d = og.empty_host(kind, n, pinned=True)
    d[:] = a
    t = og.empty_host(kind, n, pinned=True)
    r = og.sort(d, t, min_k=min_k)
    assert r is d
    assert np.array_equal(d, expected(a))


def _golden_cases(variant):
    with open(GOLDEN) as f:
        doc = json.load(f)
    cols = doc["columns"]
    var = doc["variants"][variant]
    return var, [dict(zip(cols, c)) for c in doc["cases"] if c[0] == variant]


@pytest.mark.parametrize("variant", ["a2_u32", "a2_i64", "a2_kv"])
def test_reference_digests(variant):
    """The GPU output hashes to the digest the UNMODIFIED reference produced."""
    var, cases = _golden_cases(variant)
    kind = var["kind"]
    done = 0
    for c in cases:
        if not c["ref_correct"] or c["min_k"] != 2:
            continue
        a = orc.generate(kind, c["n"], c["dist"])
        assert h(a) == c["input"]
        got = gpu_sort_device(a, kind, c["sort_n"])
        assert h(orc.keys_of(got)) == c["keys"], c
        if c["pairs"] is not None:
            assert h(orc.pairs_sorted(got).view(np.int64)) == c["pairs"]
        done += 1
    assert done >= 16


@pytest.mark.parametrize("kind", [og.U32, og.KV64])
@pytest.mark.parametrize("merge_start,sort_n", [(8, 1024), (4096, 65536), (16, 1 << 18)])
def test_merge_series(kind, merge_start, sort_n):
    n = 1 << 18
    a = make(kind, n, "uniform", seed=6)
    runs = expected(a, merge_start)  # sorted runs of merge_start
    src = to_dev(runs)
    dst = torch.empty_like(src)
    r = og.merge_series(src, dst, merge_start, sort_n, kind=kind)
    levels = int(np.log2(sort_n // merge_start))
    assert (r is dst) == (levels % 2 == 1)  # merger.h:4220-4228 ping-pong rule
    assert np.array_equal(to_host(r, a.dtype), expected(runs, sort_n))


@pytest.mark.parametrize("kind,n", [(og.U32, 1 << 26), (og.U64, 1 << 25), (og.KV64, 1 << 24),
                                    (og.U32, (1 << 28) + 12345)])
@pytest.mark.parametrize("min_k", [0, 16])  # the tuned (binary) passes, and 16-way passes
def test_large_against_torch_sort(kind, n, min_k):
    g = torch.Generator(device="cuda").manual_seed(11)
    words = 4 if kind == og.U32 else (8 if kind == og.U64 else 16)
    raw = torch.randint(0, 256, (n * words,), dtype=torch.uint8, device="cuda", generator=g)
    keep = raw.clone()
    tmp = torch.empty_like(raw)
    out = og.sort(raw, tmp, kind=kind, min_k=min_k)
    torch.cuda.synchronize()
    if kind == og.U32:
        k_in = keep.view(torch.int32).to(torch.int64) & 0xFFFFFFFF
        k_out = out.view(torch.int32).to(torch.int64) & 0xFFFFFFFF
        assert torch.equal(torch.sort(k_in).values, k_out)
    elif kind == og.U64:
        # unsigned order = signed order after flipping the top bit
        flip = torch.tensor(-(2**63), dtype=torch.int64, device="cuda")
        k_in = keep.view(torch.int64) ^ flip
        k_out = out.view(torch.int64) ^ flip
        assert torch.equal(torch.sort(k_in).values, k_out)
    else:
        kv_in = keep.view(torch.int64).view(-1, 2)
        kv_out = out.view(torch.int64).view(-1, 2)
        flip = torch.tensor(-(2**63), dtype=torch.int64, device="cuda")
        ks = torch.sort(kv_in[:, 0], stable=True)
        assert torch.equal(ks.values, kv_out[:, 0])
        assert torch.equal(kv_in[ks.indices, 1], kv_out[:, 1])  # stable: values follow input order
        del flip


@pytest.mark.parametrize("kind", [og.U32, og.U64])
@pytest.mark.parametrize("shift_items", [1, 3])
def test_misaligned_device_buffers(kind, shift_items):
    """Device buffers that are item-aligned but not 16-byte aligned are sorted
    through aligned staging; results are unchanged."""
    n = 100_003
    a = make(kind, n, "uniform", seed=9)
    ib = og.ITEM_BYTES[kind]
    raw = torch.zeros((n + 8) * ib, dtype=torch.uint8, device="cuda")
    rawt = torch.zeros_like(raw)
    d = raw[shift_items * ib: shift_items * ib + n * ib]
    t = rawt[shift_items * ib: shift_items * ib + n * ib]
    d.copy_(torch.from_numpy(a.view(np.uint8).copy()).cuda())
    r = og.sort(d, t, kind=kind)
    assert r is d
    check_against_oracle(kind, a, to_host(r, a.dtype))


@pytest.mark.parametrize("kind,n", [(og.U32, (1 << 20) + 3), (og.U32, 1 << 25), (og.KV64, 1 << 23), (og.U64, 300_007)])
def test_sort_captured_in_cuda_graph(kind, n):
    # the device sort is stream-ordered end to end (its scratch comes from the
    # stream-ordered allocator), so a CUDA graph can record it once and replay
    # it over refilled input; sizes include classes where the tuning table
    # picks 16-way passes (u32 2^25, key-value 2^23)
    words = {og.U32: 4, og.U64: 8, og.KV64: 16}[kind]
    g = torch.Generator(device="cuda").manual_seed(n)
    src = torch.randint(0, 256, (n * words,), dtype=torch.uint8, device="cuda", generator=g)
    d, t = src.clone(), torch.empty_like(src)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        og.sort(d, t, kind=kind)  # first use outside the capture (tables, kernel attributes)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        out = og.sort(d, t, kind=kind)
    expect = None
    for seed in (1, 2):
        src = torch.randint(0, 256, (n * words,), dtype=torch.uint8, device="cuda",
                            generator=torch.Generator(device="cuda").manual_seed(seed))
        d.copy_(src)
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        if kind == og.KV64:
            kv = src.view(torch.int64).view(-1, 2)
            ks = torch.sort(kv[:, 0], stable=True)
            res = out.view(torch.int64).view(-1, 2)
            assert torch.equal(ks.values, res[:, 0]) and torch.equal(kv[ks.indices, 1], res[:, 1])
        else:
            flip = torch.tensor(-(2**63), dtype=torch.int64, device="cuda")
            if kind == og.U32:
                expect = torch.sort(src.view(torch.int32).to(torch.int64) & 0xFFFFFFFF).values
                got = out.view(torch.int32).to(torch.int64) & 0xFFFFFFFF
            else:
                expect = torch.sort(src.view(torch.int64) ^ flip).values
                got = out.view(torch.int64) ^ flip
            assert torch.equal(expect, got)
