"""The autotuner and the other binary-pass merge shapes it can choose.

Every tile shape is a different merge kernel, so each is held to the same bar
as the default: bit-identical to a stable sort (the oracle's restatement of the
reference for keys) at several sizes and kinds."""
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


def make(kind, n, seed):
    rng = np.random.default_rng(seed)
    a = orc.empty(kind, n)
    k = rng.integers(0, 2**64, n, dtype=np.uint64)
    if kind == og.U32:
        a[:] = (k >> np.uint64(40)).astype(np.uint32)  # duplicates on purpose
    elif kind == og.U64:
        a[:] = k >> np.uint64(20)
    elif kind == og.I64:
        a[:] = (k >> np.uint64(20)).view(np.int64) - (1 << 43)
    else:
        a["key"] = (k >> np.uint64(44)).astype(a.dtype["key"])
        a["value"] = np.arange(n)
    return a


def expected(a):
    return a[np.argsort(orc.keys_of(a), kind="stable")]


@pytest.mark.parametrize("variant", [1, 2, 3])
@pytest.mark.parametrize("kind", [og.U32, og.U64, og.I64, og.KV64, og.KVU64])
@pytest.mark.parametrize("n", [5000, 300_007, (1 << 22) + 9])
def test_merge_shape_parity(kind, n, variant):
    a = make(kind, n, seed=n + kind)
    prev = og.tuning_get(kind, n)
    try:
        og.tuning_set(kind, n, 2, variant)
        d = torch.from_numpy(a.view(np.uint8).copy()).cuda()
        t = torch.empty_like(d)
        r = og.sort(d, t, kind=kind)
        torch.cuda.synchronize()
        got = r.cpu().numpy().view(a.dtype)
        assert np.array_equal(got, expected(a))
        # host buffers through the same tuned shape
        h = a.copy()
        og.sort(h, orc.empty(kind, n))
        assert np.array_equal(h, expected(a))
    finally:
        og.tuning_set(kind, n, *prev)


@pytest.mark.parametrize("kind", [og.U32, og.KV64])
def test_autotune_chooses_and_sorts(kind):
    n = 1 << 22
    prev = og.tuning_get(kind, n)
    try:
        r = og.autotune(kind, n)
        lines = [l for l in r["report"].splitlines() if l.startswith("fan=")]
        assert len(lines) == 7  # four binary merge shapes, fan-in 4, 8 and 16
        assert r["fan"] in (2, 4, 8, 16) and r["variant"] in (0, 1, 2, 3)
        assert og.tuning_get(kind, n) == (r["fan"], r["variant"])
        a = make(kind, n, seed=1)
        d = torch.from_numpy(a.view(np.uint8).copy()).cuda()
        out = og.sort(d, torch.empty_like(d), kind=kind)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().view(a.dtype), expected(a))
    finally:
        og.tuning_set(kind, n, *prev)


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("kind", [og.U32, og.KV64])
def test_concurrent_streams(kind, variant):
    # sorts on four streams at once: the persistent merge kernels of one sort
    # start while another's hold the SMs and claim fewer tiles; every result
    # must still equal the stable sort
    n = (1 << 21) + 5
    arrays = [make(kind, n, seed=100 + i) for i in range(4)]
    prev = og.tuning_get(kind, n)
    try:
        og.tuning_set(kind, n, 2, variant)
        streams = [torch.cuda.Stream() for _ in arrays]
        dev = [torch.from_numpy(a.view(np.uint8).copy()).cuda() for a in arrays]
        tmp = [torch.empty_like(d) for d in dev]
        torch.cuda.synchronize()
        res = [og.sort(d, t, kind=kind, stream=s.cuda_stream) for d, t, s in zip(dev, tmp, streams)]
        torch.cuda.synchronize()
        for a, r in zip(arrays, res):
            assert np.array_equal(r.cpu().numpy().view(a.dtype), expected(a))
    finally:
        og.tuning_set(kind, n, *prev)
