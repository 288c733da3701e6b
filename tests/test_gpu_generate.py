"""Device-side Writer generators (writer.h:27-35) against the oracle's
restatement of the reference's host generator.

Distributions 2 (all same), 6 (Pareto keys), 7 (Pareto back to back) and
9 (Fibonacci) are the reference's exact sequences: compared item for item.
The others draw from a counter-based generator instead of the reference's
sequential mt19937 stream and are checked by their defining property."""
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


def gen(kind, n, dist, seed=5):
    d = torch.empty(n * og.ITEM_BYTES[kind], dtype=torch.uint8, device="cuda")
    og.generate(d, dist, kind=kind, seed=seed)
    torch.cuda.synchronize()
    return d.cpu().numpy().view(orc.DTYPES[kind])


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("dist", [2, 6, 7, 9])
@pytest.mark.parametrize("n", [1, 10, 11, 1000, 123457, 1 << 21])
def test_exact_distributions_match_reference_sequence(kind, dist, n):
    assert np.array_equal(gen(kind, n, dist), orc.generate(kind, n, dist))


@pytest.mark.parametrize("kind", KINDS)
def test_uniform_sorted_reverse_almost(kind):
    n = 300_001
    u = gen(kind, n, 1)
    k = orc.keys_of(u)
    if kind == og.U32:
        assert k.max() > 0xF0000000
    elif kind == og.U64:
        assert k.max() > 0xF000_0000_0000_0000
    else:  # the reference's signed draw: [0, 2^63)
        assert int(k.min()) >= 0 and int(k.max()) > 0x7000_0000_0000_0000
    if og.ITEM_BYTES[kind] == 16:
        assert np.array_equal(u["value"].astype(np.uint64), u["key"].astype(np.uint64) + np.uint64(1))
    s = orc.keys_of(gen(kind, n, 3))
    assert np.all(s[1:] >= s[:-1]) and np.array_equal(s, np.sort(k))
    r = orc.keys_of(gen(kind, n, 4))
    assert np.array_equal(r, np.sort(k)[::-1])
    a = gen(kind, n, 5)
    ak = orc.keys_of(a)
    top = 0xFFFFFFFF if kind == og.U32 else 0x7FFF_FFFF_FFFF_FFFF
    assert np.all(ak[::7] == top)
    mask = np.ones(n, bool)
    mask[::7] = False
    assert np.array_equal(ak[mask], k[mask])


@pytest.mark.parametrize("kind", [og.U32, og.KV64])
def test_pareto_shuffled_is_a_permutation_of_back_to_back(kind):
    n = 200_003
    b2b = gen(kind, n, 7)
    sh = gen(kind, n, 8, seed=9)
    assert not np.array_equal(sh, b2b)
    assert np.array_equal(np.sort(orc.keys_of(sh)), np.sort(orc.keys_of(b2b)))
