"""The oracle (oracle/origami_oracle.c) pinned to the reference.

1. Against the committed digests the UNMODIFIED reference produced
   (tests/golden/reference_digests.json, written by tests/golden/make_golden.py):
   generated inputs, sorted keys, (key, value) multisets and the result buffer.
2. Where the reference was compiled on this machine (oracle/_ref), live
   comparisons on seeded inputs the digests do not cover.
"""
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_digests.json")


def h(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def _golden():
    with open(GOLDEN) as f:
        doc = json.load(f)
    cols = doc["columns"]
    return doc["variants"], [dict(zip(cols, c)) for c in doc["cases"]]


VARIANTS, CASES = _golden()


def _ids(c):
    return f"{c['variant']}-n{c['n']}-d{c['dist']}-s{c['sort_n']}-k{c['min_k']}"


_inputs = {}


def _input(orc, kind, n, dist):
    key = (kind, n, dist)
    if key not in _inputs:
        _inputs[key] = orc.generate(kind, n, dist)
    return _inputs[key]


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_oracle_matches_reference_digest(orc, case):
    var = VARIANTS[case["variant"]]
    kind, n = var["kind"], case["n"]
    src = _input(orc, kind, n, case["dist"])
    # the oracle's datagen::Writer restatement reproduces the reference's input bytes
    assert h(src) == case["input"]
    out, where = orc.sort_single_thread(kind, src, case["sort_n"], case["min_k"], var["p1_n"],
                                        var["p2_n"])
    keys = orc.keys_of(out)
    if case["ref_correct"]:
        # bit-identical keys to the reference
        assert h(keys) == case["keys"]
    else:
        # the reference itself mis-sorts this case; the oracle must equal std::sort
        expect = np.concatenate([np.sort(orc.keys_of(src)[c:c + case["sort_n"]])
                                 for c in range(0, n, case["sort_n"])])
        assert np.array_equal(keys, expect)
        assert h(keys) != case["keys"]
    if case["pairs"] is not None:
        assert h(orc.pairs_sorted(out).view(np.int64)) == case["pairs"]
    # same result buffer (d or tmp) as the reference build with these phase sizes
    assert where == case["result"]


def test_reference_defects_are_recorded():
    """The reference's k-way merge tree mis-sorts Pareto back-to-back inputs with
    64-bit keys (which include negative i64 keys); every other digest is a
    correct sort."""
    bad = [(c["variant"], c["dist"], c["min_k"]) for c in CASES if not c["ref_correct"]]
    assert bad and all(d == 7 and k == 4 for _, d, k in bad)


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("n", [0, 1, 7, 1000, 65537, 300001])
def test_oracle_sorts_any_size(orc, kind, n):
    rng = np.random.default_rng(n + 17 * kind)
    a = orc.empty(kind, n)
    if a.dtype.names:
        a["key"] = rng.integers(0, 1 << 20, n) if kind == 3 else rng.integers(0, 1 << 20, n)
        a["value"] = np.arange(n)
    else:
        info = np.iinfo(a.dtype)
        a[:] = rng.integers(info.min, info.max, n, dtype=a.dtype, endpoint=True)
    for min_k in (2, 8):
        out, _ = orc.sort_single_thread(kind, a, 0, min_k)
        assert np.array_equal(orc.keys_of(out), np.sort(orc.keys_of(a)))
        if a.dtype.names:
            assert np.array_equal(orc.pairs_sorted(out), orc.pairs_sorted(a))


@pytest.mark.parametrize("kind", [0, 2, 3])
def test_oracle_multi_thread(orc, kind):
    n = 3 * 131072 + 12345
    a = orc.generate(kind, n, 7 if kind else 1)
    for threads, min_k in ((4, 2), (8, 4), (3, 8)):
        out = orc.sort_multi_thread(kind, a, threads, min_k)
        assert np.array_equal(orc.keys_of(out), np.sort(orc.keys_of(a)))
        if a.dtype.names:
            assert np.array_equal(orc.pairs_sorted(out), orc.pairs_sorted(a))


def test_oracle_partition_exact_with_ties(orc):
    rng = np.random.default_rng(5)
    streams = [np.sort(rng.integers(0, 50, m).astype(np.uint32)) for m in (100, 257, 3, 0, 999)]
    total = sum(len(s) for s in streams)
    merged = np.sort(np.concatenate(streams))
    for target in (0, 1, 100, 500, total - 1, total):
        guess = [len(s) * target // total for s in streams]
        rest = target - sum(guess)
        for i, s in enumerate(streams):
            add = min(rest, len(s) - guess[i])
            guess[i] += add
            rest -= add
        S = orc.partition_ptrs(0, streams, guess)
        assert sum(S) == target
        left = np.concatenate([s[:k] for s, k in zip(streams, S)])
        right = np.concatenate([s[k:] for s, k in zip(streams, S)])
        assert np.array_equal(np.sort(left), merged[:target])
        if len(left) and len(right):
            assert left.max() <= right.min()


@pytest.mark.parametrize("variant", ["s_u32", "a2_u32", "s_i64", "a2_kv"])
def test_oracle_live_against_reference(orc, variant):
    if variant not in orc.ref_variants():
        pytest.skip("reference not compiled on this machine (x86 container only)")
    R = orc.ref_lib(variant)
    var = VARIANTS[variant]
    kind, p1, p2 = var["kind"], var["p1_n"], var["p2_n"]
    rng = np.random.default_rng(1234)
    n = 8 * p2
    for trial in range(3):
        a = orc.empty(kind, n)
        if a.dtype.names:
            a["key"] = rng.integers(0, 1 << 40, n)
            a["value"] = np.arange(n)
        else:
            a[:] = rng.integers(0, np.iinfo(a.dtype).max, n, dtype=a.dtype)
        for sort_n, min_k in ((n, 2), (2 * p2, 2), (n, 8)):
            d = orc.empty(kind, n)
            d[:] = a
            t = orc.empty(kind, n)
            buf = orc.empty(0, 64 << 20)
            r = R.ref_sort_single_thread(d.ctypes.data, t.ctypes.data, n, sort_n, min_k,
                                         buf.ctypes.data)
            ref_out = d if r == d.ctypes.data else t
            out, where = orc.sort_single_thread(kind, a, sort_n, min_k, p1, p2)
            assert np.array_equal(orc.keys_of(out), orc.keys_of(ref_out))
            assert where == ("d" if r == d.ctypes.data else "tmp")
            if a.dtype.names:
                assert np.array_equal(orc.pairs_sorted(out), orc.pairs_sorted(ref_out))
