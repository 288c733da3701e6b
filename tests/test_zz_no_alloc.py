"""The allocation-free entry point, origami_sort_noalloc_device.

It serves callers that must not allocate device memory during a sort (another
allocator owns the GPU's free memory, a latency-critical loop, a runtime that
forbids the CUDA allocator). Its splitter scratch is a fixed array in the
library's device image instead of arena memory. These tests call it through
the C ABI, twice in a row on the same device (the array keeps the previous
call's contents), and require the same bytes as the regular device entry
point, exactly: the sort is integer work, so the tolerance is zero.

The size limit and the argument checks are host logic and are tested on the
CPU (tests/test_capi.py), with buffers that are never touched.
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


def _random_bytes(n_items, kind, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    nbytes = n_items * og.ITEM_BYTES[kind]
    return torch.randint(0, 256, (nbytes,), dtype=torch.uint8, device="cuda", generator=g)


def _regular(kind, src, n, sort_n, flags=0):
    d = src.clone()
    t = torch.empty_like(d)
    res = ctypes.c_void_p()
    s = torch.cuda.current_stream().cuda_stream
    og.check(og.lib().origami_sort_device(kind, d.data_ptr(), t.data_ptr(), n, sort_n, 2, flags,
                                          ctypes.byref(res), ctypes.c_void_p(s)))
    torch.cuda.synchronize()
    return d if res.value == d.data_ptr() else t


def _noalloc(kind, src, n, sort_n, flags=0):
    d = src.clone()
    t = torch.empty_like(d)
    res = ctypes.c_void_p()
    s = torch.cuda.current_stream().cuda_stream
    og.check(og.lib().origami_sort_noalloc_device(kind, d.data_ptr(), t.data_ptr(), n, sort_n, flags,
                                                  ctypes.byref(res), ctypes.c_void_p(s)))
    torch.cuda.synchronize()
    want = t if flags & og.FLAG_RESULT_IN_TMP else d
    assert res.value == want.data_ptr()
    return want


@pytest.mark.parametrize("kind", [og.U32, og.U64, og.I64, og.KV64, og.KVU64])
@pytest.mark.parametrize("sort_n", [0, 1 << 16])
def test_noalloc_matches_regular_entry_point_twice(kind, sort_n):
    n = 3 * (1 << 20) + 77
    for call, seed in enumerate((101, 202)):  # two calls in a row share the array
        src = _random_bytes(n, kind, seed + kind)
        expect = _regular(kind, src, n, sort_n)
        got = _noalloc(kind, src, n, sort_n)
        assert torch.equal(got, expect), f"call {call}"


@pytest.mark.parametrize("flags", [og.FLAG_RESULT_IN_TMP, og.FLAG_RESULT_IN_TMP | og.FLAG_SYNC, og.FLAG_SYNC])
@pytest.mark.parametrize("kind", [og.U32, og.KV64])
def test_noalloc_result_buffer_and_sync(kind, flags):
    n = (1 << 18) + 5
    for seed in (11, 12):
        src = _random_bytes(n, kind, seed)
        expect = _regular(kind, src, n, 0, flags & og.FLAG_RESULT_IN_TMP)
        got = _noalloc(kind, src, n, 0, flags)
        assert torch.equal(got, expect)


@pytest.mark.parametrize("flags", [0, og.FLAG_RESULT_IN_TMP, og.FLAG_RESULT_IN_TMP | og.FLAG_SYNC])
def test_noalloc_zero_and_one_item(flags):
    for n in (0, 1):
        src = _random_bytes(max(n, 1), og.KV64, 5)
        got = _noalloc(og.KV64, src, n, 0, flags)
        if n == 1:
            assert torch.equal(got, src)


def test_noalloc_at_the_headline_size_twice():
    # 268,435,456 uint32 keys (1 GiB): the far end of the scratch array is used
    n = 1 << 28
    assert n <= og.lib().origami_noalloc_max_items(og.U32)
    for seed in (31, 32):
        src = _random_bytes(n, og.U32, seed)
        expect = _regular(og.U32, src, n, 0)
        got = _noalloc(og.U32, src, n, 0, og.FLAG_SYNC)
        assert torch.equal(got, expect)
        del expect, got, src
        torch.cuda.empty_cache()
