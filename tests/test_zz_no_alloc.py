"""The allocation-free entry point, origami_sort_noalloc_device.

It serves callers that must not allocate device memory during a sort (another
allocator owns the GPU's free memory, a latency-critical loop, a runtime that
forbids the CUDA allocator). Its splitter scratch is a fixed array in the
library's device image instead of arena memory. These tests call it through
the C ABI, twice in a row on the same device (the array keeps the previous
call's contents), and require the same bytes as the regular device entry
point, exactly: the sort is integer work, so the tolerance is zero.
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


def _regular(kind, src, n, sort_n):
    d = src.clone()
    t = torch.empty_like(d)
    res = ctypes.c_void_p()
    s = torch.cuda.current_stream().cuda_stream
    og.check(og.lib().origami_sort_device(kind, d.data_ptr(), t.data_ptr(), n, sort_n, 2, 0,
                                          ctypes.byref(res), ctypes.c_void_p(s)))
    torch.cuda.synchronize()
    return (d if res.value == d.data_ptr() else t).cpu().numpy()


def _noalloc(kind, src, n, sort_n):
    d = src.clone()
    t = torch.empty_like(d)
    res = ctypes.c_void_p()
    s = torch.cuda.current_stream().cuda_stream
    og.check(og.lib().origami_sort_noalloc_device(kind, d.data_ptr(), t.data_ptr(), n, sort_n, 0,
                                                  ctypes.byref(res), ctypes.c_void_p(s)))
    torch.cuda.synchronize()
    return (d if res.value == d.data_ptr() else t).cpu().numpy()


@pytest.mark.parametrize("kind", [og.U32, og.I64, og.KV64])
@pytest.mark.parametrize("sort_n", [0, 1 << 16])
def test_noalloc_matches_regular_entry_point_twice(kind, sort_n):
    n = 3 * (1 << 20) + 77
    for call, seed in enumerate((101, 202)):  # two calls in a row share the array
        src = _random_bytes(n, kind, seed + kind)
        expect = _regular(kind, src, n, sort_n)
        got = _noalloc(kind, src, n, sort_n)
        assert np.array_equal(got, expect), f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_limit():
    kind = og.U32
    limit = og.lib().origami_noalloc_max_items(kind)
    assert limit >= (1 << 28)  # the 1 GiB workload fits
    buf = torch.empty(64, dtype=torch.uint8, device="cuda")
    res = ctypes.c_void_p()
    far = buf.data_ptr() + (1 << 44)  # never dereferenced: the call is rejected first
    rc = og.lib().origami_sort_noalloc_device(kind, buf.data_ptr(), far, limit + 1, 0, 0,
                                              ctypes.byref(res), None)
    assert rc == og.ERR_INVALID
    assert b"limit" in og.lib().origami_last_error()
