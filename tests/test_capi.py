"""C-ABI checks that need no GPU: the library loads, exports every symbol
include/origami_gpu.h declares, and rejects bad arguments with the documented
status codes before touching a device."""
import ctypes
import os
import re

import numpy as np
import pytest

import origami_gpu as og

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    syms = set()
    for f in os.listdir(HDR):
        if f.endswith(".h"):
            text = open(os.path.join(HDR, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(origami_\w+)\s*\(", text))
    return sorted(syms)


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build_library()
    return og.lib()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/ but not exported"


def test_version_and_item_bytes(lib):
    assert lib.origami_version() >= 100
    assert [lib.origami_item_bytes(k) for k in range(5)] == [4, 8, 8, 16, 16]
    assert lib.origami_item_bytes(99) == 0


def _call(kind, d, tmp, n, sort_n=0, flags=0):
    res = ctypes.c_void_p()
    return og.lib().origami_sort(kind, d, tmp, n, sort_n, 0, flags, ctypes.byref(res))


def test_rejects_bad_arguments(lib):
    a = np.zeros(64, np.uint32)
    b = np.zeros(64, np.uint32)
    assert _call(9, a.ctypes.data, b.ctypes.data, 64) == og.ERR_DTYPE
    assert _call(0, None, b.ctypes.data, 64) == og.ERR_INVALID
    # sort_n must be 0, >= n or a power of two
    assert _call(0, a.ctypes.data, b.ctypes.data, 64, sort_n=12) == og.ERR_INVALID
    # overlapping buffers
    assert _call(0, a.ctypes.data, a.ctypes.data + 16, 64) == og.ERR_INVALID
    # misaligned pointer
    assert _call(0, a.ctypes.data + 1, b.ctypes.data, 8) == og.ERR_ALIGN
    # a NULL result pointer
    assert og.lib().origami_sort(0, a.ctypes.data, b.ctypes.data, 64, 0, 0, 0, None) == og.ERR_INVALID
    assert b"sort_n" in og.lib().origami_last_error() or og.lib().origami_last_error()


def test_no_device_is_reported_not_crashed(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    a = np.arange(100, dtype=np.uint32)[::-1].copy()
    b = np.zeros(100, np.uint32)
    assert _call(0, a.ctypes.data, b.ctypes.data, 100) == og.ERR_NO_DEVICE


def test_python_surface_raises_without_fallback(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(og.OrigamiError) as e:
        og.sort_single_thread(np.arange(10, dtype=np.uint32), np.zeros(10, np.uint32))
    assert e.value.code == og.ERR_NO_DEVICE


def test_server_without_device(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert lib.origami_serve_create(ctypes.byref(h), 0, 0, 0, 0) == og.ERR_NO_DEVICE
    assert not h.value
    assert lib.origami_serve_create(None, 0, 0, 0, 0) == og.ERR_INVALID
    st = og.ServerStats()
    assert lib.origami_serve_get_stats(None, ctypes.byref(st)) == og.ERR_INVALID
    assert lib.origami_serve_destroy(None) == og.ERR_INVALID


def test_tuning_table_roundtrip(lib, tmp_path):
    # the table needs no device: set, read back, save, reset, load
    for k in range(3):
        assert og.tuning_get(k, 1 << 28) == (2, 0)  # default: binary passes, first tile shape
    # built-in entries: the 16-way k-way pass where the data is about L2-sized
    assert og.tuning_get(og.U32, 1 << 25) == (16, 0)
    assert og.tuning_get(og.KV64, 1 << 23) == og.tuning_get(og.KVU64, 1 << 23) == (16, 0)
    assert og.tuning_get(og.U64, 1 << 21) == og.tuning_get(og.I64, 1 << 21) == (2, 2)
    assert og.tuning_get(og.KV64, 1 << 28) == og.tuning_get(og.KVU64, 1 << 28) == (2, 1)
    built_in = og.tuning_get(og.U32, 1 << 20)
    built_in_kv = og.tuning_get(og.KV64, 1 << 27)
    og.tuning_set(og.U32, 1 << 20, 2, 1)
    og.tuning_set(og.KV64, 1 << 27, 8, 0)
    assert og.tuning_get(og.U32, (1 << 21) - 1) == (2, 1)  # same size class
    assert og.tuning_get(og.U32, 1 << 21) == (16, 0)  # the next class keeps its own entry
    path = tmp_path / "tune.txt"
    og.tuning_save(path)
    lines = sorted(path.read_text().split("\n"))
    assert "0 20 2 1" in lines and "3 27 8 0" in lines
    og.tuning_set(og.U32, 1 << 20, 2, 0)
    og.tuning_set(og.KV64, 1 << 27, 2, 0)
    og.tuning_load(path)
    assert og.tuning_get(og.U32, 1 << 20) == (2, 1) and og.tuning_get(og.KV64, 1 << 27) == (8, 0)
    with pytest.raises(og.OrigamiError):
        og.tuning_set(og.U32, 100, 3, 0)
    with pytest.raises(og.OrigamiError):
        og.tuning_set(og.U32, 100, 4, 1)  # the tile shape choice is for binary passes
    with pytest.raises(og.OrigamiError):
        og.tuning_set(og.U32, 100, 2, 4)
    og.tuning_set(og.U64, 1 << 24, 2, 2)  # one tile per CTA
    assert og.tuning_get(og.U64, 1 << 24) == (2, 2)
    og.tuning_set(og.U64, 1 << 24, 2, 3)  # half the items per thread
    assert og.tuning_get(og.U64, 1 << 24) == (2, 3)
    og.tuning_set(og.U64, 1 << 24, 2, 0)
    og.tuning_set(og.U32, 1 << 20, *built_in)
    og.tuning_set(og.KV64, 1 << 27, *built_in_kv)


def test_noalloc_rejects_bad_arguments_on_the_host(lib):
    # pure host checks, made before the library looks for a device: no buffer
    # below is ever read or written (they are small host arrays)
    a = np.zeros(64, np.uint32)
    b = np.zeros(64, np.uint32)
    res = ctypes.c_void_p()
    limit = lib.origami_noalloc_max_items(og.U32)
    assert limit >= (1 << 28)  # the 1 GiB uint32 workload fits
    assert lib.origami_noalloc_max_items(og.KV64) >= (1 << 26)
    assert lib.origami_noalloc_max_items(9) == 0
    rc = lib.origami_sort_noalloc_device(og.U32, a.ctypes.data, b.ctypes.data, limit + 1, 0, 0,
                                         ctypes.byref(res), None)
    assert rc == og.ERR_INVALID
    assert b"limit" in lib.origami_last_error()
    # a tmp buffer is required, RESULT_IN_TMP too, even for one item
    assert lib.origami_sort_noalloc_device(og.U32, a.ctypes.data, None, 64, 0, 0, ctypes.byref(res),
                                           None) == og.ERR_INVALID
    assert lib.origami_sort_noalloc_device(og.U32, a.ctypes.data, None, 1, 0, og.FLAG_RESULT_IN_TMP,
                                           ctypes.byref(res), None) == og.ERR_INVALID
    assert lib.origami_sort_noalloc_device(9, a.ctypes.data, b.ctypes.data, 64, 0, 0, ctypes.byref(res),
                                           None) == og.ERR_DTYPE


def test_wait_limit_is_host_state(lib):
    default = lib.origami_get_wait_limit()
    assert default == 1 << 20
    assert lib.origami_set_wait_limit(77) == og.OK
    assert lib.origami_get_wait_limit() == 77
    assert lib.origami_set_wait_limit(default) == og.OK


def test_segmented_tuning_table(lib):
    assert og.seg_tuning_get(og.U32, 1 << 24, 1 << 10) == 0  # default: the first merge shape
    og.seg_tuning_set(og.U32, 1 << 24, 1 << 10, 1)
    assert og.seg_tuning_get(og.U32, (1 << 24) + 5, 1 << 10) == 1  # same mean-length class
    assert og.seg_tuning_get(og.U32, 1 << 20, 1 << 10) == 0
    og.seg_tuning_set(og.U32, 1 << 24, 1 << 10, 0)
    with pytest.raises(og.OrigamiError):
        og.seg_tuning_set(og.U32, 100, 1, 2)
    with pytest.raises(og.OrigamiError):
        og.seg_tuning_set(9, 100, 1, 0)


def test_segmented_tuning_in_the_tuning_file(lib, tmp_path):
    # the segmented table travels in the same file as the plain sort's
    og.seg_tuning_set(og.KV64, 1 << 22, 1 << 6, 1)  # mean length 2^16
    path = tmp_path / "tune.txt"
    og.tuning_save(path)
    assert "seg 3 16 1" in path.read_text().split("\n")
    og.seg_tuning_set(og.KV64, 1 << 22, 1 << 6, 0)
    og.tuning_load(path)
    assert og.seg_tuning_get(og.KV64, 1 << 16, 1) == 1
    og.seg_tuning_set(og.KV64, 1 << 22, 1 << 6, 0)


def test_profile_switch(lib):
    # host-side bookkeeping only: nothing is launched, so the report is empty
    assert lib.origami_profile_enable(-1) == og.ERR_INVALID
    og.profile_enable(True, every=7)
    assert og.profile_detail() == {}
    og.profile_enable(False)
    assert og.profile_report() == {}
