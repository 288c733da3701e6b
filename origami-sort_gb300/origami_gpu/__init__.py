"""Python host-side mirror of the Origami sorter surface over the C ABI
(include/origami_gpu.h, lib/liborigami_gpu.so).

Names and argument meaning follow the reference's C++ entry points:

    sort_single_thread(d, tmp_buf, sort_n, min_k)   sorter.h:3851-3915
    sort_multi_thread(d, out, n_threads, n_cores, min_k, kway_buf)
                                                    sorter.h:4194-4287
    merge_series(src, dst, merge_start, sort_n)     merger.h:4220-4228

Each returns whichever of its two buffers holds the sorted output, like the
reference. Buffers are numpy arrays (host memory: staged through the device
arena) or CUDA torch tensors (device memory: sorted in place, no copies).
Errors raise OrigamiError carrying the library's status code; there is no CPU
fallback - if the library is missing the import fails loudly.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "liborigami_gpu.so")

U32, U64, I64, KV64, KVU64 = 0, 1, 2, 3, 4
KIND_NAMES = {"u32": U32, "u64": U64, "i64": I64, "kv64": KV64, "kvu64": KVU64}
KV_DTYPE = np.dtype([("key", "<i8"), ("value", "<i8")])
KVU_DTYPE = np.dtype([("key", "<u8"), ("value", "<u8")])
ITEM_BYTES = {U32: 4, U64: 8, I64: 8, KV64: 16, KVU64: 16}

OK = 0
ERR_INVALID, ERR_ALIGN, ERR_OOM, ERR_CUDA, ERR_TIMEOUT = -1, -2, -3, -4, -5
ERR_DTYPE, ERR_NO_DEVICE, ERR_BUSY, ERR_CANCELLED = -6, -7, -8, -9
FLAG_RESULT_IN_TMP, FLAG_SYNC = 0x1, 0x2


class OrigamiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"origami error {code}: {msg}")
        self.code = code


class ServerStats(ctypes.Structure):
    """origami_server_stats (include/origami_gpu.h)."""
    _fields_ = [(f, ctypes.c_uint64) for f in (
        "submitted", "completed", "failed", "cancelled", "keys", "batches", "pending",
        "bytes_reserved", "peak_bytes_reserved", "max_concurrent_batches")] + \
        [(f, ctypes.c_double) for f in ("p50_ms", "p99_ms", "max_ms", "keys_per_s")] + \
        [(f, ctypes.c_uint64) for f in ("pipe_batches", "arena_bytes", "arena_grows")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python origami-sort_gb300/build.py`")
        L = ctypes.CDLL(LIB_PATH)
        vp, u64, ui, i = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint, ctypes.c_int
        L.origami_version.restype = i
        L.origami_last_error.restype = ctypes.c_char_p
        L.origami_item_bytes.restype = ui
        L.origami_item_bytes.argtypes = [i]
        L.origami_sort.restype = i
        L.origami_sort.argtypes = [i, vp, vp, u64, u64, ui, i, ctypes.POINTER(vp)]
        L.origami_sort_device.restype = i
        L.origami_sort_device.argtypes = [i, vp, vp, u64, u64, ui, i, ctypes.POINTER(vp), vp]
        L.origami_merge_series_device.restype = i
        L.origami_merge_series_device.argtypes = [i, vp, vp, u64, u64, u64, ctypes.POINTER(vp), vp]
        L.origami_merge_tree_device.restype = i
        L.origami_merge_tree_device.argtypes = [i, ctypes.POINTER(vp), ctypes.POINTER(vp), vp, ui, vp]
        L.origami_partition_device.restype = i
        L.origami_partition_device.argtypes = [i, ctypes.POINTER(vp), ctypes.POINTER(vp), ui,
                                               ctypes.POINTER(u64), u64, ctypes.POINTER(u64), vp]
        L.origami_arena_reserve.restype = i
        L.origami_arena_reserve.argtypes = [u64]
        L.origami_arena_trim.restype = i
        L.origami_arena_bytes_in_use.restype = u64
        L.origami_profile_enable.restype = i
        L.origami_profile_enable.argtypes = [i]
        L.origami_profile_report.restype = i
        L.origami_profile_report.argtypes = [ctypes.c_char_p, u64]
        L.origami_launch_count.restype = u64
        L.origami_get_wait_limit.restype = ctypes.c_uint32
        L.origami_set_wait_limit.argtypes = [ctypes.c_uint32]
        L.origami_sort_segmented_device.restype = i
        L.origami_sort_segmented_device.argtypes = [i, vp, vp, vp, u64, u64, i, vp]
        L.origami_sort_segmented.restype = i
        L.origami_sort_segmented.argtypes = [i, vp, vp, u64, i]
        L.origami_noalloc_max_items.restype = u64
        L.origami_noalloc_max_items.argtypes = [i]
        L.origami_sort_noalloc_device.restype = i
        L.origami_sort_noalloc_device.argtypes = [i, vp, vp, u64, u64, i, ctypes.POINTER(vp), vp]
        L.origami_serve_create.restype = i
        L.origami_serve_create.argtypes = [ctypes.POINTER(vp), u64, i, u64, u64]
        L.origami_serve_submit.restype = i
        L.origami_serve_submit.argtypes = [vp, i, vp, vp, u64, ctypes.POINTER(u64)]
        L.origami_serve_wait.restype = i
        L.origami_serve_wait.argtypes = [vp, u64, ctypes.c_int64]
        L.origami_serve_cancel.restype = i
        L.origami_serve_cancel.argtypes = [vp, u64]
        L.origami_serve_get_stats.restype = i
        L.origami_serve_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
        L.origami_serve_reset_stats.restype = i
        L.origami_serve_reset_stats.argtypes = [vp]
        L.origami_serve_destroy.restype = i
        L.origami_serve_destroy.argtypes = [vp]
        L.origami_autotune.restype = i
        L.origami_autotune.argtypes = [i, u64, ctypes.c_char_p, u64]
        L.origami_autotune_segmented.restype = i
        L.origami_autotune_segmented.argtypes = [i, vp, vp, vp, u64, u64, ctypes.c_char_p, u64]
        L.origami_seg_tuning_get.restype = i
        L.origami_seg_tuning_get.argtypes = [i, u64, u64, ctypes.POINTER(i)]
        L.origami_seg_tuning_set.restype = i
        L.origami_seg_tuning_set.argtypes = [i, u64, u64, i]
        L.origami_tuning_get.restype = i
        L.origami_tuning_get.argtypes = [i, u64, ctypes.POINTER(i), ctypes.POINTER(i)]
        L.origami_tuning_set.restype = i
        L.origami_tuning_set.argtypes = [i, u64, i, i]
        L.origami_tuning_save.restype = i
        L.origami_tuning_save.argtypes = [ctypes.c_char_p]
        L.origami_tuning_load.restype = i
        L.origami_tuning_load.argtypes = [ctypes.c_char_p]
        L.origami_generate_device.restype = i
        L.origami_generate_device.argtypes = [i, vp, u64, i, u64, vp]
        L.origami_seg_plan_create.restype = i
        L.origami_seg_plan_create.argtypes = [i, vp, vp, vp, u64, u64, ctypes.POINTER(vp)]
        L.origami_seg_plan_launch.restype = i
        L.origami_seg_plan_launch.argtypes = [vp, vp]
        L.origami_seg_plan_status.restype = i
        L.origami_seg_plan_status.argtypes = [vp, vp]
        L.origami_seg_plan_kernels.restype = u64
        L.origami_seg_plan_kernels.argtypes = [vp]
        L.origami_seg_plan_destroy.restype = i
        L.origami_seg_plan_destroy.argtypes = [vp]
        _lib = L
    return _lib


def check(rc):
    if rc != OK:
        raise OrigamiError(rc, lib().origami_last_error().decode(errors="replace"))
    return rc


def kind_of_dtype(dt):
    dt = np.dtype(dt)
    if dt == np.uint32:
        return U32
    if dt == np.uint64:
        return U64
    if dt == np.int64:
        return I64
    if dt == KV_DTYPE:
        return KV64
    if dt == KVU_DTYPE:
        return KVU64
    raise OrigamiError(ERR_DTYPE, f"unsupported item dtype {dt}")


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _ptr_len(x, kind):
    if x is None:
        return None, 0
    if _is_torch(x):
        return x.data_ptr(), x.numel() * x.element_size() // ITEM_BYTES[kind]
    return x.ctypes.data, len(x)


def _kind(d, kind):
    if kind is not None:
        return KIND_NAMES[kind] if isinstance(kind, str) else int(kind)
    if _is_torch(d):
        raise OrigamiError(ERR_DTYPE, "pass kind= for torch tensors (u32/u64/i64/kv64/kvu64)")
    return kind_of_dtype(d.dtype)


def sort(d, tmp=None, sort_n=0, min_k=0, kind=None, result_in_tmp=False, stream=None):
    """Sort d (chunked by sort_n). Returns d or tmp, whichever holds the output.

    Host (numpy) buffers block until the result is back in host memory. CUDA
    tensors are sorted on `stream` (default: torch's current stream) and the
    call returns once the work is enqueued."""
    k = _kind(d, kind)
    dp, n = _ptr_len(d, k)
    tp, _ = _ptr_len(tmp, k)
    res = ctypes.c_void_p()
    flags = FLAG_RESULT_IN_TMP if result_in_tmp else 0
    if _is_torch(d):
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(d.device).cuda_stream
        check(lib().origami_sort_device(k, dp, tp, n, sort_n, min_k, flags, ctypes.byref(res),
                                        ctypes.c_void_p(s)))
    else:
        check(lib().origami_sort(k, dp, tp, n, sort_n, min_k, flags, ctypes.byref(res)))
    if n == 0:
        return d
    return tmp if (tmp is not None and res.value == tp) else d


def sort_single_thread(d, tmp_buf, sort_n=0, min_k=2, interim_buf=None, kind=None):
    """origami_sorter::sort_single_thread (sorter.h:3851-3915) on the GPU."""
    del interim_buf  # the GPU merge tree keeps its buffers on chip
    return sort(d, tmp_buf, sort_n, min_k, kind=kind)


def sort_multi_thread(d, out, n_threads=1, n_cores=1, min_k=2, kway_buf=None, kind=None):
    """origami_sorter::sort_multi_thread (sorter.h:4194-4287): the whole GPU is
    used; the thread arguments are accepted for compatibility and ignored."""
    del n_threads, n_cores, kway_buf
    return sort(d, out, 0, min_k, kind=kind)


def merge_series(src, dst, merge_start, sort_n, kind=None, stream=None):
    """origami_merger::merge_series (merger.h:4220-4228) on CUDA tensors."""
    import torch
    k = _kind(src, kind)
    sp, n = _ptr_len(src, k)
    dp, _ = _ptr_len(dst, k)
    res = ctypes.c_void_p()
    s = stream if stream is not None else torch.cuda.current_stream(src.device).cuda_stream
    check(lib().origami_merge_series_device(k, sp, dp, n, merge_start, sort_n, ctypes.byref(res),
                                            ctypes.c_void_p(s)))
    return dst if res.value == dp else src


def sort_segmented(d, offsets, tmp=None, kind=None, stream=None, sync=True):
    """Sort every segment [offsets[s], offsets[s+1]) of d independently, in place.

    numpy d/offsets: host call (returns when d is sorted). CUDA tensors: d, tmp
    (same size as d, allocated if None) and offsets (uint64/int64 tensor) on the
    device; runs on `stream` and waits unless sync=False."""
    k = _kind(d, kind)
    if _is_torch(d):
        import torch
        if tmp is None:
            tmp = torch.empty_like(d)
        dp, n = _ptr_len(d, k)
        nseg = offsets.numel() - 1
        s = stream if stream is not None else torch.cuda.current_stream(d.device).cuda_stream
        check(lib().origami_sort_segmented_device(k, dp, tmp.data_ptr(), offsets.data_ptr(), nseg, n,
                                                  FLAG_SYNC if sync else 0, ctypes.c_void_p(s)))
        return d
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    check(lib().origami_sort_segmented(k, d.ctypes.data, off.ctypes.data, len(off) - 1, 0))
    return d


class SegmentedPlan:
    """CUDA-graph plan of a segmented sort over fixed device tensors
    (origami_seg_plan_*): launch() replays it on a stream."""

    def __init__(self, d, offsets, tmp, kind):
        self.kind = _kind(d, kind)
        dp, n = _ptr_len(d, self.kind)
        h = ctypes.c_void_p()
        check(lib().origami_seg_plan_create(self.kind, dp, tmp.data_ptr(), offsets.data_ptr(),
                                            offsets.numel() - 1, n, ctypes.byref(h)))
        self._h = h
        self._keep = (d, offsets, tmp)

    @property
    def kernels(self):
        return int(lib().origami_seg_plan_kernels(self._h))

    def launch(self, stream):
        check(lib().origami_seg_plan_launch(self._h, ctypes.c_void_p(stream)))

    def status(self, stream):
        check(lib().origami_seg_plan_status(self._h, ctypes.c_void_p(stream)))

    def close(self):
        if self._h is not None:
            check(lib().origami_seg_plan_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop (origami_server_* in include/origami_gpu.h).

    submit(x, out=None) queues a sort of x (numpy array, possibly pinned, or a
    CUDA tensor with kind=) into out (default: in place) and returns a request
    id; wait(id) blocks until it is sorted. The caller keeps both buffers alive,
    and out untouched, until wait() returns."""

    def __init__(self, hbm_budget_bytes=0, max_inflight=0, max_batch_items=0, max_queue=0):
        h = ctypes.c_void_p()
        check(lib().origami_serve_create(ctypes.byref(h), hbm_budget_bytes, max_inflight,
                                          max_batch_items, max_queue))
        self._h = h

    def submit(self, x, out=None, kind=None):
        """Queue a sort of x into `out` (None: in place); returns the request id."""
        k = _kind(x, kind)
        p, n = _ptr_len(x, k)
        q = p if out is None else _ptr_len(out, k)[0]
        rid = ctypes.c_uint64()
        check(lib().origami_serve_submit(self._h, k, p, q, n, ctypes.byref(rid)))
        return rid.value

    def wait(self, rid, timeout_ms=-1):
        check(lib().origami_serve_wait(self._h, rid, timeout_ms))

    def cancel(self, rid):
        check(lib().origami_serve_cancel(self._h, rid))

    def stats(self):
        st = ServerStats()
        check(lib().origami_serve_get_stats(self._h, ctypes.byref(st)))
        return st.as_dict()

    def reset_stats(self):
        check(lib().origami_serve_reset_stats(self._h))

    def close(self):
        if self._h is not None and self._h.value:
            check(lib().origami_serve_destroy(self._h))
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(kind, n):
    """Time every pass shape on n device items of `kind`; the fastest becomes the
    default for n's size class. Returns {"fan", "variant", "report"}."""
    k = KIND_NAMES[kind] if isinstance(kind, str) else int(kind)
    buf = ctypes.create_string_buffer(4096)
    check(lib().origami_autotune(k, n, buf, len(buf)))
    fan, var = tuning_get(k, n)
    return {"fan": fan, "variant": var, "report": buf.value.decode()}


def autotune_segmented(d, tmp, offsets, kind):
    """Time both merge shapes of the segmented sort on these device segments
    (d is left holding its input); the faster becomes the default for their
    mean segment length. Returns {"shape", "report"}."""
    k = KIND_NAMES[kind] if isinstance(kind, str) else int(kind)
    p, n = _ptr_len(d, k)
    nseg = offsets.numel() - 1
    buf = ctypes.create_string_buffer(1024)
    check(lib().origami_autotune_segmented(k, p, tmp.data_ptr(), offsets.data_ptr(), nseg, n, buf, len(buf)))
    return {"shape": seg_tuning_get(k, n, nseg), "report": buf.value.decode()}


def seg_tuning_get(kind, n, nseg):
    k = KIND_NAMES[kind] if isinstance(kind, str) else int(kind)
    v = ctypes.c_int()
    check(lib().origami_seg_tuning_get(k, n, nseg, ctypes.byref(v)))
    return v.value


def seg_tuning_set(kind, n, nseg, shape):
    """Merge shape (0 or 1) of segmented sorts whose mean segment length falls
    in the size class of n / nseg."""
    k = KIND_NAMES[kind] if isinstance(kind, str) else int(kind)
    check(lib().origami_seg_tuning_set(k, n, nseg, shape))


def tuning_get(kind, n):
    k = KIND_NAMES[kind] if isinstance(kind, str) else int(kind)
    f, v = ctypes.c_int(), ctypes.c_int()
    check(lib().origami_tuning_get(k, n, ctypes.byref(f), ctypes.byref(v)))
    return f.value, v.value


def tuning_set(kind, n, fan, variant=0):
    """Pass shape for n's size class: fan 2 (binary passes) with merge shape
    variant 0 or 1 (the persistent merge's two tile shapes) or 2 (one tile per
    CTA, for sorts running on several streams at once); fan 4, 8 or 16 (k-way
    passes, variant 0)."""
    k = KIND_NAMES[kind] if isinstance(kind, str) else int(kind)
    check(lib().origami_tuning_set(k, n, fan, variant))


def tuning_save(path):
    check(lib().origami_tuning_save(os.fsencode(path)))


def tuning_load(path):
    check(lib().origami_tuning_load(os.fsencode(path)))


WRITER_DISTS = {"uniform": 1, "same": 2, "sorted": 3, "reverse": 4, "almost_sorted": 5,
                "pareto": 6, "pareto_b2b": 7, "pareto_shuffled": 8, "fibonacci": 9}


def generate(d, dist, kind, seed=0, stream=None):
    """Fill the CUDA tensor d with a Writer distribution (writer.h:27-35) on the
    device: dist is 1..9 or a name from WRITER_DISTS."""
    import torch
    k = _kind(d, kind)
    p, n = _ptr_len(d, k)
    dv = WRITER_DISTS[dist] if isinstance(dist, str) else int(dist)
    s = stream if stream is not None else torch.cuda.current_stream(d.device).cuda_stream
    check(lib().origami_generate_device(k, p, n, dv, seed, ctypes.c_void_p(s)))
    return d


def _stream_bounds(streams, k):
    lo = [_ptr_len(t, k)[0] or 0 for t in streams]
    hi = [p + _ptr_len(t, k)[1] * ITEM_BYTES[k] for p, t in zip(lo, streams)]
    arr = ctypes.c_void_p * len(streams)
    return arr(*lo), arr(*hi)


def merge_tree(streams, out, kind, stream=None):
    """MergeTree::merge(X, endX, C, n, ...) (merge_tree.h:2792): merge the sorted
    CUDA tensors `streams` into `out` (ties: lower stream first)."""
    import torch
    k = _kind(out, kind)
    X, E = _stream_bounds(streams, k)
    s = stream if stream is not None else torch.cuda.current_stream(out.device).cuda_stream
    check(lib().origami_merge_tree_device(k, X, E, out.data_ptr(), len(streams), ctypes.c_void_p(s)))
    return out


def partition(streams, ranks, kind, stream=None):
    """Splits of the sorted CUDA tensors `streams` at each output rank:
    an (n_ranks, K) array; ties are ordered by stream (Partition.h:118-166)."""
    import torch
    k = _kind(streams[0], kind)
    L, R = _stream_bounds(streams, k)
    rk = np.ascontiguousarray(ranks, dtype=np.uint64)
    out = np.zeros((len(rk), len(streams)), np.uint64)
    s = stream if stream is not None else torch.cuda.current_stream(streams[0].device).cuda_stream
    check(lib().origami_partition_device(k, L, R, len(streams), rk.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                         len(rk), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                         ctypes.c_void_p(s)))
    return out


def partition_ptrs(streams, guesses, kind):
    """partition_templated::Partition_Ptrs(L, R, S, K) (Partition.h:118): moves
    the per-stream offsets `guesses` to the split of the same total rank."""
    return [int(x) for x in partition(streams, [int(sum(guesses))], kind)[0]]


def profile_enable(on=True, every=1):
    """Time kernel launches with CUDA events: every launch, or every `every`-th
    launch of each kernel (on=False switches timing off)."""
    check(lib().origami_profile_enable(max(1, int(every)) if on else 0))


def profile_detail():
    """{kernel: (launches, timed, timed_ms)} for the launches since profile_enable()."""
    buf = ctypes.create_string_buffer(1 << 16)
    rc = lib().origami_profile_report(buf, len(buf))
    if rc < 0:
        check(rc)
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms, timed = line.rsplit(",", 3)
        out[name] = (int(cnt), int(timed), float(ms))
    return out


def profile_report():
    """{kernel: (launches, total_ms)} for the launches since profile_enable();
    with sampled timing, total_ms is the timed launches' mean times `launches`."""
    return {k: (c, ms * c / t if t else 0.0) for k, (c, t, ms) in profile_detail().items()}


def launch_count():
    return int(lib().origami_launch_count())


def wait_limit():
    """Polls a merge kernel makes on a bulk copy before it gives up (default 2^20)."""
    return int(lib().origami_get_wait_limit())


def set_wait_limit(polls):
    """Sets the device-side wait bound for later launches (0: every first wait
    expires, which is how the tests drive the expiry path)."""
    check(lib().origami_set_wait_limit(int(polls)))


def empty_host(kind, n, pinned=False):
    """Host buffer for n items of `kind` (numpy; page-locked when pinned=True)."""
    k = KIND_NAMES[kind] if isinstance(kind, str) else int(kind)
    dt = {U32: np.dtype(np.uint32), U64: np.dtype(np.uint64), I64: np.dtype(np.int64),
          KV64: KV_DTYPE, KVU64: KVU_DTYPE}[k]
    if pinned:
        import torch
        t = torch.empty(n * dt.itemsize, dtype=torch.uint8, pin_memory=True)
        return t.numpy().view(dt)  # the array's base chain keeps the pinned tensor alive
    return np.empty(n, dt)
