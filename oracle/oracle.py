"""ctypes binding for the Origami oracle (oracle/origami_oracle.c) and, where it
was built, for the unmodified reference (oracle/_ref/libref_<variant>.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py, always as the checker or the CPU
baseline, never as the thing measured or shipped.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liborigami_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

U32, U64, I64, KV, KVU = 0, 1, 2, 3, 4
KIND_NAMES = {"u32": U32, "u64": U64, "i64": I64, "kv": KV, "kv64": KV, "kvu": KVU, "kvu64": KVU}
KV_DTYPE = np.dtype([("key", "<i8"), ("value", "<i8")])
KVU_DTYPE = np.dtype([("key", "<u8"), ("value", "<u8")])
DTYPES = {U32: np.dtype(np.uint32), U64: np.dtype(np.uint64), I64: np.dtype(np.int64),
          KV: KV_DTYPE, KVU: KVU_DTYPE}

# writer.h distribution ids
MT, SAME, SORTED_SEQ, REV_SORTED_SEQ, ALMOST_SORTED = 1, 2, 3, 4, 5
PARETO_NONUNIFORM, PARETO_B2B, PARETO_SHUFF, FIB_SEQ = 6, 7, 8, 9

_lib = None


def build(quiet=True):
    """Compile the oracle port (plain C) for this machine."""
    out = subprocess.run(["make", "-C", HERE, "port"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(PORT_SO):
            build()
        L = ctypes.CDLL(PORT_SO)
        vp, u64, ui, i = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint, ctypes.c_int
        L.orc_item_bytes.restype = ui
        L.orc_item_bytes.argtypes = [i]
        L.orc_p1_n.restype = u64
        L.orc_p1_n.argtypes = [i]
        L.orc_p2_n.restype = u64
        L.orc_p2_n.argtypes = [i]
        L.orc_generate.argtypes = [i, vp, u64, i]
        L.orc_sort_single_thread.restype = vp
        L.orc_sort_single_thread.argtypes = [i, vp, vp, u64, u64, ui]
        L.orc_sort_single_thread_p.restype = vp
        L.orc_sort_single_thread_p.argtypes = [i, vp, vp, u64, u64, ui, u64, u64]
        L.orc_sort_multi_thread.restype = vp
        L.orc_sort_multi_thread.argtypes = [i, vp, vp, u64, ui, ui]
        L.orc_merge_series.restype = vp
        L.orc_merge_series.argtypes = [i, vp, vp, u64, u64, u64]
        L.orc_kway_merge.argtypes = [i, ctypes.POINTER(vp), ctypes.POINTER(vp), vp, ui]
        L.orc_partition_ptrs.argtypes = [i, ctypes.POINTER(vp), ctypes.POINTER(vp),
                                         ctypes.POINTER(vp), u64]
        L.orc_is_sorted.restype = i
        L.orc_is_sorted.argtypes = [i, vp, u64]
        L.orc_chunks_sorted.restype = i
        L.orc_chunks_sorted.argtypes = [i, vp, u64, u64]
        _lib = L
    return _lib


def kind_of(kind):
    return KIND_NAMES[kind] if isinstance(kind, str) else int(kind)


def empty(kind, n, align=4096):
    """Page-aligned numpy array of n items (the reference's SIMD loads need alignment)."""
    dt = DTYPES[kind_of(kind)]
    raw = np.zeros(n * dt.itemsize + align, np.uint8)
    off = (-raw.ctypes.data) % align
    return raw[off:off + n * dt.itemsize].view(dt)


def generate(kind, n, dist=MT):
    """datagen::Writer<Item>::generate restated (writer.h:222-242)."""
    k = kind_of(kind)
    a = empty(k, n)
    lib().orc_generate(k, a.ctypes.data, n, dist)
    return a


def sort_single_thread(kind, a, sort_n=0, min_k=2, p1_n=None, p2_n=None):
    """Returns (output array, 'd' or 'tmp'); `a` is not modified."""
    k = kind_of(kind)
    n = len(a)
    d = empty(k, n)
    d[:] = a
    t = empty(k, n)
    L = lib()
    if p1_n is None:
        r = L.orc_sort_single_thread(k, d.ctypes.data, t.ctypes.data, n, sort_n, min_k)
    else:
        r = L.orc_sort_single_thread_p(k, d.ctypes.data, t.ctypes.data, n, sort_n, min_k, p1_n,
                                       p2_n)
    if n == 0 or r == d.ctypes.data:
        return d, "d"
    return t, "tmp"


def sort_multi_thread(kind, a, n_threads=8, min_k=2):
    k = kind_of(kind)
    n = len(a)
    d = empty(k, n)
    d[:] = a
    o = empty(k, n)
    r = lib().orc_sort_multi_thread(k, d.ctypes.data, o.ctypes.data, n, n_threads, min_k)
    return d if (n == 0 or r == d.ctypes.data) else o


def sort_multi_thread_inplace(kind, d, o, n_threads=8, min_k=2):
    """Timed CPU-baseline form: sorts the caller's buffers, returns the result one."""
    k = kind_of(kind)
    r = lib().orc_sort_multi_thread(k, d.ctypes.data, o.ctypes.data, len(d), n_threads, min_k)
    return d if r == d.ctypes.data else o


def kway_merge(kind, streams):
    k = kind_of(kind)
    total = sum(len(s) for s in streams)
    out = empty(k, total)
    way = len(streams)
    dt = DTYPES[k]
    X = (ctypes.c_void_p * way)(*[s.ctypes.data for s in streams])
    E = (ctypes.c_void_p * way)(*[s.ctypes.data + len(s) * dt.itemsize for s in streams])
    lib().orc_kway_merge(k, X, E, out.ctypes.data, way)
    return out


def partition_ptrs(kind, streams, guesses):
    """Partition_Ptrs over whole streams; guesses/result are per-stream offsets."""
    k = kind_of(kind)
    K = len(streams)
    dt = DTYPES[k]
    L = (ctypes.c_void_p * K)(*[s.ctypes.data for s in streams])
    R = (ctypes.c_void_p * K)(*[s.ctypes.data + len(s) * dt.itemsize for s in streams])
    S = (ctypes.c_void_p * K)(*[s.ctypes.data + g * dt.itemsize for s, g in zip(streams, guesses)])
    lib().orc_partition_ptrs(k, L, R, S, K)
    return [(S[i] - streams[i].ctypes.data) // dt.itemsize for i in range(K)]


def is_sorted(kind, a):
    return bool(lib().orc_is_sorted(kind_of(kind), a.ctypes.data, len(a)))


def chunks_sorted(kind, a, sort_n):
    return bool(lib().orc_chunks_sorted(kind_of(kind), a.ctypes.data, len(a), sort_n))


def keys_of(a):
    return a["key"] if a.dtype.names else a


def pairs_sorted(a):
    """(key, value) pairs in (key, value) order: the multiset of a KV array."""
    order = np.lexsort((a["value"], a["key"]))
    return a[order]


# --------------------------------------------------------------- reference --
def ref_variants():
    if not os.path.isdir(REF_DIR):
        return []
    return sorted(f[len("libref_"):-3] for f in os.listdir(REF_DIR)
                  if f.startswith("libref_") and f.endswith(".so"))


def ref_lib(variant):
    L = ctypes.CDLL(os.path.join(REF_DIR, f"libref_{variant}.so"))
    vp, ull, ui = ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_uint
    L.ref_sort_single_thread.restype = vp
    L.ref_sort_single_thread.argtypes = [vp, vp, ull, ull, ui, vp]
    L.ref_sort_multi_thread.restype = vp
    L.ref_sort_multi_thread.argtypes = [vp, vp, ull, ui, ui, ui, vp]
    L.ref_generate.argtypes = [vp, ull, ctypes.c_int]
    L.ref_p1_n.restype = ull
    L.ref_p2_n.restype = ull
    L.ref_item_bytes.restype = ui
    L.ref_partition_ptrs.argtypes = [ctypes.POINTER(vp)] * 3 + [ull]
    return L
