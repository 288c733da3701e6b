"""Generate tests/golden/reference_digests.json from the UNMODIFIED reference.

Run in a checkout that has the reference sources mounted (the reference cannot
travel to the GPU machines), after `make -C oracle ref`:

    python tests/golden/make_golden.py

For every reference build variant (scalar / AVX2 / AVX-512 x u32 / i64 / 64+64)
it generates inputs with the reference's own datagen::Writer (writer.h:222-242),
sorts them with origami_sorter::sort_single_thread (sorter.h:3851-3915) and
records SHA-256 digests (first 16 hex digits) of the input, of the output keys,
of the output (key, value) pairs sorted by (key, value), the buffer the result
came back in, and whether the reference's output matches std::sort of the same
chunks (it does not always: see ref_correct).
"""
import argparse
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_DIR = os.path.join(REPO, "oracle", "_ref")

# variant -> (oracle kind, reg name, key name)
VARIANTS = {
    "s_u32": 0, "a2_u32": 0, "a5_u32": 0,
    "s_i64": 2, "a2_i64": 2, "a5_i64": 2,
    "s_kv": 3, "a2_kv": 3,
}
DISTS = [1, 2, 3, 4, 5, 6, 7, 9]  # writer.h ids; 8 (PARETO_SHUFF) is seeded from random_device


def aligned(nbytes, a=4096):
    raw = np.zeros(nbytes + a, np.uint8)
    off = (-raw.ctypes.data) % a
    return raw[off:off + nbytes]


def h(b):
    return hashlib.sha256(np.ascontiguousarray(b).tobytes()).hexdigest()[:16]


def keys_of(buf, item_bytes):
    if item_bytes == 4:
        return buf.view(np.uint32)
    if item_bytes == 8:
        return buf.view(np.int64)
    return buf.view(np.int64)[0::2]


def pairs_sorted(buf):
    v = buf.view(np.int64).reshape(-1, 2)
    order = np.lexsort((v[:, 1], v[:, 0]))
    return v[order]


def load(variant):
    lib = ctypes.CDLL(os.path.join(REF_DIR, f"libref_{variant}.so"))
    lib.ref_sort_single_thread.restype = ctypes.c_void_p
    lib.ref_sort_single_thread.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_ulonglong] * 2 + [
        ctypes.c_uint, ctypes.c_void_p]
    lib.ref_generate.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_int]
    lib.ref_p1_n.restype = ctypes.c_ulonglong
    lib.ref_p2_n.restype = ctypes.c_ulonglong
    return lib


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "reference_digests.json"))
    args = ap.parse_args()
    cases = []
    variants = {}
    interim = aligned(256 << 20)
    for variant, kind in VARIANTS.items():
        lib = load(variant)
        ib = lib.ref_item_bytes()
        p1, p2 = int(lib.ref_p1_n()), int(lib.ref_p2_n())
        sizes = [4 * p2] + ([1 << 20] if ib == 4 else [])
        for n in sizes:
            for dist in DISTS:
                src = aligned(n * ib)
                lib.ref_generate(src.ctypes.data, n, dist)
                std_keys = np.sort(keys_of(src, ib))
                configs = [(n, 2), (p2, 2), (2 * p2, 2), (n, 4)]
                for sort_n, min_k in configs:
                    if min_k > 2 and (sort_n // p2) < 4:
                        continue  # the reference loops forever below 2 k-way levels
                    interim[:] = 0  # the merge tree expects a zeroed interim buffer
                    d = aligned(n * ib)
                    d[:] = src
                    t = aligned(n * ib)
                    r = lib.ref_sort_single_thread(d.ctypes.data, t.ctypes.data, n, sort_n, min_k,
                                                   interim.ctypes.data if min_k > 2 else None)
                    out = d if r == d.ctypes.data else t
                    k = keys_of(out, ib)
                    if sort_n >= n:
                        expect = std_keys
                    else:
                        expect = np.concatenate([np.sort(keys_of(src, ib)[c:c + sort_n])
                                                 for c in range(0, n, sort_n)])
                    case = [variant, n, dist, sort_n, min_k, h(src), h(k),
                            h(pairs_sorted(out)) if ib == 16 else None,
                            "d" if r == d.ctypes.data else "tmp",
                            bool(np.array_equal(k, expect))]
                    cases.append(case)
                    print(*case, file=sys.stderr)
        variants[variant] = {"kind": kind, "item_bytes": ib, "p1_n": p1, "p2_n": p2}
    doc = {
        "generator": "tests/golden/make_golden.py",
        "hash": "sha256, first 16 hex digits, little-endian item bytes",
        "columns": ["variant", "n", "dist", "sort_n", "min_k", "input", "keys", "pairs",
                    "result", "ref_correct"],
        "variants": variants,
        "cases": cases,
    }
    with open(args.out, "w") as f:
        f.write("{\n")
        for i, key in enumerate(["generator", "hash", "columns", "variants"]):
            f.write(f"{json.dumps(key)}: {json.dumps(doc[key])},\n")
        f.write('"cases": [\n')
        f.write(",\n".join(json.dumps(c, separators=(",", ":")) for c in cases))
        f.write("\n]}\n")
    print(f"wrote {len(cases)} cases to {args.out}", file=sys.stderr)


if __name__ == "__main__":
    main()
