"""Times the unmodified reference's own multi-threaded sort on this host.

TEST INFRASTRUCTURE ONLY: it loads oracle/_ref/libref_<variant>.so, the
reference compiled in place by oracle/Makefile (x86 hosts only: the reference
is written with x86 SIMD intrinsics), and nothing on the GPU path imports it.

    python oracle/time_reference.py [--pow 28] [--threads 8] [--min-k 16]
                                    [--variants a2_u32,a5_u32] [--reps 3]
                                    [--out oracle/reference_x86.json]

For each variant it sorts 2^pow uint32 keys drawn like bench_sort does
(datagen::Writer<ui>::generate(MT), writer.h:50-55) with
origami_sorter::sort_multi_thread (sorter.h:4194-4287) at the given thread
count and min_k, the same call bench_sort.cpp:27-144 times, and checks every
output against numpy's sort. (threads, min_k) must be a pair the reference
sorts correctly: 8/16 and 4/4 are; 8/8 and 4/8 are not.
Prints one JSON line per variant: best and median M keys/s over the reps, the
CPU model, core count, clock and compiler. --out also writes them to a JSON
file (the committed oracle/reference_x86.json, which bench.py quotes beside its
own host-core baseline).
"""
import argparse
import ctypes
import json
import os
import platform
import subprocess
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import oracle as orc  # noqa: E402


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def cpu_mhz():
    try:
        v = [float(line.split(":", 1)[1]) for line in open("/proc/cpuinfo") if line.startswith("cpu MHz")]
        return round(sum(v) / len(v)) if v else None
    except OSError:
        return None


def compiler():
    try:
        return subprocess.run(["g++", "--version"], capture_output=True, text=True).stdout.splitlines()[0]
    except (OSError, IndexError):
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pow", type=int, default=28)
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--min-k", type=int, default=16)
    ap.add_argument("--variants", default="a2_u32,a5_u32")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    rows = []
    n = 1 << args.pow
    have = orc.ref_variants()
    for var in args.variants.split(","):
        if var not in have:
            rows.append({"variant": var, "unavailable": "not built on this host (x86 intrinsics)"})
            print(json.dumps(rows[-1]))
            continue
        ref = orc.ref_lib(var)
        src = orc.empty(orc.U32, n)
        ref.ref_generate(src.ctypes.data, n, orc.MT)
        expect = np.sort(src)
        d = orc.empty(orc.U32, n)
        o = orc.empty(orc.U32, n)
        # the reference's k-way scratch: n_threads blocks of 8 MiB (bench_sort.cpp:55-58)
        kbuf = orc.empty(orc.U32, args.threads * (8 << 20) // 4)
        rates, ok = [], True
        for _ in range(args.reps):
            d[:] = src
            kbuf[:] = 0
            t0 = time.perf_counter()
            r = ref.ref_sort_multi_thread(d.ctypes.data, o.ctypes.data, n, args.threads, args.threads,
                                          args.min_k, kbuf.ctypes.data)
            dt = time.perf_counter() - t0
            res = d if r == d.ctypes.data else o
            ok = ok and bool(np.array_equal(res, expect))
            rates.append(n / dt / 1e6)
        rows.append({
            "variant": var, "n": n, "threads": args.threads, "min_k": args.min_k,
            "mkeys_s_best": round(max(rates), 1), "mkeys_s_median": round(float(np.median(rates)), 1),
            "reps": args.reps, "equal_to_numpy_sort": ok, "cpu": cpu_model(), "cores": os.cpu_count(),
            "mhz": cpu_mhz(), "compiler": compiler(), "flags": "-std=c++17 -O3 -march=native -fopenmp -fpermissive",
            "call": "origami_sorter::sort_multi_thread (sorter.h:4194-4287)",
        })
        print(json.dumps(rows[-1]))
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"workload": f"{n} uint32 keys, datagen::Writer MT (writer.h:50-55)", "runs": rows}, f, indent=1)
            f.write("\n")


if __name__ == "__main__":
    main()
