#!/usr/bin/env python
"""Origami GB300 mergesort benchmark.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl origami|reference]

Workload: full ascending sort of 268,435,456 uint32 keys (1 GiB) drawn
uniformly from [0, 2^32), one array per GPU (replicas: no data exchange
between GPUs, so "scaling" is weak). A step is one sort of that array.

  value   Gkeys/s with the keys already resident in HBM; each step's input is
          restored from a pristine device copy outside the step's CUDA events
          (the 1 GiB input is larger than L2, so no extra flush is needed).
  e2e     the same metric through the C ABI with pinned HOST buffers: the
          host->device copy, the sort and the device->host copy are all timed.
  roofline  the dominant kernel's algorithmic bytes per launch (read + write of
          every item once) over its average CUDA-event launch time, against the
          measured HBM copy bandwidth in MEASURED_PEAKS.json.
  cpu_baseline  the oracle (C restatement of the reference pipeline, all host
          threads) on the same workload, timed on this machine's host cores.

`--impl reference` times the reference's CPU sort instead (the compiled
reference when it loads on this host, otherwise the oracle port) and prints the
same JSON line with "impl": "reference".
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "origami-sort_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

N_KEYS = 1 << 28
METRIC = "Gkeys/s sorting 1 GB uint32 on 1 GB300 (% HBM roofline); batched p50/p99 latency"
PROFILE_EVERY = 7  # time every 7th launch of each kernel inside the timed steps
WORKLOAD = "full sort of 268,435,456 uint32 keys (1 GiB), uniform over [0, 2^32)"


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the GPU works."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, interval_ms=50):
        self.path = tempfile.mktemp(suffix=".csv")
        self.gpu = gpu_index
        self.proc = None
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", f"-lms={interval_ms}"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"],
                    "samples": 0}
        time.sleep(0.12)
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(n_full, seconds=12.0):
    """Oracle (C restatement of the reference pipeline) with every host thread, on
    a bounded sample of the workload: the largest power-of-two prefix that sorts
    in a few seconds, repeated until ~`seconds` of CPU work."""
    import numpy as np

    import oracle as orc
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(2026)
    n = min(n_full, 1 << 26)
    src = rng.integers(0, 1 << 32, n, dtype=np.uint32)
    d = orc.empty(orc.U32, n)
    o = orc.empty(orc.U32, n)
    times = []
    t_end = time.perf_counter() + seconds
    while time.perf_counter() < t_end or len(times) < 2:
        d[:] = src
        t0 = time.perf_counter()
        r = orc.sort_multi_thread_inplace(orc.U32, d, o, threads, 16)
        times.append(time.perf_counter() - t0)
        if len(times) >= 20:
            break
    assert orc.is_sorted(orc.U32, r)
    best = min(times)
    return {"value": n / best / 1e9, "unit": "Gkeys/s", "cores": threads, "kind": "port",
            "sample": f"{n} uniform uint32 keys (1/{n_full // n} of the workload), "
                      f"oracle sort_multi_thread restatement, min_k=16, best of {len(times)} runs",
            "reference_x86": reference_x86()}


def reference_x86():
    """The reference's own AVX2 / AVX-512 multi-threaded builds timed on an x86
    host (they do not build on this Arm host): oracle/reference_x86.json, written
    by oracle/time_reference.py. Quoted, not measured in this run."""
    p = os.path.join(REPO, "oracle", "reference_x86.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    out = {}
    for r in d.get("runs", []):
        if "mkeys_s_best" in r:
            out[r["variant"]] = {"gkeys_s": r["mkeys_s_best"] / 1e3, "threads": r["threads"],
                                 "min_k": r["min_k"], "n": r["n"], "cpu": r["cpu"], "cores": r["cores"],
                                 "mhz": r["mhz"], "correct": r["equal_to_numpy_sort"]}
    return out or None


def run_reference(args):
    """CPU reference arm: the reference's own multithreaded sort when it loads on
    this host (x86 builds from oracle/_ref), else the oracle port of it."""
    import numpy as np

    import oracle as orc
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    kind_label = "port"
    ref = None
    # the fastest build of the reference this host runs: AVX-512 where the CPU
    # has it, else AVX2 (x86 only; elsewhere the oracle port)
    try:
        avx512 = "avx512f" in open("/proc/cpuinfo").read()
    except OSError:
        avx512 = False
    build = "oracle port (scalar C restatement), every host thread"
    for var in (["a5_u32"] if avx512 else []) + ["a2_u32"]:
        if var in orc.ref_variants():
            try:
                ref = orc.ref_lib(var)
                kind_label = "reference"
                build = {"a5_u32": "AVX-512", "a2_u32": "AVX2"}[var] + " build of the reference, sort_multi_thread"
                break
            except OSError:
                ref = None
    orc.build()
    n = N_KEYS
    rng = np.random.default_rng(7)
    src = rng.integers(0, 1 << 32, n, dtype=np.uint32)
    d = orc.empty(orc.U32, n)
    o = orc.empty(orc.U32, n)
    kbuf = orc.empty(orc.U32, (threads * 8 << 20) // 4 + (1 << 20)) if ref is not None else None

    def one():
        d[:] = src
        t0 = time.perf_counter()
        if ref is not None:
            ref.ref_sort_multi_thread(d.ctypes.data, o.ctypes.data, n, threads, threads, 16,
                                      kbuf.ctypes.data)
        else:
            orc.sort_multi_thread_inplace(orc.U32, d, o, threads, 16)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        one()
    times = [one() for _ in range(args.steps)]
    total = sum(times)
    value = n * len(times) / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gkeys/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic: uniform uint32, numpy seed 7",
        "config": {"workload": WORKLOAD, "n": n, "threads": threads, "min_k": 16},
        "cpu_baseline": {"value": value, "unit": "Gkeys/s", "cores": threads, "kind": kind_label,
                         "sample": f"the whole {n}-key workload per step; {build}"},
        "e2e": {"value": value, "unit": "Gkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def max_over_ranks(torch, dist, value, device):
    """The largest `value` over all ranks (the slowest replica sets the time)."""
    if not dist:
        return value
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gkeys_per_s(n, steps, world, total_ms):
    """Whole-job rate: every replica sorts n keys per step."""
    return world * n * steps / (total_ms / 1e3) / 1e9


def short_workloads(torch):
    """Batched and serving measurements carried on the headline line (shorter
    runs than `--workload batched|serving`). Failures are reported, not raised."""
    import origami_gpu as og
    from origami_gpu import workloads as wl
    out = {}

    def fresh():
        # each workload starts with the device memory the previous ones cached
        # (torch's allocator, the library's pool) handed back: serving latency
        # measured right after gigabytes of cached blocks on the default stream
        # was 2-6x worse at p99 than in a fresh process
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        og.lib().origami_arena_trim()

    fresh()
    try:
        out["batched"] = wl.batched(torch, steps=3, warmup=3)
    except Exception as e:  # reported in the line
        out["batched"] = {"error": repr(e)}
    fresh()
    try:
        out["plain_configs"] = wl.plain_configs(torch)
    except Exception as e:
        out["plain_configs"] = {"error": repr(e)}
    fresh()
    try:
        out["kv_distributions"] = wl.kv_distributions(torch, steps=2, warmup=1)
    except Exception as e:
        out["kv_distributions"] = {"error": repr(e)}
    try:
        # one rate, long enough for a steady p99 (the rate sweep is --workload
        # serving), in a process of its own as a server would run: measured in
        # this process after the other workloads, p99 and saturation varied
        # 2-6x with what they had left behind on the device
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--workload", "serving",
                            "--serving-rates", "400", "--serving-seconds", "5", "--serving-pool", "64"],
                           capture_output=True, text=True, timeout=900)
        lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
        if r.returncode != 0 or not lines:
            raise RuntimeError(f"serving run exited {r.returncode}: {(r.stderr or r.stdout)[-400:]}")
        sv = json.loads(lines[-1])["detail"]
        out["serving"] = sv
        ok = [r for r in sv["rates"] if r["failed"] == 0]
        if ok:
            top = ok[-1]
            out["latency"] = {"p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
                              "offered_rate_per_s": top["offered_rate"],
                              "keys_per_s": top["keys_per_s"], "source": "serving loop",
                              # the largest request's own copies in and out at the measured link rate
                              "largest_request_link_floor_ms": sv.get("largest_request", {}).get("link_floor_ms"),
                              "saturation_vs_loop_plain": sv.get("saturation_vs_loop_plain")}
    except Exception as e:
        out["serving"] = {"error": repr(e)}
    return out


def run_workload(args, torch, world, rank):
    """`--workload batched|serving`: that workload alone, one JSON line."""
    from origami_gpu import workloads as wl
    if rank != 0:
        return
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    if args.workload == "kv":
        r = wl.kv_distributions(torch, steps=args.steps, warmup=args.warmup)
        line = {"metric": "Gkeys/s key-value sort of 134,217,728 (uint64, uint64) pairs per distribution",
                "value": min(x["gkeys_s"] for x in r.values()), "unit": "Gkeys/s", "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "kvu64", "data": "synthetic",
                "config": {"workload": "2^27 pairs, value = input index; " + ", ".join(wl.KV_DISTS)},
                "detail": r}
    elif args.workload == "plain":
        r = wl.plain_configs(torch, steps=args.steps, warmup=args.warmup)
        line = {"metric": "Gkeys/s: 1 GiB uint64 sort and 1 GiB uint32 chunked sorts",
                "value": r["u64_1GiB"]["gkeys_s"], "unit": "Gkeys/s", "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "u64/u32", "data": "synthetic", "config": {"workload": "134,217,728 uniform uint64 keys (1 GiB), full sort; 268,435,456 uniform "
                                                         "uint32 keys (1 GiB) in chunks of 2^17..2^21 keys"}, "detail": r}
    elif args.workload == "batched":
        r = wl.batched(torch, steps=args.steps, warmup=args.warmup, nseg=args.segments, hi=args.max_len,
                       loop_steps=args.loop_steps)
        line = {"metric": f"Gkeys/s batched segmented sort ({args.segments} uint32 arrays, one graph replay)",
                "value": r["segmented_gkeys_s"], "unit": "Gkeys/s", "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["segmented_graph_ms"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
                "config": {"workload": r["workload"], "l2": r["l2"]}, "detail": r}
    else:
        r = wl.serving(torch, rates=tuple(int(x) for x in args.serving_rates.split(",")),
                       duration_s=args.serving_seconds, pool_size=args.serving_pool)
        best = max(r["rates"], key=lambda x: x["keys_per_s"])
        line = {"metric": "serving throughput (keys/s) with p50/p99 latency",
                "value": best["keys_per_s"] / 1e9, "unit": "Gkeys/s", "n_gpus": 1,
                "steps": len(r["rates"]), "warmup": 1, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "mixed u32/u64/kv", "data": "synthetic",
                "config": {"workload": r["workload"]}, "detail": r}
    line["clocks"] = clocks.stop()
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="origami", choices=["origami", "reference"])
    ap.add_argument("--n", type=int, default=N_KEYS)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip timing the pass shapes before the measurement (the default shape is used)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched and serving measurements added to the line")
    ap.add_argument("--workload", default="sort", choices=["sort", "batched", "serving", "kv", "plain"],
                    help="sort: the headline line; batched / serving / kv / plain: that workload alone")
    ap.add_argument("--segments", type=int, default=65536, help="batched: number of arrays")
    ap.add_argument("--max-len", type=int, default=1 << 20, help="batched: longest array")
    ap.add_argument("--loop-steps", type=int, default=2, help="batched: timed runs of the plain-sort loop")
    ap.add_argument("--serving-rates", default="100,200,400,800,1600", help="serving: offered rates (req/s)")
    ap.add_argument("--serving-seconds", type=float, default=4.0, help="serving: seconds per rate")
    ap.add_argument("--serving-pool", type=int, default=128, help="serving: distinct requests")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    import origami_gpu as og

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    og.lib()
    if args.workload != "sort":
        run_workload(args, torch, world, rank)
        return
    n = args.n
    kind = og.U32
    dev = torch.device("cuda", local)
    g = torch.Generator(device=dev).manual_seed(1234 + rank)
    pristine = torch.randint(-(2**31), 2**31, (n,), dtype=torch.int32, device=dev, generator=g)
    d = torch.empty_like(pristine)
    tmp = torch.empty_like(pristine)

    # the autotuner times every pass shape on this size and installs the
    # fastest for it (outside the timed region); it is part of the product path
    tuning = None
    if not args.no_autotune:
        tuning = og.autotune(kind, n)

    def step():
        d.copy_(pristine)
        return og.sort(d, tmp, kind=kind)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # correctness of the measured configuration (outside the timed region)
    out = step()
    torch.cuda.synchronize()
    k = out.to(torch.int64) & 0xFFFFFFFF
    ok = bool((k[1:] >= k[:-1]).all().item()) and int(k.sum().item()) == int(
        (pristine.to(torch.int64) & 0xFFFFFFFF).sum().item())
    del k

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    # per-kernel CUDA events on every PROFILE_EVERY-th launch of each kernel:
    # an event pair between two kernels stops the second from starting while
    # the first drains (programmatic dependent launch), so bracketing every
    # launch slowed the timed sort by 3 %; 15 and 7 are coprime, so over the
    # timed steps every merge level is sampled
    og.profile_enable(True, every=PROFILE_EVERY)
    launches0 = og.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        d.copy_(pristine)
        starts[i].record()
        og.sort(d, tmp, kind=kind)
        ends[i].record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    launches = og.launch_count() - launches0
    detail = og.profile_detail()
    report = og.profile_report()
    og.profile_enable(False)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max_over_ranks(torch, dist, sum(step_ms), dev)
    value = job_gkeys_per_s(n, args.steps, world, total_ms)
    peak, peak_src = peaks()
    item = 4
    # dominant kernel and its roofline
    dom = max(report.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_ms) = dom
    per_launch_ms = dom_ms / dom_launches
    bytes_per_launch = 2 * n * item
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9
    passes = sum(c for name, (c, _) in report.items()
                 if name.startswith(("block_sort", "pair_merge", "kway_merge"))) // args.steps
    ms_step = total_ms / args.steps
    # DRAM bytes per launch need an ncu capture, which this run does not make
    traffic = None

    e2e = None
    if args.e2e_steps > 0:
        h_src = pristine.cpu().numpy().view("uint32")
        h_d = og.empty_host("u32", n, pinned=True)
        h_t = og.empty_host("u32", n, pinned=True)
        ts = []
        # a collection of the interpreter's cyclic garbage inside a timed call
        # (tens of ms with torch loaded) is not the sort's time
        import gc
        gc.collect()
        gc.disable()
        try:
            for i in range(args.e2e_steps + 1):
                h_d[:] = h_src
                t0 = time.perf_counter()
                r = og.sort(h_d, h_t)
                t1 = time.perf_counter()
                if i > 0:
                    ts.append(t1 - t0)
        finally:
            gc.enable()
        import numpy as np
        e2e_ok = bool(np.all(r[1:] >= r[:-1]))
        e2e = {"value": n / statistics.mean(ts) / 1e9, "unit": "Gkeys/s",
               "h2d_bytes_per_step": n * item, "d2h_bytes_per_step": n * item,
               "ms_per_step": 1e3 * statistics.mean(ts), "steps": len(ts), "correct": e2e_ok,
               "ms_each": [round(1e3 * x, 3) for x in ts],
               # single calls occasionally take 1.5-4x as long on these shared
               # hosts; the value above includes them, this one does not
               "value_median_call": n / statistics.median(ts) / 1e9}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(n)

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        del d, tmp, out
        torch.cuda.empty_cache()
        extras = short_workloads(torch)

    line = {
        "metric": METRIC, "value": value, "unit": "Gkeys/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic: uniform uint32 keys from torch.randint on the device (seed 1234+rank)",
        "config": {"workload": WORKLOAD, "n": n, "item_bytes": item,
                   "l2": "input (1 GiB) larger than L2; restored from a pristine copy before each step",
                   "hbm_passes": passes, "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                     "bytes_per_launch": bytes_per_launch, "launch_ms": per_launch_ms,
                     "launches_timed": detail[dom_name][1],
                     "traffic": traffic,
                     "pipeline_frac": (2 * n * item * passes / (ms_step / 1e3) / 1e9) / peak,
                     # one read + write of the array at peak (P = 1), and all passes
                     "pass_floor_ms": 2 * n * item / (peak * 1e9) * 1e3,
                     "passes_floor_ms": 2 * n * item * passes / (peak * 1e9) * 1e3},
        "kernels": {k: {"launches": c, "timed": t, "ms_per_launch": (ms / t if t else None)}
                    for k, (c, t, ms) in detail.items()},
        "gpu_launches": launches,
        "tuning": tuning,
        "correct": ok,
        "clocks": clk,
        "e2e": e2e,
        "cpu_baseline": cpu,
        **extras,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
