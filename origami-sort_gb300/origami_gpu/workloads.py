"""Batched and serving workloads: synthetic inputs and their measurement.

batched  65,536 independent uint32 arrays, lengths log-uniform on
         [32, 1,048,576], keys uniform: one CUDA-graph replay of the batched
         segmented sort per step, against looping the plain single-array sort
         over the same arrays.
serving  sort requests with Poisson arrivals at swept rates through the serving
         loop (origami_server_*): lengths log-uniform on [1,024, 67,108,864],
         kinds 50% uint32 / 30% uint64 / 20% uint64-key+uint64-value pairs, keys
         uniform or Zipf(1.0) over 2^20 distinct values, 50/50 per request.
         Reports throughput and p50/p99 latency per rate.

Inputs are generated on the device with torch (seeded) and, for serving, copied
into pinned host buffers: requests arrive from host memory and their sorted
output is written back to host memory inside the measured latency.
"""
import ctypes
import time

import numpy as np

from . import KVU64, U32, U64, SegmentedPlan, Server, check, lib

ZIPF_DISTINCT = 1 << 20


def log_uniform_lengths(rng, count, lo, hi):
    x = np.exp(rng.uniform(np.log(lo), np.log(hi + 1), count))
    return np.clip(np.floor(x).astype(np.int64), lo, hi)


def device_keys(torch, n, gen, dev, zipf=False, words=1):
    """n keys of `words` 32-bit words (int32 storage), uniform, or Zipf(1.0)
    over 2^20 distinct values: rank r has probability ~ 1/r, drawn by inverting
    the continuous approximation of the harmonic CDF, then spread over the key
    space by multiplying with an odd constant (a bijection)."""
    if not zipf:
        return torch.randint(-(2**31), 2**31, (n * words,), dtype=torch.int32, device=dev, generator=gen)
    u = torch.rand(n, device=dev, generator=gen, dtype=torch.float64)
    rank = torch.floor(torch.exp(u * np.log(ZIPF_DISTINCT + 1.0))).to(torch.int64)  # 1..2^20
    rank = torch.clamp(rank, 1, ZIPF_DISTINCT)
    if words == 1:
        k = (rank * 0x9E3779B1) & 0xFFFFFFFF
        return torch.where(k >= 2**31, k - 2**32, k).to(torch.int32)
    return (rank * -0x61C8864680B583EB).view(torch.int32)  # x 0x9E3779B97F4A7C15 mod 2^64


# ------------------------------------------------------------------ batched --
CHUNK = 1 << 28


def u32_sum(torch, x):
    """Sum of the uint32 keys held in int32 tensor x, exact, in bounded chunks."""
    tot = 0
    for i in range(0, x.numel(), CHUNK):
        tot += int((x[i:i + CHUNK].to(torch.int64) & 0xFFFFFFFF).sum().item())
    return tot


def segments_sorted_u32(torch, x, off):
    """Every segment [off[s], off[s+1]) of the uint32 keys in x is ascending."""
    flip = x ^ torch.tensor(-(2**31), dtype=torch.int32, device=x.device)  # unsigned order as signed
    ok = True
    for i in range(0, x.numel() - 1, CHUNK):
        j = min(i + CHUNK, x.numel() - 1)
        up = flip[i + 1:j + 1] >= flip[i:j]
        b = off[(off > i) & (off <= j)] - 1 - i  # a segment starts at b + 1
        if len(b):
            up[torch.from_numpy(b).to(x.device)] = True
        ok &= bool(up.all().item())
    del flip
    return ok

def batched(torch, steps=5, warmup=3, nseg=65536, lo=32, hi=1 << 20, seed=4, loop_steps=1,
            dev=None):
    dev = dev or torch.device("cuda", torch.cuda.current_device())
    rng = np.random.default_rng(seed)
    lens = log_uniform_lengths(rng, nseg, lo, hi)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    n = int(off[-1])
    gen = torch.Generator(device=dev).manual_seed(seed)
    pristine = device_keys(torch, n, gen, dev)
    d = torch.empty_like(pristine)
    tmp = torch.empty_like(pristine)
    offs = torch.from_numpy(off).to(dev)
    stream = torch.cuda.current_stream(dev)
    # the segmented tuning table's merge shape for these segments, timed on them
    # (outside the measurement); the plan takes its shape from the table
    from . import autotune_segmented
    d.copy_(pristine)
    tuning = autotune_segmented(d, tmp, offs, U32)
    plan = SegmentedPlan(d, offs, tmp, kind=U32)
    for _ in range(warmup):
        d.copy_(pristine)
        plan.launch(stream.cuda_stream)
    plan.status(stream.cuda_stream)
    # properties of the result: every segment ascending, same multiset sum
    d.copy_(pristine)
    plan.launch(stream.cuda_stream)
    plan.status(stream.cuda_stream)
    ok = segments_sorted_u32(torch, d, off) and u32_sum(torch, d) == u32_sum(torch, pristine)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    l0 = int(lib().origami_launch_count())
    for a, b in ev:
        d.copy_(pristine)
        a.record(stream)
        plan.launch(stream.cuda_stream)
        b.record(stream)
    torch.cuda.synchronize()
    seg_launches = (int(lib().origami_launch_count()) - l0) // steps
    seg_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    plan.close()
    # per-kernel split of the same sort (outside the graph, one call)
    from . import profile_enable, profile_report, sort_segmented
    d.copy_(pristine)
    torch.cuda.synchronize()
    profile_enable(True)
    sort_segmented(d, offs, tmp, kind=U32, stream=stream.cuda_stream)
    kernels = {k: {"launches": c, "ms": round(ms, 3)} for k, (c, ms) in profile_report().items()}
    profile_enable(False)

    cpu = cpu_segments(pristine, off, lens, target_keys=1 << 26)

    # the plain single-array sort looped over the same arrays, from C-ABI calls
    L = lib()
    res = ctypes.c_void_p()
    st = ctypes.c_void_p(stream.cuda_stream)
    base_d, base_t = d.data_ptr(), tmp.data_ptr()
    ptrs = [(base_d + 4 * int(o), base_t + 4 * int(o), int(m)) for o, m in zip(off[:-1], lens)]
    fn = L.origami_sort_device

    def loop():
        for pd, pt, m in ptrs:
            rc = fn(U32, pd, pt, m, 0, 0, 0, ctypes.byref(res), st)
            if rc:
                check(rc)

    d.copy_(pristine)
    loop()  # warm-up: arena growth
    torch.cuda.synchronize()
    loop_ms = []
    for _ in range(loop_steps):
        d.copy_(pristine)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        loop()
        b.record(stream)
        torch.cuda.synchronize()
        loop_ms.append(a.elapsed_time(b))
    loop_ms = float(np.mean(loop_ms))
    del pristine, d, tmp
    torch.cuda.empty_cache()
    return {
        "workload": f"{nseg} uint32 arrays, lengths log-uniform on [{lo}, {hi}] (numpy seed {seed}), "
                    f"keys uniform (torch seed {seed}); {n} keys in total",
        "keys": n, "segments": nseg, "correct": ok,
        "segmented_graph_ms": seg_ms, "segmented_gkeys_s": n / seg_ms / 1e6,
        "kernels_per_replay": seg_launches, "kernels": kernels, "tuning": tuning,
        "loop_plain_ms": loop_ms, "loop_plain_gkeys_s": n / loop_ms / 1e6,
        "speedup_vs_loop": loop_ms / seg_ms,
        "cpu_segments": cpu,
        "l2": "inputs (GBs) larger than L2; restored from a pristine copy before each step",
    }


def cpu_segments(pristine, off, lens, target_keys):
    """Host comparator for the batched form (not the reference, which has no
    batched form): numpy's sort of each array on all host cores, over the first
    arrays up to target_keys keys."""
    import concurrent.futures
    import os
    k = int(np.searchsorted(off, target_keys, side="right")) - 1
    k = max(1, min(k, len(lens)))
    host = pristine[: int(off[k])].cpu().numpy().view(np.uint32)
    threads = os.cpu_count() or 1
    segs = [(int(off[i]), int(off[i + 1])) for i in range(k)]

    def work(idx):
        for i in idx:
            a, b = segs[i]
            np.sort(host[a:b], kind="quicksort")

    parts = [list(range(t, k, threads)) for t in range(threads)]
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, parts))  # warm-up
        t0 = time.perf_counter()
        list(ex.map(work, parts))
        dt = time.perf_counter() - t0
    keys = int(off[k])
    return {"gkeys_s": keys / dt / 1e9, "threads": threads, "arrays": k, "keys": keys,
            "sample": f"the first {k} arrays ({keys} keys), numpy sort per array, {threads} host threads; "
                      "not the reference (it has no batched form)"}


# ------------------------------------------------------------------ serving --
KIND_WORDS = {U32: 1, U64: 2, KVU64: 4}


class RequestPool:
    """`count` request inputs in pinned host memory (generated on the device)."""

    def __init__(self, torch, count, seed, lo=1024, hi=1 << 26, max_bytes=8 << 30, dev=None):
        dev = dev or torch.device("cuda", torch.cuda.current_device())
        rng = np.random.default_rng(seed)
        kinds = rng.choice([U32, U64, KVU64], size=count, p=[0.5, 0.3, 0.2])
        lens = log_uniform_lengths(rng, count, lo, hi)
        zipf = rng.random(count) < 0.5
        # keep the pinned pool bounded: shrink the longest requests' share
        words = np.array([KIND_WORDS[int(k)] for k in kinds])
        while int((lens * words * 4).sum()) > max_bytes:
            i = int(np.argmax(lens * words))
            lens[i] //= 2
        gen = torch.Generator(device=dev).manual_seed(seed)
        self.items = []
        for k, n, z, w in zip(kinds, lens, zipf, words):
            k, n, w = int(k), int(n), int(w)
            if k == KVU64:
                key = device_keys(torch, n, gen, dev, zipf=bool(z), words=2).view(torch.int64)
                val = torch.arange(n, device=dev, dtype=torch.int64)
                x = torch.stack([key, val], dim=1).reshape(-1).view(torch.int32)
            else:
                x = device_keys(torch, n, gen, dev, zipf=bool(z), words=w)
            h = torch.empty(x.numel(), dtype=torch.int32, pin_memory=True)
            h.copy_(x)
            out = torch.empty_like(h, pin_memory=True)
            self.items.append({"kind": k, "n": n, "zipf": bool(z), "in": h, "out": out})
        torch.cuda.synchronize()
        self.keys = int(lens.sum())
        self.bytes = int((lens * words * 4).sum())


def serve_rate(server, pool, rate, duration_s, seed, max_requests=None):
    """Open-loop Poisson arrivals at `rate` requests/s (None: all at once) for
    `duration_s` or `max_requests`; every request is waited for. Returns the
    server's statistics for this rate."""
    rng = np.random.default_rng(seed)
    server.reset_stats()
    L = lib()
    rid = ctypes.c_uint64()
    ids = []
    slot_ids = {}
    t0 = time.perf_counter()
    t_next = t0
    i = 0
    while max_requests is None or i < max_requests:
        if rate is not None:
            t_next += rng.exponential(1.0 / rate)
            if t_next - t0 > duration_s:
                break
        j = i % len(pool.items)
        it = pool.items[j]
        if j in slot_ids:  # the output buffer is reused: its last request must be done
            check(L.origami_serve_wait(server._h, slot_ids.pop(j), -1))
        now = time.perf_counter()
        if t_next > now:
            time.sleep(t_next - now)
        check(L.origami_serve_submit(server._h, it["kind"], it["in"].data_ptr(), it["out"].data_ptr(),
                                      it["n"], ctypes.byref(rid)))
        slot_ids[j] = rid.value
        ids.append(rid.value)
        i += 1
    for r in slot_ids.values():
        check(L.origami_serve_wait(server._h, r, -1))
    st = server.stats()
    st["offered_rate"] = rate
    st["requests"] = len(ids)
    st["elapsed_s"] = time.perf_counter() - t0
    return st


def serving(torch, rates=(100, 200, 400, 800), duration_s=3.0, pool_size=96, seed=11,
            budget=120 << 30, check_results=True, dev=None):
    pool = RequestPool(torch, pool_size, seed, dev=dev)
    out = {"workload": "Poisson arrivals; lengths log-uniform on [1024, 67108864]; kinds 50% u32 / "
                       "30% u64 / 20% u64+u64 pairs; uniform or Zipf(1.0) keys 50/50; "
                       f"{pool_size} distinct pinned-host requests reused round robin "
                       f"({pool.bytes / 2**30:.1f} GiB); HBM budget {budget >> 30} GiB",
           "rates": []}
    fields = ("offered_rate", "requests", "completed", "failed", "keys", "batches", "pipe_batches",
              "max_concurrent_batches", "peak_bytes_reserved", "arena_bytes", "arena_grows", "p50_ms", "p99_ms",
              "max_ms", "keys_per_s")
    with Server(hbm_budget_bytes=budget) as s:
        # warm-up: every request once (arena growth, first touch of host pages)
        serve_rate(s, pool, None, 0, seed, max_requests=len(pool.items))
        for r in rates:
            st = serve_rate(s, pool, r, duration_s, seed + r)
            out["rates"].append({k: st[k] for k in fields})
        # saturation: two rounds of the pool submitted back to back, three
        # times (one such run lasts about 0.1 s and varied by +-20 % between
        # runs); keys/s over all three, latency and counts of the median run
        runs = [serve_rate(s, pool, None, 0, seed + i, max_requests=2 * len(pool.items)) for i in range(3)]
        med = sorted(runs, key=lambda r: r["keys_per_s"])[1]
        out["saturation"] = {k: med[k] for k in fields if k != "offered_rate"}
        secs = sum(r["keys"] / r["keys_per_s"] for r in runs if r["keys_per_s"] > 0)
        out["saturation"]["keys_per_s"] = sum(r["keys"] for r in runs) / secs if secs > 0 else 0.0
        out["saturation"]["keys_per_s_runs"] = [r["keys_per_s"] for r in runs]
    if check_results:
        bad = 0
        for it in pool.items:
            h = it["out"]
            if it["kind"] == U32:
                k = h.numpy().view(np.uint32)
            elif it["kind"] == U64:
                k = h.numpy().view(np.uint64)
            else:
                k = h.numpy().view(np.uint64)[0::2]
            bad += int(not np.all(k[1:] >= k[:-1]))
        out["outputs_sorted"] = bad == 0
    # the plain single-array sort called once per request, same requests,
    # two rounds of the pool
    L = lib()
    res = ctypes.c_void_p()
    dt = 0.0
    for _ in range(2):
        for it in pool.items:
            it["out"].copy_(it["in"])
            t0 = time.perf_counter()
            check(L.origami_sort(it["kind"], it["out"].data_ptr(), None, it["n"], 0, 0, 0, ctypes.byref(res)))
            dt += time.perf_counter() - t0
    out["loop_plain_keys_per_s"] = 2 * pool.keys / dt
    if out.get("saturation", {}).get("keys_per_s"):
        out["saturation_vs_loop_plain"] = out["saturation"]["keys_per_s"] / out["loop_plain_keys_per_s"]
    # the host link: what the largest request's copies cost at the least
    big = max(pool.items, key=lambda it: it["in"].numel())
    nbytes = big["in"].numel() * 4
    dev_buf = torch.empty(big["in"].numel(), dtype=torch.int32, device=dev or "cuda")
    ts_in, ts_out = [], []
    for _ in range(3):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        c = torch.cuda.Event(enable_timing=True)
        a.record()
        dev_buf.copy_(big["in"], non_blocking=True)
        b.record()
        big["out"].copy_(dev_buf, non_blocking=True)
        c.record()
        torch.cuda.synchronize()
        ts_in.append(a.elapsed_time(b))
        ts_out.append(b.elapsed_time(c))
    del dev_buf
    out["largest_request"] = {"kind": big["kind"], "n": big["n"], "bytes": nbytes,
                              "copy_in_ms": min(ts_in), "copy_out_ms": min(ts_out),
                              "host_link_in_gbs": nbytes / min(ts_in) / 1e6,
                              "host_link_out_gbs": nbytes / min(ts_out) / 1e6,
                              "link_floor_ms": min(ts_in) + min(ts_out)}
    return out


# ------------------------------------------------- key-value distributions --
KV_DISTS = ("uniform", "zipf", "sorted", "reverse", "equal", "runs8")


def kv_input(torch, n, dist, gen, dev):
    """n uint64 keys (int64 storage) of one distribution; values are added by
    the caller. uniform over [0, 2^64); Zipf(1.0) over 2^20 ranks, key = rank
    times an odd 64-bit constant; sorted / reverse sorted uniform keys; one
    seeded value; 8 interleaved ascending runs (item i in run i mod 8)."""
    def uniform(m):
        lo = torch.randint(0, 2**32, (m,), dtype=torch.int64, device=dev, generator=gen)
        hi = torch.randint(0, 2**32, (m,), dtype=torch.int64, device=dev, generator=gen)
        return (hi << 32) | lo

    def unsigned_sorted(k):  # ascending as uint64: sort the sign-flipped values
        flip = k ^ (-(2**63))
        return torch.sort(flip).values ^ (-(2**63))

    if dist == "uniform":
        return uniform(n)
    if dist == "zipf":
        return device_keys(torch, n, gen, dev, zipf=True, words=2).view(torch.int64)
    if dist == "sorted":
        return unsigned_sorted(uniform(n))
    if dist == "reverse":
        return unsigned_sorted(uniform(n)).flip(0)
    if dist == "equal":
        return uniform(1).expand(n).contiguous()
    if dist == "runs8":
        m = (n + 7) // 8
        runs = torch.stack([unsigned_sorted(uniform(m)) for _ in range(8)], dim=1)  # [m, 8]
        return runs.reshape(-1)[:n].contiguous()
    raise ValueError(dist)


def kv_distributions(torch, n=1 << 27, steps=3, warmup=2, seed=3, dev=None):
    """Sort n (uint64 key, uint64 value = original index) pairs under every
    distribution. Checks on the device: keys ascending, and the pairs intact
    (key[i] == input key[value[i]], values a permutation) with equal keys in
    input order (stable)."""
    import ctypes
    from . import KVU64
    dev = dev or torch.device("cuda", torch.cuda.current_device())
    gen = torch.Generator(device=dev).manual_seed(seed)
    stream = torch.cuda.current_stream(dev)
    out = {}
    for dist in KV_DISTS:
        keys = kv_input(torch, n, dist, gen, dev)
        pristine = torch.stack([keys, torch.arange(n, device=dev, dtype=torch.int64)], dim=1).contiguous()
        d = torch.empty_like(pristine)
        tmp = torch.empty_like(pristine)
        res = ctypes.c_void_p()
        L = lib()

        def one():
            check(L.origami_sort_device(KVU64, d.data_ptr(), tmp.data_ptr(), n, 0, 0, 0, ctypes.byref(res),
                                        ctypes.c_void_p(stream.cuda_stream)))

        for _ in range(warmup):
            d.copy_(pristine)
            one()
        ms = []
        for _ in range(steps):
            d.copy_(pristine)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            one()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        k, v = d[:, 0], d[:, 1]
        flip = k ^ (-(2**63))
        asc = bool((flip[1:] >= flip[:-1]).all().item())
        intact = bool((keys[v] == k).all().item())
        perm = bool((torch.sort(v).values == torch.arange(n, device=dev)).all().item())
        same = k[1:] == k[:-1]
        stable = bool(((v[1:] > v[:-1]) | ~same).all().item())
        t = float(np.mean(ms))
        out[dist] = {"ms": t, "gkeys_s": n / t / 1e6, "sorted": asc, "pairs_intact": intact and perm,
                     "stable": stable}
        del keys, pristine, d, tmp, k, v, flip, same
        torch.cuda.empty_cache()
    return out


def plain_configs(torch, steps=3, warmup=2, dev=None):
    """1 GiB as 134,217,728 uniform uint64 keys, and the 1 GiB uint32 array
    sorted in chunks of 128K..2M keys (device-resident, CUDA events)."""
    import ctypes
    from . import U64
    dev = dev or torch.device("cuda", torch.cuda.current_device())
    gen = torch.Generator(device=dev).manual_seed(5)
    stream = torch.cuda.current_stream(dev)
    L = lib()
    res = ctypes.c_void_p()

    def timed(kind, pristine, d, tmp, n, sort_n):
        def one():
            check(L.origami_sort_device(kind, d.data_ptr(), tmp.data_ptr(), n, sort_n, 0, 0, ctypes.byref(res),
                                        ctypes.c_void_p(stream.cuda_stream)))
        for _ in range(warmup):
            d.copy_(pristine)
            one()
        ms = []
        for _ in range(steps):
            d.copy_(pristine)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            one()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.mean(ms))

    out = {}
    # 1,048,576 uint32 keys (4 MiB, L2-resident, launch-bound): device time and
    # the host call the reference's bench_sort makes (pageable buffers)
    n1 = 1 << 20
    p1 = torch.randint(-(2**31), 2**31, (n1,), dtype=torch.int32, device=dev, generator=gen)
    d1, t1 = torch.empty_like(p1), torch.empty_like(p1)
    ms1 = []
    for i in range(warmup + 20):
        d1.copy_(p1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        check(L.origami_sort_device(U32, d1.data_ptr(), t1.data_ptr(), n1, 0, 0, 0, ctypes.byref(res),
                                    ctypes.c_void_p(stream.cuda_stream)))
        b.record(stream)
        torch.cuda.synchronize()
        if i >= warmup:
            ms1.append(a.elapsed_time(b))
    h_in = p1.cpu().numpy().view(np.uint32)
    h = h_in.copy()
    ht = np.empty_like(h)
    host_ms = []
    for i in range(warmup + 10):
        h[:] = h_in
        t0 = time.perf_counter()
        check(L.origami_sort(U32, h.ctypes.data, ht.ctypes.data, n1, 0, 0, 0, ctypes.byref(res)))
        if i >= warmup:
            host_ms.append((time.perf_counter() - t0) * 1e3)
    out["u32_1M"] = {"n": n1, "device_ms": float(np.median(ms1)), "device_gkeys_s": n1 / float(np.median(ms1)) / 1e6,
                     "host_ms": float(np.median(host_ms)), "host_gkeys_s": n1 / float(np.median(host_ms)) / 1e6,
                     "equal_to_numpy_sort": bool(np.array_equal(h, np.sort(h_in)))}
    del p1, d1, t1
    n64 = 1 << 27
    p = torch.randint(-(2**63), 2**63 - 1, (n64,), dtype=torch.int64, device=dev, generator=gen)
    d, tmp = torch.empty_like(p), torch.empty_like(p)
    t = timed(U64, p, d, tmp, n64, 0)
    flip = d ^ (-(2**63))
    out["u64_1GiB"] = {"n": n64, "ms": t, "gkeys_s": n64 / t / 1e6,
                       "sorted": bool((flip[1:] >= flip[:-1]).all().item())}
    del p, d, tmp, flip
    n32 = 1 << 28
    p = torch.randint(-(2**31), 2**31, (n32,), dtype=torch.int32, device=dev, generator=gen)
    d, tmp = torch.empty_like(p), torch.empty_like(p)
    chunks = {}
    for sh in range(17, 22):
        s = 1 << sh
        t = timed(U32, p, d, tmp, n32, s)
        flip = (d ^ (-(2**31))).view(-1, s)
        ok = bool((flip[:, 1:] >= flip[:, :-1]).all().item())
        chunks[str(s)] = {"ms": t, "gkeys_s": n32 / t / 1e6, "sorted_chunks": ok}
        del flip
    out["u32_1GiB_chunked"] = chunks
    del p, d, tmp
    torch.cuda.empty_cache()
    return out
