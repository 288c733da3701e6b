// Host orchestration of the plain sort: K1 tile sort, then binary merge passes
// (K4 splitters + K3 tile merges) until the runs reach the chunk size. Restates
// the control flow of the reference's sort_single_thread (sorter.h:3851-3915):
// phase 1-2 (tile sort) then phase 3 (merge levels over DRAM-resident runs),
// with the ping-pong buffer bookkeeping that decides where the result lands.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "kway.cuh"
#include "profiler.h"
#include "sort_kernels.cuh"

namespace origami {

template <class T>
struct Config;
// K1 tile (K1_NT*K1_VT) must be a multiple of the merge tile (M_NT*M_VT)/2 so
// that a merge tile never straddles two run pairs.
template <>
struct Config<uint32_t> {
    // K1: warps sort 32*32 keys in registers, then shared-memory rounds to 8192
    static constexpr bool WARP_K1 = true;
    // 8 warps sort 1024 keys each; 9 warps share the merge rounds (265 blocks)
    static constexpr int K1_NW = 8, K1_NWT = 9, K1_VT = 32, K1_MINB = 3;
    static constexpr int K1_RUN0 = 1024;  // register merges up to the whole warp's 1024 keys
    static constexpr int K1_NT = 256, K1_VTS = 32, K1_VTM = 32;  // (block K1, unused)
    // binary pass tiles (P_BULK: the persistent bulk-copy merge kernel)
    static constexpr int P_NT = 160, P_VT = 32, P_TILE = 4096, P_MINB = 6;
    static constexpr bool P_BULK = true;
    static constexpr int P2_NT = 288, P2_VT = 32, P2_TILE = 8192, P2_MINB = 3;  // second tile shape
    static constexpr bool P2_BULK = true;
    static constexpr int PI_MINB = 1;  // the first shape as one tile per CTA (variant 2)
    // variant 3: the first shape's tile with half the keys per thread
    static constexpr int P3_NT = 288, P3_VT = 16, P3_MINB = 4;
    static constexpr bool STABLE = false;
};
template <>
struct Config<uint64_t> {
    static constexpr bool WARP_K1 = true;
    static constexpr int K1_NW = 8, K1_NWT = 9, K1_VT = 16, K1_MINB = 3;
    static constexpr int K1_RUN0 = 128;  // register merges to runs of 128 keys, shared-memory rounds from there
    static constexpr int K1_NT = 512, K1_VTS = 8, K1_VTM = 16;
    static constexpr int P_NT = 160, P_VT = 16, P_TILE = 2048, P_MINB = 6;
    static constexpr bool P_BULK = true;
    static constexpr int P2_NT = 288, P2_VT = 16, P2_TILE = 4096, P2_MINB = 3;
    static constexpr bool P2_BULK = true;
    static constexpr int PI_MINB = 8;
    static constexpr int P3_NT = 320, P3_VT = 8, P3_MINB = 3;
    static constexpr bool STABLE = false;
};
template <>
struct Config<KV64> {
    static constexpr bool WARP_K1 = false;  // key-value items need stable merges
    static constexpr int K1_NW = 8, K1_NWT = 8, K1_VT = 8, K1_MINB = 1;
    static constexpr int K1_RUN0 = 256;  // (the warp tile sort serves keys-only items)
    static constexpr int K1_NT = 256, K1_VTS = 8, K1_VTM = 11;  // 2048 items (32 KiB), serial blocks of 11
    static constexpr int P_NT = 96, P_VT = 11, P_TILE = 1024, P_MINB = 4;  // serial merge blocks of 11
    static constexpr bool P_BULK = true;
    static constexpr int P2_NT = 192, P2_VT = 11, P2_TILE = 2048, P2_MINB = 3;
    static constexpr bool P2_BULK = true;
    static constexpr int PI_MINB = 1;
    static constexpr int P3_NT = 160, P3_VT = 7, P3_MINB = 5;  // serial blocks of 7
    static constexpr bool STABLE = true;
};

template <class T>
using K1Shape = BlockSortShape<T, Config<T>::K1_NT, Config<T>::K1_VTS, Config<T>::K1_VTM, Config<T>::STABLE>;
template <class T>
using K1WShape = WarpSortShape<T, Config<T>::K1_NW, Config<T>::K1_VT, Config<T>::K1_NWT>;
template <class T>
constexpr int k1_tile() {
    return Config<T>::WARP_K1 ? K1WShape<T>::TILE : K1Shape<T>::TILE;
}
template <class T>
constexpr int merge_tile() {
    return Config<T>::P_TILE;
}
template <class T>
constexpr size_t k1_smem() {
    return Config<T>::WARP_K1 ? K1WShape<T>::SMEM : K1Shape<T>::SMEM;
}
template <class T>
using PShape = PairShape<T, Config<T>::P_NT, Config<T>::P_VT, Config<T>::STABLE, Config<T>::P_TILE>;
// Launch of a kernel that may start before the previous kernel in the stream
// has finished (programmatic dependent launch): the kernel itself waits for it
// (grid_dep_wait) before it touches memory, so only the launch latency and the
// CTA start-up overlap the previous kernel's tail. Partition and bulk merge
// kernels go this way: 1,048,576 uint32 keys sort in 0.113 ms instead of
// 0.141 ms, 16 M keys in 0.57 ms instead of 0.63 ms.
template <class... KArgs, class... Args>
cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                             Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// One binary-pass merge shape: pair_merge_kernel (one tile per CTA, cp.async
// staging) or, with BULK, pair_merge_bulk_kernel (persistent, double-buffered
// bulk copies, as many CTAs as fit on the GPU at once).
template <class T, int NT, int VT, int TILE, int MINB, bool BULK>
struct PairMerge {
    static constexpr bool ST = Config<T>::STABLE;
    static constexpr size_t SMEM = BULK ? PairBulkShape<T, NT, VT, ST, TILE>::SMEM : PairShape<T, NT, VT, ST, TILE>::SMEM;
    static void configure() {
        if constexpr (BULK)
            cudaFuncSetAttribute(pair_merge_bulk_kernel<T, NT, VT, ST, TILE, MINB>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
        else
            cudaFuncSetAttribute(pair_merge_kernel<T, NT, VT, ST, TILE, MINB>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
    }
    // resident CTAs on the whole GPU (the persistent grid)
    static uint64_t resident() {
        static const uint64_t r = [] {
            configure();
            int dev = 0, sms = 0, per = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, pair_merge_bulk_kernel<T, NT, VT, ST, TILE, MINB>, NT,
                                                          SMEM);
            return (uint64_t)sms * (uint64_t)(per > 0 ? per : 1);
        }();
        return r;
    }
    // claim: the tile counter pair_partition_kernel reset just before
    static void launch(const T* cur, T* nxt, uint64_t n, uint64_t run, const int64_t* splits, uint64_t tiles,
                       uint64_t xo, unsigned* claim, int* err, cudaStream_t st) {
        if constexpr (BULK) {
            const uint64_t g = tiles < resident() ? tiles : resident();
            launch_dependent(pair_merge_bulk_kernel<T, NT, VT, ST, TILE, MINB>, dim3((unsigned)g), dim3(NT), SMEM, st,
                             cur, nxt, n, run, splits, tiles, xo, claim, ~0u, err, wait_limit());
        } else {
            (void)claim;
            pair_merge_kernel<T, NT, VT, ST, TILE, MINB><<<(unsigned)tiles, NT, SMEM, st>>>(cur, nxt, n, run, splits, xo,
                                                                                           err);
        }
    }
};
template <class T>
using PairMerge1 = PairMerge<T, Config<T>::P_NT, Config<T>::P_VT, Config<T>::P_TILE, Config<T>::P_MINB, Config<T>::P_BULK>;
template <class T>
using PairMerge2 =
    PairMerge<T, Config<T>::P2_NT, Config<T>::P2_VT, Config<T>::P2_TILE, Config<T>::P2_MINB, Config<T>::P2_BULK>;
// The first shape with one tile per CTA: several sorts on concurrent streams
// interleave at CTA granularity, so one sort's latency-bound splitter searches
// overlap another's merges (a persistent kernel holds the SMs until it drains).
template <class T>
using PairMergeI = PairMerge<T, Config<T>::P_NT, Config<T>::P_VT, Config<T>::P_TILE, Config<T>::PI_MINB, false>;
// The first shape's tile merged with half the items per thread (more threads,
// fewer registers each): the autotuner's choice of items per thread.
template <class T>
using PairMerge3 = PairMerge<T, Config<T>::P3_NT, Config<T>::P3_VT, Config<T>::P_TILE, Config<T>::P3_MINB, true>;

// Resident CTAs of the k-way merge kernel on the whole GPU (its persistent grid).
template <class T>
uint64_t kb_resident() {
    static const uint64_t r = [] {
        cudaFuncSetAttribute(kb_merge_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KbShape<T>::SMEM);
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb_merge_kernel<T>, KbCfg<T>::NT, KbShape<T>::SMEM);
        return (uint64_t)sms * (uint64_t)(per > 0 ? per : 1);
    }();
    return r;
}

static_assert(Config<uint32_t>::P2_TILE >= Config<uint32_t>::P_TILE && Config<uint64_t>::P2_TILE >= Config<uint64_t>::P_TILE &&
                  Config<KV64>::P2_TILE >= Config<KV64>::P_TILE,
              "the splitter array is sized by the first (smallest) tile");

// A pass shape code: merge fan-in in the low byte (2 = binary passes, 4/8/16 =
// k-way), the binary-pass merge shape above it (0 = P_*, 1 = P2_*, 2 = P_* one
// tile per CTA). Chosen per kind and size by the tuning table (capi.cu).
inline int shape_fan(int code) { return code & 0xFF; }
inline int shape_variant(int code) { return code >> 8; }
inline int shape_code(int fan, int variant) { return fan | (variant << 8); }

// Number of binary merge passes after K1 for runs to reach `limit` items.
inline int merge_passes(uint64_t limit, uint64_t tile) {
    int p = 0;
    for (uint64_t r = tile; r < limit; r <<= 1) ++p;
    return p;
}

struct LaunchStats {
    int kernels = 0;  // kernel launches issued
    int passes = 0;   // HBM passes (K1 + merge passes)
};

// int64 slots the binary-pass splitter array needs (one per merge tile + 1).
template <class T>
inline uint64_t merge_split_slots(uint64_t n) {
    return n / merge_tile<T>() + 2;
}

// One merge pass of the plan: runs of `run` items merged `fan` at a time.
struct PassPlan {
    uint64_t run;
    int fan;          // 2 = binary pass (K4 pair partition + K3 pair merge)
    uint64_t groups;  // k-way: groups of `fan` runs
    int rpg;          // k-way: exact ranges per group (1 = the group is one range)
};

inline int next_pow2_int(uint64_t v) {
    int p = 1;
    while ((uint64_t)p < v && p < (1 << 30)) p <<= 1;
    return p;
}

// The merge passes after K1 for runs to reach `limit` (chunk size or n).
// fan == 2 gives the binary pipeline; fan in {4, 8, 16} the k-way one, whose
// last pass uses the smallest fan-in that still reaches `limit`.
template <class T>
std::vector<PassPlan> plan_passes(uint64_t n, uint64_t limit, int fan, uint64_t start_run = 0) {
    std::vector<PassPlan> v;
    uint64_t run = start_run ? start_run : k1_tile<T>();
    while (run < limit) {
        PassPlan p{run, 2, 0, 1};
        if (fan > 2) {
            const uint64_t need = (limit + run - 1) / run;
            p.fan = need < (uint64_t)fan ? next_pow2_int(need) : fan;
            if (p.fan < 2) p.fan = 2;
            const uint64_t G = run * (uint64_t)p.fan;
            p.groups = (n + G - 1) / G;
            p.rpg = kb_ranges_per_group<T>(run, p.fan);
        }
        v.push_back(p);
        run *= (uint64_t)p.fan;
    }
    return v;
}

inline uint64_t chunk_limit(uint64_t n, uint64_t sort_n) {
    return (sort_n == 0 || sort_n >= n) ? n : sort_n;
}

// Device scratch of one sort, in this order (each part 256-byte aligned):
//   splits     binary passes: one int64 per merge tile + 2
//   k-way passes (only when the plan has some, kway_bulk.cuh):
//   bnd0       super-sample splits of the range boundaries, [groups][rpg+1][16]
//   cut q/key/run  the ranges' tile cuts (KbCuts), [ranges][TPR+1]([16])
//   tiles      the pass's tile list (slots), ranges * TPR
//   samp 0/1   samples (one key per S items) of the runs a pass reads / writes
//   ssamp 0/1  super-samples (one key per S*64 items)
//   tail       256 bytes: the error word, the merge kernels' claim counter
//              (+64), the k-way passes' two tile counters (+128, +132)
template <class T>
struct PipeScratch {
    using K = typename Traits<T>::Key;
    uint64_t bytes = 0;  // total, tail included
    int64_t* splits = nullptr;
    int64_t* bnd0 = nullptr;
    KbCuts cuts{nullptr, nullptr, nullptr};
    uint32_t* tiles = nullptr;
    unsigned* tcount = nullptr;  // [2]: pass p counts its tiles in tcount[p & 1]
    K* samp[2] = {nullptr, nullptr};
    K* ssamp[2] = {nullptr, nullptr};
    int* err = nullptr;
    unsigned* claim = nullptr;
    PipeScratch(void* base, uint64_t n, uint64_t sort_n, int code, uint64_t start_run) {
        char* b = static_cast<char*>(base);
        uint64_t o = 0;
        auto take = [&](uint64_t sz) {
            char* r = b ? b + o : nullptr;
            o += (sz + 255) & ~255ull;
            return r;
        };
        uint64_t bnd_b = 0, rng = 0;
        bool kway = false;
        for (const PassPlan& p : plan_passes<T>(n, chunk_limit(n, sort_n), shape_fan(code), start_run)) {
            if (p.fan <= 2) continue;
            kway = true;
            if (p.rpg > 1) bnd_b = std::max<uint64_t>(bnd_b, p.groups * (uint64_t)(p.rpg + 1) * KWAY_MAX * 8);
            rng = std::max<uint64_t>(rng, p.groups * (uint64_t)p.rpg);
        }
        splits = reinterpret_cast<int64_t*>(take(merge_split_slots<T>(n) * sizeof(int64_t)));
        if (kway) {
            constexpr uint64_t S = KbCfg<T>::S;
            const uint64_t rows = rng * (uint64_t)(KbShape<T>::TPR + 1);
            if (bnd_b) bnd0 = reinterpret_cast<int64_t*>(take(bnd_b));
            cuts.q = reinterpret_cast<uint32_t*>(take(rows * KWAY_MAX * 4));
            cuts.key = take(rows * sizeof(K));
            cuts.run = reinterpret_cast<int*>(take(rows * 4));
            tiles = reinterpret_cast<uint32_t*>(take(rows * 4));
            for (int i = 0; i < 2; ++i) samp[i] = reinterpret_cast<K*>(take((n / S + 1) * sizeof(K)));
            for (int i = 0; i < 2; ++i) ssamp[i] = reinterpret_cast<K*>(take((n / (S * KB_SS) + 1) * sizeof(K)));
        }
        err = reinterpret_cast<int*>(take(256));
        claim = b ? reinterpret_cast<unsigned*>(reinterpret_cast<char*>(err) + 64) : nullptr;
        tcount = b ? reinterpret_cast<unsigned*>(reinterpret_cast<char*>(err) + 128) : nullptr;
        bytes = o;
    }
};

// Device scratch (bytes) one sort needs (PipeScratch); the error word is the
// first int of its last 256 bytes.
template <class T>
uint64_t pipeline_scratch_bytes(uint64_t n, uint64_t sort_n, int code, uint64_t start_run = 0) {
    return PipeScratch<T>(nullptr, n, sort_n, code, start_run).bytes;
}

// Sorts in[0..n) in chunks of sort_n (0 = one full sort) into out[0..n).
// The first kernel reads `in` once and the last pass writes `out` once; the
// passes in between ping-pong between the work buffers wa and wb (the pass
// before the last writes wa, the one before that wb, ...). `in` may be one of
// the work buffers (the first kernel sorts tiles in place) and out may be wb;
// in and out may also be host memory the device can address (pinned or, with
// address translation services, pageable), which streams the data over the
// host link inside the first and last kernels instead of separate copies.
// xin is XORed into every key as the first kernel reads it, xout as the last
// kernel writes it (the sign flip of signed keys; see common.cuh).
// start_run > 0 skips the first kernel: `in` already holds sorted runs of
// start_run items (a multiple of the tile, keys already flipped by xin), and
// only the merge passes from there to the chunk size run (at least one).
// `scratch` holds pipeline_scratch_bytes<T>(n, sort_n, fan, start_run) bytes of
// device memory.
template <class T>
cudaError_t sort_pipeline_io(const T* in, T* out, T* wa, T* wb, uint64_t n, uint64_t sort_n, uint64_t xin,
                             uint64_t xout, uint64_t start_run, int code, void* scratch, cudaStream_t st,
                             LaunchStats* stats) {
    using C = Config<T>;
    using KC = KwayCfg<T>;
    constexpr int T1 = k1_tile<T>();
    const int fan = shape_fan(code);
    const int variant = shape_variant(code);
    const int MT = variant == 1 ? C::P2_TILE : merge_tile<T>();
    if (n == 0) return cudaSuccess;
    const bool full = (sort_n == 0 || sort_n >= n);
    const uint64_t limit = chunk_limit(n, sort_n);
    const std::vector<PassPlan> plan = plan_passes<T>(n, limit, fan, start_run);
    const int passes = (int)plan.size();
    if (start_run && passes == 0) return cudaErrorInvalidValue;
    const int k1_chunk = (int)(limit < (uint64_t)T1 ? (full ? T1 : limit) : T1);
    // buffer written by step k (0 = the first kernel, k = pass k): out for the
    // last, then wa, wb, wa, ... going backwards
    auto written_by = [&](int k) -> T* { return k == passes ? out : (((passes - k) & 1) ? wa : wb); };
    const T* cur = start_run ? in : written_by(0);
    const PipeScratch<T> sc(scratch, n, sort_n, code, start_run);
    int64_t* splits = sc.splits;
    int* err = sc.err;
    unsigned* claim = sc.claim;
    using K = typename Traits<T>::Key;
    // samples for the first k-way pass: written by the tile sort, or gathered
    // from runs the caller gave (start_run)
    const bool kw_first = passes > 0 && plan[0].fan > 2;
    K* k1_samp = (kw_first && !start_run) ? sc.samp[0] : nullptr;
    K* k1_ssamp = (kw_first && !start_run) ? sc.ssamp[0] : nullptr;

    // kernel attributes, once per process (thread-safe static initialisation)
    static const bool configured = [] {
        if constexpr (C::WARP_K1) {
            cudaFuncSetAttribute(warp_block_sort_kernel<T, C::K1_NW, C::K1_VT, C::K1_NWT, C::K1_MINB, false, C::K1_RUN0>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k1_smem<T>());
            cudaFuncSetAttribute(warp_block_sort_kernel<T, C::K1_NW, C::K1_VT, C::K1_NWT, C::K1_MINB, true, C::K1_RUN0>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k1_smem<T>());
        } else
            cudaFuncSetAttribute(block_sort_kernel<T, C::K1_NT, C::K1_VTS, C::K1_VTM, C::STABLE>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k1_smem<T>());
        PairMerge1<T>::configure();
        PairMerge2<T>::configure();
        PairMergeI<T>::configure();
        PairMerge3<T>::configure();
        cudaFuncSetAttribute(range_merge_kernel<T, RunLists<T>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)KwayLayout<T>::SMEM);
        cudaFuncSetAttribute(kb_cut_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)KbShape<T>::CUT_SMEM);
        cudaFuncSetAttribute(kb_merge_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KbShape<T>::SMEM);
        return true;
    }();
    (void)configured;

    static const std::string n_k1 = std::string("block_sort<") + TypeName<T>::v + ">";
    static const std::string n_k4 = std::string("pair_partition<") + TypeName<T>::v + ">";
    static const std::string n_k3 = std::string("pair_merge<") + TypeName<T>::v + ">";
    static const std::string n_ks = std::string("kway_split<") + TypeName<T>::v + ">";
    static const std::string n_kc = std::string("kway_cut<") + TypeName<T>::v + ">";
    static const std::string n_km = std::string("kway_merge<") + TypeName<T>::v + ">";
    static const std::string n_kg = std::string("kway_samples<") + TypeName<T>::v + ">";
    const uint64_t tiles1 = (n + T1 - 1) / T1;
    // the tile sort prefetches into L2 the tile one wave of resident CTAs
    // further on (input in device memory only; 1 GiB: 1.89 -> 1.82 ms)
    uint32_t ahead = 0;
    if constexpr (C::WARP_K1) {  // (the key-value tile sort measured no gain)
        static const uint32_t wave = [] {
            int dev = 0, sms = 0, per = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per, warp_block_sort_kernel<T, C::K1_NW, C::K1_VT, C::K1_NWT, C::K1_MINB, false, C::K1_RUN0>, C::K1_NWT * 32,
                k1_smem<T>());
            return (uint32_t)(sms * (per > 0 ? per : 1));
        }();
        if (!start_run && tiles1 > wave) {
            cudaPointerAttributes pa;
            if (cudaPointerGetAttributes(&pa, in) != cudaSuccess)
                cudaGetLastError();  // not a CUDA pointer (pageable host memory): no prefetch
            else if (pa.type == cudaMemoryTypeDevice)
                ahead = wave;
        }
    }
    // the error word starts at 0: the tile sort clears it, else a memset
    if (start_run) cudaMemsetAsync(err, 0, sizeof(int), st);
    if (!start_run) {
        T* k1_out = written_by(0);
        launch(n_k1.c_str(), st, [&] {
            if constexpr (C::WARP_K1) {
                if (k1_samp)
                    warp_block_sort_kernel<T, C::K1_NW, C::K1_VT, C::K1_NWT, C::K1_MINB, true, C::K1_RUN0>
                        <<<(unsigned)tiles1, C::K1_NWT * 32, k1_smem<T>(), st>>>(
                            in, k1_out, n, k1_chunk, xin, passes == 0 ? xout : 0, ahead, err, k1_samp, k1_ssamp);
                else
                    warp_block_sort_kernel<T, C::K1_NW, C::K1_VT, C::K1_NWT, C::K1_MINB, false, C::K1_RUN0>
                        <<<(unsigned)tiles1, C::K1_NWT * 32, k1_smem<T>(), st>>>(
                            in, k1_out, n, k1_chunk, xin, passes == 0 ? xout : 0, ahead, err);
            } else
                block_sort_kernel<T, C::K1_NT, C::K1_VTS, C::K1_VTM, C::STABLE>
                    <<<(unsigned)tiles1, C::K1_NT, k1_smem<T>(), st>>>(in, k1_out, n, k1_chunk, xin,
                                                                       passes == 0 ? xout : 0, err, k1_samp,
                                                                       k1_ssamp);
        });
        if (stats) {
            stats->kernels++;
            stats->passes++;
        }
    }
    for (int pi = 0; pi < passes; ++pi) {
        const PassPlan& p = plan[pi];
        T* nxt = written_by(pi + 1);
        const uint64_t xo = pi + 1 == passes ? xout : 0;
        if (p.fan == 2) {
            const uint64_t tiles = (n + MT - 1) / MT;
            // small blocks spread the latency-bound searches over more SMs
            const unsigned pblocks = (unsigned)((tiles + 1 + 63) / 64);
            const uint64_t run = p.run;
            launch(n_k4.c_str(), st, [&] {
                launch_dependent(pair_partition_kernel<T>, dim3(pblocks), dim3(64), 0, st, cur, n, run, MT, tiles,
                                 splits, claim);
            });
            launch(n_k3.c_str(), st, [&] {
                if (variant == 1)
                    PairMerge2<T>::launch(cur, nxt, n, run, splits, tiles, xo, claim, err, st);
                else if (variant == 2)
                    PairMergeI<T>::launch(cur, nxt, n, run, splits, tiles, xo, claim, err, st);
                else if (variant == 3)
                    PairMerge3<T>::launch(cur, nxt, n, run, splits, tiles, xo, claim, err, st);
                else
                    PairMerge1<T>::launch(cur, nxt, n, run, splits, tiles, xo, claim, err, st);
            });
            if (stats) stats->kernels += 2;
        } else {
            // sampled k-way pass (kway_bulk.cuh): samples of `cur` are in set
            // pi & 1; the pass writes set (pi+1) & 1 when a k-way pass follows
            constexpr uint64_t S = KbCfg<T>::S, SS = KB_SS;
            K* s_in = sc.samp[pi & 1];
            K* ss_in = sc.ssamp[pi & 1];
            const bool more = pi + 1 < passes && plan[pi + 1].fan > 2;
            K* s_out = more ? sc.samp[(pi + 1) & 1] : nullptr;
            K* ss_out = more ? sc.ssamp[(pi + 1) & 1] : nullptr;
            if (pi == 0 && start_run) {
                const uint64_t ns = n / S;
                const unsigned gb = (unsigned)std::min<uint64_t>((ns + 255) / 256 + 1, 152ull * 16);
                launch(n_kg.c_str(), st, [&] { kb_gather_samples_kernel<T><<<gb, 256, 0, st>>>(cur, n, s_in, ss_in); });
                if (stats) stats->kernels++;
            }
            if (p.rpg > 1) {
                launch(n_ks.c_str(), st, [&] {
                    kway_split_kernel<K, RunLists<K>><<<(unsigned)(p.groups * (p.rpg + 1)), 256, 0, st>>>(
                        RunLists<K>{ss_in, n / (S * SS), p.run / (S * SS), p.fan}, p.rpg, 0, sc.bnd0, err);
                });
                if (stats) stats->kernels++;
            }
            const uint64_t ranges = p.groups * (uint64_t)p.rpg;
            // pass pi lists its tiles in tcount[pi & 1]; the first k-way pass's
            // counter starts at 0 here, each merge kernel zeroes the next one
            unsigned* tc = sc.tcount + (pi & 1);
            if (pi == 0) cudaMemsetAsync(tc, 0, sizeof(unsigned), st);
            launch(n_kc.c_str(), st, [&] {
                kb_cut_kernel<T><<<(unsigned)ranges, KB_CUT_NT, KbShape<T>::CUT_SMEM, st>>>(
                    s_in, n, p.run, p.fan, p.rpg, sc.bnd0, sc.cuts, sc.tiles, tc, claim, err);
            });
            const uint64_t nslots = ranges * (uint64_t)KbShape<T>::TPR;
            const uint64_t grid = std::min<uint64_t>(nslots, kb_resident<T>());
            launch(n_km.c_str(), st, [&] {
                kb_merge_kernel<T><<<(unsigned)grid, KbCfg<T>::NT, KbShape<T>::SMEM, st>>>(
                    cur, nxt, n, p.run, p.fan, p.rpg, sc.cuts, sc.tiles, tc, more ? sc.tcount + ((pi + 1) & 1) : nullptr,
                    xo, s_out, ss_out, claim, err, wait_limit());
            });
            if (stats) stats->kernels += 2;
        }
        if (stats) stats->passes++;
        cur = nxt;
    }
    return cudaGetLastError();
}

// One k-way pass merging the F runs of `run` items in[0..n) (n <= run * F,
// one group) into out, launched in `slices` parts by output range so that the
// caller can start consuming finished output while later parts merge: after
// each part, on_slice(o0, o1) is called with the output items [o0, o1) it
// completed (enqueue work after them on `st`). Keys are already in the
// internal order; xout is applied as they are written.
// `scratch` holds kway_pass_scratch_bytes<T>(n) bytes.
template <class T>
uint64_t kway_pass_err_offset(uint64_t n) {
    const uint64_t rpg = (n + KwayCfg<T>::RANGE - 1) / KwayCfg<T>::RANGE;
    return (rpg + 1) * KWAY_MAX * sizeof(int64_t);
}
template <class T>
uint64_t kway_pass_scratch_bytes(uint64_t n) {
    return kway_pass_err_offset<T>(n) + 256;
}

template <class T, class OnSlice>
cudaError_t kway_pass_sliced(const T* in, T* out, uint64_t n, uint64_t run, int fan, uint64_t xout, void* scratch,
                             cudaStream_t st, int slices, OnSlice&& on_slice) {
    using KC = KwayCfg<T>;
    static const std::string n_ks = std::string("kway_split<") + TypeName<T>::v + ">";
    static const std::string n_km = std::string("kway_merge<") + TypeName<T>::v + ">";
    static const bool configured = [] {
        cudaFuncSetAttribute(range_merge_kernel<T, RunLists<T>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)KwayLayout<T>::SMEM);
        return true;
    }();
    (void)configured;
    if (n == 0) return cudaSuccess;
    const uint64_t rpg = (n + KC::RANGE - 1) / KC::RANGE;
    int64_t* bnd = static_cast<int64_t*>(scratch);
    int* err = reinterpret_cast<int*>(static_cast<char*>(scratch) + kway_pass_err_offset<T>(n));
    const RunLists<T> lists{in, n, run, fan};
    cudaMemsetAsync(err, 0, sizeof(int), st);
    if (rpg > 1)
        launch(n_ks.c_str(), st, [&] {
            kway_split_kernel<T, RunLists<T>><<<(unsigned)(rpg + 1), 256, 0, st>>>(lists, (int)rpg, 0, bnd, err);
        });
    if (slices < 1) slices = 1;
    if ((uint64_t)slices > rpg) slices = (int)rpg;
    for (int sl = 0; sl < slices; ++sl) {
        const uint64_t b0 = rpg * sl / slices, b1 = rpg * (sl + 1) / slices;
        launch(n_km.c_str(), st, [&] {
            range_merge_kernel<T, RunLists<T>><<<(unsigned)(b1 - b0), KC::NT, KwayLayout<T>::SMEM, st>>>(
                lists, out, (int)rpg, rpg > 1 ? bnd : nullptr, 0, xout, (uint32_t)b0, NoProbe(), err);
        });
        // range b starts at output b * n / rpg (kway_split_kernel's boundaries)
        on_slice((uint64_t)(((unsigned __int128)b0 * n) / rpg), (uint64_t)(((unsigned __int128)b1 * n) / rpg));
    }
    return cudaGetLastError();
}

// Sorts d[0..n) in chunks of sort_n into `want` (d or tmp), ping-ponging
// between the two: the last pass writes want, so the one before writes the
// other buffer. With an even number of merge passes the first kernel writes
// want itself (in place when want == d).
template <class T>
cudaError_t sort_pipeline(T* d, T* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, T* want,
                          int fan, void* scratch, cudaStream_t st, LaunchStats* stats) {
    T* other = (want == d) ? tmp : d;
    return sort_pipeline_io<T>(d, want, other, want, n, sort_n, key_mask, key_mask, 0, fan, scratch, st, stats);
}

}  // namespace origami
