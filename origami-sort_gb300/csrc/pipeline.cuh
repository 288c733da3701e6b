// Host orchestration of the plain sort: K1 tile sort, then binary merge passes
// (K4 splitters + K3 tile merges) until the runs reach the chunk size. Restates
// the control flow of the reference's sort_single_thread (sorter.h:3851-3915):
// phase 1-2 (tile sort) then phase 3 (merge levels over DRAM-resident runs),
// with the ping-pong buffer bookkeeping that decides where the result lands.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "profiler.h"
#include "sort_kernels.cuh"

namespace origami {

template <class T>
struct Config;
// K1 tile (K1_NT*K1_VT) must be a multiple of the merge tile (M_NT*M_VT)/2 so
// that a merge tile never straddles two run pairs.
template <>
struct Config<uint32_t> {
    static constexpr int K1_NT = 512, K1_VT = 16;  // 8192-item tiles (32 KiB)
    static constexpr int M_NT = 256, M_VT = 16;    // 4096-item merge tiles
    static constexpr bool STABLE = false;
};
template <>
struct Config<uint64_t> {
    static constexpr int K1_NT = 512, K1_VT = 8;  // 4096 items (32 KiB)
    static constexpr int M_NT = 256, M_VT = 8;    // 2048
    static constexpr bool STABLE = false;
};
template <>
struct Config<KV64> {
    static constexpr int K1_NT = 256, K1_VT = 8;  // 2048 items (32 KiB)
    static constexpr int M_NT = 256, M_VT = 8;    // 2048
    static constexpr bool STABLE = true;
};

template <class T>
constexpr int k1_tile() {
    return Config<T>::K1_NT * Config<T>::K1_VT;
}
template <class T>
constexpr int merge_tile() {
    return Config<T>::M_NT * Config<T>::M_VT;
}
template <class T>
constexpr size_t k1_smem() {
    return (size_t)padded_items<T>(k1_tile<T>() + Config<T>::K1_VT) * sizeof(T);
}
template <class T>
constexpr size_t merge_smem() {
    return (size_t)padded_items<T>(merge_tile<T>() + Config<T>::M_VT) * sizeof(T);
}

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

// Sorts d[0..n) in chunks of sort_n (0 = one full sort). The output lands in
// `want` (d or tmp); `key_mask` is XORed into every key on the way in and out.
// `splits` must hold merge_split_slots(n) int64 values (device memory).
template <class T>
inline uint64_t merge_split_slots(uint64_t n) {
    return n / merge_tile<T>() + 2;
}

template <class T>
cudaError_t sort_pipeline(T* d, T* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, T* want,
                          int64_t* splits, cudaStream_t st, LaunchStats* stats) {
    using C = Config<T>;
    constexpr int T1 = k1_tile<T>();
    constexpr int MT = merge_tile<T>();
    if (n == 0) return cudaSuccess;
    const bool full = (sort_n == 0 || sort_n >= n);
    const uint64_t limit = full ? n : sort_n;
    const int passes = limit > (uint64_t)T1 ? merge_passes(limit, T1) : 0;
    const int k1_chunk = (int)(limit < (uint64_t)T1 ? (full ? T1 : limit) : T1);
    // the last writer must target `want`: with an even number of merge passes
    // K1 writes there itself (in place when want == d)
    T* other = (want == d) ? tmp : d;
    T* cur = (passes % 2 == 0) ? want : other;

    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(block_sort_kernel<T, C::K1_NT, C::K1_VT, C::STABLE>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k1_smem<T>());
        cudaFuncSetAttribute(pair_merge_kernel<T, C::M_NT, C::M_VT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)merge_smem<T>());
        configured = true;
    }

    static const std::string n_k1 = std::string("block_sort<") + TypeName<T>::v + ">";
    static const std::string n_k4 = std::string("pair_partition<") + TypeName<T>::v + ">";
    static const std::string n_k3 = std::string("pair_merge<") + TypeName<T>::v + ">";
    const uint64_t tiles1 = (n + T1 - 1) / T1;
    launch(n_k1.c_str(), st, [&] {
        block_sort_kernel<T, C::K1_NT, C::K1_VT, C::STABLE><<<(unsigned)tiles1, C::K1_NT, k1_smem<T>(), st>>>(
            d, cur, n, k1_chunk, key_mask, passes == 0 ? key_mask : 0);
    });
    if (stats) {
        stats->kernels++;
        stats->passes++;
    }
    uint64_t run = T1;
    for (int p = 0; p < passes; ++p) {
        T* nxt = (cur == want) ? other : want;
        const uint64_t tiles = (n + MT - 1) / MT;
        const unsigned pblocks = (unsigned)((tiles + 1 + 255) / 256);
        launch(n_k4.c_str(), st, [&] {
            pair_partition_kernel<T><<<pblocks, 256, 0, st>>>(cur, n, run, MT, tiles, splits);
        });
        launch(n_k3.c_str(), st, [&] {
            pair_merge_kernel<T, C::M_NT, C::M_VT><<<(unsigned)tiles, C::M_NT, merge_smem<T>(), st>>>(
                cur, nxt, n, run, splits, p + 1 == passes ? key_mask : 0);
        });
        if (stats) {
            stats->kernels += 2;
            stats->passes++;
        }
        cur = nxt;
        run <<= 1;
    }
    return cudaGetLastError();
}

}  // namespace origami
