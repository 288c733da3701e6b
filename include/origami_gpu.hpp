// origami_gpu.hpp - C++ surface of the GB300 Origami mergesort, with the
// reference's names and argument meaning, over the C ABI of origami_gpu.h.
//
//   sort_single_thread<Item>(d, tmp_buf, end, sort_n, min_k, interim_buf)
//       origami_sorter::sort_single_thread (reference sorter.h:3851-3915)
//   sort_multi_thread<Item>(d, out, n, n_threads, n_cores, min_k, kway_buf)
//       origami_sorter::sort_multi_thread (sorter.h:4194-4287); the thread
//       counts do not apply to one GPU and are ignored
//   merge_series<Item>(src, dst, n, merge_start, sort_n)
//       origami_merger::merge_series (merger.h:4220-4228), device buffers
//   MergeTree<Item>::merge_init / merge / merge_cleanup
//       origami_merge_tree::MergeTreeEven/Odd (merge_tree.h:2577-3735),
//       device buffers; both merge forms (equal chunks, pointer-bounded streams)
//   Partition_Ptrs<Item>(L, R, S, K)
//       partition_templated::Partition_Ptrs (Partition.h:118-166), device
//       buffers; S moves to the split of the rank sum(S[k] - L[k])
//
// Every function returns like the reference (a pointer to the buffer holding
// the result where the reference returns one) and throws origami_gpu::error
// with the library's status code where the reference would print and exit.
// Item: uint32_t, uint64_t, int64_t, KeyValue<int64_t, int64_t>,
// KeyValue<uint64_t, uint64_t>.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "origami_gpu.h"

namespace origami_gpu {

// Same layout as the reference's KeyValue (commons.h:51-72): key, then value.
template <class K, class V>
struct KeyValue {
    K key;
    V value;
};
static_assert(sizeof(KeyValue<int64_t, int64_t>) == 16, "16-byte key-value items");

template <class Item>
struct kind_of;
template <>
struct kind_of<uint32_t> : std::integral_constant<int, ORIGAMI_U32> {};
template <>
struct kind_of<uint64_t> : std::integral_constant<int, ORIGAMI_U64> {};
template <>
struct kind_of<int64_t> : std::integral_constant<int, ORIGAMI_I64> {};
template <>
struct kind_of<KeyValue<int64_t, int64_t>> : std::integral_constant<int, ORIGAMI_KV64> {};
template <>
struct kind_of<KeyValue<uint64_t, uint64_t>> : std::integral_constant<int, ORIGAMI_KVU64> {};

class error : public std::runtime_error {
public:
    error(int code, const char* msg) : std::runtime_error(msg ? msg : "origami error"), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc) {
    if (rc != ORIGAMI_OK) throw error(rc, origami_last_error());
}

// Host or device buffers (see origami_sort): returns d or tmp_buf.
template <class Item>
Item* sort_single_thread(Item* d, Item* tmp_buf, Item* end, uint64_t sort_n, unsigned min_k = 2,
                         Item* interim_buf = nullptr) {
    (void)interim_buf;  // the GPU merge keeps its interim tiles on chip
    void* res = nullptr;
    check(origami_sort(kind_of<Item>::value, d, tmp_buf, (uint64_t)(end - d), sort_n, min_k, 0, &res));
    return static_cast<Item*>(res);
}

template <class Item>
Item* sort_multi_thread(Item* d, Item* out, uint64_t n_items, unsigned n_threads, unsigned n_cores,
                        unsigned min_k = 2, Item* kway_buf = nullptr) {
    (void)n_threads;
    (void)n_cores;
    (void)kway_buf;
    void* res = nullptr;
    check(origami_sort(kind_of<Item>::value, d, out, n_items, 0, min_k, 0, &res));
    return static_cast<Item*>(res);
}

// Device buffers; runs on `stream` (a cudaStream_t, NULL = legacy default).
template <class Item>
Item* merge_series(Item* src, Item* dst, uint64_t n, uint64_t merge_start, uint64_t sort_n,
                   void* stream = nullptr) {
    void* res = nullptr;
    check(origami_merge_series_device(kind_of<Item>::value, src, dst, n, merge_start, sort_n, &res, stream));
    return static_cast<Item*>(res);
}

// Device buffers. The interim buffer and the L1/L2 buffer sizes of the
// reference's tree are accepted and ignored: tiles are staged in shared memory
// and interim levels come from the library's device arena.
template <class Item>
class MergeTree {
public:
    void merge_init(unsigned WAY, Item* buf = nullptr, unsigned buf_n = 0, unsigned l2_buf_n = 0,
                    void* stream = nullptr) {
        (void)buf;
        (void)buf_n;
        (void)l2_buf_n;
        way_ = WAY;
        stream_ = stream;
    }
    void merge_cleanup() { way_ = 0; }

    // WAY equal chunks A[i*chunk, (i+1)*chunk) -> C (merge_tree.h:2618)
    void merge(Item* A, Item* C, uint64_t chunk, unsigned buf_n, unsigned l2_buf_n, Item* buf, unsigned WAY) {
        (void)buf_n;
        (void)l2_buf_n;
        (void)buf;
        std::vector<void*> X(WAY), E(WAY);
        for (unsigned i = 0; i < WAY; ++i) {
            X[i] = A + (uint64_t)i * chunk;
            E[i] = A + (uint64_t)(i + 1) * chunk;
        }
        check(origami_merge_tree_device(kind_of<Item>::value, X.data(), E.data(), C, WAY, stream_));
    }

    // streams [X[i], endX[i]) -> C (merge_tree.h:2792); n is their total
    void merge(Item** X, Item** endX, Item* C, uint64_t n, unsigned buf_n, unsigned l2_buf_n, Item* buf,
               unsigned WAY) {
        (void)n;
        (void)buf_n;
        (void)l2_buf_n;
        (void)buf;
        check(origami_merge_tree_device(kind_of<Item>::value, reinterpret_cast<void* const*>(X),
                                        reinterpret_cast<void* const*>(endX), C, WAY, stream_));
    }

    unsigned way() const { return way_; }

private:
    unsigned way_ = 0;
    void* stream_ = nullptr;
};

// Device buffers. Moves S[k] (L[k] <= S[k] <= R[k]) to the split that keeps
// sum(S[k] - L[k]) items on the left with every left item ordered before every
// right item (ties by stream). Waits for `stream`.
template <class Item>
void Partition_Ptrs(Item** L, Item** R, Item** S, uint64_t K, void* stream = nullptr) {
    uint64_t rank = 0;
    for (uint64_t k = 0; k < K; ++k) rank += (uint64_t)(S[k] - L[k]);
    std::vector<uint64_t> split(K);
    check(origami_partition_device(kind_of<Item>::value, reinterpret_cast<void* const*>(L),
                                   reinterpret_cast<void* const*>(R), (unsigned)K, &rank, 1, split.data(), stream));
    for (uint64_t k = 0; k < K; ++k) S[k] = L[k] + split[k];
}

}  // namespace origami_gpu
