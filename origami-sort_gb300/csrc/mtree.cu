// C ABI of the merge tree and the partitioner (merge_tree.cuh), instantiated
// for the three item widths.
#include <cstring>
#include <vector>

#include "../../include/origami_gpu.h"
#include "dispatch.h"
#include "merge_tree.cuh"

namespace {

using namespace origami;

unsigned item_bytes(int kind) { return kind == ORIGAMI_U32 ? 4u : (kind <= ORIGAMI_I64 ? 8u : 16u); }
uint64_t key_mask(int kind) {
    return (kind == ORIGAMI_I64 || kind == ORIGAMI_KV64) ? 0x8000000000000000ull : 0ull;
}

int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return ORIGAMI_OK;
    cudaGetLastError();
    return api_fail(e == cudaErrorMemoryAllocation ? ORIGAMI_ERR_OOM : ORIGAMI_ERR_CUDA, what);
}

// Validates K device streams [lo[i], hi[i]) of `kind`: ordered bounds, item
// alignment (16 bytes for key-value items, which the merge copies whole with
// 16-byte cp.async). Fills ptr/cnt.
int streams(int kind, const void* const* lo, const void* const* hi, unsigned K, std::vector<const void*>& ptr,
            std::vector<uint64_t>& cnt, uint64_t& total) {
    const unsigned ib = item_bytes(kind);
    const unsigned al = ib;  // u32: 4, u64/i64: 8, key-value: 16
    ptr.resize(K);
    cnt.resize(K);
    total = 0;
    for (unsigned i = 0; i < K; ++i) {
        const char* a = static_cast<const char*>(lo[i]);
        const char* b = static_cast<const char*>(hi[i]);
        if ((!a || !b) && a != b) return api_fail(ORIGAMI_ERR_INVALID, "stream bound is NULL");
        if (b < a) return api_fail(ORIGAMI_ERR_INVALID, "stream end precedes its start");
        if ((uintptr_t)a % al || (b - a) % ib)
            return api_fail(ORIGAMI_ERR_ALIGN, "stream not aligned to the item size");
        ptr[i] = a;
        cnt[i] = (uint64_t)(b - a) / ib;
        total += cnt[i];
    }
    return ORIGAMI_OK;
}

}  // namespace

extern "C" {

int origami_merge_tree_device(int kind, void* const* X, void* const* endX, void* C, unsigned way,
                              void* stream) {
    if (kind < ORIGAMI_U32 || kind > ORIGAMI_KVU64) return api_fail(ORIGAMI_ERR_DTYPE, "unknown item kind");
    if (way == 0) return ORIGAMI_OK;
    if (!X || !endX) return api_fail(ORIGAMI_ERR_INVALID, "X and endX are required");
    std::vector<const void*> ptr;
    std::vector<uint64_t> cnt;
    uint64_t total = 0;
    int rc = streams(kind, X, endX, way, ptr, cnt, total);
    if (rc != ORIGAMI_OK) return rc;
    if (total == 0) return ORIGAMI_OK;
    if (!C) return api_fail(ORIGAMI_ERR_INVALID, "C is NULL");
    const unsigned ib = item_bytes(kind);
    if ((uintptr_t)C % (ib > 8 ? 8 : ib)) return api_fail(ORIGAMI_ERR_ALIGN, "C not aligned to the item size");
    const char* c0 = static_cast<const char*>(C);
    const char* c1 = c0 + total * ib;
    for (unsigned i = 0; i < way; ++i) {
        const char* a = static_cast<const char*>(ptr[i]);
        if (cnt[i] && a < c1 && c0 < a + cnt[i] * ib)
            return api_fail(ORIGAMI_ERR_INVALID, "C overlaps an input stream");
    }
    if ((rc = arena_init()) != ORIGAMI_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint64_t m = key_mask(kind);
    cudaError_t e;
    switch (kind) {
        case ORIGAMI_U32:
            e = MergeTreeOps<uint32_t>::merge(reinterpret_cast<const uint32_t* const*>(ptr.data()), cnt.data(), way,
                                              static_cast<uint32_t*>(C), m, st);
            break;
        case ORIGAMI_U64:
        case ORIGAMI_I64:
            e = MergeTreeOps<uint64_t>::merge(reinterpret_cast<const uint64_t* const*>(ptr.data()), cnt.data(), way,
                                              static_cast<uint64_t*>(C), m, st);
            break;
        default:
            e = MergeTreeOps<KV64>::merge(reinterpret_cast<const KV64* const*>(ptr.data()), cnt.data(), way,
                                          static_cast<KV64*>(C), m, st);
            break;
    }
    return cuda_status(e, "merge tree");
}

int origami_partition_device(int kind, void* const* L, void* const* R, unsigned K,
                             const uint64_t* ranks, uint64_t n_ranks, uint64_t* splits,
                             void* stream) {
    if (kind < ORIGAMI_U32 || kind > ORIGAMI_KVU64) return api_fail(ORIGAMI_ERR_DTYPE, "unknown item kind");
    if (K == 0 || n_ranks == 0) return ORIGAMI_OK;
    if (K > (unsigned)RANK_SPLIT_MAX_K) return api_fail(ORIGAMI_ERR_INVALID, "at most 1024 streams");
    if (!L || !R || !ranks || !splits) return api_fail(ORIGAMI_ERR_INVALID, "L, R, ranks and splits are required");
    if (n_ranks > (1u << 30)) return api_fail(ORIGAMI_ERR_INVALID, "too many ranks");
    std::vector<const void*> ptr;
    std::vector<uint64_t> cnt;
    uint64_t total = 0;
    int rc = streams(kind, L, R, K, ptr, cnt, total);
    if (rc != ORIGAMI_OK) return rc;
    if ((rc = arena_init()) != ORIGAMI_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // one device block: pointers | counts | ranks | splits
    const uint64_t b_ptr = (uint64_t)K * 8, b_cnt = (uint64_t)K * 8, b_rank = n_ranks * 8;
    const uint64_t b_out = n_ranks * K * 8;
    char* dev = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&dev), b_ptr + b_cnt + b_rank + b_out, st);
    if (e != cudaSuccess) return cuda_status(e, "partition scratch");
    std::vector<char> host(b_ptr + b_cnt + b_rank);
    std::memcpy(host.data(), ptr.data(), b_ptr);
    std::memcpy(host.data() + b_ptr, cnt.data(), b_cnt);
    std::memcpy(host.data() + b_ptr + b_cnt, ranks, b_rank);
    e = cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, st);
    uint64_t* out = reinterpret_cast<uint64_t*>(dev + b_ptr + b_cnt + b_rank);
    const uint64_t* dcnt = reinterpret_cast<const uint64_t*>(dev + b_ptr);
    const uint64_t* drank = reinterpret_cast<const uint64_t*>(dev + b_ptr + b_cnt);
    const uint64_t m = key_mask(kind);
    if (e == cudaSuccess) {
        switch (kind) {
            case ORIGAMI_U32:
                e = MergeTreeOps<uint32_t>::split(reinterpret_cast<const uint32_t* const*>(dev), dcnt, (int)K, drank,
                                                  n_ranks, m, out, st);
                break;
            case ORIGAMI_U64:
            case ORIGAMI_I64:
                e = MergeTreeOps<uint64_t>::split(reinterpret_cast<const uint64_t* const*>(dev), dcnt, (int)K, drank,
                                                  n_ranks, m, out, st);
                break;
            default:
                e = MergeTreeOps<KV64>::split(reinterpret_cast<const KV64* const*>(dev), dcnt, (int)K, drank, n_ranks,
                                              m, out, st);
                break;
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(splits, out, b_out, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(dev, st);
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = es;
    return cuda_status(e, "partition");
}

}  // extern "C"
