// Instantiation of the plain-sort pipeline for KV64 items.
#include "dispatch.h"
#include "pipeline.cuh"

namespace origami {

cudaError_t sort_kv(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                     int64_t* splits, cudaStream_t st, LaunchStats* stats) {
    return sort_pipeline<KV64>(static_cast<KV64*>(d), static_cast<KV64*>(tmp), n, sort_n, key_mask,
                              static_cast<KV64*>(want), splits, st, stats);
}

uint64_t split_slots_kv(uint64_t n) { return merge_split_slots<KV64>(n); }

}  // namespace origami
