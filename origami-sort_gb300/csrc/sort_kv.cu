// Instantiation of the plain-sort pipeline for KV64 items.
#include "dispatch.h"
#include "pipeline.cuh"

namespace origami {

cudaError_t sort_kv(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                     int fan, void* scratch, cudaStream_t st, LaunchStats* stats) {
    return sort_pipeline<KV64>(static_cast<KV64*>(d), static_cast<KV64*>(tmp), n, sort_n, key_mask,
                              static_cast<KV64*>(want), fan, scratch, st, stats);
}

uint64_t scratch_bytes_kv(uint64_t n, uint64_t sort_n, int fan) {
    return pipeline_scratch_bytes<KV64>(n, sort_n, fan);
}

}  // namespace origami
