// Instantiation of the plain-sort pipeline for uint64_t items.
#include "dispatch.h"
#include "pipeline.cuh"

namespace origami {

cudaError_t sort_u64(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                     int fan, void* scratch, cudaStream_t st, LaunchStats* stats) {
    return sort_pipeline<uint64_t>(static_cast<uint64_t*>(d), static_cast<uint64_t*>(tmp), n, sort_n, key_mask,
                              static_cast<uint64_t*>(want), fan, scratch, st, stats);
}

uint64_t scratch_bytes_u64(uint64_t n, uint64_t sort_n, int fan) {
    return pipeline_scratch_bytes<uint64_t>(n, sort_n, fan);
}

}  // namespace origami
