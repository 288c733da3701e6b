// Instantiation of the plain-sort pipeline for uint32_t items.
#include "dispatch.h"
#include "pipeline.cuh"

namespace origami {

cudaError_t sort_u32(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                     int fan, void* scratch, cudaStream_t st, LaunchStats* stats) {
    return sort_pipeline<uint32_t>(static_cast<uint32_t*>(d), static_cast<uint32_t*>(tmp), n, sort_n, key_mask,
                              static_cast<uint32_t*>(want), fan, scratch, st, stats);
}

uint64_t scratch_bytes_u32(uint64_t n, uint64_t sort_n, int fan) {
    return pipeline_scratch_bytes<uint32_t>(n, sort_n, fan);
}

}  // namespace origami
