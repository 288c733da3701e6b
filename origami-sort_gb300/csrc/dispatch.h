// Typed entry points compiled in one translation unit per item type
// (sort_u32.cu, sort_u64.cu, sort_kv.cu) and dispatched on by the C ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace origami {

struct LaunchStats;

// Sorts d[0..n) in chunks of sort_n into `want` (d or tmp); see pipeline.cuh.
cudaError_t sort_u32(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                     int64_t* splits, cudaStream_t st, LaunchStats* stats);
cudaError_t sort_u64(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                     int64_t* splits, cudaStream_t st, LaunchStats* stats);
cudaError_t sort_kv(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                    int64_t* splits, cudaStream_t st, LaunchStats* stats);
// int64 slots the splitter scratch needs for n items of the given kind.
uint64_t split_slots(int kind, uint64_t n);

}  // namespace origami
