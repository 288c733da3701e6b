// Instantiation of the plain-sort pipeline for uint32_t items.
#include "dispatch.h"
#include "pipeline.cuh"
#include "seg_host.cuh"

namespace origami {

cudaError_t sort_u32(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                     int fan, void* scratch, cudaStream_t st, LaunchStats* stats) {
    return sort_pipeline<uint32_t>(static_cast<uint32_t*>(d), static_cast<uint32_t*>(tmp), n, sort_n, key_mask,
                              static_cast<uint32_t*>(want), fan, scratch, st, stats);
}

cudaError_t sort_io_u32(const void* in, void* out, void* wa, void* wb, uint64_t n, uint64_t sort_n,
                        uint64_t xin, uint64_t xout, uint64_t start_run, int fan, void* scratch, cudaStream_t st) {
    return sort_pipeline_io<uint32_t>(static_cast<const uint32_t*>(in), static_cast<uint32_t*>(out), static_cast<uint32_t*>(wa),
                                static_cast<uint32_t*>(wb), n, sort_n, xin, xout, start_run, fan, scratch, st, nullptr);
}

uint64_t scratch_bytes_io_u32(uint64_t n, uint64_t sort_n, int fan, uint64_t start_run) {
    return pipeline_scratch_bytes<uint32_t>(n, sort_n, fan, start_run);
}

uint64_t tile_u32() { return k1_tile<uint32_t>(); }

cudaError_t kway_final_u32(const void* in, void* out, uint64_t n, uint64_t run, int fan, uint64_t xout,
                          void* scratch, cudaStream_t st, int slices, void (*on_slice)(void*, uint64_t, uint64_t),
                          void* ctx) {
    return kway_pass_sliced<uint32_t>(static_cast<const uint32_t*>(in), static_cast<uint32_t*>(out), n, run, fan, xout, scratch, st,
                                slices, [&](uint64_t o0, uint64_t o1) { on_slice(ctx, o0, o1); });
}

uint64_t kway_final_err_u32(uint64_t n) { return kway_pass_err_offset<uint32_t>(n); }

uint64_t scratch_bytes_u32(uint64_t n, uint64_t sort_n, int fan) {
    return pipeline_scratch_bytes<uint32_t>(n, sort_n, fan);
}

int seg_levels_u32(uint64_t n) { return seg_levels_for<uint32_t>(n); }

uint64_t seg_scratch_bytes_u32(uint64_t n, uint64_t nseg, int maxl) {
    return seg_scratch_bytes<uint32_t>(n, nseg, maxl);
}

cudaError_t seg_sort_u32(void* d, void* tmp, const uint64_t* off, uint64_t nseg, uint64_t n,
                          uint64_t key_mask, void* scratch, int maxl, int shape, cudaStream_t st) {
    return seg_sort<uint32_t>(static_cast<uint32_t*>(d), static_cast<uint32_t*>(tmp), off, nseg, n, key_mask, scratch,
                          maxl, shape, st);
}

int seg_prepare_u32() { return seg_grid<uint32_t>(); }

int seg_err_offset_u32(uint64_t n, uint64_t nseg, int maxl) {
    SegState s = seg_state<uint32_t>(nullptr, nullptr, n, nseg, maxl);
    return (int)(reinterpret_cast<char*>(s.err) - static_cast<char*>(nullptr));
}

}  // namespace origami
