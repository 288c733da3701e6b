// Instantiation of the plain-sort pipeline for KV64 items.
#include "dispatch.h"
#include "pipeline.cuh"
#include "seg_host.cuh"

namespace origami {

cudaError_t sort_kv(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, void* want,
                     int fan, void* scratch, cudaStream_t st, LaunchStats* stats) {
    return sort_pipeline<KV64>(static_cast<KV64*>(d), static_cast<KV64*>(tmp), n, sort_n, key_mask,
                              static_cast<KV64*>(want), fan, scratch, st, stats);
}

cudaError_t sort_io_kv(const void* in, void* out, void* wa, void* wb, uint64_t n, uint64_t sort_n,
                        uint64_t xin, uint64_t xout, uint64_t start_run, int fan, void* scratch, cudaStream_t st) {
    return sort_pipeline_io<KV64>(static_cast<const KV64*>(in), static_cast<KV64*>(out), static_cast<KV64*>(wa),
                                static_cast<KV64*>(wb), n, sort_n, xin, xout, start_run, fan, scratch, st, nullptr);
}

uint64_t scratch_bytes_io_kv(uint64_t n, uint64_t sort_n, int fan, uint64_t start_run) {
    return pipeline_scratch_bytes<KV64>(n, sort_n, fan, start_run);
}

uint64_t tile_kv() { return k1_tile<KV64>(); }

cudaError_t kway_final_kv(const void* in, void* out, uint64_t n, uint64_t run, int fan, uint64_t xout,
                          void* scratch, cudaStream_t st, int slices, void (*on_slice)(void*, uint64_t, uint64_t),
                          void* ctx) {
    return kway_pass_sliced<KV64>(static_cast<const KV64*>(in), static_cast<KV64*>(out), n, run, fan, xout, scratch, st,
                                slices, [&](uint64_t o0, uint64_t o1) { on_slice(ctx, o0, o1); });
}

uint64_t kway_final_err_kv(uint64_t n) { return kway_pass_err_offset<KV64>(n); }

uint64_t scratch_bytes_kv(uint64_t n, uint64_t sort_n, int fan) {
    return pipeline_scratch_bytes<KV64>(n, sort_n, fan);
}

int seg_levels_kv(uint64_t n) { return seg_levels_for<KV64>(n); }

uint64_t seg_scratch_bytes_kv(uint64_t n, uint64_t nseg, int maxl) {
    return seg_scratch_bytes<KV64>(n, nseg, maxl);
}

cudaError_t seg_sort_kv(void* d, void* tmp, const uint64_t* off, uint64_t nseg, uint64_t n,
                          uint64_t key_mask, void* scratch, int maxl, int shape, cudaStream_t st) {
    return seg_sort<KV64>(static_cast<KV64*>(d), static_cast<KV64*>(tmp), off, nseg, n, key_mask, scratch,
                          maxl, shape, st);
}

int seg_prepare_kv() { return seg_grid<KV64>(); }

int seg_err_offset_kv(uint64_t n, uint64_t nseg, int maxl) {
    SegState s = seg_state<KV64>(nullptr, nullptr, n, nseg, maxl);
    return (int)(reinterpret_cast<char*>(s.err) - static_cast<char*>(nullptr));
}

}  // namespace origami
