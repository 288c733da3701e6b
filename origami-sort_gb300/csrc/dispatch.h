// Typed entry points compiled in one translation unit per item type
// (sort_u32.cu, sort_u64.cu, sort_kv.cu) and dispatched on by the C ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace origami {

struct LaunchStats;

// Sorts d[0..n) in chunks of sort_n into `want` (d or tmp) with merge fan-in
// `fan` (2 = binary passes, 4/8/16 = k-way passes); see pipeline.cuh.
#define ORIGAMI_DECLARE_SORT(name)                                                              \
    cudaError_t sort_##name(void* d, void* tmp, uint64_t n, uint64_t sort_n, uint64_t key_mask, \
                            void* want, int fan, void* scratch, cudaStream_t st,                \
                            LaunchStats* stats);                                                \
    uint64_t scratch_bytes_##name(uint64_t n, uint64_t sort_n, int fan);                          \
    cudaError_t sort_io_##name(const void* in, void* out, void* wa, void* wb, uint64_t n, uint64_t sort_n, \
                               uint64_t xin, uint64_t xout, uint64_t start_run, int fan, void* scratch,   \
                               cudaStream_t st);                                                          \
    uint64_t scratch_bytes_io_##name(uint64_t n, uint64_t sort_n, int fan, uint64_t start_run);          \
    uint64_t tile_##name();                                                                               \
    cudaError_t kway_final_##name(const void* in, void* out, uint64_t n, uint64_t run, int fan, uint64_t xout, \
                                  void* scratch, cudaStream_t st, int slices,                            \
                                  void (*on_slice)(void*, uint64_t, uint64_t), void* ctx);         \
    uint64_t kway_final_err_##name(uint64_t n); /* error word's offset in kway_final's scratch */
ORIGAMI_DECLARE_SORT(u32)
ORIGAMI_DECLARE_SORT(u64)
ORIGAMI_DECLARE_SORT(kv)
#undef ORIGAMI_DECLARE_SORT

// Batched segmented sort (segmented.cuh): levels to plan for, scratch bytes,
// the launch sequence, and where the error word sits inside the scratch.
#define ORIGAMI_DECLARE_SEG(name)                                                                 \
    int seg_levels_##name(uint64_t n);                                                           \
    uint64_t seg_scratch_bytes_##name(uint64_t n, uint64_t nseg, int maxl);                      \
    cudaError_t seg_sort_##name(void* d, void* tmp, const uint64_t* off, uint64_t nseg, uint64_t n, \
                                uint64_t key_mask, void* scratch, int maxl, int shape, cudaStream_t st); \
    int seg_err_offset_##name(uint64_t n, uint64_t nseg, int maxl);                               \
    int seg_prepare_##name(); /* one-time kernel attributes; call outside stream capture */
ORIGAMI_DECLARE_SEG(u32)
ORIGAMI_DECLARE_SEG(u64)
ORIGAMI_DECLARE_SEG(kv)
#undef ORIGAMI_DECLARE_SEG

// Kind-generic form of the above (capi.cu), shared by the C ABI and the
// serving loop: the plan for n items in nseg segments, then the launch
// sequence on `st` with caller-provided scratch of plan.scratch_bytes. The
// device error word (0 ok, 1 a bounded wait ran out, 2 bad offsets) is the int
// at scratch + plan.err_offset once the stream has passed the launch.
struct SegPlan {
    int maxl;
    uint64_t scratch_bytes;
    int err_offset;
    int shape;  // merge shape of the level merges (0 or 1), from the segmented tuning table
};
SegPlan seg_plan(int kind, uint64_t n, uint64_t nseg);
void seg_prepare(int kind);
cudaError_t seg_launch(int kind, void* d, void* tmp, const uint64_t* off, uint64_t nseg, uint64_t n,
                       void* scratch, const SegPlan& p, cudaStream_t st);

// Status of a device error word (bulk.cuh): 1 and 3 mean a bounded bulk-copy
// wait expired (ORIGAMI_ERR_TIMEOUT), 2 bad segment offsets
// (ORIGAMI_ERR_INVALID), 0 none.
inline bool err_word_timeout(int w) { return w == 1 || w == 3; }

// capi.cu: the pipelined sort of one array whose buffers the device can
// address (host memory the GPU reads through its mapping or page tables, or
// device memory): chunks copied in while earlier chunks sort, then one k-way
// pass whose output slices leave while later slices merge. host_pipe_bytes is
// the device memory it needs (one block, caller-owned); host_pipe_sort runs it
// on `st` and the calling thread's helper streams and returns once the result
// is in `out` (ORIGAMI_ERR_INVALID when a buffer is not device-addressable).
uint64_t host_pipe_bytes(int kind, uint64_t n);
int host_pipe_sort(int kind, const void* in, void* out, uint64_t n, void* block, cudaStream_t st);

// capi.cu: sets the thread's last-error message; makes the stream-ordered pool
// the caching device arena (returns an ORIGAMI_* status).
int api_fail(int code, const char* msg);
int arena_init();

}  // namespace origami
