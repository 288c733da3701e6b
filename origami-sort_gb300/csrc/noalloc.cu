// Allocation-free sort entry point (include/origami_gpu.h:
// origami_sort_noalloc_device).
//
// Who needs it: callers that must not allocate device memory during the call,
// for example code that runs while another allocator owns the GPU's free
// memory (a framework's caching allocator, a serving process that reserved
// its whole budget up front), code that cannot let an allocation stall or
// synchronize the device in a latency-critical loop, or runtimes that forbid
// the CUDA allocator outright. The regular entry points take their splitter
// scratch from the stream-ordered allocator; this one keeps it in a
// fixed-size array in the library's own device image instead.
//
// The scratch array below is part of every device image that loads the
// library and stays allocated on each GPU that uses it until the process
// exits. Its device address is looked up once per device (first call with that
// device current), so the first call on a device should happen before any
// stream capture begins. Every call shares the one
// array: two calls whose work overlaps on the GPU (different streams, or
// different host threads) race on it and must be serialized by the caller.
#include <cstdint>
#include <mutex>

#include "../../include/origami_gpu.h"
#include "dispatch.h"
#include "pipeline.cuh"

namespace origami {
int noalloc_fail(int code, const char* msg);  // capi.cu: sets origami_last_error()
int noalloc_check(int kind, const void* d, const void* tmp, uint64_t n, uint64_t sort_n,
                  void** result);  // capi.cu: the regular argument checks
}  // namespace origami

using namespace origami;

namespace {

// Binary-pass splitter slots (one per merge tile + 2) plus the pipeline's
// 256-byte status tail.
constexpr uint64_t kSlots = ORIGAMI_NOALLOC_SPLIT_SLOTS;
__device__ __align__(256) int64_t g_noalloc_scratch[kSlots + 32];

constexpr int kMaxDevices = 64;
int64_t* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_mu;

int64_t* scratch_for(int dev, cudaError_t* err) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        // host code must not use g_noalloc_scratch directly: that name is a
        // host-side stand-in, not the device address
        void* p = nullptr;
        *err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (*err != cudaSuccess) return nullptr;
        g_scratch_ptr[dev] = static_cast<int64_t*>(p);
    }
    *err = cudaSuccess;
    return g_scratch_ptr[dev];
}

// Bytes of scratch a binary-pass sort of n items uses: its splitter slots
// (rounded up to 256 bytes), then the 256-byte status tail whose first int is
// the sort's error word.
uint64_t scratch_needed(int kind, uint64_t n, uint64_t sort_n) {
    switch (kind) {
        case ORIGAMI_U32: return scratch_bytes_u32(n, sort_n, 2);
        case ORIGAMI_U64:
        case ORIGAMI_I64: return scratch_bytes_u64(n, sort_n, 2);
        default: return scratch_bytes_kv(n, sort_n, 2);
    }
}

}  // namespace

extern "C" uint64_t origami_noalloc_max_items(int kind) {
    switch (kind) {
        case ORIGAMI_U32: return (kSlots - 2) * (uint64_t)merge_tile<uint32_t>();
        case ORIGAMI_U64:
        case ORIGAMI_I64: return (kSlots - 2) * (uint64_t)merge_tile<uint64_t>();
        case ORIGAMI_KV64:
        case ORIGAMI_KVU64: return (kSlots - 2) * (uint64_t)merge_tile<KV64>();
        default: return 0;
    }
}

extern "C" int origami_sort_noalloc_device(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n,
                                           int flags, void** result, void* stream) {
    // the size limit first: it holds whatever the buffers are
    if (origami_noalloc_max_items(kind) > 0 && n > origami_noalloc_max_items(kind))
        return noalloc_fail(ORIGAMI_ERR_INVALID,
                            "n exceeds the no-alloc limit (origami_noalloc_max_items)");
    int rc = noalloc_check(kind, d, tmp, n, sort_n, result);
    if (rc != ORIGAMI_OK) return rc;
    if (n > 1 && !tmp) return noalloc_fail(ORIGAMI_ERR_INVALID, "the no-alloc sort needs a tmp buffer");
    if ((((uintptr_t)d) | ((uintptr_t)tmp)) & 15)
        return noalloc_fail(ORIGAMI_ERR_ALIGN, "the no-alloc sort needs 16-byte aligned device buffers");
    const bool in_tmp = (flags & ORIGAMI_FLAG_RESULT_IN_TMP) != 0;
    if (in_tmp && !tmp) return noalloc_fail(ORIGAMI_ERR_INVALID, "RESULT_IN_TMP needs a tmp buffer");
    *result = in_tmp ? tmp : d;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n <= 1) {
        cudaError_t e = cudaSuccess;
        if (n == 1 && in_tmp) e = cudaMemcpyAsync(tmp, d, origami_item_bytes(kind), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess && (flags & ORIGAMI_FLAG_SYNC)) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return noalloc_fail(ORIGAMI_ERR_CUDA, cudaGetErrorString(e));
        return ORIGAMI_OK;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return noalloc_fail(ORIGAMI_ERR_NO_DEVICE, "no usable CUDA device");
    int64_t* scratch = scratch_for(dev, &e);
    if (!scratch) return noalloc_fail(ORIGAMI_ERR_CUDA, cudaGetErrorString(e));
    if (scratch_needed(kind, n, sort_n) > sizeof(g_noalloc_scratch))  // defensive: implied by the limit above
        return noalloc_fail(ORIGAMI_ERR_INVALID, "n exceeds the no-alloc limit");
    const uint64_t m = (kind == ORIGAMI_I64 || kind == ORIGAMI_KV64) ? 0x8000000000000000ull : 0ull;
    void* want = in_tmp ? tmp : d;
    // binary merge passes only: their scratch is the splitter array
    switch (kind) {
        case ORIGAMI_U32: e = sort_u32(d, tmp, n, sort_n, m, want, 2, scratch, st, nullptr); break;
        case ORIGAMI_U64:
        case ORIGAMI_I64: e = sort_u64(d, tmp, n, sort_n, m, want, 2, scratch, st, nullptr); break;
        default: e = sort_kv(d, tmp, n, sort_n, m, want, 2, scratch, st, nullptr); break;
    }
    if (e != cudaSuccess) return noalloc_fail(ORIGAMI_ERR_CUDA, cudaGetErrorString(e));
    if (flags & ORIGAMI_FLAG_SYNC) {
        // the sort's error word opens the 256-byte tail of the scratch it
        // uses; the tile sort cleared it at the start of this call. The copy
        // goes to the stack (the driver stages it; nothing is allocated).
        int word = 0;
        e = cudaMemcpyAsync(&word, reinterpret_cast<const char*>(scratch) + scratch_needed(kind, n, sort_n) - 256,
                            sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return noalloc_fail(ORIGAMI_ERR_CUDA, cudaGetErrorString(e));
        if (err_word_timeout(word))
            return noalloc_fail(ORIGAMI_ERR_TIMEOUT, "a merge kernel's bulk-copy wait expired");
    }
    return ORIGAMI_OK;
}
