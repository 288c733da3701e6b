// C ABI (include/origami_gpu.h): argument validation, the pooled device arena,
// host-pointer staging and dispatch onto the typed pipelines.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/origami_gpu.h"
#include "dispatch.h"
#include "pipeline.cuh"
#include "profiler.h"

namespace origami {

// ---- launch accounting / profiling (profiler.h) ----
namespace {
std::atomic<uint64_t> g_launches{0};
std::atomic<bool> g_prof_on{false};
std::mutex g_prof_mu;
struct ProfRec {
    std::string name;
    cudaEvent_t a, b;
};
std::vector<ProfRec> g_recs;
std::vector<cudaEvent_t> g_event_pool;
std::map<std::string, uint64_t> g_prof_seen;  // launches per kernel since profiling was enabled
uint32_t g_prof_every = 1;                     // time every k-th launch of each kernel

cudaEvent_t take_event() {
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

namespace {
thread_local bool t_capturing = false;
}
// Launches recorded into a CUDA graph are not bracketed by events: the graph
// replays as one unit and is timed as one.
bool profiling_on() { return g_prof_on.load(std::memory_order_relaxed) && !t_capturing; }
void set_capturing(bool on) { t_capturing = on; }
uint64_t launches_so_far() { return g_launches.load(std::memory_order_relaxed); }
void count_launches(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int prof_begin(const char* name, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    uint64_t& seen = g_prof_seen[name];
    const bool timed = seen % g_prof_every == 0;
    ++seen;
    if (!timed) return -1;
    ProfRec r{name, take_event(), take_event()};
    cudaEventRecord(r.a, st);
    g_recs.push_back(r);
    return (int)g_recs.size() - 1;
}

void prof_end(int slot, cudaStream_t st) {
    if (slot < 0) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEventRecord(g_recs[slot].b, st);
}
std::atomic<uint32_t> g_wait_limit{BULK_SPIN_LIMIT};
uint32_t wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }

uint64_t scratch_bytes(int kind, uint64_t n, uint64_t sort_n, int fan) {
    switch (kind) {
        case ORIGAMI_U32: return scratch_bytes_u32(n, sort_n, fan);
        case ORIGAMI_U64:
        case ORIGAMI_I64: return scratch_bytes_u64(n, sort_n, fan);
        default: return scratch_bytes_kv(n, sort_n, fan);
    }
}
}  // namespace origami

using namespace origami;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(ORIGAMI_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return fail(ORIGAMI_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Device error words (bulk.cuh) of the sorts a call enqueues, copied into
// pinned host memory behind each sort; read once the stream has drained.
// Slots come from a per-thread pinned block in stack order, so a watch made
// inside another (a nested call) takes the slots after the outer one's.
constexpr int ERR_SLOTS = 256;
thread_local int* t_err_host = nullptr;
thread_local int t_err_top = 0;

struct ErrWatch {
    int base, top;
    ErrWatch() : base(t_err_top), top(t_err_top) {
        if (!t_err_host && cudaHostAlloc(&t_err_host, ERR_SLOTS * sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            t_err_host = nullptr;
        }
    }
    ~ErrWatch() { t_err_top = base; }
    ErrWatch(const ErrWatch&) = delete;
    ErrWatch& operator=(const ErrWatch&) = delete;
    // Enqueues the copy of the error word at dev_err (device memory) on st.
    cudaError_t watch(const void* dev_err, cudaStream_t st) {
        if (!t_err_host || top >= ERR_SLOTS) return cudaSuccess;  // no slot left: not watched
        int* h = t_err_host + top++;
        t_err_top = top;
        *h = 0;
        return cudaMemcpyAsync(h, dev_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    }
    // After the streams have drained: true when a watched sort timed out.
    bool timed_out() const {
        for (int i = base; i < top; ++i)
            if (t_err_host && err_word_timeout(t_err_host[i])) return true;
        return false;
    }
};

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

bool valid_kind(int kind) { return kind >= ORIGAMI_U32 && kind <= ORIGAMI_KVU64; }

unsigned item_bytes(int kind) {
    switch (kind) {
        case ORIGAMI_U32: return 4;
        case ORIGAMI_U64:
        case ORIGAMI_I64: return 8;
        default: return 16;
    }
}

uint64_t k1_tile_of(int kind) {
    switch (kind) {
        case ORIGAMI_U32: return tile_u32();
        case ORIGAMI_U64:
        case ORIGAMI_I64: return tile_u64();
        default: return tile_kv();
    }
}

uint64_t key_mask(int kind) {
    return (kind == ORIGAMI_I64 || kind == ORIGAMI_KV64) ? 0x8000000000000000ull : 0ull;
}

// The stream-ordered allocator's default pool is the device arena: freed blocks
// stay cached (release threshold = max) so repeated calls do not return memory
// to the driver.
std::once_flag g_pool_once;
int g_pool_status = ORIGAMI_OK;

int ensure_device() {
    std::call_once(g_pool_once, [] {
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
            cudaGetLastError();
            g_pool_status = ORIGAMI_ERR_NO_DEVICE;
            return;
        }
        int dev = 0;
        cudaGetDevice(&dev);
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    });
    if (g_pool_status != ORIGAMI_OK) return fail(g_pool_status, "no CUDA device available");
    return ORIGAMI_OK;
}

cudaStream_t worker_stream() {
    thread_local cudaStream_t s = nullptr;
    if (!s) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    return s;
}

bool is_device_pointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int check_args(int kind, const void* d, const void* tmp, uint64_t n, uint64_t sort_n, void** result) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    if (!result) return fail(ORIGAMI_ERR_INVALID, "result pointer is NULL");
    if (n > 0 && !d) return fail(ORIGAMI_ERR_INVALID, "d is NULL with n = %llu", (unsigned long long)n);
    const unsigned s = item_bytes(kind);
    const unsigned align = s > 8 ? 8 : s;
    if (((uintptr_t)d % align) || (tmp && ((uintptr_t)tmp % align)))
        return fail(ORIGAMI_ERR_ALIGN, "buffers must be %u-byte aligned", align);
    if (n > (1ull << 40)) return fail(ORIGAMI_ERR_INVALID, "n = %llu is too large", (unsigned long long)n);
    if (sort_n != 0 && sort_n < n && (sort_n & (sort_n - 1)) != 0)
        return fail(ORIGAMI_ERR_INVALID, "sort_n = %llu must be 0, >= n or a power of two",
                    (unsigned long long)sort_n);
    if (d && tmp && n > 0) {
        const char* a = (const char*)d;
        const char* b = (const char*)tmp;
        const uint64_t bytes = n * s;
        if (a < b + bytes && b < a + bytes) return fail(ORIGAMI_ERR_INVALID, "d and tmp overlap");
    }
    return ORIGAMI_OK;
}

// Merge fan-in for a min_k request: 2 keeps binary passes, 3..16 round up to
// a power of two, larger values are capped at 16.
int fan_of(unsigned min_k) {
    if (min_k <= 2) return 2;
    int f = 4;
    while ((unsigned)f < min_k && f < 16) f <<= 1;
    return f;
}

// ---- tuning table: pass shape per kind and size class (floor(log2 n)) ----
// Default: binary passes with the first tile shape (the measured best at
// 1 GiB). origami_autotune() times the candidates and stores the winner.
constexpr int TUNE_CLASSES = 41;
std::atomic<int> g_tune[5][TUNE_CLASSES];
std::once_flag g_tune_once;

int size_class(uint64_t n) {
    int c = 0;
    while (c + 1 < TUNE_CLASSES && (2ull << c) <= n) ++c;
    return c;
}

void tune_init();

// Pass shape code for a sort of n items: min_k = 0 takes the table's choice,
// min_k <= 2 binary passes with the table's tile shape, larger min_k k-way.
int shape_for(int kind, uint64_t n, unsigned min_k) {
    std::call_once(g_tune_once, tune_init);
    const int code = g_tune[kind][size_class(n)].load(std::memory_order_relaxed);
    if (min_k == 0) return code;
    if (min_k <= 2) return shape_code(2, shape_fan(code) == 2 ? shape_variant(code) : 0);
    return shape_code(fan_of(min_k), 0);
}

// Segmented sorts: the level merges' merge shape (0 / 1, SegMergeCfg) per
// kind and size class of the mean segment length. Default 0.
std::atomic<int> g_seg_tune[5][TUNE_CLASSES];

int seg_class(uint64_t n, uint64_t nseg) { return size_class(nseg ? n / nseg : n); }

int seg_shape_for(int kind, uint64_t n, uint64_t nseg) {
    std::call_once(g_tune_once, tune_init);
    return g_seg_tune[kind][seg_class(n, nseg)].load(std::memory_order_relaxed);
}

cudaError_t run_typed(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n, void* want,
                      int fan, void* scratch, cudaStream_t st) {
    const uint64_t m = key_mask(kind);
    switch (kind) {
        case ORIGAMI_U32: return sort_u32(d, tmp, n, sort_n, m, want, fan, scratch, st, nullptr);
        case ORIGAMI_U64:
        case ORIGAMI_I64: return sort_u64(d, tmp, n, sort_n, m, want, fan, scratch, st, nullptr);
        default: return sort_kv(d, tmp, n, sort_n, m, want, fan, scratch, st, nullptr);
    }
}

// Device-resident sort; the caller has validated the arguments. `watch`
// (optional) collects the sort's device error word; with ORIGAMI_FLAG_SYNC and
// no outer watch the call checks it itself and returns ORIGAMI_ERR_TIMEOUT
// when a bounded wait of a merge kernel expired.
int sort_device_impl(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                     int flags, void** result, cudaStream_t st, ErrWatch* watch = nullptr) {
    const bool in_tmp = (flags & ORIGAMI_FLAG_RESULT_IN_TMP) != 0;
    if (in_tmp && !tmp) return fail(ORIGAMI_ERR_INVALID, "RESULT_IN_TMP needs a tmp buffer");
    // device kernels move whole items with vector loads and cp.async
    const unsigned ib = item_bytes(kind);
    if (((uintptr_t)d % ib) || (tmp && ((uintptr_t)tmp % ib)))
        return fail(ORIGAMI_ERR_ALIGN, "device buffers must be %u-byte aligned", ib);
    *result = in_tmp ? tmp : d;
    if (n <= 1) {
        if (n == 1 && in_tmp)
            CK(cudaMemcpyAsync(tmp, d, item_bytes(kind), cudaMemcpyDeviceToDevice, st), "copy");
        if (flags & ORIGAMI_FLAG_SYNC) CK(cudaStreamSynchronize(st), "stream sync");
        return ORIGAMI_OK;
    }
    // the kernels move 16-byte vectors: caller buffers that are not 16-byte
    // aligned are sorted in aligned arena copies
    if ((((uintptr_t)d) | ((uintptr_t)tmp)) & 15) {
        const uint64_t bytes = n * item_bytes(kind);
        void* ad = nullptr;
        void* at = nullptr;
        CK(cudaMallocAsync(&ad, bytes, st), "aligned staging");
        cudaError_t e0 = cudaMallocAsync(&at, bytes, st);
        if (e0 != cudaSuccess) {
            cudaFreeAsync(ad, st);
            return cuda_fail(e0, "aligned staging");
        }
        void* r = nullptr;
        int rc = ORIGAMI_OK;
        ErrWatch local;
        ErrWatch* w = watch ? watch : &local;
        e0 = cudaMemcpyAsync(ad, d, bytes, cudaMemcpyDeviceToDevice, st);
        if (e0 == cudaSuccess) rc = sort_device_impl(kind, ad, at, n, sort_n, min_k, 0, &r, st, w);
        if (e0 == cudaSuccess && rc == ORIGAMI_OK)
            e0 = cudaMemcpyAsync(in_tmp ? tmp : d, r, bytes, cudaMemcpyDeviceToDevice, st);
        cudaFreeAsync(ad, st);
        cudaFreeAsync(at, st);
        if (rc != ORIGAMI_OK) return rc;
        if (e0 != cudaSuccess) return cuda_fail(e0, "aligned staging copy");
        if (flags & ORIGAMI_FLAG_SYNC) {
            CK(cudaStreamSynchronize(st), "stream sync");
            if (!watch && local.timed_out()) return fail(ORIGAMI_ERR_TIMEOUT, "a merge kernel's bulk-copy wait expired");
        }
        return ORIGAMI_OK;
    }
    void* scratch = nullptr;
    if (!tmp) CK(cudaMallocAsync(&scratch, n * item_bytes(kind), st), "scratch allocation");
    const int fan = shape_for(kind, n, min_k);
    void* work = nullptr;
    cudaError_t e = cudaMallocAsync(&work, scratch_bytes(kind, n, sort_n, fan), st);
    if (e != cudaSuccess) {
        if (scratch) cudaFreeAsync(scratch, st);
        return cuda_fail(e, "splitter allocation");
    }
    e = run_typed(kind, d, tmp ? tmp : scratch, n, sort_n, in_tmp ? tmp : d, fan, work, st);
    // the pipeline's error word: the last 256 bytes of its scratch
    ErrWatch local;
    ErrWatch* w = watch ? watch : ((flags & ORIGAMI_FLAG_SYNC) ? &local : nullptr);
    if (e == cudaSuccess && w)
        e = w->watch(static_cast<char*>(work) + scratch_bytes(kind, n, sort_n, fan) - 256, st);
    cudaFreeAsync(work, st);
    if (scratch) cudaFreeAsync(scratch, st);
    if (e != cudaSuccess) return cuda_fail(e, "sort launch");
    if (flags & ORIGAMI_FLAG_SYNC) {
        CK(cudaStreamSynchronize(st), "stream sync");
        if (!watch && local.timed_out()) return fail(ORIGAMI_ERR_TIMEOUT, "a merge kernel's bulk-copy wait expired");
    }
    return ORIGAMI_OK;
}

// Device view of a host buffer the GPU can address: the mapped pointer of
// pinned memory, or the pointer itself for pageable memory when the device
// reads it through the host's page tables (address translation services on
// Grace). nullptr when neither applies or ORIGAMI_HOST_DIRECT=0.
void* device_view(void* p) {
    static const bool enabled = [] {
        const char* e = std::getenv("ORIGAMI_HOST_DIRECT");
        return !(e && e[0] == '0');
    }();
    if (!enabled) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    if (a.type == cudaMemoryTypeUnregistered) {
        int dev = 0, pageable = 0, host_tables = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
        if (pageable && host_tables) return p;
    }
    return nullptr;
}

cudaError_t typed_io(int kind, const void* in, void* out, void* wa, void* wb, uint64_t n, uint64_t sort_n,
                     uint64_t xin, uint64_t xout, uint64_t start_run, int fan, void* scratch, cudaStream_t st) {
    switch (kind) {
        case ORIGAMI_U32: return sort_io_u32(in, out, wa, wb, n, sort_n, xin, xout, start_run, fan, scratch, st);
        case ORIGAMI_U64:
        case ORIGAMI_I64: return sort_io_u64(in, out, wa, wb, n, sort_n, xin, xout, start_run, fan, scratch, st);
        default: return sort_io_kv(in, out, wa, wb, n, sort_n, xin, xout, start_run, fan, scratch, st);
    }
}

uint64_t typed_scratch_io(int kind, uint64_t n, uint64_t sort_n, int fan, uint64_t start_run) {
    switch (kind) {
        case ORIGAMI_U32: return scratch_bytes_io_u32(n, sort_n, fan, start_run);
        case ORIGAMI_U64:
        case ORIGAMI_I64: return scratch_bytes_io_u64(n, sort_n, fan, start_run);
        default: return scratch_bytes_io_kv(n, sort_n, fan, start_run);
    }
}

// Per-thread helper streams of the host pipeline: 0 .. HOST_LANES-3 sort
// chunks beside the caller's stream, HOST_LANES-1 carries the copies. Six
// compute streams: the chunk sorts of a 1 GiB u32 call end 7.27 ms after the
// first copy starts with six, 7.40 with four, 7.51 with three, 7.97 with two,
// 7.28 with eight.
constexpr int HOST_LANES = 7;
static_assert(HOST_LANES - 1 >= 4, "the first chunk's four pieces sort on four lanes");
cudaStream_t aux_stream(int which) {
    thread_local cudaStream_t s[HOST_LANES] = {};
    if (!s[which]) cudaStreamCreateWithFlags(&s[which], cudaStreamNonBlocking);
    return s[which];
}

bool is_pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Host buffers the device can address (view pointers vin / vout).
//  * Small sorts, fan-in > 2, or chunk sizes of at most one chunk: one
//    pipeline whose first kernel reads the host input and whose last pass
//    writes the host output, with the passes in between in two arena buffers.
//  * Large sorts: the input is cut into chunks of chunk_n (a power of two of
//    at least 2^22 items; 4 to 16 chunks, more than 8 above 2^26 items). Each
//    chunk lands in HBM (a copy-engine transfer for pinned memory, a copy
//    kernel for pageable memory; device input stays where it is; the first
//    chunk in four pieces) and is sorted on one of six compute streams
//    while the next chunks are in flight; one k-way pass across the chunks
//    follows and writes the host output itself, or (the serving loop, pinned
//    output) is cut into output slices that go to the host by copies while
//    the next slices merge.
//    The host link carries each byte once each way, overlapped with the sorts.
cudaError_t typed_kway_final(int kind, const void* in, void* out, uint64_t n, uint64_t run, int fan, uint64_t xout,
                             void* scratch, cudaStream_t st, int slices, void (*cb)(void*, uint64_t, uint64_t),
                             void* ctx) {
    switch (kind) {
        case ORIGAMI_U32: return kway_final_u32(in, out, n, run, fan, xout, scratch, st, slices, cb, ctx);
        case ORIGAMI_U64:
        case ORIGAMI_I64: return kway_final_u64(in, out, n, run, fan, xout, scratch, st, slices, cb, ctx);
        default: return kway_final_kv(in, out, n, run, fan, xout, scratch, st, slices, cb, ctx);
    }
}

// Scratch bytes of kway_pass_sliced (the final pass of the chunked host pipeline).
uint64_t kway_final_bytes(int kind, uint64_t n);

// Byte offset of the error word in kway_pass_sliced's scratch.
uint64_t typed_kway_final_err(int kind, uint64_t n) {
    switch (kind) {
        case ORIGAMI_U32: return kway_final_err_u32(n);
        case ORIGAMI_U64:
        case ORIGAMI_I64: return kway_final_err_u64(n);
        default: return kway_final_err_kv(n);
    }
}

uint64_t kway_final_bytes(int kind, uint64_t n) { return typed_kway_final_err(kind, n) + 256; }

// Copies each finished slice of the final pass to the host on the copy stream.
struct SliceCopy {
    cudaStream_t st, sc;
    const char* dev;
    char* host;
    uint64_t ib;
    std::vector<cudaEvent_t>* evs;
    cudaError_t e;
    static void on(void* p, uint64_t o0, uint64_t o1) {
        auto* c = static_cast<SliceCopy*>(p);
        if (c->e != cudaSuccess || o1 <= o0) return;
        cudaEvent_t ev;
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        cudaEventRecord(ev, c->st);
        c->evs->push_back(ev);
        cudaStreamWaitEvent(c->sc, ev, 0);
        c->e = cudaMemcpyAsync(c->host + o0 * c->ib, c->dev + o0 * c->ib, (o1 - o0) * c->ib, cudaMemcpyDeviceToHost,
                               c->sc);
    }
};

}  // namespace

namespace origami {
// Moves `bytes` from host memory the device reads through the host's page
// tables (pageable memory on Grace) into HBM: 16-byte loads, four in flight
// per thread, grid-stride; the last bytes % 16 by the first threads. One CTA
// of 256 threads per SM keeps the host link busy (211 GB/s with mapped pinned
// memory from 152 CTAs on, the copy engines' rate) and leaves the SMs' other
// slots to the chunk sorts.
__global__ void __launch_bounds__(256) link_copy_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                        uint64_t nvec, const unsigned char* __restrict__ tsrc,
                                                        unsigned char* __restrict__ tdst, unsigned tail) {
    constexpr int U = 4;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * U;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x * U + threadIdx.x; i < nvec; i += stride) {
        uint4 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t j = i + (uint64_t)u * blockDim.x;
            if (j < nvec) v[u] = src[j];
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t j = i + (uint64_t)u * blockDim.x;
            if (j < nvec) dst[j] = v[u];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < tail) tdst[threadIdx.x] = tsrc[threadIdx.x];
}
}  // namespace origami

namespace {
using origami::link_copy_kernel;

cudaError_t link_copy(const void* src, void* dst, uint64_t bytes, cudaStream_t st) {
    static const unsigned grid = [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return (unsigned)(sms > 0 ? sms : 1);
    }();
    const uint64_t nvec = bytes / 16;
    const unsigned tail = (unsigned)(bytes % 16);
    launch("link_copy", st, [&] {
        link_copy_kernel<<<grid, 256, 0, st>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), nvec,
                                                static_cast<const unsigned char*>(src) + nvec * 16,
                                                static_cast<unsigned char*>(dst) + nvec * 16, tail);
    });
    return cudaGetLastError();
}

// The host pipeline's plan: whether it runs chunked, the pass shapes, and the
// device memory it takes from one block (each part 256-byte aligned).
struct HostPipePlan {
    bool chunked = false;
    // pinned output of a chunked sort: copies of finished output slices (the
    // SMs stay free for other work while the link drains them), or the final
    // pass writing the host buffer itself (ends sooner: 1 GiB u32 13.4 against
    // 13.75 ms per call, as the first bytes leave without waiting for the
    // slice boundaries and a first slice)
    bool slice_copies = false;
    uint64_t chunk_n = 0;
    int fan = 0, cfan = 0, mfan = 0;
    // host input: the first chunk lands in this many pieces, each sorted as
    // it lands, then merged into the chunk's run by one k-way pass
    int first_pieces = 1;
    uint64_t data = 0, ws = 0, wm = 0, total = 0;  // A and B (data each), lane scratch, merge scratch
};

uint64_t a256(uint64_t b) { return (b + 255) & ~255ull; }

HostPipePlan host_pipe_plan(int kind, uint64_t n, uint64_t sort_n, unsigned min_k) {
    HostPipePlan p;
    const uint64_t limit = (sort_n == 0 || sort_n >= n) ? n : sort_n;
    p.fan = shape_for(kind, n, min_k);
    p.chunk_n = 1ull << 22;
    // at most 16 chunks, so that one k-way pass of fan-in 16 merges them, and
    // more than 8 where the chunks are larger than the smallest size. The
    // chunk sorts are bound by the GPU's sorting throughput, not by the link:
    // the smaller the chunks, the earlier the first one arrives and the fewer
    // levels the chunk sorts merge before the final pass, whose levels hide
    // under its writes to the host (1 GiB u32 from pinned memory: 16 chunks
    // 13.74 ms per call, 8 chunks 14.09 ms; the last chunk sort ends 7.40
    // against 7.86 ms after the first copy starts)
    while (p.chunk_n * 16 < n) p.chunk_n <<= 1;
    p.chunked = n >= 4 * p.chunk_n && limit > p.chunk_n;
    p.data = a256(n * item_bytes(kind));
    if (!p.chunked) {
        p.ws = a256(typed_scratch_io(kind, n, sort_n, p.fan, 0));
        p.total = 2 * p.data + p.ws;
        return p;
    }
    // chunks sort on HOST_LANES-1 streams at once: by default with 16-way
    // passes (a 1 GiB u32 call from pinned memory: 14.03 ms per call, against
    // 14.35 with binary passes of the one-tile-per-CTA shape, whose launches
    // from the different streams interleave, 14.46 with the persistent binary
    // kernel and 14.27 with 8-way passes); min_k = 2 keeps binary passes of the
    // interleaving shape, larger min_k that fan-in
    p.cfan = min_k > 2 ? shape_code(fan_of(min_k), 0) : (min_k == 2 ? shape_code(2, 2) : shape_code(16, 0));
    // the GPU would wait for a whole first chunk before any sorting starts:
    // copied in four pieces it starts after a quarter (1 GiB u32 call from
    // pinned memory 13.33-13.40 -> 13.25-13.28 ms); needs chunk passes of
    // fan-in 4 or more, so that the pieces merge in one pass
    p.first_pieces = shape_fan(p.cfan) >= 4 ? 4 : 1;
    p.ws = a256(std::max(typed_scratch_io(kind, p.chunk_n, 0, p.cfan, 0),
                         typed_scratch_io(kind, p.chunk_n, 0, p.cfan, p.chunk_n / p.first_pieces)));
    // the merges across chunks are one k-way pass: bound by the host link it
    // writes (1 GiB in ~5.6 ms), which hides its cost per level
    const uint64_t need = (limit + p.chunk_n - 1) / p.chunk_n;
    p.mfan = 2;
    while ((uint64_t)p.mfan < need && p.mfan < 16) p.mfan <<= 1;
    p.wm = a256(std::max(typed_scratch_io(kind, n, sort_n, p.mfan, p.chunk_n), kway_final_bytes(kind, n)));
    p.total = 2 * p.data + (HOST_LANES - 1) * p.ws + p.wm;
    return p;
}

// Sorts n items from `host_in` into `host_out` (host memory the device can
// address through vin / vout, or device memory) with the memory of one block
// of plan.total bytes, on `st` and this thread's helper streams; returns when
// the result is in place. Large sorts are cut into chunks: each chunk lands
// in HBM (a copy-engine transfer for pinned memory, a copy kernel for
// pageable memory) and is sorted on one of six streams while the next chunks
// are in flight; the merge across chunks follows as one k-way pass that
// writes the host output (or, with plan.slice_copies and pinned output, is
// cut into output slices copied to the host while the next slices merge).
// Small sorts run one pipeline whose first kernel reads the input and whose
// last pass writes the output.
int host_pipe_run(int kind, void* host_in, void* host_out, const void* vin, void* vout, uint64_t n, uint64_t sort_n,
                  const HostPipePlan& p, void* block, cudaStream_t st) {
    const uint64_t ib = item_bytes(kind);
    const uint64_t m = key_mask(kind);
    const uint64_t limit = (sort_n == 0 || sort_n >= n) ? n : sort_n;
    char* blk = static_cast<char*>(block);
    char* a = blk;
    char* b = blk + p.data;
    ErrWatch watch;  // every sort's error word, read after the final sync
    cudaError_t e = cudaSuccess;
    std::vector<cudaEvent_t> evs;
    if (!p.chunked) {
        void* w = b + p.data;
        e = typed_io(kind, vin, vout, a, b, n, sort_n, m, m, 0, p.fan, w, st);
        if (e == cudaSuccess)
            e = watch.watch(static_cast<char*>(w) + typed_scratch_io(kind, n, sort_n, p.fan, 0) - 256, st);
    } else {
        const uint64_t chunk_n = p.chunk_n;
        char* w[HOST_LANES - 1];
        for (int i = 0; i < HOST_LANES - 1; ++i) w[i] = b + p.data + (uint64_t)i * p.ws;
        char* wm = b + p.data + (HOST_LANES - 1) * p.ws;
        // host chunks land in HBM before they sort: pinned memory by the copy
        // engines, pageable memory by link_copy_kernel. A chunk sort whose
        // first kernel read the host link itself held its SMs for the
        // transfer (1 GiB u32 from pageable memory: 16.3 ms per call). Device
        // input (a serving request) is sorted where it is.
        const bool pinned_in = is_pinned(host_in);
        const bool device_in = !pinned_in && is_device_pointer(host_in);
        const int np = device_in ? 1 : p.first_pieces;
        cudaStream_t lanes[HOST_LANES - 1] = {st};
        for (int i = 1; i < HOST_LANES - 1; ++i) lanes[i] = aux_stream(i - 1);
        cudaStream_t sc = aux_stream(HOST_LANES - 1);
        auto land = [&](char* dst, uint64_t off_items, uint64_t items) -> cudaError_t {
            if (pinned_in)
                return cudaMemcpyAsync(dst, static_cast<const char*>(host_in) + off_items * ib, items * ib,
                                       cudaMemcpyHostToDevice, sc);
            return link_copy(static_cast<const char*>(vin) + off_items * ib, dst, items * ib, sc);
        };
        auto event_on = [&](cudaStream_t s) {
            cudaEvent_t ev;
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            cudaEventRecord(ev, s);
            evs.push_back(ev);
            return ev;
        };
        const cudaEvent_t ready = event_on(st);  // the block's earlier users are done
        for (int i = 1; i < HOST_LANES - 1; ++i) cudaStreamWaitEvent(lanes[i], ready, 0);
        cudaStreamWaitEvent(sc, ready, 0);
        for (uint64_t off = 0, c = 0; e == cudaSuccess && off < n; off += chunk_n, ++c) {
            const uint64_t cn = n - off < chunk_n ? n - off : chunk_n;
            const int lane = (int)(c % (HOST_LANES - 1));
            cudaStream_t cst = lanes[lane];
            const void* src = static_cast<const char*>(vin) + off * ib;
            if (c == 0 && np > 1) {
                // piece q lands in A, is sorted into B on lane q; one pass of
                // fan-in np then merges B's runs into the chunk's run in A
                const uint64_t pn = chunk_n / np;
                for (int q = 0; q < np && e == cudaSuccess; ++q) {
                    char* pa = a + q * pn * ib;
                    char* pb = b + q * pn * ib;
                    e = land(pa, q * pn, pn);
                    cudaStreamWaitEvent(lanes[q], event_on(sc), 0);
                    if (e == cudaSuccess) e = typed_io(kind, pa, pb, pa, pb, pn, 0, m, 0, 0, p.cfan, w[q], lanes[q]);
                    if (e == cudaSuccess) e = watch.watch(w[q] + typed_scratch_io(kind, pn, 0, p.cfan, 0) - 256, lanes[q]);
                }
                for (int q = 1; q < np; ++q) cudaStreamWaitEvent(lanes[0], event_on(lanes[q]), 0);
                if (e == cudaSuccess) e = typed_io(kind, b, a, a, b, chunk_n, 0, 0, 0, pn, p.cfan, w[0], lanes[0]);
                if (e == cudaSuccess)
                    e = watch.watch(w[0] + typed_scratch_io(kind, chunk_n, 0, p.cfan, pn) - 256, lanes[0]);
                continue;
            }
            if (!device_in) {
                e = land(a + off * ib, off, cn);
                cudaStreamWaitEvent(cst, event_on(sc), 0);
                src = a + off * ib;
            }
            if (e == cudaSuccess)
                e = typed_io(kind, src, a + off * ib, b + off * ib, a + off * ib, cn, 0, m, 0, 0, p.cfan, w[lane],
                             cst);
            // the lane's next chunk sort clears the word again: read it now
            if (e == cudaSuccess)
                e = watch.watch(w[lane] + typed_scratch_io(kind, cn, 0, p.cfan, 0) - 256, cst);
        }
        if (e == cudaSuccess) {
            for (int i = 1; i < HOST_LANES - 1; ++i) cudaStreamWaitEvent(st, event_on(lanes[i]), 0);
            if (limit == n && p.slice_copies && is_pinned(host_out)) {
                // one k-way pass into HBM in 16 slices; each finished slice goes
                // to the host on the copy stream while the next ones merge (at
                // 1 GiB, 8 slices finish 0.1-0.2 ms later and 32 about 1 ms later)
                SliceCopy sc_ctx{st, sc, b, static_cast<char*>(host_out), ib, &evs, cudaSuccess};
                e = typed_kway_final(kind, a, b, n, chunk_n, p.mfan, m, wm, st, 16, &SliceCopy::on, &sc_ctx);
                if (e == cudaSuccess) e = sc_ctx.e;
                if (e == cudaSuccess) e = watch.watch(wm + typed_kway_final_err(kind, n), st);
                cudaStreamWaitEvent(st, event_on(sc), 0);  // the block is free after the copies
            } else {
                // merges from runs of chunk_n (one pass unless more than 16
                // chunks form a run); a pass must not write A while the first
                // one reads it; the last pass writes the output directly
                int passes = 0;
                for (uint64_t r = chunk_n; r < limit; r *= (uint64_t)p.mfan) ++passes;
                void* wa = ((passes - 1) & 1) ? (void*)b : (void*)a;
                void* wb = ((passes - 1) & 1) ? (void*)a : (void*)b;
                e = typed_io(kind, a, vout, wa, wb, n, sort_n, 0, m, chunk_n, p.mfan, wm, st);
                if (e == cudaSuccess)
                    e = watch.watch(wm + typed_scratch_io(kind, n, sort_n, p.mfan, chunk_n) - 256, st);
            }
        }
    }
    const cudaError_t es = cudaStreamSynchronize(st);
    for (cudaEvent_t ev : evs) cudaEventDestroy(ev);
    if (e != cudaSuccess) return cuda_fail(e, "host sort");
    if (es != cudaSuccess) return cuda_fail(es, "stream sync");
    if (watch.timed_out()) return fail(ORIGAMI_ERR_TIMEOUT, "a merge kernel's bulk-copy wait expired");
    return ORIGAMI_OK;
}

int sort_host_direct(int kind, void* host_in, void* host_out, const void* vin, void* vout, uint64_t n,
                     uint64_t sort_n, unsigned min_k, cudaStream_t st) {
    const HostPipePlan p = host_pipe_plan(kind, n, sort_n, min_k);
    void* block = nullptr;
    CK(cudaMallocAsync(&block, p.total, st), "arena allocation");
    const int rc = host_pipe_run(kind, host_in, host_out, vin, vout, n, sort_n, p, block, st);
    cudaFreeAsync(block, st);
    return rc;
}

// Tuning file: one entry per line. "kind class fan variant": the plain sort's
// pass shape for a size class; "seg kind class shape": the segmented sort's
// merge shape for a class of mean segment length. Other lines are skipped.
int tune_load_file(const char* path) {
    FILE* f = std::fopen(path, "r");
    if (!f) return fail(ORIGAMI_ERR_INVALID, "cannot open tuning file %s", path);
    char line[256];
    int kind, cls, fan, var, loaded = 0;
    while (std::fgets(line, sizeof line, f)) {
        if (std::sscanf(line, "seg %d %d %d", &kind, &cls, &var) == 3) {
            if (kind < 0 || kind > 4 || cls < 0 || cls >= TUNE_CLASSES || (var != 0 && var != 1)) continue;
            g_seg_tune[kind][cls].store(var, std::memory_order_relaxed);
            ++loaded;
            continue;
        }
        if (std::sscanf(line, "%d %d %d %d", &kind, &cls, &fan, &var) != 4) continue;
        if (kind < 0 || kind > 4 || cls < 0 || cls >= TUNE_CLASSES) continue;
        if (fan != 2 && fan != 4 && fan != 8 && fan != 16) continue;
        if (var < 0 || var > 3 || (fan != 2 && var != 0)) continue;
        g_tune[kind][cls].store(shape_code(fan, var), std::memory_order_relaxed);
        ++loaded;
    }
    std::fclose(f);
    return loaded;
}

// Built-in pass shapes: the autotuner's choice on one GB300 (two sweeps, the
// same winner in both, ahead of binary passes with the first tile shape by at
// least 1.5 %), for size classes floor(log2 n). Every other class keeps binary
// passes with the first tile shape. Signed kinds share their unsigned kind's
// kernels and entries. The sampled 16-way pass wins where the data is about
// the size of L2 (u32 2^25 keys: 1.00 against 1.02 ms; key-value 2^23 pairs:
// 0.91 against 0.95 ms).
struct TuneDefault {
    int kind, cls, fan, variant;
};
constexpr TuneDefault kTuneDefaults[] = {
    {ORIGAMI_U32, 18, 16, 0},  {ORIGAMI_U32, 19, 2, 3},   {ORIGAMI_U32, 20, 2, 3},   {ORIGAMI_U32, 21, 16, 0},
    {ORIGAMI_U32, 22, 2, 3},   {ORIGAMI_U32, 23, 2, 2},   {ORIGAMI_U32, 25, 16, 0},  {ORIGAMI_U64, 17, 16, 0},
    {ORIGAMI_U64, 18, 2, 3},   {ORIGAMI_U64, 19, 2, 3},   {ORIGAMI_U64, 20, 16, 0},  {ORIGAMI_U64, 21, 2, 2},
    {ORIGAMI_U64, 22, 2, 2},   {ORIGAMI_U64, 23, 2, 1},   {ORIGAMI_KV64, 17, 2, 3},  {ORIGAMI_KV64, 19, 16, 0},
    {ORIGAMI_KV64, 20, 16, 0}, {ORIGAMI_KV64, 22, 16, 0}, {ORIGAMI_KV64, 23, 16, 0}, {ORIGAMI_KV64, 24, 2, 1},
    {ORIGAMI_KV64, 25, 2, 1},  {ORIGAMI_KV64, 26, 2, 1},   {ORIGAMI_KV64, 27, 2, 1},   {ORIGAMI_KV64, 28, 2, 1},
};

void tune_init() {
    for (auto& row : g_tune)
        for (auto& c : row) c.store(shape_code(2, 0), std::memory_order_relaxed);
    for (const TuneDefault& t : kTuneDefaults) {
        g_tune[t.kind][t.cls].store(shape_code(t.fan, t.variant), std::memory_order_relaxed);
        const int twin = t.kind == ORIGAMI_U64 ? ORIGAMI_I64 : (t.kind == ORIGAMI_KV64 ? ORIGAMI_KVU64 : -1);
        if (twin >= 0) g_tune[twin][t.cls].store(shape_code(t.fan, t.variant), std::memory_order_relaxed);
    }
    for (auto& row : g_seg_tune)
        for (auto& c : row) c.store(0, std::memory_order_relaxed);
    if (const char* path = std::getenv("ORIGAMI_TUNING")) tune_load_file(path);
}

// Host buffers: stage through the arena, sort on the device, copy the result
// back into d (or tmp) and return when it is there.
int sort_host_impl(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                   int flags, void** result) {
    const bool in_tmp = (flags & ORIGAMI_FLAG_RESULT_IN_TMP) != 0;
    if (in_tmp && !tmp) return fail(ORIGAMI_ERR_INVALID, "RESULT_IN_TMP needs a tmp buffer");
    void* out = in_tmp ? tmp : d;
    *result = out;
    if (n == 0) return ORIGAMI_OK;
    const uint64_t bytes = n * item_bytes(kind);
    cudaStream_t st = worker_stream();
    if (n > 1) {
        void* vin = device_view(d);
        void* vout = vin ? device_view(out) : nullptr;
        if (vin && vout && !((((uintptr_t)vin) | ((uintptr_t)vout)) & 15))
            return sort_host_direct(kind, d, out, vin, vout, n, sort_n, min_k, st);
    }
    void* dd = nullptr;
    void* dt = nullptr;
    CK(cudaMallocAsync(&dd, bytes, st), "arena allocation");
    cudaError_t e = cudaMallocAsync(&dt, bytes, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(dd, st);
        return cuda_fail(e, "arena allocation");
    }
    int rc = ORIGAMI_OK;
    void* dres = nullptr;
    ErrWatch watch;
    e = cudaMemcpyAsync(dd, d, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        rc = sort_device_impl(kind, dd, dt, n, sort_n, min_k, 0, &dres, st, &watch);
        if (rc == ORIGAMI_OK) e = cudaMemcpyAsync(out, dres, bytes, cudaMemcpyDeviceToHost, st);
    }
    cudaFreeAsync(dd, st);
    cudaFreeAsync(dt, st);
    cudaError_t es = cudaStreamSynchronize(st);
    if (rc != ORIGAMI_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "host staging copy");
    if (es != cudaSuccess) return cuda_fail(es, "stream sync");
    if (watch.timed_out()) return fail(ORIGAMI_ERR_TIMEOUT, "a merge kernel's bulk-copy wait expired");
    return ORIGAMI_OK;
}

}  // namespace

namespace origami {
// The serving loop's large requests: the pipelined host sort with binary
// passes of the interleaving shape for the chunks (min_k = 2), because the
// loop's other batches run beside it; persistent 16-way chunk sorts hold
// every SM while they run (400 requests/s: p50 0.35 -> 3.6 ms, p99 14 -> 108 ms).
uint64_t host_pipe_bytes(int kind, uint64_t n) { return host_pipe_plan(kind, n, 0, 2).total; }

int host_pipe_sort(int kind, const void* in, void* out, uint64_t n, void* block, cudaStream_t st) {
    auto view = [](const void* p) -> void* {
        if (is_device_pointer(p)) return const_cast<void*>(p);
        return device_view(const_cast<void*>(p));
    };
    void* vin = view(in);
    void* vout = view(out);
    if (!vin || !vout || ((((uintptr_t)vin) | ((uintptr_t)vout)) & 15))
        return fail(ORIGAMI_ERR_INVALID, "buffers the device cannot address directly");
    HostPipePlan p = host_pipe_plan(kind, n, 0, 2);
    p.slice_copies = true;  // the loop's other batches run beside this one
    return host_pipe_run(kind, const_cast<void*>(in), out, vin, vout, n, 0, p, block, st);
}

int noalloc_fail(int code, const char* msg) { return fail(code, "%s", msg); }
int noalloc_check(int kind, const void* d, const void* tmp, uint64_t n, uint64_t sort_n,
                  void** result) {
    return check_args(kind, d, tmp, n, sort_n, result);
}
int api_fail(int code, const char* msg) { return fail(code, "%s", msg); }
int arena_init() { return ensure_device(); }

SegPlan seg_plan(int kind, uint64_t n, uint64_t nseg) {
    SegPlan p{};
    p.shape = seg_shape_for(kind, n, nseg);
    switch (kind) {
        case ORIGAMI_U32:
            p.maxl = seg_levels_u32(n);
            p.scratch_bytes = seg_scratch_bytes_u32(n, nseg, p.maxl);
            p.err_offset = seg_err_offset_u32(n, nseg, p.maxl);
            break;
        case ORIGAMI_U64:
        case ORIGAMI_I64:
            p.maxl = seg_levels_u64(n);
            p.scratch_bytes = seg_scratch_bytes_u64(n, nseg, p.maxl);
            p.err_offset = seg_err_offset_u64(n, nseg, p.maxl);
            break;
        default:
            p.maxl = seg_levels_kv(n);
            p.scratch_bytes = seg_scratch_bytes_kv(n, nseg, p.maxl);
            p.err_offset = seg_err_offset_kv(n, nseg, p.maxl);
            break;
    }
    return p;
}

void seg_prepare(int kind) {
    switch (kind) {
        case ORIGAMI_U32: seg_prepare_u32(); break;
        case ORIGAMI_U64:
        case ORIGAMI_I64: seg_prepare_u64(); break;
        default: seg_prepare_kv(); break;
    }
}

cudaError_t seg_launch(int kind, void* d, void* tmp, const uint64_t* off, uint64_t nseg, uint64_t n,
                       void* scratch, const SegPlan& p, cudaStream_t st) {
    const uint64_t m = key_mask(kind);
    switch (kind) {
        case ORIGAMI_U32: return seg_sort_u32(d, tmp, off, nseg, n, m, scratch, p.maxl, p.shape, st);
        case ORIGAMI_U64:
        case ORIGAMI_I64: return seg_sort_u64(d, tmp, off, nseg, n, m, scratch, p.maxl, p.shape, st);
        default: return seg_sort_kv(d, tmp, off, nseg, n, m, scratch, p.maxl, p.shape, st);
    }
}
}  // namespace origami

extern "C" {

int origami_version(void) { return ORIGAMI_GPU_VERSION; }

const char* origami_last_error(void) { return g_last_error.c_str(); }

unsigned origami_item_bytes(int kind) { return valid_kind(kind) ? item_bytes(kind) : 0; }

int origami_sort_device(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                        int flags, void** result, void* stream) {
    int rc = check_args(kind, d, tmp, n, sort_n, result);
    if (rc != ORIGAMI_OK) return rc;
    if ((rc = ensure_device()) != ORIGAMI_OK) return rc;
    return sort_device_impl(kind, d, tmp, n, sort_n, min_k, flags, result, (cudaStream_t)stream);
}

int origami_sort(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                 int flags, void** result) {
    int rc = check_args(kind, d, tmp, n, sort_n, result);
    if (rc != ORIGAMI_OK) return rc;
    if ((rc = ensure_device()) != ORIGAMI_OK) return rc;
    if (n > 0 && is_device_pointer(d)) {
        if (tmp && !is_device_pointer(tmp))
            return fail(ORIGAMI_ERR_INVALID, "d is device memory but tmp is not");
        return sort_device_impl(kind, d, tmp, n, sort_n, min_k, flags | ORIGAMI_FLAG_SYNC, result, 0);
    }
    return sort_host_impl(kind, d, tmp, n, sort_n, min_k, flags, result);
}

#define ORIGAMI_TYPED(name, KIND)                                                                  \
    int origami_sort_##name(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,      \
                            int flags, void** result) {                                            \
        return origami_sort(KIND, d, tmp, n, sort_n, min_k, flags, result);                        \
    }                                                                                              \
    int origami_sort_##name##_device(void* d, void* tmp, uint64_t n, uint64_t sort_n,             \
                                     unsigned min_k, int flags, void** result, void* stream) {     \
        return origami_sort_device(KIND, d, tmp, n, sort_n, min_k, flags, result, stream);         \
    }
ORIGAMI_TYPED(u32, ORIGAMI_U32)
ORIGAMI_TYPED(u64, ORIGAMI_U64)
ORIGAMI_TYPED(i64, ORIGAMI_I64)
ORIGAMI_TYPED(kv64, ORIGAMI_KV64)
ORIGAMI_TYPED(kvu64, ORIGAMI_KVU64)

int origami_merge_series_device(int kind, void* src, void* dst, uint64_t n, uint64_t merge_start,
                                uint64_t sort_n, void** result, void* stream) {
    int rc = check_args(kind, src, dst, n, sort_n, result);
    if (rc != ORIGAMI_OK) return rc;
    if (!dst && n > 0) return fail(ORIGAMI_ERR_INVALID, "dst is NULL");
    if (merge_start == 0 || (merge_start & (merge_start - 1)) || sort_n == 0 ||
        (sort_n & (sort_n - 1)) || merge_start > sort_n)
        return fail(ORIGAMI_ERR_INVALID, "merge_start and sort_n must be powers of two, merge_start <= sort_n");
    if ((rc = ensure_device()) != ORIGAMI_OK) return rc;
    // merger.h:4220-4228 swaps src/dst once per level and returns src: the
    // output is in src after an even number of levels, in dst after an odd one.
    int levels = 0;
    for (uint64_t r = merge_start; r < sort_n; r <<= 1) ++levels;
    const int flags = (levels & 1) ? ORIGAMI_FLAG_RESULT_IN_TMP : 0;
    // Merging sorted runs stably up to sort_n gives exactly the stable chunk
    // sort of the input, which is what the pipeline computes.
    return sort_device_impl(kind, src, dst, n, sort_n, 2, flags, result, (cudaStream_t)stream);
}

// ------------------------------------------------------------ segmented --
int origami_sort_segmented_device(int kind, void* d, void* tmp, const uint64_t* offsets,
                                  uint64_t nseg, uint64_t n, int flags, void* stream) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    if (nseg == 0 || n == 0) return ORIGAMI_OK;
    if (!d || !tmp || !offsets) return fail(ORIGAMI_ERR_INVALID, "d, tmp and offsets are required");
    if (nseg >= (1ull << 32) - 1) return fail(ORIGAMI_ERR_INVALID, "too many segments");
    if (n > (1ull << 40)) return fail(ORIGAMI_ERR_INVALID, "n is too large");
    if ((((uintptr_t)d) | ((uintptr_t)tmp)) & 15)
        return fail(ORIGAMI_ERR_ALIGN, "segmented sort needs 16-byte aligned device buffers");
    int rc = ensure_device();
    if (rc != ORIGAMI_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const SegPlan plan = seg_plan(kind, n, nseg);
    void* scratch = nullptr;
    CK(cudaMallocAsync(&scratch, plan.scratch_bytes, st), "segmented scratch");
    cudaError_t e = seg_launch(kind, d, tmp, offsets, nseg, n, scratch, plan, st);
    int herr = 0;
    if (e == cudaSuccess && (flags & ORIGAMI_FLAG_SYNC)) {
        e = cudaMemcpyAsync(&herr, static_cast<char*>(scratch) + plan.err_offset, sizeof(int),
                            cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFreeAsync(scratch, st);
    if (e != cudaSuccess) return cuda_fail(e, "segmented sort");
    if (err_word_timeout(herr)) return fail(ORIGAMI_ERR_TIMEOUT, "a merge job waited past its budget");
    if (herr == 2) return fail(ORIGAMI_ERR_INVALID, "segment offsets decrease");
    return ORIGAMI_OK;
}

int origami_sort_segmented(int kind, void* d, const uint64_t* offsets, uint64_t nseg, int flags) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    if (nseg == 0) return ORIGAMI_OK;
    if (!offsets) return fail(ORIGAMI_ERR_INVALID, "offsets is NULL");
    const uint64_t n = offsets[nseg];
    if (offsets[0] != 0) return fail(ORIGAMI_ERR_INVALID, "offsets[0] must be 0");
    for (uint64_t s = 0; s < nseg; ++s)
        if (offsets[s + 1] < offsets[s]) return fail(ORIGAMI_ERR_INVALID, "segment offsets decrease");
    if (n == 0) return ORIGAMI_OK;
    if (!d) return fail(ORIGAMI_ERR_INVALID, "d is NULL");
    int rc = ensure_device();
    if (rc != ORIGAMI_OK) return rc;
    (void)flags;
    const uint64_t bytes = n * item_bytes(kind);
    cudaStream_t st = worker_stream();
    void *dd = nullptr, *dt = nullptr, *doff = nullptr;
    CK(cudaMallocAsync(&dd, bytes, st), "arena allocation");
    cudaError_t e = cudaMallocAsync(&dt, bytes, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&doff, (nseg + 1) * sizeof(uint64_t), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dd, d, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(doff, offsets, (nseg + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        rc = origami_sort_segmented_device(kind, dd, dt, static_cast<const uint64_t*>(doff), nseg, n,
                                           ORIGAMI_FLAG_SYNC, st);
        if (rc == ORIGAMI_OK) e = cudaMemcpyAsync(d, dd, bytes, cudaMemcpyDeviceToHost, st);
    }
    if (dd) cudaFreeAsync(dd, st);
    if (dt) cudaFreeAsync(dt, st);
    if (doff) cudaFreeAsync(doff, st);
    cudaError_t es = cudaStreamSynchronize(st);
    if (rc != ORIGAMI_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "segmented sort staging");
    if (es != cudaSuccess) return cuda_fail(es, "stream sync");
    return ORIGAMI_OK;
}

int origami_arena_reserve(uint64_t bytes) {
    int rc = ensure_device();
    if (rc != ORIGAMI_OK) return rc;
    void* p = nullptr;
    cudaStream_t st = worker_stream();
    CK(cudaMallocAsync(&p, bytes, st), "arena reserve");
    CK(cudaFreeAsync(p, st), "arena reserve");
    CK(cudaStreamSynchronize(st), "arena reserve");
    return ORIGAMI_OK;
}

int origami_arena_trim(void) {
    int rc = ensure_device();
    if (rc != ORIGAMI_OK) return rc;
    int dev = 0;
    cudaMemPool_t pool;
    CK(cudaGetDevice(&dev), "arena trim");
    CK(cudaDeviceGetDefaultMemPool(&pool, dev), "arena trim");
    CK(cudaDeviceSynchronize(), "arena trim");
    CK(cudaMemPoolTrimTo(pool, 0), "arena trim");
    return ORIGAMI_OK;
}

uint64_t origami_arena_bytes_in_use(void) {
    if (ensure_device() != ORIGAMI_OK) return 0;
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess)
        return 0;
    uint64_t v = 0;
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &v);
    return v;
}

int origami_profile_enable(int on) {
    if (on < 0) return fail(ORIGAMI_ERR_INVALID, "profile_enable: negative argument");
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto& r : g_recs) {
        g_event_pool.push_back(r.a);
        g_event_pool.push_back(r.b);
    }
    g_recs.clear();
    g_prof_seen.clear();
    g_prof_every = on > 1 ? (uint32_t)on : 1u;
    g_prof_on.store(on != 0);
    return ORIGAMI_OK;
}

int origami_profile_report(char* buf, uint64_t cap) {
    if (!buf || cap == 0) return fail(ORIGAMI_ERR_INVALID, "report buffer is NULL");
    std::lock_guard<std::mutex> lk(g_prof_mu);
    std::map<std::string, std::pair<uint64_t, double>> agg;  // timed launches, their total ms
    for (auto& r : g_recs) {
        CK(cudaEventSynchronize(r.b), "profile sync");
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, r.a, r.b), "profile elapsed");
        auto& e = agg[r.name];
        e.first += 1;
        e.second += ms;
    }
    std::string out;
    char line[256];
    for (auto& kv : g_prof_seen) {
        const auto it = agg.find(kv.first);
        const uint64_t timed = it == agg.end() ? 0 : it->second.first;
        const double ms = it == agg.end() ? 0.0 : it->second.second;
        snprintf(line, sizeof line, "%s,%llu,%.6f,%llu\n", kv.first.c_str(), (unsigned long long)kv.second, ms,
                 (unsigned long long)timed);
        out += line;
    }
    if (out.size() + 1 > cap) return fail(ORIGAMI_ERR_INVALID, "report buffer too small");
    memcpy(buf, out.c_str(), out.size() + 1);
    return (int)out.size();
}

uint64_t origami_launch_count(void) { return g_launches.load(); }

uint32_t origami_get_wait_limit(void) { return wait_limit(); }

int origami_set_wait_limit(uint32_t polls) {
    g_wait_limit.store(polls, std::memory_order_relaxed);
    return ORIGAMI_OK;
}

// ------------------------------------------------------------- tuning --
int origami_tuning_get(int kind, uint64_t n, int* fan, int* variant) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    const int code = shape_for(kind, n, 0);
    if (fan) *fan = shape_fan(code);
    if (variant) *variant = shape_variant(code);
    return ORIGAMI_OK;
}

int origami_tuning_set(int kind, uint64_t n, int fan, int variant) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    if (fan != 2 && fan != 4 && fan != 8 && fan != 16) return fail(ORIGAMI_ERR_INVALID, "fan must be 2, 4, 8 or 16");
    if (variant < 0 || variant > 3 || (fan != 2 && variant != 0))
        return fail(ORIGAMI_ERR_INVALID, "variant must be 0 to 3 (1 to 3 only with fan 2)");
    std::call_once(g_tune_once, tune_init);
    g_tune[kind][size_class(n)].store(shape_code(fan, variant), std::memory_order_relaxed);
    return ORIGAMI_OK;
}

int origami_tuning_save(const char* path) {
    if (!path) return fail(ORIGAMI_ERR_INVALID, "path is NULL");
    std::call_once(g_tune_once, tune_init);
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(ORIGAMI_ERR_INVALID, "cannot write tuning file %s", path);
    for (int k = 0; k < 5; ++k)
        for (int c = 0; c < TUNE_CLASSES; ++c) {
            const int code = g_tune[k][c].load(std::memory_order_relaxed);
            if (code != shape_code(2, 0)) std::fprintf(f, "%d %d %d %d\n", k, c, shape_fan(code), shape_variant(code));
        }
    for (int k = 0; k < 5; ++k)
        for (int c = 0; c < TUNE_CLASSES; ++c) {
            const int shape = g_seg_tune[k][c].load(std::memory_order_relaxed);
            if (shape != 0) std::fprintf(f, "seg %d %d %d\n", k, c, shape);
        }
    std::fclose(f);
    return ORIGAMI_OK;
}

int origami_tuning_load(const char* path) {
    if (!path) return fail(ORIGAMI_ERR_INVALID, "path is NULL");
    std::call_once(g_tune_once, tune_init);
    const int r = tune_load_file(path);
    return r < 0 ? r : ORIGAMI_OK;
}

// Times every pass shape on n uniform device items of `kind` (binary passes
// with either tile shape, k-way passes with fan-in 4, 8, 16; each the best of
// three sorts after a warm-up) and stores the fastest for n's size class.
int origami_autotune(int kind, uint64_t n, char* report, uint64_t cap) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    if (n < 2) return fail(ORIGAMI_ERR_INVALID, "autotune needs at least 2 items");
    int rc = ensure_device();
    if (rc != ORIGAMI_OK) return rc;
    std::call_once(g_tune_once, tune_init);
    const uint64_t bytes = n * item_bytes(kind);
    cudaStream_t st = worker_stream();
    void *p = nullptr, *d = nullptr, *t = nullptr, *work = nullptr;
    CK(cudaMallocAsync(&p, bytes, st), "autotune buffers");
    cudaError_t e = cudaMallocAsync(&d, bytes, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&t, bytes, st);
    const int codes[] = {shape_code(2, 0), shape_code(2, 1), shape_code(2, 2), shape_code(2, 3),
                         shape_code(4, 0), shape_code(8, 0), shape_code(16, 0)};
    uint64_t wbytes = 0;
    for (int c : codes) wbytes = std::max<uint64_t>(wbytes, scratch_bytes(kind, n, 0, c));
    if (e == cudaSuccess) e = cudaMallocAsync(&work, wbytes, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && origami_generate_device(kind, p, n, 1, 2024, st) != ORIGAMI_OK) e = cudaErrorUnknown;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    std::string rep;
    int best = codes[0];
    float best_ms = 1e30f;
    for (int c : codes) {
        if (e != cudaSuccess) break;
        if (shape_fan(c) > 2 && (n + k1_tile_of(kind) - 1) / k1_tile_of(kind) <= 2) continue;  // one level
        float ms_best = 1e30f;
        for (int it = 0; it < 4 && e == cudaSuccess; ++it) {
            e = cudaMemcpyAsync(d, p, bytes, cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess) e = cudaEventRecord(a, st);
            if (e == cudaSuccess) e = run_typed(kind, d, t, n, 0, d, c, work, st);
            if (e == cudaSuccess) e = cudaEventRecord(b, st);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            float ms = 0;
            if (e == cudaSuccess && it > 0 && cudaEventElapsedTime(&ms, a, b) == cudaSuccess) ms_best = std::min(ms_best, ms);
        }
        char line[128];
        std::snprintf(line, sizeof line, "fan=%d variant=%d ms=%.4f\n", shape_fan(c), shape_variant(c), ms_best);
        rep += line;
        if (ms_best < best_ms) {
            best_ms = ms_best;
            best = c;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (work) cudaFreeAsync(work, st);
    if (t) cudaFreeAsync(t, st);
    if (d) cudaFreeAsync(d, st);
    cudaFreeAsync(p, st);
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "autotune");
    if (es != cudaSuccess) return cuda_fail(es, "autotune");
    g_tune[kind][size_class(n)].store(best, std::memory_order_relaxed);
    char line[128];
    std::snprintf(line, sizeof line, "chosen fan=%d variant=%d size_class=%d\n", shape_fan(best), shape_variant(best),
                  size_class(n));
    rep += line;
    if (report && cap) {
        std::strncpy(report, rep.c_str(), cap - 1);
        report[cap - 1] = 0;
    }
    return ORIGAMI_OK;
}


// ---------------------------------------------------- segmented tuning --
int origami_seg_tuning_get(int kind, uint64_t n, uint64_t nseg, int* shape) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    if (!shape) return fail(ORIGAMI_ERR_INVALID, "shape is NULL");
    *shape = seg_shape_for(kind, n, nseg);
    return ORIGAMI_OK;
}

int origami_seg_tuning_set(int kind, uint64_t n, uint64_t nseg, int shape) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    if (shape != 0 && shape != 1) return fail(ORIGAMI_ERR_INVALID, "shape must be 0 or 1");
    std::call_once(g_tune_once, tune_init);
    g_seg_tune[kind][seg_class(n, nseg)].store(shape, std::memory_order_relaxed);
    return ORIGAMI_OK;
}

// Times both merge shapes of the segmented sort on the caller's own segments
// (device buffers; d is restored to its input after every run) and stores the
// faster for their mean segment length. Best of three after a warm-up each.
int origami_autotune_segmented(int kind, void* d, void* tmp, const uint64_t* offsets, uint64_t nseg, uint64_t n,
                               char* report, uint64_t cap) {
    if (!valid_kind(kind)) return fail(ORIGAMI_ERR_DTYPE, "unknown item kind %d", kind);
    if (nseg == 0 || n == 0) return fail(ORIGAMI_ERR_INVALID, "autotune needs segments");
    if (!d || !tmp || !offsets) return fail(ORIGAMI_ERR_INVALID, "d, tmp and offsets are required");
    if ((((uintptr_t)d) | ((uintptr_t)tmp)) & 15)
        return fail(ORIGAMI_ERR_ALIGN, "segmented sort needs 16-byte aligned device buffers");
    int rc = ensure_device();
    if (rc != ORIGAMI_OK) return rc;
    std::call_once(g_tune_once, tune_init);
    const uint64_t bytes = n * item_bytes(kind);
    cudaStream_t st = worker_stream();
    SegPlan plan = seg_plan(kind, n, nseg);
    void *keep = nullptr, *scratch = nullptr;
    CK(cudaMallocAsync(&keep, bytes, st), "autotune buffers");
    cudaError_t e = cudaMallocAsync(&scratch, plan.scratch_bytes, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(keep, d, bytes, cudaMemcpyDeviceToDevice, st);
    cudaEvent_t a = nullptr, b = nullptr;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    std::string rep;
    int best = 0;
    float best_ms = 1e30f;
    for (int shape = 0; shape < 2 && e == cudaSuccess; ++shape) {
        plan.shape = shape;
        float ms_best = 1e30f;
        for (int it = 0; it < 4 && e == cudaSuccess; ++it) {
            e = cudaMemcpyAsync(d, keep, bytes, cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess) e = cudaEventRecord(a, st);
            if (e == cudaSuccess) e = seg_launch(kind, d, tmp, offsets, nseg, n, scratch, plan, st);
            if (e == cudaSuccess) e = cudaEventRecord(b, st);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            float ms = 0;
            if (e == cudaSuccess && it > 0 && cudaEventElapsedTime(&ms, a, b) == cudaSuccess)
                ms_best = std::min(ms_best, ms);
        }
        char line[128];
        std::snprintf(line, sizeof line, "shape=%d ms=%.4f\n", shape, ms_best);
        rep += line;
        if (ms_best < best_ms) {
            best_ms = ms_best;
            best = shape;
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, keep, bytes, cudaMemcpyDeviceToDevice, st);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (scratch) cudaFreeAsync(scratch, st);
    cudaFreeAsync(keep, st);
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "segmented autotune");
    if (es != cudaSuccess) return cuda_fail(es, "segmented autotune");
    g_seg_tune[kind][seg_class(n, nseg)].store(best, std::memory_order_relaxed);
    char line[128];
    std::snprintf(line, sizeof line, "chosen shape=%d mean_len_class=%d\n", best, seg_class(n, nseg));
    rep += line;
    if (report && cap) {
        std::strncpy(report, rep.c_str(), cap - 1);
        report[cap - 1] = 0;
    }
    return ORIGAMI_OK;
}

}  // extern "C"
