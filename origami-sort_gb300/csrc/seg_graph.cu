// Segmented-sort plans: the launch sequence of one batched segmented sort over
// fixed buffers, recorded once into a CUDA graph and replayed per call.
//
// A plan owns its scratch (allocated once at creation), so a replay makes no
// allocation and issues one graph launch instead of the memset and the
// 4 + 2 x levels kernel launches of the plain call. This is the form for a
// caller that sorts the same set of segment buffers repeatedly (a batch slot
// refilled between calls).
#include <mutex>

#include "../../include/origami_gpu.h"
#include "dispatch.h"
#include "profiler.h"

struct origami_seg_plan {
    int kind = 0;
    uint64_t n = 0, nseg = 0;
    origami::SegPlan plan{};
    void* scratch = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;  // kernel launches recorded in the graph
};

namespace {
const char* graph_name(int kind) {
    switch (kind) {
        case ORIGAMI_U32: return "segmented_graph<u32>";
        case ORIGAMI_U64:
        case ORIGAMI_I64: return "segmented_graph<u64>";
        default: return "segmented_graph<kv64>";
    }
}

int destroy(origami_seg_plan* p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->scratch) cudaFree(p->scratch);
    delete p;
    return ORIGAMI_OK;
}
}  // namespace

extern "C" {

int origami_seg_plan_create(int kind, void* d, void* tmp, const uint64_t* offsets, uint64_t nseg,
                            uint64_t n, origami_seg_plan** out) {
    using origami::api_fail;
    if (!out) return api_fail(ORIGAMI_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (kind < ORIGAMI_U32 || kind > ORIGAMI_KVU64) return api_fail(ORIGAMI_ERR_DTYPE, "unknown item kind");
    if (nseg == 0 || n == 0) return api_fail(ORIGAMI_ERR_INVALID, "a plan needs at least one item");
    if (!d || !tmp || !offsets) return api_fail(ORIGAMI_ERR_INVALID, "d, tmp and offsets are required");
    if (nseg >= (1ull << 32) - 1 || n > (1ull << 40)) return api_fail(ORIGAMI_ERR_INVALID, "too large");
    if ((((uintptr_t)d) | ((uintptr_t)tmp)) & 15)
        return api_fail(ORIGAMI_ERR_ALIGN, "segmented sort needs 16-byte aligned device buffers");
    int rc = origami::arena_init();
    if (rc != ORIGAMI_OK) return rc;
    auto* p = new origami_seg_plan();
    p->kind = kind;
    p->n = n;
    p->nseg = nseg;
    p->plan = origami::seg_plan(kind, n, nseg);
    if (cudaMalloc(&p->scratch, p->plan.scratch_bytes) != cudaSuccess) {
        cudaGetLastError();
        destroy(p);
        return api_fail(ORIGAMI_ERR_OOM, "plan scratch allocation failed");
    }
    cudaStream_t cap = nullptr;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) {
        destroy(p);
        return api_fail(ORIGAMI_ERR_CUDA, "stream creation failed");
    }
    origami::seg_prepare(kind);
    const uint64_t l0 = origami::launches_so_far();
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        origami::set_capturing(true);
        cudaError_t el = origami::seg_launch(kind, d, tmp, offsets, nseg, n, p->scratch, p->plan, cap);
        origami::set_capturing(false);
        e = cudaStreamEndCapture(cap, &p->graph);
        if (el != cudaSuccess) e = el;
    }
    p->kernels = origami::launches_so_far() - l0;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        destroy(p);
        return api_fail(ORIGAMI_ERR_CUDA, "graph capture of the segmented sort failed");
    }
    *out = p;
    return ORIGAMI_OK;
}

int origami_seg_plan_launch(origami_seg_plan* p, void* stream) {
    if (!p) return origami::api_fail(ORIGAMI_ERR_INVALID, "plan is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int slot = origami::profiling_on() ? origami::prof_begin(graph_name(p->kind), st) : -1;
    const cudaError_t e = cudaGraphLaunch(p->exec, st);
    origami::prof_end(slot, st);
    origami::count_launches(p->kernels);
    if (e != cudaSuccess) return origami::api_fail(ORIGAMI_ERR_CUDA, cudaGetErrorString(e));
    return ORIGAMI_OK;
}

int origami_seg_plan_status(origami_seg_plan* p, void* stream) {
    if (!p) return origami::api_fail(ORIGAMI_ERR_INVALID, "plan is NULL");
    int herr = 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(&herr, static_cast<char*>(p->scratch) + p->plan.err_offset, sizeof(int),
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return origami::api_fail(ORIGAMI_ERR_CUDA, cudaGetErrorString(e));
    if (origami::err_word_timeout(herr)) return origami::api_fail(ORIGAMI_ERR_TIMEOUT, "a merge job waited past its budget");
    if (herr == 2) return origami::api_fail(ORIGAMI_ERR_INVALID, "segment offsets decrease");
    return ORIGAMI_OK;
}

uint64_t origami_seg_plan_kernels(const origami_seg_plan* p) { return p ? p->kernels : 0; }

int origami_seg_plan_destroy(origami_seg_plan* p) {
    if (!p) return origami::api_fail(ORIGAMI_ERR_INVALID, "plan is NULL");
    cudaDeviceSynchronize();
    return destroy(p);
}

}  // extern "C"
