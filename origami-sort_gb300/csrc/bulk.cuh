// Bulk asynchronous copies between global and shared memory (the TMA unit's
// untiled form, cp.async.bulk) and the shared-memory mbarriers that track them.
//
// Every wait is bounded: mbar_wait() gives up after a number of polls (the
// kernel's `spin` argument, BULK_SPIN_LIMIT by default) and returns false, so a
// kernel can record an error and leave instead of spinning forever. A kernel
// whose wait expired drains its own copies with the full limit before it
// returns (bulk_drain), so that no bulk load lands in shared memory that a
// later CTA owns.
//
// Error words written by the kernels (int, 0 = no error):
//   1  a bulk-copy wait expired; the copies it waited for were drained
//   2  (segmented sort) decreasing or out-of-range segment offsets
//   3  a bulk-copy wait expired and a drain wait expired too: copies may still
//      have been in flight when the CTA returned
//   5  merge splits that are inconsistent: the runs given to a merge were not
//      sorted (the tile was clamped so that every access stays in bounds)
// A merge kernel that finds 1 or 3 already set returns at once: the passes
// after an expired wait would merge runs that are not sorted.
#pragma once
#include <cstdint>

namespace origami {

constexpr uint32_t BULK_SPIN_LIMIT = 1u << 20;
constexpr int ERR_WAIT_EXPIRED = 1;
constexpr int ERR_WAIT_UNDRAINED = 3;
constexpr int ERR_BAD_RUNS = 5;

__device__ __forceinline__ bool err_wait_set(const int* err) {
    const int w = *(volatile const int*)err;
    return w == ERR_WAIT_EXPIRED || w == ERR_WAIT_UNDRAINED;
}
// Records a first error (an earlier one is kept).
__device__ __forceinline__ void err_first(int* err, int code) { atomicCAS(err, 0, code); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// One-arrival barrier: the thread that issues the copies arrives once (with the
// byte count it expects) and the copies complete the phase.
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the copy engine and other threads
// (followed by a block barrier).
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Polls the barrier until the phase with the given parity has completed;
// false when it has not after `limit` polls (0: gives up at once).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = BULK_SPIN_LIMIT) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Global -> shared copy of `bytes` (a multiple of 16; both addresses 16-byte
// aligned), completing on `bar`.
__device__ __forceinline__ void bulk_load(void* smem, const void* gmem, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(smem)),
        "l"(gmem), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Asks the copy engine to bring `bytes` (a multiple of 16; 16-byte aligned
// address) of global memory into L2; nothing waits for it.
__device__ __forceinline__ void bulk_prefetch_l2(const void* gmem, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(gmem), "r"(bytes) : "memory");
}

// Orders this thread's generic shared-memory writes before later bulk copies
// that read (or overwrite) the same bytes.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// Shared -> global copy of `bytes` (a multiple of 16; both addresses 16-byte
// aligned) in the issuing thread's current bulk group.
__device__ __forceinline__ void bulk_store(void* gmem, const void* smem, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(gmem), "r"(smem_u32(smem)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }

// Waits until at most N of this thread's bulk groups still read shared memory.
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
// Waits until all of this thread's bulk groups have completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

// Error path of a CTA whose wait on a bulk load expired (thread 0, the thread
// that issued every copy of the CTA): records ERR_WAIT_EXPIRED, waits for its
// bulk stores, then for each barrier in `bars` whose load is outstanding
// (`pending` bit i set) waits with the full limit for the phase `parity` bit i.
// If one of those waits expires as well, records ERR_WAIT_UNDRAINED.
template <int NB>
__device__ __forceinline__ void bulk_drain(int* err, uint64_t* bars, uint32_t pending, uint32_t parity) {
    atomicCAS(err, 0, ERR_WAIT_EXPIRED);
    atomicCAS(err, ERR_BAD_RUNS, ERR_WAIT_EXPIRED);
    bulk_wait_all();
    bool drained = true;
#pragma unroll
    for (int i = 0; i < NB; ++i)
        if ((pending >> i) & 1u) drained = mbar_wait(&bars[i], (parity >> i) & 1u) && drained;
    if (!drained) atomicExch(err, ERR_WAIT_UNDRAINED);
}

// Programmatic dependent launch. A kernel launched with the programmatic
// stream serialization attribute may start while the kernel before it in the
// stream still runs; grid_dep_wait() returns once that kernel has completed and
// its writes are visible, so a dependent kernel calls it before it touches
// memory the previous kernel reads or writes. grid_dep_launch() lets the next
// such kernel start launching. Both do nothing in a kernel launched normally.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

}  // namespace origami
