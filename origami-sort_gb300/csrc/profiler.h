// Launch accounting and optional per-kernel CUDA-event timing.
//
// Every kernel the library launches goes through launch(): it always counts
// the launch, and while profiling is switched on (origami_profile_enable) it
// brackets the launch with two CUDA events recorded on the launching stream.
// origami_profile_report() turns the recorded pairs into per-kernel launch
// counts and total device milliseconds.
#pragma once
#include <cuda_runtime.h>

namespace origami {

bool profiling_on();
void count_launch();
// CUDA-graph support: launches made while the calling thread captures a graph
// are counted but not timed; a replay adds the graph's kernel count.
void set_capturing(bool on);
uint64_t launches_so_far();
void count_launches(uint64_t k);
// Records the begin event; returns a slot id (or -1 when profiling is off).
int prof_begin(const char* name, cudaStream_t st);
void prof_end(int slot, cudaStream_t st);

// Polls a kernel makes on a bulk-copy barrier before it gives up, reports an
// expired wait and returns (bulk.cuh). Read when a kernel is launched;
// origami_set_wait_limit() changes it (default 2^20).
uint32_t wait_limit();

template <class F>
inline void launch(const char* name, cudaStream_t st, F&& f) {
    count_launch();
    if (!profiling_on()) {
        f();
        return;
    }
    const int slot = prof_begin(name, st);
    f();
    prof_end(slot, st);
}

template <class T>
struct TypeName;
template <>
struct TypeName<uint32_t> {
    static constexpr const char* v = "u32";
};
template <>
struct TypeName<uint64_t> {
    static constexpr const char* v = "u64";
};
struct KV64;
template <>
struct TypeName<KV64> {
    static constexpr const char* v = "kv64";
};

}  // namespace origami
