// Shared pieces of the GPU benchmark drivers: argument parsing helpers, item
// kinds by name, device buffers and CUDA-event timing.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "origami_gpu.h"

namespace bench {

inline int kind_of(const std::string& s) {
    if (s == "u32") return ORIGAMI_U32;
    if (s == "u64") return ORIGAMI_U64;
    if (s == "i64") return ORIGAMI_I64;
    if (s == "kv64") return ORIGAMI_KV64;
    if (s == "kvu64") return ORIGAMI_KVU64;
    std::fprintf(stderr, "unknown kind %s (u32, u64, i64, kv64, kvu64)\n", s.c_str());
    std::exit(2);
}

inline const char* kind_name(int k) {
    static const char* names[] = {"u32", "u64", "i64", "kv64", "kvu64"};
    return names[k];
}

inline void ck(int rc, const char* what) {
    if (rc != ORIGAMI_OK) {
        std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, origami_last_error());
        std::exit(1);
    }
}

inline void ckc(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "%s failed: %s\n", what, cudaGetErrorString(e));
        std::exit(1);
    }
}

struct DeviceBuf {
    void* p = nullptr;
    explicit DeviceBuf(uint64_t bytes) { ckc(cudaMalloc(&p, bytes ? bytes : 16), "cudaMalloc"); }
    ~DeviceBuf() { cudaFree(p); }
    DeviceBuf(const DeviceBuf&) = delete;
    DeviceBuf& operator=(const DeviceBuf&) = delete;
};

struct Timer {
    cudaEvent_t a, b;
    Timer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~Timer() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    void start(cudaStream_t s = nullptr) { cudaEventRecord(a, s); }
    float stop_ms(cudaStream_t s = nullptr) {
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        return ms;
    }
};

// Sortedness of every chunk of sort_n items (the reference's
// sort_correctness_checker, utils.h:38-47), on a host copy of the keys.
inline bool chunks_sorted(int kind, const void* h, uint64_t n, uint64_t sort_n) {
    if (sort_n == 0 || sort_n > n) sort_n = n;
    for (uint64_t c = 0; c < n; c += sort_n) {
        const uint64_t e = c + sort_n < n ? c + sort_n : n;
        for (uint64_t i = c + 1; i < e; ++i) {
            bool ok;
            switch (kind) {
                case ORIGAMI_U32: ok = ((const uint32_t*)h)[i - 1] <= ((const uint32_t*)h)[i]; break;
                case ORIGAMI_U64: ok = ((const uint64_t*)h)[i - 1] <= ((const uint64_t*)h)[i]; break;
                case ORIGAMI_I64: ok = ((const int64_t*)h)[i - 1] <= ((const int64_t*)h)[i]; break;
                case ORIGAMI_KV64: ok = ((const int64_t*)h)[2 * (i - 1)] <= ((const int64_t*)h)[2 * i]; break;
                default: ok = ((const uint64_t*)h)[2 * (i - 1)] <= ((const uint64_t*)h)[2 * i]; break;
            }
            if (!ok) return false;
        }
    }
    return true;
}

// --name value options after the positional arguments
inline std::string opt(int argc, char** argv, const char* name, const char* dflt) {
    for (int i = 1; i + 1 < argc; ++i)
        if (std::strcmp(argv[i], name) == 0) return argv[i + 1];
    return dflt;
}
inline bool flag(int argc, char** argv, const char* name) {
    for (int i = 1; i < argc; ++i)
        if (std::strcmp(argv[i], name) == 0) return true;
    return false;
}
// positional arguments come first, as in the reference's drivers
inline std::vector<std::string> positional(int argc, char** argv) {
    std::vector<std::string> p;
    for (int i = 1; i < argc && std::strncmp(argv[i], "--", 2) != 0; ++i) p.push_back(argv[i]);
    return p;
}

inline double peak_hbm_gbs() {
    const char* e = std::getenv("ORIGAMI_HBM_GBS");
    return e ? std::atof(e) : 0.0;
}

}  // namespace bench
