// GPU form of the reference's bench_sort driver (bench_sort.cpp:27-145).
//
//   bench_sort <size_pow> <n_threads> [n_cores] <min_k> [--kind u32] [--dist 1]
//              [--repeat 3] [--device] [--seed 1]
//
// Sorts 2^size_pow bytes of `kind` items (n_cores is read when n_threads > 1,
// as in the reference; thread counts do not apply to one GPU). Input comes
// from the device-side Writer generator (distribution --dist, 1..9). Default:
// host buffers through origami_gpu::sort_single_thread / sort_multi_thread,
// the reference's own call, so each timed sort includes the host<->device
// copies. --device times the device-resident sort alone with CUDA events.
// Prints the reference's lines ("Speed: X M keys/sec") and one JSON line.
#include <chrono>
#include <cstdio>
#include <vector>

#include "bench_common.hpp"
#include "origami_gpu.hpp"

// The reference's call (bench_sort.cpp:95-101) on host buffers.
template <class Item>
void* host_sort(void* d, void* t, uint64_t n, unsigned n_threads, unsigned n_cores, unsigned min_k) {
    Item* D = static_cast<Item*>(d);
    Item* T = static_cast<Item*>(t);
    if (n_threads <= 1) return origami_gpu::sort_single_thread<Item>(D, T, D + n, n, min_k, nullptr);
    return origami_gpu::sort_multi_thread<Item>(D, T, n, n_threads, n_cores, min_k, nullptr);
}

void* host_sort_kind(int kind, void* d, void* t, uint64_t n, unsigned n_threads, unsigned n_cores, unsigned min_k) {
    using namespace origami_gpu;
    switch (kind) {
        case ORIGAMI_U32: return host_sort<uint32_t>(d, t, n, n_threads, n_cores, min_k);
        case ORIGAMI_U64: return host_sort<uint64_t>(d, t, n, n_threads, n_cores, min_k);
        case ORIGAMI_I64: return host_sort<int64_t>(d, t, n, n_threads, n_cores, min_k);
        case ORIGAMI_KV64: return host_sort<KeyValue<int64_t, int64_t>>(d, t, n, n_threads, n_cores, min_k);
        default: return host_sort<KeyValue<uint64_t, uint64_t>>(d, t, n, n_threads, n_cores, min_k);
    }
}

int main(int argc, char** argv) {
    const auto pos = bench::positional(argc, argv);
    if (pos.size() < 3) {
        std::fprintf(stderr,
                     "usage: bench_sort <size_pow> <n_threads> [n_cores] <min_k> [--kind u32|u64|i64|kv64|kvu64]"
                     " [--dist 1..9] [--repeat R] [--device] [--seed S]\n");
        return 2;
    }
    const unsigned size_pow = (unsigned)std::atoi(pos[0].c_str());
    const unsigned n_threads = (unsigned)std::atoi(pos[1].c_str());
    unsigned n_cores = 1, min_k = 2;
    if (n_threads > 1) {
        if (pos.size() < 4) {
            std::fprintf(stderr, "n_threads > 1 needs n_cores and min_k\n");
            return 2;
        }
        n_cores = (unsigned)std::atoi(pos[2].c_str());
        min_k = (unsigned)std::atoi(pos[3].c_str());
    } else {
        min_k = (unsigned)std::atoi(pos[2].c_str());
    }
    const int kind = bench::kind_of(bench::opt(argc, argv, "--kind", "u32"));
    const int dist = std::atoi(bench::opt(argc, argv, "--dist", "1").c_str());
    const int repeat = std::atoi(bench::opt(argc, argv, "--repeat", "3").c_str());
    const uint64_t seed = std::strtoull(bench::opt(argc, argv, "--seed", "1").c_str(), nullptr, 10);
    const bool device = bench::flag(argc, argv, "--device");
    const uint64_t ib = origami_item_bytes(kind);
    const uint64_t bytes = 1ull << size_pow;
    const uint64_t n = bytes / ib;

    std::printf("Running origami-sort --> n: %llu (%s, dist %d, %s) ...\n", (unsigned long long)n,
                bench::kind_name(kind), dist, device ? "device buffers" : "host buffers");
    bench::DeviceBuf pristine(bytes), d(bytes), tmp(bytes);
    bench::ck(origami_generate_device(kind, pristine.p, n, dist, seed, nullptr), "generate");
    bench::ckc(cudaDeviceSynchronize(), "generate");
    std::vector<char> h_in, h_d, h_t;
    if (!device) {
        h_in.resize(bytes);
        h_d.resize(bytes);
        h_t.resize(bytes);
        bench::ckc(cudaMemcpy(h_in.data(), pristine.p, bytes, cudaMemcpyDeviceToHost), "copy input");
    }

    double avg = 0;
    bool ok = true;
    std::vector<char> check(bytes);
    for (int it = 0; it < repeat; ++it) {
        double ms;
        const void* out;
        if (device) {
            bench::ckc(cudaMemcpy(d.p, pristine.p, bytes, cudaMemcpyDeviceToDevice), "restore");
            bench::Timer t;
            t.start();
            void* res = nullptr;
            bench::ck(origami_sort_device(kind, d.p, tmp.p, n, 0, min_k, 0, &res, nullptr), "sort");
            ms = t.stop_ms();
            bench::ckc(cudaMemcpy(check.data(), res, bytes, cudaMemcpyDeviceToHost), "copy result");
            out = check.data();
        } else {
            std::memcpy(h_d.data(), h_in.data(), bytes);
            const auto t0 = std::chrono::steady_clock::now();
            void* res = nullptr;
            try {
                res = host_sort_kind(kind, h_d.data(), h_t.data(), n, n_threads, n_cores, min_k);
            } catch (const origami_gpu::error& e) {
                std::fprintf(stderr, "sort failed (%d): %s\n", e.code(), e.what());
                return 1;
            }
            ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            out = res;
        }
        const double sp = (double)n / ms / 1e3;
        avg += sp;
        if (!bench::chunks_sorted(kind, out, n, n)) {
            std::printf("Correctness error @ %d\n", it);
            ok = false;
        }
        std::printf("\rIter: %d / %d", it + 1, repeat);
        std::fflush(stdout);
    }
    avg /= repeat;
    std::printf("\nSpeed: %.2f M keys/sec\n", avg);
    std::printf("{\"driver\": \"bench_sort\", \"kind\": \"%s\", \"n\": %llu, \"dist\": %d, \"min_k\": %u, "
                "\"n_threads\": %u, \"n_cores\": %u, \"buffers\": \"%s\", \"mkeys_per_s\": %.3f, \"correct\": %s}\n",
                bench::kind_name(kind), (unsigned long long)n, dist, min_k, n_threads, n_cores,
                device ? "device" : "host", avg, ok ? "true" : "false");
    return ok ? 0 : 1;
}
