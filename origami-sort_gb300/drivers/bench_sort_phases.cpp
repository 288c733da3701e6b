// GPU form of the reference's bench_sort_phases driver
// (bench_sort_phases.cpp:1108-1542): one table per phase of the pipeline.
//
//   bench_sort_phases [phase1|phase2|phase3|phase4|all] [--kind u32] [--pow 30]
//                     [--dist 1] [--repeat 5]
//
//   phase1  tile sort alone: chunked sort with sort_n = the tile that the first
//           kernel sorts in registers and shared memory (Table 9's phase 1)
//   phase2  chunked sorts for sort_n from 32 up to 128K items: the sizes the
//           reference keeps in L2 (sort_sliding_test, Table 10)
//   phase3  chunked sorts for sort_n from 256K items up to the whole array
//           (Table 11), including the chunk sweep 128K..2M of the README
//   phase4  the full sort at every merge fan-in min_k = 2, 4, 8, 16 (the
//           switch point between binary and k-way passes; Tables 13-14)
// Every line gives Mkeys/s, the number of HBM passes (launches of the sort and
// merge kernels) and the kernels' share of the time, from the library's
// per-launch CUDA events. Device buffers; the input is restored from a
// pristine device copy outside the timed region.
#include <cstdio>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "bench_common.hpp"

namespace {

struct Result {
    double mkeys = 0, ms = 0;
    int passes = 0;
    std::string kernels;
};

// {kernel: (launches, total ms)} from origami_profile_report's
// "kernel,launches,timed_ms,timed" lines (every launch is timed here).
std::map<std::string, std::pair<long, double>> report() {
    std::vector<char> buf(1 << 16);
    std::map<std::string, std::pair<long, double>> m;
    const int len = origami_profile_report(buf.data(), buf.size());
    if (len < 0) return m;
    std::istringstream in(std::string(buf.data(), (size_t)len));
    std::string line;
    while (std::getline(in, line)) {
        const size_t c3 = line.rfind(',');
        if (c3 == std::string::npos || c3 == 0) continue;
        const size_t c2 = line.rfind(',', c3 - 1);
        if (c2 == std::string::npos || c2 == 0) continue;
        const size_t c1 = line.rfind(',', c2 - 1);
        if (c1 == std::string::npos) continue;
        m[line.substr(0, c1)] = {std::stol(line.substr(c1 + 1, c2 - c1 - 1)), std::stod(line.substr(c2 + 1, c3 - c2 - 1))};
    }
    return m;
}

Result run(int kind, void* pristine, void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k, int repeat,
           void* check) {
    const uint64_t bytes = n * origami_item_bytes(kind);
    Result r;
    void* res = nullptr;
    bench::ckc(cudaMemcpy(d, pristine, bytes, cudaMemcpyDeviceToDevice), "restore");  // warm-up
    bench::ck(origami_sort_device(kind, d, tmp, n, sort_n, min_k, 0, &res, nullptr), "sort");
    bench::ckc(cudaDeviceSynchronize(), "sort");
    origami_profile_enable(1);
    double total = 0;
    for (int i = 0; i < repeat; ++i) {
        bench::ckc(cudaMemcpy(d, pristine, bytes, cudaMemcpyDeviceToDevice), "restore");
        bench::Timer t;
        t.start();
        bench::ck(origami_sort_device(kind, d, tmp, n, sort_n, min_k, 0, &res, nullptr), "sort");
        total += t.stop_ms();
    }
    auto rep = report();
    origami_profile_enable(0);
    r.ms = total / repeat;
    r.mkeys = (double)n / r.ms / 1e3;
    double ktot = 0;
    for (auto& kv : rep) ktot += kv.second.second;
    std::ostringstream ks;
    for (auto& kv : rep) {
        const std::string& name = kv.first;
        if (name.rfind("block_sort", 0) == 0 || name.rfind("pair_merge", 0) == 0 || name.rfind("kway_merge", 0) == 0)
            r.passes += (int)(kv.second.first / repeat);
        ks << (ks.tellp() > 0 ? ", " : "") << name << " " << (int)(100.0 * kv.second.second / ktot + 0.5) << "%";
    }
    r.kernels = ks.str();
    bench::ckc(cudaMemcpy(check, res, bytes, cudaMemcpyDeviceToHost), "copy result");
    if (!bench::chunks_sorted(kind, check, n, sort_n)) {
        std::printf("Correctness error at sort_n %llu\n", (unsigned long long)sort_n);
        std::exit(1);
    }
    return r;
}

void line(const char* phase, int kind, uint64_t n, uint64_t sort_n, unsigned min_k, const Result& r) {
    const double gbs = 2.0 * n * origami_item_bytes(kind) * r.passes / (r.ms / 1e3) / 1e9;
    std::printf("%-7s sort_n %10llu  min_k %2u  %9.3f ms  %9.1f Mkeys/s  passes %2d  %8.1f GB/s moved  [%s]\n", phase,
                (unsigned long long)sort_n, min_k, r.ms, r.mkeys, r.passes, gbs, r.kernels.c_str());
    std::printf("{\"driver\": \"bench_sort_phases\", \"phase\": \"%s\", \"kind\": \"%s\", \"n\": %llu, \"sort_n\": %llu, "
                "\"min_k\": %u, \"ms\": %.4f, \"mkeys_per_s\": %.2f, \"passes\": %d, \"gbs_moved\": %.1f}\n",
                phase, bench::kind_name(kind), (unsigned long long)n, (unsigned long long)sort_n, min_k, r.ms,
                r.mkeys, r.passes, gbs);
    std::fflush(stdout);
}

}  // namespace

int main(int argc, char** argv) {
    const auto pos = bench::positional(argc, argv);
    const std::string which = pos.empty() ? "all" : pos[0];
    const int kind = bench::kind_of(bench::opt(argc, argv, "--kind", "u32"));
    const unsigned pw = (unsigned)std::atoi(bench::opt(argc, argv, "--pow", "30").c_str());
    const int dist = std::atoi(bench::opt(argc, argv, "--dist", "1").c_str());
    const int repeat = std::atoi(bench::opt(argc, argv, "--repeat", "5").c_str());
    const uint64_t ib = origami_item_bytes(kind);
    const uint64_t n = (1ull << pw) / ib;
    const uint64_t bytes = n * ib;
    bench::DeviceBuf pristine(bytes), d(bytes), tmp(bytes);
    std::vector<char> check(bytes);
    bench::ck(origami_generate_device(kind, pristine.p, n, dist, 1, nullptr), "generate");
    bench::ckc(cudaDeviceSynchronize(), "generate");
    std::printf("bench_sort_phases: %s, n = %llu (%llu bytes), dist %d, %d timed runs per line\n",
                bench::kind_name(kind), (unsigned long long)n, (unsigned long long)bytes, dist, repeat);
    const uint64_t tile = ib == 4 ? 8192 : (ib == 8 ? 4096 : 2048);  // first kernel's tile per kind
    auto want = [&](const char* p) { return which == "all" || which == p; };
    if (want("phase1")) line("phase1", kind, n, tile, 2, run(kind, pristine.p, d.p, tmp.p, n, tile, 2, repeat, check.data()));
    if (want("phase2"))
        for (uint64_t s = 32; s <= (1ull << 17) && s < n; s <<= 1)
            line("phase2", kind, n, s, 2, run(kind, pristine.p, d.p, tmp.p, n, s, 2, repeat, check.data()));
    if (want("phase3"))
        for (uint64_t s = 1ull << 17; s <= n; s <<= 1)
            line("phase3", kind, n, s, 2, run(kind, pristine.p, d.p, tmp.p, n, s, 2, repeat, check.data()));
    if (want("phase4"))
        for (unsigned k : {2u, 4u, 8u, 16u})
            line("phase4", kind, n, 0, k, run(kind, pristine.p, d.p, tmp.p, n, 0, k, repeat, check.data()));
    return 0;
}
