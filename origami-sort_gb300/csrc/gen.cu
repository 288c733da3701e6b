// Device-side input generators for the reference's Writer distributions
// (writer.h:27-35), so benchmarks fill HBM without a host round trip.
//
//   1 uniform          counter-based: splitmix64 of (seed, index); same value
//                      ranges as the reference (u32 and u64 full range, signed
//                      and key-value keys in [0, 2^63)), not its mt19937 stream
//   2 all same         the reference's value: first std::mt19937_64 draw >> 1
//   3 sorted / 4 reverse   uniform, then sorted on the device by this library
//   5 almost sorted    uniform with every 7th item set to the kind's maximum
//   6 Pareto keys      exact: the reference's LCG y-sequence, evaluated per
//                      item by LCG jump-ahead
//   7 Pareto back to back  exact: runs of the LCG x-sequence with Pareto run
//                      lengths; run starts from a device prefix sum, the last
//                      few runs (where the reference may skip draws) on one
//                      thread
//   8 Pareto shuffled  distribution 7 permuted by sorting on random keys (the
//                      reference shuffles with a random_device seed, so its
//                      order is not reproducible either)
//   9 Fibonacci        exact: the reference's sequence repeats every 94 items
// Key-value items get value = key + 1, as in the reference.
#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "../../include/origami_gpu.h"
#include "common.cuh"
#include "dispatch.h"
#include "profiler.h"

namespace origami {
namespace {

constexpr uint64_t LCG_A = 6364136223846793005ull, LCG_C = 1442695040888963407ull;
constexpr uint64_t FIB_PERIOD = 94;

__host__ __device__ __forceinline__ uint64_t splitmix(uint64_t seed, uint64_t i) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// k steps of v -> v * LCG_A + LCG_C, in O(log k) (affine maps composed by
// repeated squaring).
__host__ __device__ __forceinline__ uint64_t lcg_skip(uint64_t v, uint64_t k) {
    uint64_t am = 1, ap = 0, cm = LCG_A, cp = LCG_C;
    while (k) {
        if (k & 1) {
            am *= cm;
            ap = ap * cm + cp;
        }
        cp = (cm + 1) * cp;
        cm *= cm;
        k >>= 1;
    }
    return am * v + ap;
}

// Pareto run length of the reference (writer.h:83-84): alpha 1, beta 7,
// rounded up, capped at 100000. IEEE double arithmetic, as on the host.
__host__ __device__ __forceinline__ uint64_t pareto_f(uint64_t y) {
    const double u = (double)y / 18446744073709551616.0;
    const double fd = ceil(7.0 * (1.0 / (1.0 - u) - 1.0));
    return fd < 100000.0 ? (uint64_t)fd : 100000ull;
}

__device__ __forceinline__ void put(int kind, void* d, uint64_t i, uint64_t x) {
    switch (kind) {
        case ORIGAMI_U32: static_cast<uint32_t*>(d)[i] = (uint32_t)x; break;
        case ORIGAMI_U64:
        case ORIGAMI_I64: static_cast<uint64_t*>(d)[i] = x; break;
        default: static_cast<KV64*>(d)[i] = KV64{x, x + 1}; break;
    }
}

__global__ void fill_uniform(int kind, void* d, uint64_t n, uint64_t seed) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t z = splitmix(seed, i);
        put(kind, d, i, (kind == ORIGAMI_U32 || kind == ORIGAMI_U64) ? z : (z >> 1));
    }
}

__global__ void fill_const(int kind, void* d, uint64_t n, uint64_t x) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        put(kind, d, i, x);
}

__global__ void mark_every_7th(int kind, void* d, uint64_t n) {
    for (uint64_t i = 7 * (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x); i < n; i += 7ull * gridDim.x * blockDim.x) {
        switch (kind) {
            case ORIGAMI_U32: static_cast<uint32_t*>(d)[i] = 0xFFFFFFFFu; break;
            case ORIGAMI_U64:
            case ORIGAMI_I64: static_cast<uint64_t*>(d)[i] = 0x7FFFFFFFFFFFFFFFull; break;
            default: static_cast<KV64*>(d)[i].key = 0x7FFFFFFFFFFFFFFFull; break;  // the value is kept
        }
    }
}

template <class T>
__global__ void reverse_items(T* d, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n / 2; i += (uint64_t)gridDim.x * blockDim.x) {
        const T a = d[i];
        d[i] = d[n - 1 - i];
        d[n - 1 - i] = a;
    }
}

// Pareto keys: item i holds the run length drawn at step i (y after i+1 steps).
constexpr int PARETO_VT = 16;
__global__ void fill_pareto(int kind, void* d, uint64_t n) {
    const uint64_t i0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) * PARETO_VT;
    if (i0 >= n) return;
    uint64_t y = lcg_skip(889, i0 + 1);
    for (int k = 0; k < PARETO_VT && i0 + k < n; ++k) {
        put(kind, d, i0 + k, pareto_f(y));
        y = y * LCG_A + LCG_C;
    }
}

// Back-to-back runs, step j in [j0, j0 + m): len[j - j0] = its run length.
__global__ void pareto_lengths(uint64_t j0, uint64_t m, uint64_t* len) {
    const uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) * PARETO_VT;
    if (t >= m) return;
    uint64_t y = lcg_skip(889, j0 + t + 1);
    for (int k = 0; k < PARETO_VT && t + k < m; ++k) {
        len[t + k] = pareto_f(y);
        y = y * LCG_A + LCG_C;
    }
}

// Items [0, limit) of runs 0..m-1; next[r] is the start of run r + 1. Item p
// belongs to run r, the first with next[r] > p, whose key is x after r + 1
// steps of the LCG.
__global__ void fill_runs(int kind, void* d, const uint64_t* next, uint64_t m, uint64_t limit) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < limit; p += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t a = 0, e = m;
        while (a < e) {
            const uint64_t mid = (a + e) >> 1;
            if (next[mid] <= p)
                a = mid + 1;
            else
                e = mid;
        }
        put(kind, d, p, lcg_skip(1, a + 1));
    }
}

// The reference's loop from step j with i items written (writer.h:78-120):
// runs that fit are taken, a run that does not fit is skipped unless at most
// ten items remain, which are then filled with its key.
__global__ void pareto_tail(int kind, void* d, uint64_t n, uint64_t i, uint64_t j) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint64_t x = lcg_skip(1, j), y = lcg_skip(889, j);
    // a skip needs a draw of at least the remaining count (> 10 items), which
    // happens with probability below 0.42 per draw: the bound is never reached
    for (uint64_t guard = 0; i < n && guard < (1ull << 22); ++guard) {
        x = x * LCG_A + LCG_C;
        y = y * LCG_A + LCG_C;
        const uint64_t f = pareto_f(y);
        if (i + f < n) {
            for (uint64_t q = 0; q < f; ++q) put(kind, d, i + q, x);
            i += f;
        } else if (i + 10 >= n) {
            for (; i < n; ++i) put(kind, d, i, x);
        }
    }
}

__global__ void fill_fib(int kind, void* d, uint64_t n, const uint64_t* table) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        put(kind, d, i, table[i % FIB_PERIOD]);
}

// ---- exclusive prefix sum of uint64 (in place), blocks of 4096 ----------
constexpr int SCAN_NT = 1024, SCAN_VT = 4, SCAN_TILE = SCAN_NT * SCAN_VT;

__global__ void __launch_bounds__(SCAN_NT) scan_tiles(uint64_t* v, uint64_t m, uint64_t* sums) {
    __shared__ uint64_t warp_tot[SCAN_NT / 32];
    const uint64_t base = blockIdx.x * (uint64_t)SCAN_TILE + threadIdx.x * (uint64_t)SCAN_VT;
    uint64_t x[SCAN_VT], t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_VT; ++k) {
        x[k] = base + k < m ? v[base + k] : 0;
        t += x[k];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t inc = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint64_t s = warp_tot[lane], si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, si, o);
            if (lane >= o) si += y;
        }
        warp_tot[lane] = si - s;  // exclusive over warps
        if (lane == 31) sums[blockIdx.x] = si;
    }
    __syncthreads();
    uint64_t run = inc - t + warp_tot[w];
#pragma unroll
    for (int k = 0; k < SCAN_VT; ++k) {
        if (base + k < m) v[base + k] = run;
        run += x[k];
    }
}

__global__ void add_tile_offsets(uint64_t* v, uint64_t m, const uint64_t* sums) {
    const uint64_t b = blockIdx.x;
    const uint64_t add = sums[b];
    for (uint64_t i = b * SCAN_TILE + threadIdx.x; i < m && i < (b + 1) * SCAN_TILE; i += blockDim.x) v[i] += add;
}

cudaError_t exclusive_scan(uint64_t* v, uint64_t m, cudaStream_t st) {
    if (m == 0) return cudaSuccess;
    const uint64_t tiles = (m + SCAN_TILE - 1) / SCAN_TILE;
    uint64_t* sums = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&sums), tiles * 8, st);
    if (e != cudaSuccess) return e;
    launch("gen_scan", st, [&] { scan_tiles<<<(unsigned)tiles, SCAN_NT, 0, st>>>(v, m, sums); });
    if (tiles > 1) {
        e = exclusive_scan(sums, tiles, st);
        if (e == cudaSuccess)
            launch("gen_scan_add", st, [&] { add_tile_offsets<<<(unsigned)tiles, SCAN_NT, 0, st>>>(v, m, sums); });
    }
    cudaFreeAsync(sums, st);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

unsigned grid_for(uint64_t n) {
    const uint64_t b = (n + 255) / 256;
    return (unsigned)(b < 152ull * 64 ? (b ? b : 1) : 152ull * 64);
}

uint64_t ib_of(int kind) { return kind == ORIGAMI_U32 ? 4 : (kind <= ORIGAMI_I64 ? 8 : 16); }

cudaError_t pareto_b2b(int kind, void* d, uint64_t n, cudaStream_t st) {
    // steps 0..m-1 as prefix sums; m grows until their runs cover n items
    uint64_t m = n / 16 + 4096;
    for (;;) {
        uint64_t* len = nullptr;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&len), (m + 1) * 8, st);
        if (e != cudaSuccess) return e;
        const unsigned blocks = (unsigned)((m + 256ull * PARETO_VT - 1) / (256ull * PARETO_VT));
        launch("gen_pareto_len", st, [&] { pareto_lengths<<<blocks, 256, 0, st>>>(0, m, len); });
        cudaMemsetAsync(len + m, 0, 8, st);
        e = exclusive_scan(len, m + 1, st);  // len[j] = start of run j, len[m] = total
        uint64_t total = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&total, len + m, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaFreeAsync(len, st);
            return e;
        }
        if (total < n) {  // not enough runs yet
            cudaFreeAsync(len, st);
            m *= 4;
            continue;
        }
        // first step whose run does not end before n: start[j+1] >= n
        std::vector<uint64_t> h(m + 1);
        e = cudaMemcpyAsync(h.data(), len, (m + 1) * 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaFreeAsync(len, st);
            return e;
        }
        const uint64_t j = (uint64_t)(std::lower_bound(h.begin() + 1, h.end(), n) - (h.begin() + 1));
        const uint64_t covered = h[j];  // runs 0..j-1 fit, back to back
        launch("gen_pareto_fill", st, [&] {
            fill_runs<<<grid_for(covered), 256, 0, st>>>(kind, d, len + 1, j, covered);
        });
        launch("gen_pareto_tail", st, [&] { pareto_tail<<<1, 32, 0, st>>>(kind, d, n, covered, j); });
        cudaFreeAsync(len, st);
        return cudaGetLastError();
    }
}

// Shuffle by sorting (random key, item key) pairs on the device.
__global__ void tag_random(int kind, const void* d, KV64* t, uint64_t n, uint64_t seed) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k;
        switch (kind) {
            case ORIGAMI_U32: k = static_cast<const uint32_t*>(d)[i]; break;
            case ORIGAMI_U64:
            case ORIGAMI_I64: k = static_cast<const uint64_t*>(d)[i]; break;
            default: k = static_cast<const KV64*>(d)[i].key; break;
        }
        t[i] = KV64{splitmix(seed, i), k};
    }
}
__global__ void untag(int kind, void* d, const KV64* t, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        put(kind, d, i, t[i].value);
}

}  // namespace
}  // namespace origami

using namespace origami;

extern "C" int origami_generate_device(int kind, void* d, uint64_t n, int dist, uint64_t seed, void* stream) {
    if (kind < ORIGAMI_U32 || kind > ORIGAMI_KVU64) return api_fail(ORIGAMI_ERR_DTYPE, "unknown item kind");
    if (dist < 1 || dist > 9) return api_fail(ORIGAMI_ERR_INVALID, "distribution must be 1..9");
    if (n == 0) return ORIGAMI_OK;
    if (!d) return api_fail(ORIGAMI_ERR_INVALID, "d is NULL");
    if ((uintptr_t)d % ib_of(kind)) return api_fail(ORIGAMI_ERR_ALIGN, "d not aligned to the item size");
    int rc = arena_init();
    if (rc != ORIGAMI_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned g = grid_for(n);
    cudaError_t e = cudaSuccess;
    switch (dist) {
        case 1:
        case 3:
        case 4:
        case 5:
            launch("gen_uniform", st, [&] { fill_uniform<<<g, 256, 0, st>>>(kind, d, n, seed); });
            break;
        case 2: {
            std::mt19937_64 eng;  // default seed, as the reference's all_same
            const uint64_t x = eng() >> 1;
            launch("gen_const", st, [&] { fill_const<<<g, 256, 0, st>>>(kind, d, n, x); });
            break;
        }
        case 6: {
            const unsigned b = (unsigned)((n + 256ull * PARETO_VT - 1) / (256ull * PARETO_VT));
            launch("gen_pareto", st, [&] { fill_pareto<<<b, 256, 0, st>>>(kind, d, n); });
            break;
        }
        case 7:
        case 8:
            e = pareto_b2b(kind, d, n, st);
            break;
        case 9: {
            std::vector<uint64_t> fib(FIB_PERIOD);
            fib[0] = 0;
            fib[1] = 1;
            for (uint64_t i = 2; i < FIB_PERIOD; ++i) fib[i] = fib[i - 1] + fib[i - 2];
            uint64_t* t = nullptr;
            e = cudaMallocAsync(reinterpret_cast<void**>(&t), FIB_PERIOD * 8, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(t, fib.data(), FIB_PERIOD * 8, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) launch("gen_fib", st, [&] { fill_fib<<<g, 256, 0, st>>>(kind, d, n, t); });
            if (t) cudaFreeAsync(t, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host table must outlive the copy
            break;
        }
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess && (dist == 3 || dist == 4)) {
        void* res = nullptr;
        rc = origami_sort_device(kind, d, nullptr, n, 0, 0, 0, &res, stream);
        if (rc != ORIGAMI_OK) return rc;
        if (dist == 4) {
            const uint64_t ib = ib_of(kind);
            launch("gen_reverse", st, [&] {
                if (ib == 4)
                    reverse_items<<<g, 256, 0, st>>>(static_cast<uint32_t*>(d), n);
                else if (ib == 8)
                    reverse_items<<<g, 256, 0, st>>>(static_cast<uint64_t*>(d), n);
                else
                    reverse_items<<<g, 256, 0, st>>>(static_cast<KV64*>(d), n);
            });
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && dist == 5) {
        launch("gen_mark7", st, [&] { mark_every_7th<<<g, 256, 0, st>>>(kind, d, n); });
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && dist == 8) {
        KV64* t = nullptr;
        e = cudaMallocAsync(reinterpret_cast<void**>(&t), n * sizeof(KV64), st);
        if (e == cudaSuccess) {
            launch("gen_tag", st, [&] { tag_random<<<g, 256, 0, st>>>(kind, d, t, n, seed); });
            void* res = nullptr;
            rc = origami_sort_device(ORIGAMI_KVU64, t, nullptr, n, 0, 0, 0, &res, stream);
            if (rc == ORIGAMI_OK) launch("gen_untag", st, [&] { untag<<<g, 256, 0, st>>>(kind, d, t, n); });
            cudaFreeAsync(t, st);
            if (rc != ORIGAMI_OK) return rc;
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return api_fail(e == cudaErrorMemoryAllocation ? ORIGAMI_ERR_OOM : ORIGAMI_ERR_CUDA, "generator");
    }
    return ORIGAMI_OK;
}
