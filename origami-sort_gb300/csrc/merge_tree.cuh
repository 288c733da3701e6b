// Merge tree and partition over independent device streams: the GPU forms of
// the reference's MergeTree::merge(X, endX, C, n, ...) (merge_tree.h:2792-3010)
// and partition_templated::Partition_Ptrs (Partition.h:118-166).
//
// merge_streams: way sorted streams -> C. Up to 16 streams are merged in one
// HBM pass by the k-way kernels of the sort pipeline (kway.cuh) over a
// StreamLists group: kway_split_kernel cuts the output into ranges of RANGE
// items, range_merge_kernel merges each range through shared memory. More
// streams are merged in levels of 16 (consecutive streams per group, so ties
// keep stream order), through interim buffers from the stream-ordered pool.
//
// rank_split_kernel: for K sorted streams (K up to 1024) and a list of output
// ranks, the split of every stream at every rank: S[i] items of stream i are
// among the r smallest, ties ordered by stream index. One block per rank,
// one thread per stream. The r-th item's key t is found by bisection over the
// key space (32 or 64 rounds); each round every thread counts its stream's
// items <= the probe inside a window that only shrinks, and a block reduction
// sums the counts. Equal keys at t are then handed out in stream order.
#pragma once
#include <string>
#include <vector>

#include "kway.cuh"
#include "profiler.h"

namespace origami {

constexpr int RANK_SPLIT_MAX_K = 1024;

template <class T>
__global__ void __launch_bounds__(RANK_SPLIT_MAX_K) rank_split_kernel(
    const T* const* __restrict__ ptr, const uint64_t* __restrict__ cnt, int K,
    const uint64_t* __restrict__ ranks, uint64_t xin, uint64_t* __restrict__ out) {
    using K_t = typename Traits<T>::Key;
    __shared__ unsigned long long part[RANK_SPLIT_MAX_K / 32];
    __shared__ unsigned long long total;
    const int i = threadIdx.x;
    const int lane = i & 31, warp = i >> 5, nw = (blockDim.x + 31) >> 5;
    const uint64_t r = ranks[blockIdx.x];
    const T* p = i < K ? ptr[i] : nullptr;
    const uint64_t len = i < K ? cnt[i] : 0;

    auto block_sum = [&](uint64_t v) -> uint64_t {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        __syncthreads();
        if (lane == 0) part[warp] = v;
        __syncthreads();
        if (i == 0) {
            unsigned long long s = 0;
            for (int w = 0; w < nw; ++w) s += part[w];
            total = s;
        }
        __syncthreads();
        return total;
    };
    // items of this stream with key <= v, searching [a, e)
    auto count_le = [&](K_t v, uint64_t a, uint64_t e) -> uint64_t {
        while (a < e) {
            const uint64_t m = a + ((e - a) >> 1);
            if (ckey(p[m], xin) <= v)
                a = m + 1;
            else
                e = m;
        }
        return a;
    };

    const uint64_t G = block_sum(len);
    uint64_t s;
    if (r >= G) {
        s = len;
    } else if (r == 0) {
        s = 0;
    } else {
        // smallest key t with (items <= t) > r; ub window [wlo, whi] per stream
        K_t lo = 0, hi = (K_t)~(K_t)0;
        uint64_t wlo = 0, whi = len;
        while (lo < hi) {
            const K_t mid = lo + ((hi - lo) >> 1);
            const uint64_t c = count_le(mid, wlo, whi);
            if (block_sum(c) > r) {
                hi = mid;
                whi = c;
            } else {
                lo = mid + 1;
                wlo = c;
            }
        }
        // the windows have closed on t: wlo items are < t, whi items are <= t
        const uint64_t lt = wlo;
        const uint64_t eq = whi - wlo;
        // hand the equal items out in stream order: exclusive scan of eq
        const uint64_t need = r - block_sum(lt);
        uint64_t before = eq;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, before, o);
            if (lane >= o) before += y;
        }
        __syncthreads();
        if (lane == 31) part[warp] = before;
        __syncthreads();
        uint64_t wbase = 0;
        for (int w = 0; w < warp; ++w) wbase += part[w];
        before = before - eq + wbase;  // equal items in streams < i
        const uint64_t take = need > before ? (need - before < eq ? need - before : eq) : 0;
        s = lt + take;
    }
    if (i < K) out[blockIdx.x * (uint64_t)K + i] = s;
}

template <class T>
struct MergeTreeOps {
    using C = KwayCfg<T>;

    static void configure() {
        static const bool done = [] {
            cudaFuncSetAttribute(range_merge_kernel<T, StreamLists<T>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)KwayLayout<T>::SMEM);
            return true;
        }();
        (void)done;
    }

    // One pass: up to KWAY_MAX streams into dst. xin/xout: flips on read/write.
    static cudaError_t pass(const StreamLists<T>& sl, T* dst, uint64_t xin, uint64_t xout, cudaStream_t st) {
        static const std::string n_ks = std::string("mtree_split<") + TypeName<T>::v + ">";
        static const std::string n_km = std::string("mtree_merge<") + TypeName<T>::v + ">";
        if (sl.G == 0) return cudaSuccess;
        const uint64_t rpg = (sl.G + C::RANGE - 1) / C::RANGE;
        int64_t* bnd = nullptr;
        int* err = nullptr;
        if (rpg > 1) {
            cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&bnd),
                                            (rpg + 1) * KWAY_MAX * sizeof(int64_t) + 256, st);
            if (e != cudaSuccess) return e;
            err = reinterpret_cast<int*>(reinterpret_cast<char*>(bnd) + (rpg + 1) * KWAY_MAX * sizeof(int64_t));
            cudaMemsetAsync(err, 0, sizeof(int), st);
            launch(n_ks.c_str(), st, [&] {
                kway_split_kernel<T, StreamLists<T>><<<(unsigned)(rpg + 1), 256, 0, st>>>(sl, (int)rpg, xin, bnd,
                                                                                         err);
            });
        }
        launch(n_km.c_str(), st, [&] {
            range_merge_kernel<T, StreamLists<T>><<<(unsigned)rpg, C::NT, KwayLayout<T>::SMEM, st>>>(
                sl, dst, (int)rpg, bnd, xin, xout, 0, NoProbe(), err);
        });
        if (bnd) cudaFreeAsync(bnd, st);
        return cudaGetLastError();
    }

    // way streams (ptr[i], cnt[i]) -> dst, ties by stream index.
    static cudaError_t merge(const T* const* ptr, const uint64_t* cnt, uint64_t way, T* dst, uint64_t xmask,
                             cudaStream_t st) {
        configure();
        std::vector<const T*> cur(ptr, ptr + way);
        std::vector<uint64_t> len(cnt, cnt + way);
        uint64_t G = 0;
        for (uint64_t i = 0; i < way; ++i) G += len[i];
        if (G == 0) return cudaSuccess;
        T* tmp[2] = {nullptr, nullptr};
        int which = 0;
        uint64_t xin = xmask;  // the first level reads the caller's items
        cudaError_t e = cudaSuccess;
        while (e == cudaSuccess) {
            const bool last = cur.size() <= (size_t)KWAY_MAX;
            T* out = dst;
            if (!last) {
                if (!tmp[which]) {
                    e = cudaMallocAsync(reinterpret_cast<void**>(&tmp[which]), G * sizeof(T), st);
                    if (e != cudaSuccess) break;
                }
                out = tmp[which];
            }
            std::vector<const T*> nxt;
            std::vector<uint64_t> nlen;
            uint64_t o = 0;
            for (size_t g0 = 0; g0 < cur.size() && e == cudaSuccess; g0 += KWAY_MAX) {
                StreamLists<T> sl{};
                const size_t g1 = g0 + KWAY_MAX < cur.size() ? g0 + KWAY_MAX : cur.size();
                sl.nr = (int)(g1 - g0);
                sl.G = 0;
                for (size_t q = g0; q < g1; ++q) {
                    sl.ptr[q - g0] = cur[q];
                    sl.cnt[q - g0] = len[q];
                    sl.G += len[q];
                }
                e = pass(sl, out + o, xin, last ? xmask : 0, st);
                nxt.push_back(out + o);
                nlen.push_back(sl.G);
                o += sl.G;
            }
            if (last) break;
            cur.swap(nxt);
            len.swap(nlen);
            xin = 0;  // interim levels hold flipped keys
            which ^= 1;
        }
        if (tmp[0]) cudaFreeAsync(tmp[0], st);
        if (tmp[1]) cudaFreeAsync(tmp[1], st);
        return e;
    }

    // splits[j*K + i] for every rank j (device arrays ptr, cnt, ranks, out).
    static cudaError_t split(const T* const* ptr, const uint64_t* cnt, int K, const uint64_t* ranks,
                             uint64_t n_ranks, uint64_t xmask, uint64_t* out, cudaStream_t st) {
        static const std::string n_rs = std::string("rank_split<") + TypeName<T>::v + ">";
        const int threads = ((K + 31) / 32) * 32;
        launch(n_rs.c_str(), st, [&] {
            rank_split_kernel<T><<<(unsigned)n_ranks, threads, 0, st>>>(ptr, cnt, K, ranks, xmask, out);
        });
        return cudaGetLastError();
    }
};

}  // namespace origami
