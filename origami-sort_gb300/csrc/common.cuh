// Shared device-side definitions: item traits, shared-memory layout and the
// merge primitives every kernel is built from.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace origami {

// 16-byte key-value item, same layout as the reference's packed
// KeyValue<i64,i64> (commons.h:51-72): key first, then value.
struct __align__(16) KV64 {
    uint64_t key;
    uint64_t value;
};

// Keys are compared as unsigned integers. Signed 64-bit keys (the reference's
// i64 and KeyValue<i64,i64>) are mapped onto the same order by flipping the sign
// bit when an item is first read from the caller's buffer and flipping it back
// when the final pass writes it: k -> k ^ 2^63 is an order-preserving bijection
// from int64 to uint64.
template <class T>
struct Traits;

template <>
struct Traits<uint32_t> {
    using Key = uint32_t;
    static constexpr bool kStable = false;  // keys only: equal items are identical
    static __host__ __device__ __forceinline__ Key key(uint32_t v) { return v; }
    static __device__ __forceinline__ uint32_t flip(uint32_t v, uint64_t x) { return v ^ (uint32_t)x; }
    static __device__ __forceinline__ uint32_t max_item() { return 0xFFFFFFFFu; }
};

template <>
struct Traits<uint64_t> {
    using Key = uint64_t;
    static constexpr bool kStable = false;
    static __host__ __device__ __forceinline__ Key key(uint64_t v) { return v; }
    static __device__ __forceinline__ uint64_t flip(uint64_t v, uint64_t x) { return v ^ x; }
    static __device__ __forceinline__ uint64_t max_item() { return ~0ull; }
};

template <>
struct Traits<KV64> {
    using Key = uint64_t;
    static constexpr bool kStable = true;  // values must keep their input order
    static __host__ __device__ __forceinline__ Key key(const KV64& v) { return v.key; }
    static __device__ __forceinline__ KV64 flip(KV64 v, uint64_t x) {
        v.key ^= x;
        return v;
    }
    static __device__ __forceinline__ KV64 max_item() { return KV64{~0ull, ~0ull}; }
};

template <class T>
__device__ __forceinline__ bool less(const T& a, const T& b) {
    return Traits<T>::key(a) < Traits<T>::key(b);
}

// Shared-memory index padding: one spare item after every 128 bytes, so that a
// warp storing VT consecutive items per thread (blocked layout, VT a power of
// two) hits distinct banks.
template <class T>
__host__ __device__ constexpr int pad_stride() {
    return 128 / (int)sizeof(T);
}
template <class T>
__host__ __device__ __forceinline__ int pad(int i) {
    return i + i / pad_stride<T>();
}
template <class T>
__host__ __device__ constexpr int padded_items(int n) {
    return n + n / pad_stride<T>() + 1;
}

// Compare-exchange into ascending order.
template <class T>
__device__ __forceinline__ void cx(T& a, T& b) {
    const bool sw = less(b, a);
    const T lo = sw ? b : a;
    const T hi = sw ? a : b;
    a = lo;
    b = hi;
}
template <>
__device__ __forceinline__ void cx<uint32_t>(uint32_t& a, uint32_t& b) {
    const uint32_t lo = min(a, b);
    b = max(a, b);
    a = lo;
}
template <>
__device__ __forceinline__ void cx<uint64_t>(uint64_t& a, uint64_t& b) {
    const uint64_t lo = min(a, b);
    b = max(a, b);
    a = lo;
}

// In-thread sort of VT register items, every aligned block of `chunk` items
// (chunk a power of two) sorted independently.
//  - keys only: bitonic network in the variant that leaves every merged block
//    ascending (first stage of each merge compares i with i^(k-1)), so the
//    network can stop at any block size;
//  - stable (key-value): odd-even transposition, which only swaps neighbours
//    that are strictly out of order and so keeps equal keys in input order.
template <class T, int VT, bool STABLE>
__device__ __forceinline__ void thread_sort(T (&v)[VT], int chunk) {
    if constexpr (STABLE) {
#pragma unroll
        for (int r = 0; r < VT; ++r) {
#pragma unroll
            for (int i = r & 1; i + 1 < VT; i += 2) {
                const bool same_chunk = (chunk >= VT) || (((i + 1) & (chunk - 1)) != 0);
                if (same_chunk && less(v[i + 1], v[i])) {
                    const T t = v[i];
                    v[i] = v[i + 1];
                    v[i + 1] = t;
                }
            }
        }
    } else {
#pragma unroll
        for (int k = 2; k <= VT; k <<= 1) {
            if (k <= chunk) {
#pragma unroll
                for (int i = 0; i < VT; ++i) {
                    const int j = i ^ (k - 1);
                    if (j > i) cx(v[i], v[j]);
                }
#pragma unroll
                for (int s = k >> 2; s > 0; s >>= 1) {
#pragma unroll
                    for (int i = 0; i < VT; ++i) {
                        const int j = i ^ s;
                        if (j > i) cx(v[i], v[j]);
                    }
                }
            }
        }
    }
}

// Merge path (Odeh et al., "Merge Path - parallel merging made simple") over two
// sorted lists in global memory, A[0 .. na) and B[0 .. nb): how many of the
// first `diag` merged items come from A, A winning ties (every merge is stable:
// A is always the earlier run). Used by the pass partition kernels, with a few
// interpolation steps before the bisection. When the bracket is wide (late
// passes: runs of millions of items), the two ends are probed together, then
// up to three steps each place a probe x by linear interpolation of
// g(i) = key(A[i]) - key(B[diag-1-i]), which rises with i, and two guard
// probes at x -+ d, d about twice the square root of the bracket (the spread
// of the interpolation's error on evenly spread keys). The three probes of a
// step are independent loads, one latency; the split lands between two of
// them, so both ends of the bracket move (a single probe moves only one, and
// the far end stays where it was). Bisection finishes the narrowed bracket.
// The chain of dependent global loads is the partition's whole latency: on
// uniform keys it falls from log2(run) to about eight, and on any other
// distribution the steps cost at most three latencies before a bisection of
// what is left. The split is the first i with g(i) > 0 (A[i] > B[diag-1-i]:
// equal keys go to A first); every decision is an exact integer compare, g
// (in float) only places probes.
// `interp` off: plain bisection (data that fits in L2, where each bisection
// step is a short L2 hit and the interpolation arithmetic does not pay).
template <class T>
__device__ __forceinline__ int64_t global_merge_path_interp(const T* A, int64_t na, const T* B, int64_t nb,
                                                            int64_t diag, bool interp = true) {
    int64_t lo = diag - nb > 0 ? diag - nb : 0;
    int64_t hi = diag < na ? diag : na;
    if (interp && hi - lo >= 4096) {
        const auto al = Traits<T>::key(A[lo]), bl = Traits<T>::key(B[diag - 1 - lo]);
        const auto ar = Traits<T>::key(A[hi - 1]), br = Traits<T>::key(B[diag - hi]);
        if (al > bl) return lo;     // the split is lo
        if (!(ar > br)) return hi;  // every candidate goes to A
        // g(xl) <= 0 < g(xr): the split is in (xl, xr]
        int64_t xl = lo, xr = hi - 1;
        float gl = (float)al - (float)bl, gr = (float)ar - (float)br;
#pragma unroll 1
        for (int step = 0; step < 3 && xr - xl > 64 && gr > gl; ++step) {
            const int64_t span = xr - xl;
            const float f = -gl / (gr - gl);
            int64_t x = xl + 1 + (int64_t)(f * (float)(span - 1));
            x = x < xl + 1 ? xl + 1 : (x > xr - 1 ? xr - 1 : x);
            int64_t d = (int64_t)(2.0f * sqrtf((float)span));
            d = d < 16 ? 16 : d;
            // xl < x0 <= x <= x2 < xr: every probe inside both lists
            const int64_t x0 = x - d > xl + 1 ? x - d : xl + 1;
            const int64_t x2 = x + d < xr - 1 ? x + d : xr - 1;
            const auto a0 = Traits<T>::key(A[x0]), b0 = Traits<T>::key(B[diag - 1 - x0]);
            const auto a1 = Traits<T>::key(A[x]), b1 = Traits<T>::key(B[diag - 1 - x]);
            const auto a2 = Traits<T>::key(A[x2]), b2 = Traits<T>::key(B[diag - 1 - x2]);
            // g rises with i: the first probe with g > 0 closes the bracket
            // on the right, the one before it on the left
            if (a0 > b0) {
                xr = x0;
                gr = (float)a0 - (float)b0;
            } else if (a1 > b1) {
                xl = x0;
                gl = (float)a0 - (float)b0;
                xr = x;
                gr = (float)a1 - (float)b1;
            } else if (a2 > b2) {
                xl = x;
                gl = (float)a1 - (float)b1;
                xr = x2;
                gr = (float)a2 - (float)b2;
            } else {
                xl = x2;
                gl = (float)a2 - (float)b2;
            }
        }
        lo = xl + 1;
        hi = xr;
    }
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (!less(B[diag - 1 - mid], A[mid]))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Items of run A that one merge tile takes: the tile covers outputs [d0, d0 +
// total) of the pair (A of la items, B of lb), s0 and a1 are the merge-path
// splits at its two ends (each from a bounded search, so s0 lies in [max(0,
// d0-lb), min(d0, la)]). For sorted runs the splits are consistent and a1 - s0
// is returned unchanged. Otherwise (runs that are not sorted) the count is
// clamped so that both slices lie inside their runs, and *bad is set: every
// access stays in bounds whatever the data.
__device__ __forceinline__ int tile_split(int64_t s0, int64_t a1, int64_t d0, int total, int64_t la, int64_t lb,
                                          bool* bad) {
    const int64_t na = a1 - s0;
    const int64_t lo = (int64_t)total - (lb - (d0 - s0));
    const int64_t hi = la - s0;
    int64_t c = na < lo ? lo : na;
    c = c > hi ? hi : c;
    c = c < 0 ? 0 : (c > total ? total : c);
    *bad = c != na;
    return (int)c;
}

// 16-byte vector view of items (all buffers the kernels touch are 16-byte
// aligned: the C ABI stages misaligned caller buffers through aligned scratch).
template <class T>
struct Vec {
    static constexpr int N = 16 / (int)sizeof(T);  // items per vector
};

// Asynchronous 16-byte global -> shared copy (cp.async.cg); both addresses
// 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit_all() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

// Stages items [p, p + cnt) of a 16-byte aligned global array `g` into shared
// memory with 16-byte copies: the enclosing aligned vectors are copied to
// `s` (16-byte aligned), and the first item lands at s[return value]. Reads at
// most one partial vector past either end, never outside the enclosing
// 16-byte chunks (so never across a page). All NT threads call it.
template <class T, int NT>
__device__ __forceinline__ int stage_vec(T* s, const T* g, uint64_t p, int cnt) {
    constexpr int V = Vec<T>::N;
    const int lead = (int)(p % V);
    const uint64_t p0 = p - lead;
    const int nv = (lead + cnt + V - 1) / V;
    for (int i = threadIdx.x; i < nv; i += NT) cp_async16(s + (size_t)i * V, g + p0 + (uint64_t)i * V);
    return lead;
}

}  // namespace origami
