// Merge rounds in shared memory: the core step of the tile sort (K1) and of the
// k-way tile merge (K3).
//
// A round merges adjacent pairs of sorted lists (A_p, B_p) from `src` into
// `dst`, every pair writing its output over the positions it occupies. The
// output of a pair is cut into blocks of VT items and one thread owns a block:
// it finds where its block starts in A by merge path (Odeh et al.) and reads
// where it ends from the next block's search, so its outputs are exactly the
// merge of A[a0, a1) and B[b0, b1).
//
//  keys only  - the thread loads A[a0, a1) ascending and B[b0, b1) descending
//               into VT registers (a bitonic sequence; a short block is filled
//               with the largest key between the two parts) and sorts it with a
//               bitonic half-cleaner network: VT/2*log2(VT) compare-exchanges,
//               every load independent of the others;
//  stable     - (key-value items) the thread merges serially, A first on equal
//               keys, so equal keys keep their input order.
#pragma once
#include "common.cuh"

namespace origami {

// Bitonic half-cleaner sort of a bitonic register sequence into ascending order.
template <class T, int VT>
__device__ __forceinline__ void bitonic_clean(T (&v)[VT]) {
#pragma unroll
    for (int s = VT / 2; s > 0; s >>= 1) {
#pragma unroll
        for (int i = 0; i < VT; ++i)
            if ((i & s) == 0) cx(v[i], v[i + s]);
    }
}

// Merges one block: outputs [o, o + cnt) of the pair whose A part starts at
// ia0 - sa, taking na = ea - sa items from A (starting at ia0) and the rest from
// B (starting at ib0).
template <class T, int VT, bool STABLE>
__device__ __forceinline__ void merge_block(const T* src, T* dst, int ia0, int ib0, int na, int cnt,
                                            int o) {
    const int nb = cnt - na;
    if constexpr (STABLE) {
        int ia = ia0, ib = ib0;
        const int aEnd = ia0 + na, bEnd = ib0 + nb;
        T x = src[pad<T>(ia)];
        T y = src[pad<T>(ib)];
#pragma unroll
        for (int i = 0; i < VT; ++i) {
            if (i < cnt) {
                const bool takeA = (ib >= bEnd) || (ia < aEnd && !less(y, x));
                dst[pad<T>(o + i)] = takeA ? x : y;
                const int nxt = takeA ? ++ia : ++ib;
                const T vv = src[pad<T>(nxt)];
                x = takeA ? vv : x;
                y = takeA ? y : vv;
            }
        }
    } else {
        T v[VT];
#pragma unroll
        for (int i = 0; i < VT; ++i) {
            // [A ascending | largest key ... | B descending] is bitonic
            const bool fromA = i < na;
            const bool fromB = (VT - 1 - i) < nb;
            const int idx = fromA ? (ia0 + i) : (fromB ? ib0 + (VT - 1 - i) : ia0);
            const T t = src[pad<T>(idx)];
            v[i] = (fromA || fromB) ? t : Traits<T>::max_item();
        }
        bitonic_clean<T, VT>(v);
#pragma unroll
        for (int i = 0; i < VT; ++i)
            if (i < cnt) dst[pad<T>(o + i)] = v[i];
    }
}

// Round over pairs of equal width w (lists [2p*w, (2p+1)*w) and
// [(2p+1)*w, (2p+2)*w) within `total` items; the last pair may be short or
// absent). Used by the tile sort, where every list is a power-of-two run.
// `split` is shared scratch of total/VT + 1 ints.
template <class T, int NT, int VT, bool STABLE>
__device__ __forceinline__ void merge_round_uniform(const T* src, T* dst, int w, int total, int* split) {
    const int tid = threadIdx.x;
    const int nblk = (total + VT - 1) / VT;
    for (int blk = tid; blk < nblk; blk += NT) {
        const int o = blk * VT;
        const int a0 = o & ~(2 * w - 1);
        const int b0 = min(a0 + w, total), e0 = min(a0 + 2 * w, total);
        split[blk] = smem_merge_path(src, a0, b0 - a0, b0, e0 - b0, o - a0);
    }
    __syncthreads();
    for (int blk = tid; blk < nblk; blk += NT) {
        const int o = blk * VT;
        const int a0 = o & ~(2 * w - 1);
        const int b0 = min(a0 + w, total), e0 = min(a0 + 2 * w, total);
        const int diag = o - a0;
        const int cnt = min(VT, e0 - o);
        const int sa = split[blk];
        const int ea = (o + VT < e0) ? split[blk + 1] : (b0 - a0);
        merge_block<T, VT, STABLE>(src, dst, a0 + sa, b0 + (diag - sa), ea - sa, cnt, o);
    }
    __syncthreads();
}

// Round over pairs of arbitrary lists: list i is [off[i*stride], off[(i+1)*stride])
// and pair p = lists (2p, 2p+1), p < npairs <= MAXP. Blocks of VT outputs are
// numbered pair by pair. `split` is shared scratch of total/VT + npairs + 1 ints.
template <class T, int NT, int VT, int MAXP, bool STABLE>
__device__ __forceinline__ void merge_round_lists(const T* src, T* dst, const int* off, int stride,
                                                  int npairs, int* split) {
    const int tid = threadIdx.x;
    // bp[p] = first block of pair p (registers, unrolled)
    int bp[MAXP + 1];
    {
        int acc = 0;
#pragma unroll
        for (int p = 0; p < MAXP; ++p) {
            bp[p] = acc;
            if (p < npairs) acc += (off[(2 * p + 2) * stride] - off[(2 * p) * stride] + VT - 1) / VT;
        }
        bp[MAXP] = acc;
    }
    const int nblk = bp[MAXP];
    // pair of a block and the first block of that pair and of the next
    auto locate = [&](int blk, int& p, int& first, int& next) {
        p = 0;
        first = 0;
        next = bp[1];
#pragma unroll
        for (int q = 1; q < MAXP; ++q) {
            if (q < npairs && bp[q] <= blk) {
                p = q;
                first = bp[q];
                next = bp[q + 1];
            }
        }
    };
    for (int blk = tid; blk < nblk; blk += NT) {
        int p, first, next;
        locate(blk, p, first, next);
        const int a0 = off[(2 * p) * stride], b0 = off[(2 * p + 1) * stride];
        const int e0 = off[(2 * p + 2) * stride];
        split[blk] = smem_merge_path(src, a0, b0 - a0, b0, e0 - b0, (blk - first) * VT);
    }
    __syncthreads();
    for (int blk = tid; blk < nblk; blk += NT) {
        int p, first, next;
        locate(blk, p, first, next);
        const int a0 = off[(2 * p) * stride], b0 = off[(2 * p + 1) * stride];
        const int e0 = off[(2 * p + 2) * stride];
        const int diag = (blk - first) * VT;
        const int cnt = min(VT, e0 - a0 - diag);
        const int sa = split[blk];
        const int ea = (blk + 1 < next) ? split[blk + 1] : (b0 - a0);
        merge_block<T, VT, STABLE>(src, dst, a0 + sa, b0 + (diag - sa), ea - sa, cnt, a0 + diag);
    }
    __syncthreads();
}

// Merges `nl` (a power of two <= 2*MAXP) lists held back to back in `src`
// (list i = [off[i], off[i+1]), off[nl] = total) by log2(nl) rounds,
// ping-ponging with `dst`. Returns the buffer holding the result. The lower
// list wins ties in every round, so the result is ordered by (key, list).
template <class T, int NT, int VT, int MAXP, bool STABLE>
__device__ T* merge_lists(T* src, T* dst, const int* off, int nl, int* split) {
    for (int r = 0; (nl >> r) > 1; ++r) {
        merge_round_lists<T, NT, VT, MAXP, STABLE>(src, dst, off, 1 << r, nl >> (r + 1), split);
        T* t = src;
        src = dst;
        dst = t;
    }
    return src;
}

}  // namespace origami
