// Merge rounds in shared memory: the core step of the tile sort (K1) and of the
// k-way tile merge (K3).
//
// A round merges adjacent pairs of sorted lists (A_p, B_p) from `src` into
// `dst`; every pair writes its output over the positions it occupies. A pair's
// output is cut into blocks of VO items and one thread owns a block: it finds
// where its block starts in A by merge path (Odeh et al.) and reads where it
// ends from the next block's search, so its outputs are exactly the merge of
// A[a0, a1) and B[b0, b1).
//
//  keys only  - VO = VT - 1. The thread loads A[a0, a1) ascending, then the
//               largest key, then B[b0, b1) descending into VT registers (a
//               bitonic sequence) and sorts it with a bitonic half-cleaner
//               network (VT/2*log2(VT) compare-exchanges); the loads are
//               independent of each other.
//  stable     - (key-value items) VO = VT. The thread merges serially, A first
//               on equal keys, so equal keys keep their input order.
//
// Buffers are unpadded. VO is odd, so the blocks of the 32 threads of a warp
// start 31 (or 7, 15) items apart and their stores fall on different banks.
// A source may instead use the padded layout (one spare slot per 32 items),
// which the tile sort uses once, for the blocked store after its register sort.
#pragma once
#include "common.cuh"

namespace origami {

// Index maps of a source buffer.
struct LinIdx {
    static __device__ __forceinline__ int at(int i) { return i; }
};
template <class T>
struct PadIdx {
    static __device__ __forceinline__ int at(int i) { return pad<T>(i); }
};

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

template <class T, int VT, bool STABLE>
struct Block {
    static constexpr int VO = STABLE ? VT : VT - 1;  // outputs per block
};

// Merge path on a source with index map IX.
template <class T, class IX>
__device__ __forceinline__ int merge_path_ix(const T* s, int a0, int na, int b0, int nb, int diag) {
    int lo = max(0, diag - nb);
    int hi = min(diag, na);
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const T a = s[IX::at(a0 + mid)];
        const T b = s[IX::at(b0 + diag - 1 - mid)];
        if (!less(b, a))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Merges one block: cnt outputs at dst[o..], na of them from A starting at
// src index ia0, the rest from B starting at ib0.
template <class T, int VT, bool STABLE, class IX>
__device__ __forceinline__ void merge_block(const T* src, T* dst, int ia0, int ib0, int na, int cnt,
                                            int o) {
    const int nb = cnt - na;
    if constexpr (STABLE) {
        int ia = ia0, ib = ib0;
        const int aEnd = ia0 + na, bEnd = ib0 + nb;
        T x = src[IX::at(ia)];
        T y = src[IX::at(ib)];
#pragma unroll
        for (int i = 0; i < VT; ++i) {
            if (i < cnt) {
                const bool takeA = (ib >= bEnd) || (ia < aEnd && !less(y, x));
                dst[o + i] = takeA ? x : y;
                const int nxt = takeA ? ++ia : ++ib;
                const T vv = src[IX::at(nxt)];
                x = takeA ? vv : x;
                y = takeA ? y : vv;
            }
        }
    } else {
        T v[VT];
        const int pb = ib0 + VT - 1;  // B is read backwards: slot i holds B[pb - i]
#pragma unroll
        for (int i = 0; i < VT; ++i) {
            const bool fromA = i < na;
            const T t = src[IX::at(fromA ? ia0 + i : pb - i)];
            // slots between the A part and the B part hold the largest key
            v[i] = (fromA || i >= VT - nb) ? t : Traits<T>::max_item();
        }
        bitonic_clean<T, VT>(v);
        if (cnt == VT - 1) {
#pragma unroll
            for (int i = 0; i < VT - 1; ++i) dst[o + i] = v[i];
        } else {
#pragma unroll
            for (int i = 0; i < VT - 1; ++i)
                if (i < cnt) dst[o + i] = v[i];
        }
    }
}

// merge_block into registers: out[0 .. cnt) receive the block's outputs, so
// that the caller can overwrite the source buffer once every thread is done
// reading it.
template <class T, int VT, bool STABLE>
__device__ __forceinline__ void merge_block_regs(const T* src, int ia0, int ib0, int na, int cnt, T (&out)[VT]) {
    const int nb = cnt - na;
    if constexpr (STABLE) {
        int ia = ia0, ib = ib0;
        const int aEnd = ia0 + na, bEnd = ib0 + nb;
        T x = src[ia];
        T y = src[ib];
#pragma unroll
        for (int i = 0; i < VT; ++i) {
            if (i < cnt) {
                const bool takeA = (ib >= bEnd) || (ia < aEnd && !less(y, x));
                out[i] = takeA ? x : y;
                const int nxt = takeA ? ++ia : ++ib;
                const T vv = src[nxt];
                x = takeA ? vv : x;
                y = takeA ? y : vv;
            }
        }
    } else {
        const int pb = ib0 + VT - 1;  // B is read backwards: slot i holds B[pb - i]
#pragma unroll
        for (int i = 0; i < VT; ++i) {
            const bool fromA = i < na;
            const T t = src[fromA ? ia0 + i : pb - i];
            out[i] = (fromA || i >= VT - nb) ? t : Traits<T>::max_item();
        }
        bitonic_clean<T, VT>(out);
    }
}

// Round over pairs of equal width w inside `total` items (the last pair may be
// short or absent): the tile sort's rounds. `split` is shared scratch of
// blocks + 1 ints, blocks = ceil(total / VO) + total / (2w) + 1.
template <class T, int NT, int VT, bool STABLE, class IX>
__device__ __forceinline__ void merge_round_uniform(const T* src, T* dst, int w, int total, int* split) {
    constexpr int VO = Block<T, VT, STABLE>::VO;
    const int tid = threadIdx.x;
    const int bpp = (2 * w + VO - 1) / VO;  // blocks per full pair
    const int npairs = (total + 2 * w - 1) / (2 * w);
    const int nblk = npairs * bpp;
    for (int blk = tid; blk < nblk; blk += NT) {
        const int p = blk / bpp;
        const int a0 = p * 2 * w;
        const int b0 = min(a0 + w, total), e0 = min(a0 + 2 * w, total);
        const int diag = min((blk - p * bpp) * VO, e0 - a0);
        split[blk] = merge_path_ix<T, IX>(src, a0, b0 - a0, b0, e0 - b0, diag);
    }
    __syncthreads();
    for (int blk = tid; blk < nblk; blk += NT) {
        const int p = blk / bpp;
        const int a0 = p * 2 * w;
        const int b0 = min(a0 + w, total), e0 = min(a0 + 2 * w, total);
        const int diag = (blk - p * bpp) * VO;
        const int cnt = min(VO, e0 - a0 - diag);
        if (cnt <= 0) continue;
        const int sa = split[blk];
        const int ea = (blk + 1 < (p + 1) * bpp) ? split[blk + 1] : (b0 - a0);
        merge_block<T, VT, STABLE, IX>(src, dst, a0 + sa, b0 + (diag - sa), ea - sa, cnt, a0 + diag);
    }
    __syncthreads();
}

// Round over pairs of arbitrary lists: list i is [off[i*stride], off[(i+1)*stride])
// and pair p = lists (2p, 2p+1), p < npairs <= MAXP. Blocks are numbered pair by
// pair. `split` is shared scratch of total/VO + npairs + 1 ints.
template <class T, int NT, int VT, int MAXP, bool STABLE, class IX>
__device__ __forceinline__ void merge_round_lists(const T* src, T* dst, const int* off, int stride,
                                                  int npairs, int* split) {
    constexpr int VO = Block<T, VT, STABLE>::VO;
    const int tid = threadIdx.x;
    int bp[MAXP + 1];  // first block of each pair (registers, unrolled)
    {
        int acc = 0;
#pragma unroll
        for (int p = 0; p < MAXP; ++p) {
            bp[p] = acc;
            if (p < npairs) acc += (off[(2 * p + 2) * stride] - off[(2 * p) * stride] + VO - 1) / VO;
        }
        bp[MAXP] = acc;
    }
    const int nblk = bp[MAXP];
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
        split[blk] = merge_path_ix<T, IX>(src, a0, b0 - a0, b0, e0 - b0, (blk - first) * VO);
    }
    __syncthreads();
    for (int blk = tid; blk < nblk; blk += NT) {
        int p, first, next;
        locate(blk, p, first, next);
        const int a0 = off[(2 * p) * stride], b0 = off[(2 * p + 1) * stride];
        const int e0 = off[(2 * p + 2) * stride];
        const int diag = (blk - first) * VO;
        const int cnt = min(VO, e0 - a0 - diag);
        const int sa = split[blk];
        const int ea = (blk + 1 < next) ? split[blk + 1] : (b0 - a0);
        merge_block<T, VT, STABLE, IX>(src, dst, a0 + sa, b0 + (diag - sa), ea - sa, cnt, a0 + diag);
    }
    __syncthreads();
}

// One merge round over a single pair that writes its output over its own
// input: `buf` holds A at [as, as+na) and B at [bs, bs+nb) and receives the
// merge at [0, na+nb).
// Every thread owns at most one block (NT * VO >= na + nb), keeps it in
// registers while the others read, then stores it. The output may therefore
// share the input's shared memory, which halves the footprint of a tile.
template <class T, int NT, int VT, bool STABLE>
__device__ __forceinline__ void merge_pair_round_inplace(T* buf, int as, int na, int bs, int nb, int* split) {
    constexpr int VO = Block<T, VT, STABLE>::VO;
    const int tid = threadIdx.x;
    const int total = na + nb;
    const int nblk = (total + VO - 1) / VO;
    if (tid < nblk) split[tid] = merge_path_ix<T, LinIdx>(buf, as, na, bs, nb, tid * VO);
    __syncthreads();
    T r[VT];
    const int diag = tid * VO;
    const int cnt = tid < nblk ? min(VO, total - diag) : 0;
    if (tid < nblk) {
        const int sa = split[tid];
        const int ea = (tid + 1 < nblk) ? split[tid + 1] : na;
        merge_block_regs<T, VT, STABLE>(buf, as + sa, bs + (diag - sa), ea - sa, cnt, r);
    }
    __syncthreads();
    if (cnt == VO) {
#pragma unroll
        for (int i = 0; i < VO; ++i) buf[diag + i] = r[i];
    } else {
#pragma unroll
        for (int i = 0; i < VO; ++i)
            if (i < cnt) buf[diag + i] = r[i];
    }
    __syncthreads();
}

// Merges `nl` (a power of two <= 2*MAXP) lists held back to back in `src`
// (list i = [off[i], off[i+1]), off[nl] = total) by log2(nl) rounds,
// ping-ponging with `dst` (both unpadded). Returns the buffer holding the
// result. The lower list wins ties in every round, so the result is ordered by
// (key, list).
template <class T, int NT, int VT, int MAXP, bool STABLE>
__device__ T* merge_lists(T* src, T* dst, const int* off, int nl, int* split) {
    for (int r = 0; (nl >> r) > 1; ++r) {
        merge_round_lists<T, NT, VT, MAXP, STABLE, LinIdx>(src, dst, off, 1 << r, nl >> (r + 1), split);
        T* t = src;
        src = dst;
        dst = t;
    }
    return src;
}

}  // namespace origami
