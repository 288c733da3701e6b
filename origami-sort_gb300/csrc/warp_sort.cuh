// Register and warp-shuffle sorting for keys-only items (the GPU form of the
// reference's in-register phase, sorter.h:30-1907: sorting networks over
// registers, then merges across registers).
//
// Each lane holds VT keys. warp_sort() sorts the lane's keys with a bitonic
// network, then merges lanes pairwise, by fours, ... up to the whole warp with
// bitonic merges whose cross-lane stages are __shfl_xor_sync exchanges. The
// result is the warp's 32*VT keys sorted in blocked order (lane l holds items
// l*VT .. l*VT+VT-1). No shared memory and no barriers are involved.
// `chunk` (a power of two) stops the process once runs of `chunk` keys are
// sorted, for chunked sorts.
#pragma once
#include "common.cuh"

namespace origami {

template <class T>
__device__ __forceinline__ T min_max_sel(T a, T b, bool keep_min) {
    const T lo = less(b, a) ? b : a;
    const T hi = less(b, a) ? a : b;
    return keep_min ? lo : hi;
}

// Bitonic sort of VT registers (every merged block ascending).
template <class T, int VT>
__device__ __forceinline__ void lane_sort(T (&v)[VT], int chunk) {
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

// Merges sorted runs of VT*g/2 keys held by half-groups of g/2 lanes into runs
// of VT*g keys (blocked over the g lanes of each group).
template <class T, int VT>
__device__ __forceinline__ void lane_group_merge(T (&v)[VT], int g) {
    const int lane = threadIdx.x & 31;
    // flip stage: item k of lane l meets item VT-1-k of lane l ^ (g-1)
    const bool lower = (lane & (g >> 1)) == 0;
    if constexpr (VT == 1) {
        const T a = __shfl_xor_sync(0xFFFFFFFFu, v[0], g - 1);
        v[0] = min_max_sel(v[0], a, lower);
    }
#pragma unroll
    for (int k = 0; k < VT / 2; ++k) {
        const T a = __shfl_xor_sync(0xFFFFFFFFu, v[VT - 1 - k], g - 1);
        const T b = __shfl_xor_sync(0xFFFFFFFFu, v[k], g - 1);
        v[k] = min_max_sel(v[k], a, lower);
        v[VT - 1 - k] = min_max_sel(v[VT - 1 - k], b, lower);
    }
    // half-cleaners across lanes
    for (int d = g >> 2; d >= 1; d >>= 1) {
        const bool lo = (lane & d) == 0;
#pragma unroll
        for (int k = 0; k < VT; ++k) {
            const T o = __shfl_xor_sync(0xFFFFFFFFu, v[k], d);
            v[k] = min_max_sel(v[k], o, lo);
        }
    }
    // half-cleaners inside the lane
#pragma unroll
    for (int s = VT / 2; s > 0; s >>= 1) {
#pragma unroll
        for (int i = 0; i < VT; ++i)
            if ((i & s) == 0) cx(v[i], v[i + s]);
    }
}

template <class T, int VT>
__device__ __forceinline__ void warp_sort(T (&v)[VT], int chunk) {
    lane_sort<T, VT>(v, chunk);
    for (int g = 2; g <= 32 && VT * g <= chunk; g <<= 1) lane_group_merge<T, VT>(v, g);
}

}  // namespace origami
