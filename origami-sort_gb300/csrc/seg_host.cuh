// Host launcher of the batched segmented sort (segmented.cuh).
#pragma once
#include <string>

#include "profiler.h"
#include "segmented.cuh"

namespace origami {

// Grids of the strided kernels: every SM full (resident CTAs per SM x SMs).
template <class T>
struct SegGrids {
    int tile = 0, merge[2] = {0, 0}, part = 0;  // merge: per merge shape
};

template <class T>
const SegGrids<T>& seg_grids() {
    static const SegGrids<T> grids = [] {  // thread-safe static initialisation
        SegGrids<T> g;
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(seg_tile_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SegShape<T>::SMEM);
        cudaFuncSetAttribute(seg_merge_kernel<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)SegMergeShape<T, 0>::SMEM);
        cudaFuncSetAttribute(seg_merge_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)SegMergeShape<T, 1>::SMEM);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, seg_tile_kernel<T>, SegShape<T>::NTM, SegShape<T>::SMEM);
        const int tile = sms * (per > 0 ? per : 1);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, seg_merge_kernel<T, 0>, SegMergeCfg<T, 0>::NT,
                                                      SegMergeShape<T, 0>::SMEM);
        g.merge[0] = sms * (per > 0 ? per : 1);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, seg_merge_kernel<T, 1>, SegMergeCfg<T, 1>::NT,
                                                      SegMergeShape<T, 1>::SMEM);
        g.merge[1] = sms * (per > 0 ? per : 1);
        g.part = sms * 8;
        g.tile = tile;
        return g;
    }();
    return grids;
}

template <class T>
int seg_grid() {
    return seg_grids<T>().tile;
}

// Sorts every segment of d in place (result in d; tmp is the ping-pong
// buffer). off: device array of nseg+1 offsets, off[nseg] == n. shape: the
// level merges' merge shape (SegMergeCfg).
template <class T>
cudaError_t seg_sort(T* d, T* tmp, const uint64_t* off, uint64_t nseg, uint64_t n, uint64_t xmask,
                     void* scratch, int maxl, int shape, cudaStream_t st) {
    if (nseg == 0) return cudaSuccess;
    SegState s = seg_state<T>(scratch, off, n, nseg, maxl);
    s.spin = wait_limit();
    s.mtile = shape ? Config<T>::P2_TILE : Config<T>::P_TILE;
    const SegGrids<T>& g = seg_grids<T>();
    cudaMemsetAsync(s.err, 0, sizeof(int), st);
    const unsigned b = (unsigned)((nseg + 255) / 256);
    static const std::string n_plan = std::string("seg_plan<") + TypeName<T>::v + ">";
    static const std::string n_scan = std::string("seg_scan<") + TypeName<T>::v + ">";
    static const std::string n_fill = std::string("seg_fill<") + TypeName<T>::v + ">";
    static const std::string n_tile = std::string("seg_tile<") + TypeName<T>::v + ">";
    static const std::string n_part = std::string("seg_partition<") + TypeName<T>::v + ">";
    static const std::string n_merge = std::string("seg_merge<") + TypeName<T>::v + ">";
    launch(n_plan.c_str(), st, [&] { seg_plan_kernel<T><<<b, 256, 0, st>>>(s); });
    launch(n_scan.c_str(), st, [&] { seg_scan_kernel<T><<<(unsigned)(maxl + 1), 1024, 0, st>>>(s); });
    launch(n_fill.c_str(), st, [&] { seg_fill_kernel<T><<<b, 256, 0, st>>>(s); });
    launch(n_tile.c_str(), st, [&] {
        seg_tile_kernel<T><<<g.tile, SegShape<T>::NTM, SegShape<T>::SMEM, st>>>(s, d, tmp, xmask);
    });
    for (int l = 0; l < maxl; ++l) {
        launch(n_part.c_str(), st, [&] { seg_part_kernel<T><<<g.part, 256, 0, st>>>(s, l, d, tmp); });
        launch(n_merge.c_str(), st, [&] {
            if (shape)
                seg_merge_kernel<T, 1><<<g.merge[1], SegMergeCfg<T, 1>::NT, SegMergeShape<T, 1>::SMEM, st>>>(
                    s, l, d, tmp, xmask);
            else
                seg_merge_kernel<T, 0><<<g.merge[0], SegMergeCfg<T, 0>::NT, SegMergeShape<T, 0>::SMEM, st>>>(
                    s, l, d, tmp, xmask);
        });
    }
    return cudaGetLastError();
}

}  // namespace origami
