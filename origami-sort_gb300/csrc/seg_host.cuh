// Host launcher of the batched segmented sort (segmented.cuh).
#pragma once
#include <string>

#include "profiler.h"
#include "segmented.cuh"

namespace origami {

template <class T>
int seg_grid() {
    static int g = 0;
    if (g == 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(seg_persistent_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)SegShape<T>::SMEM);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, seg_persistent_kernel<T>, SegShape<T>::NT,
                                                      SegShape<T>::SMEM);
        g = sms * (per > 0 ? per : 1);
    }
    return g;
}

// Sorts every segment of d in place (result in d; tmp is the ping-pong
// buffer). off: device array of nseg+1 offsets, off[nseg] == n.
template <class T>
cudaError_t seg_sort(T* d, T* tmp, const uint64_t* off, uint64_t nseg, uint64_t n, uint64_t xmask,
                     void* scratch, int maxl, cudaStream_t st) {
    if (nseg == 0) return cudaSuccess;
    SegState s = seg_state<T>(scratch, off, n, nseg, maxl);
    cudaMemsetAsync(s.err, 0, sizeof(int), st);
    const unsigned b = (unsigned)((nseg + 255) / 256);
    static const std::string n_plan = std::string("seg_plan<") + TypeName<T>::v + ">";
    static const std::string n_scan = std::string("seg_scan<") + TypeName<T>::v + ">";
    static const std::string n_fill = std::string("seg_fill<") + TypeName<T>::v + ">";
    static const std::string n_run = std::string("seg_persistent<") + TypeName<T>::v + ">";
    launch(n_plan.c_str(), st, [&] { seg_plan_kernel<T><<<b, 256, 0, st>>>(s); });
    launch(n_scan.c_str(), st, [&] { seg_scan_kernel<T><<<(unsigned)(maxl + 2), 1024, 0, st>>>(s); });
    launch(n_fill.c_str(), st, [&] { seg_fill_kernel<T><<<b, 256, 0, st>>>(s); });
    const int grid = seg_grid<T>();
    launch(n_run.c_str(), st, [&] {
        seg_persistent_kernel<T><<<grid, SegShape<T>::NT, SegShape<T>::SMEM, st>>>(s, d, tmp, xmask);
    });
    return cudaGetLastError();
}

}  // namespace origami
