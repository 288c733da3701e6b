// Batched segmented sort: many independent arrays of uneven length, sorted by
// ONE persistent launch that pulls jobs from a device work queue.
//
// Segment s is items [off[s], off[s+1]) of the caller's buffer. Size classes:
//   warp    len <= 32*WVT      one warp sorts it in registers (warp_sort.cuh)
//   tile    len <= TILE        one CTA sorts it (register + shared-memory tile sort)
//   large   len >  TILE        ceil(len/TILE) tile jobs, then L = ceil(log2(tiles))
//                              binary merge levels of ceil(len/MT) merge jobs each
// Queue A holds CTA jobs in dependency order: every tile job first, then merge
// level 0 of every large segment, level 1, ... A merge job of level l may start
// once its segment has finished all tile jobs and levels < l (a per-segment
// completion counter). Jobs are handed out in increasing order and never
// depend on later ones, so every wait is for work already running on some
// CTA; waits are still bounded (clock budget, then an error flag and exit).
// Queue B holds the warp-class segments; warps take them once queue A is empty.
//
// The job lists are built on the device (plan -> per-class scans -> fill), so
// the whole batched call is a fixed sequence of launches and can be captured
// in a CUDA graph.
#pragma once
#include "common.cuh"
#include "merge_core.cuh"
#include "warp_sort.cuh"

namespace origami {

template <class T>
struct SegCfg;
template <>
struct SegCfg<uint32_t> {
    static constexpr int NW = 8, VT = 32;  // tile: 8 warps x 32 lanes x 32 keys = 8192
    static constexpr int TILE = NW * 32 * VT;
    static constexpr int MT = 8192;        // merge job output tile
    static constexpr bool WARP_CLASS = true;
    static constexpr bool STABLE = false;
};
template <>
struct SegCfg<uint64_t> {
    static constexpr int NW = 8, VT = 16;  // 4096
    static constexpr int TILE = NW * 32 * VT;
    static constexpr int MT = 4096;
    static constexpr bool WARP_CLASS = true;
    static constexpr bool STABLE = false;
};
template <>
struct SegCfg<KV64> {
    static constexpr int NW = 8, VT = 8;   // 2048, stable block sort
    static constexpr int TILE = NW * 32 * VT;
    static constexpr int MT = 2048;
    static constexpr bool WARP_CLASS = false;
    static constexpr bool STABLE = true;
};

template <class T>
inline int seg_levels_for(uint64_t len) {
    const uint64_t tiles = (len + SegCfg<T>::TILE - 1) / SegCfg<T>::TILE;
    int l = 0;
    while ((1ull << l) < tiles) ++l;
    return l;
}

// Device-resident plan and queue state (all pointers into one scratch block).
struct SegState {
    const uint64_t* off;   // [nseg+1] segment offsets (caller's)
    uint64_t n;            // items in the buffers: every segment must lie in [0, n)
    uint32_t nseg;
    int maxl;              // merge levels planned for
    uint32_t* cnt;         // [(maxl+2) * nseg] per-class job counts, then prefixes
    uint32_t* tot;         // [maxl+2] class totals: 0 = tile jobs, 1 = warp segs, 2+l = level l
    uint64_t* jobs;        // queue A: (segment << 32 | local index)
    uint32_t* wsegs;       // queue B: warp-class segment ids
    uint32_t* done;        // [nseg] finished CTA jobs per segment
    uint32_t* heads;       // [2] queue heads
    int* err;              // 1 = wait budget exhausted
};

template <class T>
struct SegGeom {
    uint64_t len;
    uint32_t tiles, levels, mjobs;
    int cls;  // 0 warp, 1 tile, 2 large
    // An invalid segment (decreasing offsets or past the buffer) is treated as
    // empty; the plan kernel reports it.
    __device__ __forceinline__ SegGeom(const uint64_t* off, uint32_t s, uint64_t n) {
        using C = SegCfg<T>;
        const uint64_t a = off[s], b = off[s + 1];
        len = (a <= b && b <= n) ? b - a : 0;
        tiles = (uint32_t)((len + C::TILE - 1) / C::TILE);
        levels = 0;
        while ((1ull << levels) < tiles) ++levels;
        mjobs = (uint32_t)((len + C::MT - 1) / C::MT);
        if (C::WARP_CLASS && len <= 32ull * C::VT)
            cls = 0;
        else if (len <= (uint64_t)C::TILE)
            cls = 1;
        else
            cls = 2;
    }
};

// 1. per segment: job counts of every class (cnt[q * nseg + s])
template <class T>
__global__ void seg_plan_kernel(SegState st) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= st.nseg) return;
    if (st.off[s + 1] < st.off[s] || st.off[s + 1] > st.n) atomicExch(st.err, 2);
    const SegGeom<T> g(st.off, s, st.n);
    const uint32_t n = st.nseg;
    st.cnt[0 * n + s] = (g.cls == 0) ? 0u : (g.cls == 1 ? 1u : g.tiles);
    st.cnt[1 * n + s] = (g.cls == 0) ? 1u : 0u;
    for (int l = 0; l < st.maxl; ++l) st.cnt[(2 + l) * n + s] = (g.cls == 2 && (uint32_t)l < g.levels) ? g.mjobs : 0u;
    st.done[s] = 0;
}

// 2. exclusive scan of one class per block (block q scans cnt[q*nseg ..]); the
//    class total goes to tot[q]. 1024 threads, chunked.
template <class T>
__global__ void __launch_bounds__(1024) seg_scan_kernel(SegState st) {
    __shared__ uint32_t part[1024];
    const uint32_t n = st.nseg;
    uint32_t* a = st.cnt + (size_t)blockIdx.x * n;
    const uint32_t chunk = (n + 1023) / 1024;
    const uint32_t b = threadIdx.x * chunk, e = min(n, b + chunk);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += a[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {  // inclusive Hillis-Steele scan of the partials
        const uint32_t v = threadIdx.x >= (unsigned)d ? part[threadIdx.x - d] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t acc = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (uint32_t i = b; i < e; ++i) {
        const uint32_t v = a[i];
        a[i] = acc;
        acc += v;
    }
    if (threadIdx.x == 1023) st.tot[blockIdx.x] = part[1023];
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st.heads[0] = 0;
        st.heads[1] = 0;
    }
}

// 3. fill the queues: queue A = [tile jobs | level 0 | level 1 | ...]
template <class T>
__global__ void seg_fill_kernel(SegState st) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= st.nseg) return;
    const SegGeom<T> g(st.off, s, st.n);
    const uint32_t n = st.nseg;
    if (g.cls == 0) {
        st.wsegs[st.cnt[1 * n + s]] = s;
        return;
    }
    uint64_t base = st.cnt[0 * n + s];
    const uint32_t nt = (g.cls == 1) ? 1u : g.tiles;
    for (uint32_t t = 0; t < nt; ++t) st.jobs[base + t] = ((uint64_t)s << 32) | t;
    uint64_t lvl_base = st.tot[0];
    for (int l = 0; l < st.maxl; ++l) {
        if (g.cls == 2 && (uint32_t)l < g.levels) {
            const uint64_t b = lvl_base + st.cnt[(2 + l) * n + s];
            for (uint32_t t = 0; t < g.mjobs; ++t) st.jobs[b + t] = ((uint64_t)s << 32) | t;
        }
        lvl_base += st.tot[2 + l];
    }
}

// ------------------------------------------------------ persistent kernel --
template <class T>
struct SegShape {
    using C = SegCfg<T>;
    static constexpr int NT = C::NW * 32;
    static constexpr int BUF = padded_items<T>(C::TILE + C::VT + 1);
    static constexpr size_t BUF_BYTES = (((size_t)BUF * sizeof(T)) + 15) & ~(size_t)15;
    static constexpr int V = Vec<T>::N;
    static constexpr int IN_CAP = C::MT + 4 * V + C::VT + 4;
    static constexpr size_t IN_BYTES = (((size_t)IN_CAP * sizeof(T)) + 15) & ~(size_t)15;
    static constexpr size_t SMEM = (2 * BUF_BYTES > IN_BYTES + BUF_BYTES) ? 2 * BUF_BYTES : IN_BYTES + BUF_BYTES;
    static constexpr int SPLITS = C::TILE / (C::VT - 1) + C::TILE / (2 * C::VT) + 8;
};

// bounded wait on a completion counter (thread 0 only)
__device__ __forceinline__ bool seg_wait(const uint32_t* ctr, uint32_t target, int* err) {
    const long long budget = 2000000000ll;  // ~1 s of SM clock
    const long long t0 = clock64();
    while (*(volatile const uint32_t*)ctr < target) {
        if (clock64() - t0 > budget || *(volatile int*)err) {
            atomicExch(err, 1);
            return false;
        }
        __nanosleep(200);
    }
    __threadfence();
    return true;
}

// Sorts items [p0, p0+cnt) of `src` (cnt <= TILE) into `dst` at the same
// positions: register/warp sort, then shared-memory rounds up to the tile.
template <class T>
__device__ void seg_tile_sort(const T* src, T* dst, uint64_t p0, int cnt, uint64_t xin, uint64_t xout,
                              unsigned char* smem, int* split) {
    using C = SegCfg<T>;
    using Sh = SegShape<T>;
    constexpr int NT = Sh::NT, VT = C::VT, TILE = C::TILE, WT = 32 * VT;
    T* sa = reinterpret_cast<T*>(smem);
    T* sb = reinterpret_cast<T*>(smem + Sh::BUF_BYTES);
    const int tid = threadIdx.x;
#pragma unroll
    for (int k = 0; k < VT; ++k) {
        const int i = k * NT + tid;
        sa[pad<T>(i)] = (i < cnt) ? Traits<T>::flip(src[p0 + i], xin) : Traits<T>::max_item();
    }
    __syncthreads();
    // the sorted span: the smallest power of two >= cnt (at least one warp run)
    int span = WT;
    while (span < cnt) span <<= 1;
    if constexpr (C::STABLE) {
        T v[VT];
#pragma unroll
        for (int k = 0; k < VT; ++k) v[k] = sa[pad<T>(tid * VT + k)];
        thread_sort<T, VT, true>(v, VT);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < VT; ++k) sa[pad<T>(tid * VT + k)] = v[k];
        __syncthreads();
        merge_round_uniform<T, NT, VT - 1, true, PadIdx<T>>(sa, sb, VT, TILE, split);
        T* s0 = sb;
        T* s1 = sa;
        for (int w = 2 * VT; w < TILE && w < span; w <<= 1) {
            merge_round_uniform<T, NT, VT - 1, true, LinIdx>(s0, s1, w, TILE, split);
            T* t = s0;
            s0 = s1;
            s1 = t;
        }
        for (int i = tid; i < cnt; i += NT) dst[p0 + i] = Traits<T>::flip(s0[i], xout);
    } else {
        const int lane = tid & 31, w0 = (tid >> 5) * WT;
        T v[VT];
#pragma unroll
        for (int k = 0; k < VT; ++k) v[k] = sa[pad<T>(w0 + lane * VT + k)];
        warp_sort<T, VT>(v, WT);
        __syncwarp();
#pragma unroll
        for (int k = 0; k < VT; ++k) sa[pad<T>(w0 + lane * VT + k)] = v[k];
        __syncthreads();
        if (span > WT) {
            merge_round_uniform<T, NT, VT, false, PadIdx<T>>(sa, sb, WT, TILE, split);
            T* s0 = sb;
            T* s1 = sa;
            for (int w = 2 * WT; w < span; w <<= 1) {
                merge_round_uniform<T, NT, VT, false, LinIdx>(s0, s1, w, TILE, split);
                T* t = s0;
                s0 = s1;
                s1 = t;
            }
            for (int i = tid; i < cnt; i += NT) dst[p0 + i] = Traits<T>::flip(s0[i], xout);
        } else {
            for (int i = tid; i < cnt; i += NT) dst[p0 + i] = Traits<T>::flip(sa[pad<T>(i)], xout);
        }
    }
}

// One warp sorts a whole segment of len <= 32*VT keys in registers.
template <class T, int VT>
__device__ __forceinline__ void seg_warp_sort(T* d, uint64_t base, int len, uint64_t xmask) {
    const int lane = threadIdx.x & 31;
    T v[VT];
#pragma unroll
    for (int k = 0; k < VT; ++k) {
        const int i = lane * VT + k;
        v[k] = (i < len) ? Traits<T>::flip(d[base + i], xmask) : Traits<T>::max_item();
    }
    warp_sort<T, VT>(v, 32 * VT);
#pragma unroll
    for (int k = 0; k < VT; ++k) {
        const int i = lane * VT + k;
        if (i < len) d[base + i] = Traits<T>::flip(v[k], xmask);
    }
}

template <class T>
__global__ void __launch_bounds__(SegShape<T>::NT) seg_persistent_kernel(SegState st, T* d, T* tmp,
                                                                        uint64_t xmask) {
    using C = SegCfg<T>;
    using Sh = SegShape<T>;
    constexpr int NT = Sh::NT, V = Sh::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int split[Sh::SPLITS];
    __shared__ uint64_t job_s;
    __shared__ int ok_s;
    __shared__ int64_t msplit[2];
    const int tid = threadIdx.x;
    const uint32_t nA = st.tot[0] + [&] {
        uint32_t t = 0;
        for (int l = 0; l < st.maxl; ++l) t += st.tot[2 + l];
        return t;
    }();

    // ---------------- queue A: CTA jobs
    for (;;) {
        if (tid == 0) {
            const uint32_t j = atomicAdd(&st.heads[0], 1u);
            job_s = (j < nA && !*(volatile int*)st.err) ? ((uint64_t)j | (1ull << 63)) : 0ull;
        }
        __syncthreads();
        const uint64_t jw = job_s;
        __syncthreads();
        if (!(jw >> 63)) break;
        const uint32_t j = (uint32_t)jw;
        const uint64_t e = st.jobs[j];
        const uint32_t s = (uint32_t)(e >> 32), t = (uint32_t)e;
        const SegGeom<T> g(st.off, s, st.n);
        const uint64_t base = st.off[s];
        // buffer holding level l's input: tiles write to `first`, so the last
        // level (or the tile sort itself) lands in d
        T* first = (g.levels % 2 == 0) ? d : tmp;
        if (j < st.tot[0]) {
            // tile job: sort tile t of segment s (or the whole segment)
            const uint64_t p0 = base + (uint64_t)t * C::TILE;
            const int cnt = (int)min((uint64_t)C::TILE, g.len - (uint64_t)t * C::TILE);
            const bool last = (g.levels == 0);
            seg_tile_sort<T>(d, first, p0, cnt, xmask, last ? xmask : 0, smem_raw, split);
        } else {
            // merge job: level l, output tile t
            int l = 0;
            uint32_t acc = st.tot[0];
            while (l + 1 < st.maxl && j >= acc + st.tot[2 + l]) acc += st.tot[2 + l++];
            if (tid == 0) ok_s = seg_wait(&st.done[s], g.tiles + (uint32_t)l * g.mjobs, st.err);
            __syncthreads();
            if (!ok_s) break;
            const T* src = ((l & 1) == 0) ? first : (first == d ? tmp : d);
            T* dst = (src == d) ? tmp : d;
            const uint64_t run = (uint64_t)C::TILE << l;
            const uint64_t o = (uint64_t)t * C::MT;
            const uint64_t pb = (o / (2 * run)) * (2 * run);
            const uint64_t la = min(run, g.len - pb);
            const uint64_t lb = min(run, g.len - pb - la);
            const uint64_t d0 = o - pb;
            const uint64_t d1 = min(d0 + (uint64_t)C::MT, la + lb);
            const T* A = src + base + pb;
            const T* B = A + la;
            const int wid = tid >> 5;
            if (wid < 2) {
                const int64_t r = warp_merge_path(A, (int64_t)la, B, (int64_t)lb, (int64_t)(wid ? d1 : d0));
                if ((tid & 31) == 0) msplit[wid] = r;
            }
            __syncthreads();
            const int64_t a0 = msplit[0], a1 = msplit[1];
            const int na = (int)(a1 - a0);
            const int total = (int)(d1 - d0);
            const int nb = total - na;
            T* sin = reinterpret_cast<T*>(smem_raw);
            T* sout = reinterpret_cast<T*>(smem_raw + Sh::IN_BYTES);
            const int a_lead = stage_vec<T, NT>(sin, src, base + pb + (uint64_t)a0, na);
            const int b_base = ((a_lead + na + V - 1) / V) * V;
            const int b_lead = stage_vec<T, NT>(sin + b_base, src, base + pb + la + (d0 - (uint64_t)a0), nb);
            cp_async_commit_all();
            cp_async_wait_all();
            __syncthreads();
            merge_pair_round<T, NT, C::STABLE ? C::VT - 1 : C::VT, C::STABLE>(sin, a_lead, na, b_base + b_lead,
                                                                               nb, sout, split);
            const uint64_t xo = ((uint32_t)l + 1 == g.levels) ? xmask : 0;
            T* op = dst + base + o;
            for (int i = tid; i < total; i += NT) op[i] = Traits<T>::flip(sout[i], xo);
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicAdd(&st.done[s], 1u);
        }
    }

    // ---------------- queue B: warp-class segments, one warp each
    if constexpr (C::WARP_CLASS) {
        const int lane = tid & 31;
        const uint32_t nB = st.tot[1];
        for (;;) {
            uint32_t j = 0;
            if (lane == 0) j = atomicAdd(&st.heads[1], 1u);
            j = __shfl_sync(0xFFFFFFFFu, j, 0);
            if (j >= nB) break;
            const uint32_t s = st.wsegs[j];
            const uint64_t base = st.off[s];
            const int len = (int)SegGeom<T>(st.off, s, st.n).len;
            // smallest lane width that holds the segment
            if (len <= 32 * 1)
                seg_warp_sort<T, 1>(d, base, len, xmask);
            else if (len <= 32 * 2)
                seg_warp_sort<T, 2>(d, base, len, xmask);
            else if (len <= 32 * 4)
                seg_warp_sort<T, 4>(d, base, len, xmask);
            else if (len <= 32 * 8)
                seg_warp_sort<T, 8>(d, base, len, xmask);
            else if (len <= 32 * 16)
                seg_warp_sort<T, 16>(d, base, len, xmask);
            else if constexpr (C::VT >= 32)
                seg_warp_sort<T, 32>(d, base, len, xmask);
        }
    }
}

}  // namespace origami

namespace origami {

// Upper bound of queue A's length for nseg segments of n items in total.
template <class T>
inline uint64_t seg_max_jobs(uint64_t n, uint64_t nseg, int maxl) {
    using C = SegCfg<T>;
    return (n / C::TILE + nseg) + (uint64_t)maxl * (n / C::MT + nseg) + 16;
}

// Scratch bytes for the plan and queues.
template <class T>
inline uint64_t seg_scratch_bytes(uint64_t n, uint64_t nseg, int maxl) {
    const uint64_t q = (uint64_t)maxl + 2;
    uint64_t b = 0;
    b += ((q * nseg * 4 + 255) & ~255ull);              // cnt
    b += ((q * 4 + 255) & ~255ull);                     // tot
    b += ((seg_max_jobs<T>(n, nseg, maxl) * 8 + 255) & ~255ull);  // jobs
    b += ((nseg * 4 + 255) & ~255ull);                  // wsegs
    b += ((nseg * 4 + 255) & ~255ull);                  // done
    b += 256;                                           // heads, err
    return b;
}

template <class T>
inline SegState seg_state(void* scratch, const uint64_t* off, uint64_t n, uint64_t nseg, int maxl) {
    SegState s;
    const uint64_t q = (uint64_t)maxl + 2;
    char* p = static_cast<char*>(scratch);
    auto take = [&](uint64_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~255ull;
        return r;
    };
    s.off = off;
    s.n = n;
    s.nseg = (uint32_t)nseg;
    s.maxl = maxl;
    s.cnt = reinterpret_cast<uint32_t*>(take(q * nseg * 4));
    s.tot = reinterpret_cast<uint32_t*>(take(q * 4));
    s.jobs = reinterpret_cast<uint64_t*>(take(seg_max_jobs<T>(n, nseg, maxl) * 8));
    s.wsegs = reinterpret_cast<uint32_t*>(take(nseg * 4));
    s.done = reinterpret_cast<uint32_t*>(take(nseg * 4));
    char* tail = take(256);
    s.heads = reinterpret_cast<uint32_t*>(tail);
    s.err = reinterpret_cast<int*>(tail + 16);
    return s;
}

}  // namespace origami
