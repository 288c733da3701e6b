// Batched segmented sort: many independent arrays of uneven length, sorted
// together, level by level, with the plain sort's tile bodies.
//
// Segment s is items [off[s], off[s+1]) of the caller's buffer d. With T1 the
// tile of the first kernel (8192 / 4096 / 2048 items) and MT the merge tile
// of a binary pass (pipeline.cuh):
//   tile phase   every segment is cut into ceil(len / T1) tiles (a short
//                segment is one partial tile); one CTA sorts a tile in
//                registers and shared memory;
//   level l      every segment longer than T1 << l merges its runs of
//                T1 << l pairwise: a partition kernel finds each output tile's
//                merge-path split, a merge kernel merges the tiles (the
//                binary-pass merge body: shared-memory staging, output written
//                over the input, one block per thread).
// A segment with L levels alternates between d and tmp so that its last step
// writes d: its tiles go to tmp when L is odd.
//
// Each kernel is launched once per phase or level for all segments together,
// with a fixed grid that strides over that phase's job list. The job lists are
// counted on the device (plan, then one prefix scan per list), so the host
// never waits and the whole sequence can be captured in a CUDA graph. A level
// that no segment needs finds an empty list and returns at once.
#pragma once
#include "common.cuh"
#include "merge_core.cuh"
#include "pipeline.cuh"
#include "warp_sort.cuh"

namespace origami {

template <class T>
struct SegCfg;
template <>
struct SegCfg<uint32_t> {
    static constexpr int NW = 8, VT = 32;  // tile: 8 warps x 32 lanes x 32 keys = 8192
    static constexpr int TILE = NW * 32 * VT;
    static constexpr bool STABLE = false;
    static constexpr int VTM = VT;  // (stable rounds only)
    static constexpr int NWT = 9;  // warps in the shared-memory rounds (one merge block per thread)
    static constexpr int TILE_MINB = 3, MERGE_MINB = 8;  // CTAs per SM the register budget allows
};
template <>
struct SegCfg<uint64_t> {
    static constexpr int NW = 8, VT = 16;  // 4096
    static constexpr int TILE = NW * 32 * VT;
    static constexpr bool STABLE = false;
    static constexpr int VTM = VT;
    static constexpr int NWT = 9;
    static constexpr int TILE_MINB = 2, MERGE_MINB = 8;
};
template <>
struct SegCfg<KV64> {
    static constexpr int NW = 8, VT = 8;  // 2048, stable block sort
    static constexpr int TILE = NW * 32 * VT;
    static constexpr bool STABLE = true;
    static constexpr int VTM = 11;  // serial merge blocks of the shared-memory rounds
    static constexpr int NWT = 8;
    static constexpr int TILE_MINB = 3, MERGE_MINB = 6;
};

// Merge levels for a segment of len items (runs of TILE doubled until one).
template <class T>
__host__ __device__ inline int seg_levels_for(uint64_t len) {
    const uint64_t tiles = (len + SegCfg<T>::TILE - 1) / SegCfg<T>::TILE;
    int l = 0;
    while ((1ull << l) < tiles) ++l;
    return l;
}

// Device-resident plan (all pointers into one scratch block).
struct SegState {
    const uint64_t* off;  // [nseg+1] segment offsets (caller's)
    uint64_t n;           // items in the buffers: every segment must lie in [0, n)
    uint32_t nseg;
    int maxl;             // merge levels planned for
    uint32_t* cnt;        // [(maxl+1) * nseg] jobs per segment: row 0 tiles, row 1+l
                          // level-l merge tiles; exclusive prefixes after the scan
    uint32_t* tot;        // [maxl+1] jobs per row
    int64_t* splits;      // merge-path split of each merge tile of the current level
    uint32_t* segof;      // segment of each merge tile of the current level
    uint32_t* tileseg;    // segment of each tile job
    int* err;             // 2 = bad offsets
};

template <class T>
struct SegGeom {
    uint64_t len;
    uint32_t tiles, levels, mtiles;
    // An invalid segment (decreasing offsets or past the buffer) is treated as
    // empty; the plan kernel reports it.
    __device__ __forceinline__ SegGeom(const uint64_t* off, uint32_t s, uint64_t n) {
        const uint64_t a = off[s], b = off[s + 1];
        len = (a <= b && b <= n) ? b - a : 0;
        tiles = (uint32_t)((len + SegCfg<T>::TILE - 1) / SegCfg<T>::TILE);
        levels = (uint32_t)seg_levels_for<T>(len);
        mtiles = (uint32_t)((len + Config<T>::P_TILE - 1) / Config<T>::P_TILE);
    }
};

// The segment whose job range [pref[s], pref[s] + cnt[s]) holds job j
// (segments without jobs have empty ranges and are skipped).
__device__ __forceinline__ uint32_t seg_of_job(const uint32_t* pref, uint32_t nseg, uint32_t j) {
    uint32_t a = 0, e = nseg;
    while (a < e) {
        const uint32_t m = (a + e) >> 1;
        if (pref[m] <= j)
            a = m + 1;
        else
            e = m;
    }
    return a - 1;
}

// Buffer a segment with L levels holds after step k (0 = tile phase).
template <class T>
__device__ __forceinline__ T* seg_buf(uint32_t L, uint32_t k, T* d, T* tmp) {
    return ((L - k) & 1) ? tmp : d;
}

// 1. per segment: jobs of every row
template <class T>
__global__ void seg_plan_kernel(SegState st) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= st.nseg) return;
    if (st.off[s + 1] < st.off[s] || st.off[s + 1] > st.n) atomicExch(st.err, 2);
    const SegGeom<T> g(st.off, s, st.n);
    const uint32_t n = st.nseg;
    st.cnt[s] = g.tiles;
    for (int l = 0; l < st.maxl; ++l) st.cnt[(1 + l) * (size_t)n + s] = ((uint32_t)l < g.levels) ? g.mtiles : 0u;
}

// 2. exclusive scan of one row per block (block q scans row q); the row total
//    goes to tot[q]. 1024 threads, chunked.
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
}

// 3. the segment of every tile job (one thread per segment)
template <class T>
__global__ void seg_fill_kernel(SegState st) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= st.nseg) return;
    const SegGeom<T> g(st.off, s, st.n);
    const uint32_t b = st.cnt[s];
    for (uint32_t t = 0; t < g.tiles; ++t) st.tileseg[b + t] = s;
}

// ------------------------------------------------------------ tile phase --
template <class T>
struct SegShape {
    using C = SegCfg<T>;
    static constexpr int NT = C::NW * 32;   // threads that load and sort in registers
    static constexpr int NTM = C::NWT * 32; // threads of the CTA (all take part in the rounds)
    static constexpr int BUF = padded_items<T>(C::TILE + C::VT + 1);
    static constexpr size_t BUF_BYTES = (((size_t)BUF * sizeof(T)) + 15) & ~(size_t)15;
    static constexpr size_t SMEM = 2 * BUF_BYTES;
    static constexpr int VO = C::STABLE ? C::VTM : C::VT - 1;  // outputs per merge block of the rounds
    static constexpr int SPLITS = C::TILE / VO + C::TILE / (2 * C::VT) + 8;
};

// Sorts items [p0, p0+cnt) of `src` (cnt <= TILE) into `dst` at the same
// positions: register/warp sort, then shared-memory rounds up to the tile.
// Any alignment of p0: loads and stores are plain and coalesced.
template <class T>
__device__ void seg_tile_sort(const T* src, T* dst, uint64_t p0, int cnt, uint64_t xin, uint64_t xout,
                              unsigned char* smem, int* split) {
    using C = SegCfg<T>;
    using Sh = SegShape<T>;
    constexpr int NT = Sh::NT, NTM = Sh::NTM, VT = C::VT, TILE = C::TILE, WT = 32 * VT;
    T* sa = reinterpret_cast<T*>(smem);
    T* sb = reinterpret_cast<T*>(smem + Sh::BUF_BYTES);
    const int tid = threadIdx.x;
    // the sorted span: the smallest power of two >= cnt (at least one warp run)
    int span = WT;
    while (span < cnt) span <<= 1;
    if constexpr (C::STABLE) {
#pragma unroll
        for (int k = 0; k < VT; ++k) {
            const int i = k * NT + tid;
            if (tid < NT) sa[pad<T>(i)] = (i < cnt) ? Traits<T>::flip(src[p0 + i], xin) : Traits<T>::max_item();
        }
        __syncthreads();
        T v[VT];
        if (tid < NT) {
#pragma unroll
            for (int k = 0; k < VT; ++k) v[k] = sa[pad<T>(tid * VT + k)];
            thread_sort<T, VT, true>(v, VT);
        }
        __syncthreads();
        if (tid < NT) {
#pragma unroll
            for (int k = 0; k < VT; ++k) sa[pad<T>(tid * VT + k)] = v[k];
        }
        __syncthreads();
        merge_round_uniform<T, NTM, C::VTM, true, PadIdx<T>>(sa, sb, VT, TILE, split);
        T* s0 = sb;
        T* s1 = sa;
        for (int w = 2 * VT; w < TILE && w < span; w <<= 1) {
            merge_round_uniform<T, NTM, C::VTM, true, LinIdx>(s0, s1, w, TILE, split);
            T* t = s0;
            s0 = s1;
            s1 = t;
        }
        for (int i = tid; i < cnt; i += NTM) dst[p0 + i] = Traits<T>::flip(s0[i], xout);
    } else {
        // each sorting warp loads its WT slots striped (one 128-byte line per
        // instruction) straight into registers: which keys a lane starts with
        // does not matter once the warp's run is sorted
        const int lane = tid & 31, warp = tid >> 5, w0 = warp * WT;
        if (warp < C::NW) {
            T v[VT];
#pragma unroll
            for (int k = 0; k < VT; ++k) {
                const int i = w0 + k * 32 + lane;
                v[k] = (i < cnt) ? Traits<T>::flip(src[p0 + i], xin) : Traits<T>::max_item();
            }
            warp_sort<T, VT>(v, WT);
#pragma unroll
            for (int k = 0; k < VT; ++k) sa[pad<T>(w0 + lane * VT + k)] = v[k];
        }
        __syncthreads();
        if (span > WT) {
            merge_round_uniform<T, NTM, VT, false, PadIdx<T>>(sa, sb, WT, TILE, split);
            T* s0 = sb;
            T* s1 = sa;
            for (int w = 2 * WT; w < span; w <<= 1) {
                merge_round_uniform<T, NTM, VT, false, LinIdx>(s0, s1, w, TILE, split);
                T* t = s0;
                s0 = s1;
                s1 = t;
            }
            for (int i = tid; i < cnt; i += NTM) dst[p0 + i] = Traits<T>::flip(s0[i], xout);
        } else {
            for (int i = tid; i < cnt; i += NTM) dst[p0 + i] = Traits<T>::flip(sa[pad<T>(i)], xout);
        }
    }
}

// 4. tile phase: a grid of CTAs strides over the tile jobs
template <class T>
__global__ void __launch_bounds__(SegShape<T>::NTM, SegCfg<T>::TILE_MINB) seg_tile_kernel(SegState st, T* d, T* tmp,
                                                                                          uint64_t xmask) {
    using C = SegCfg<T>;
    using Sh = SegShape<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int split[Sh::SPLITS];
    const uint32_t total = st.tot[0];
    for (uint32_t j = blockIdx.x; j < total; j += gridDim.x) {
        const uint32_t s = st.tileseg[j];
        const SegGeom<T> g(st.off, s, st.n);
        const uint32_t t = j - st.cnt[s];
        const uint64_t p0 = st.off[s] + (uint64_t)t * C::TILE;
        const int cnt = (int)min((uint64_t)C::TILE, g.len - (uint64_t)t * C::TILE);
        seg_tile_sort<T>(d, seg_buf<T>(g.levels, 0, d, tmp), p0, cnt, xmask, g.levels == 0 ? xmask : 0, smem_raw,
                         split);
        __syncthreads();
    }
}

// Geometry of merge tile u (MT outputs) of a segment of len items at level l.
struct SegPair {
    uint64_t pb, la, lb, d0, d1;
    __device__ __forceinline__ SegPair(uint64_t len, uint64_t run, uint64_t u, uint64_t mt) {
        const uint64_t o = u * mt;
        pb = (o / (2 * run)) * (2 * run);
        la = min(run, len - pb);
        lb = min(run, len - pb - la);
        d0 = o - pb;
        d1 = min(d0 + mt, la + lb);
    }
};

// 5. level l, partition: one thread per merge tile
template <class T>
__global__ void seg_part_kernel(SegState st, int l, const T* d, const T* tmp) {
    const uint32_t* pref = st.cnt + (size_t)(1 + l) * st.nseg;
    const uint32_t total = st.tot[1 + l];
    const uint64_t run = (uint64_t)SegCfg<T>::TILE << l;
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < total;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = seg_of_job(pref, st.nseg, (uint32_t)j);
        const SegGeom<T> g(st.off, s, st.n);
        const SegPair p(g.len, run, j - pref[s], Config<T>::P_TILE);
        const T* A = seg_buf<const T>(g.levels, l, d, tmp) + st.off[s] + p.pb;
        st.splits[j] = global_merge_path(A, (int64_t)p.la, A + p.la, (int64_t)p.lb, (int64_t)p.d0);
        st.segof[j] = s;
    }
}

// 6. level l, merge: a grid of CTAs strides over the merge tiles
template <class T>
__global__ void __launch_bounds__(Config<T>::P_NT, SegCfg<T>::MERGE_MINB) seg_merge_kernel(SegState st, int l, T* d,
                                                                                           T* tmp, uint64_t xmask) {
    using C = Config<T>;
    using Sh = PShape<T>;
    constexpr int NT = C::P_NT, V = Sh::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int split[Sh::SPLITS];
    T* sin = reinterpret_cast<T*>(smem_raw);
    const int tid = threadIdx.x;
    const uint32_t* pref = st.cnt + (size_t)(1 + l) * st.nseg;
    const uint32_t total = st.tot[1 + l];
    const uint64_t run = (uint64_t)SegCfg<T>::TILE << l;
    for (uint32_t j = blockIdx.x; j < total; j += gridDim.x) {
        const uint32_t s = st.segof[j];
        const SegGeom<T> g(st.off, s, st.n);
        const SegPair p(g.len, run, j - pref[s], C::P_TILE);
        const T* src = seg_buf<T>(g.levels, l, d, tmp);
        T* dst = seg_buf<T>(g.levels, l + 1, d, tmp);
        const uint64_t base = st.off[s] + p.pb;
        const int64_t a0 = st.splits[j];
        const int64_t a1 = (p.d1 < p.la + p.lb) ? st.splits[j + 1] : (int64_t)p.la;  // next tile, same pair
        const int na = (int)(a1 - a0);
        const int tot = (int)(p.d1 - p.d0);
        const int nb = tot - na;
        const int a_lead = stage_vec<T, NT>(sin, src, base + (uint64_t)a0, na);
        const int b_base = ((a_lead + na + V - 1) / V) * V;
        const int b_lead = stage_vec<T, NT>(sin + b_base, src, base + p.la + (p.d0 - (uint64_t)a0), nb);
        cp_async_commit_all();
        cp_async_wait_all();
        __syncthreads();
        merge_pair_round_inplace<T, NT, C::P_VT, C::STABLE>(sin, a_lead, na, b_base + b_lead, nb, split);
        const uint64_t xo = ((uint32_t)l + 1 == g.levels) ? xmask : 0;
        T* op = dst + base + p.d0;  // any alignment: plain coalesced stores
        for (int i = tid; i < tot; i += NT) op[i] = Traits<T>::flip(sin[i], xo);
        __syncthreads();
    }
}

// ------------------------------------------------------------ scratch ----
template <class T>
inline uint64_t seg_tile_slots(uint64_t n, uint64_t nseg) {
    return n / Config<T>::P_TILE + nseg + 2;  // merge tiles of one level, upper bound
}

// Tile jobs: every segment's tiles, upper bound.
template <class T>
inline uint64_t seg_tile_jobs(uint64_t n, uint64_t nseg) {
    return n / SegCfg<T>::TILE + nseg + 2;
}

template <class T>
inline uint64_t seg_scratch_bytes(uint64_t n, uint64_t nseg, int maxl) {
    const uint64_t q = (uint64_t)maxl + 1;
    uint64_t b = ((seg_tile_jobs<T>(n, nseg) * 4 + 255) & ~255ull);  // tileseg
    b += ((q * nseg * 4 + 255) & ~255ull);                      // cnt
    b += ((q * 4 + 255) & ~255ull);                             // tot
    b += ((seg_tile_slots<T>(n, nseg) * 8 + 255) & ~255ull);    // splits
    b += ((seg_tile_slots<T>(n, nseg) * 4 + 255) & ~255ull);    // segof
    b += 256;                                                   // err
    return b;
}

template <class T>
inline SegState seg_state(void* scratch, const uint64_t* off, uint64_t n, uint64_t nseg, int maxl) {
    SegState s;
    const uint64_t q = (uint64_t)maxl + 1;
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
    s.splits = reinterpret_cast<int64_t*>(take(seg_tile_slots<T>(n, nseg) * 8));
    s.segof = reinterpret_cast<uint32_t*>(take(seg_tile_slots<T>(n, nseg) * 4));
    s.err = reinterpret_cast<int*>(take(256));
    s.tileseg = reinterpret_cast<uint32_t*>(take(seg_tile_jobs<T>(n, nseg) * 4));
    return s;
}

}  // namespace origami
