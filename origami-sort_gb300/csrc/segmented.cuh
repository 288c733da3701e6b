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
//                merge-path split and records the tile's geometry, a
//                persistent merge kernel merges the tiles (the binary-pass
//                merge body with double-buffered bulk copies and claimed
//                tiles, as pair_merge_bulk_kernel).
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
    static constexpr int TILE_MINB = 3;  // CTAs per SM the register budget allows
    static constexpr int RUN0 = 1024;    // register merges up to the warp's whole run
};
template <>
struct SegCfg<uint64_t> {
    static constexpr int NW = 8, VT = 16;  // 4096
    static constexpr int TILE = NW * 32 * VT;
    static constexpr bool STABLE = false;
    static constexpr int VTM = VT;
    static constexpr int NWT = 9;
    static constexpr int TILE_MINB = 2;
    static constexpr int RUN0 = 128;  // register merges to runs of 128, shared-memory rounds from there
};
template <>
struct SegCfg<KV64> {
    static constexpr int NW = 8, VT = 8;  // 2048, stable block sort
    static constexpr int TILE = NW * 32 * VT;
    static constexpr bool STABLE = true;
    static constexpr int VTM = 11;  // serial merge blocks of the shared-memory rounds
    static constexpr int NWT = 8;
    static constexpr int TILE_MINB = 3;
    static constexpr int RUN0 = 8;  // (stable tiles sort in registers, then merge rounds)
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
    struct SegTileRec* rec;  // geometry of each merge tile of the current level
    unsigned* claim;      // [maxl] tile counter of each level's merge kernel
    uint32_t* tileseg;    // segment of each tile job
    int* err;             // 1 / 3 = a bulk-copy wait expired (bulk.cuh), 2 = bad offsets
    uint32_t spin;        // polls before a bulk-copy wait gives up
    uint32_t mtile;       // merge tile of the level merges (the merge shape's, SegMergeCfg)
};

template <class T>
struct SegGeom {
    uint64_t len;
    uint32_t tiles, levels, mtiles;
    // An invalid segment (decreasing offsets or past the buffer) is treated as
    // empty; the plan kernel reports it.
    // mt: merge tile of the level merges (only mtiles depends on it)
    __device__ __forceinline__ SegGeom(const uint64_t* off, uint32_t s, uint64_t n,
                                       uint64_t mt = Config<T>::P_TILE) {
        const uint64_t a = off[s], b = off[s + 1];
        len = (a <= b && b <= n) ? b - a : 0;
        tiles = (uint32_t)((len + SegCfg<T>::TILE - 1) / SegCfg<T>::TILE);
        levels = (uint32_t)seg_levels_for<T>(len);
        mtiles = (uint32_t)((len + mt - 1) / mt);
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
    const SegGeom<T> g(st.off, s, st.n, st.mtile);
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
// Any alignment of p0.
//  - key-value items: plain coalesced loads and stores;
//  - keys: the tile arrives by one bulk copy (the 16-byte chunks enclosing
//    it), warps read their keys from shared memory, only the warps whose keys
//    lie inside the sorted span (the smallest power of two >= cnt) sort, and
//    the last round writes its output shifted by p0's misalignment so that
//    the whole 16-byte chunks leave by one bulk store (the items before and
//    after them directly). `bar`/`phase`: the CTA's load barrier. Returns
//    false when a bulk-copy wait expired (err set).
template <class T>
__device__ bool seg_tile_sort(const T* src, T* dst, uint64_t p0, int cnt, uint64_t xin, uint64_t xout,
                              unsigned char* smem, int* split, uint64_t* bar, uint32_t& phase, int* err,
                              uint32_t spin) {
    using C = SegCfg<T>;
    using Sh = SegShape<T>;
    constexpr int NT = Sh::NT, NTM = Sh::NTM, VT = C::VT, TILE = C::TILE, WT = 32 * VT;
    constexpr int R0 = C::RUN0 < WT ? C::RUN0 : WT;  // runs the register merges stop at
    static_assert((R0 & (R0 - 1)) == 0 && R0 >= VT, "runs of a power of two, at least one lane's");
    T* sa = reinterpret_cast<T*>(smem);
    T* sb = reinterpret_cast<T*>(smem + Sh::BUF_BYTES);
    const int tid = threadIdx.x;
    // the sorted span: the smallest power of two >= cnt (at least one warp run)
    int span = WT;
    while (span < cnt) span <<= 1;
    if constexpr (C::STABLE) {
        (void)bar;
        (void)phase;
        (void)err;
        (void)spin;
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
        return true;
    } else {
        constexpr int V = Vec<T>::N;
        const int lane = tid & 31, warp = tid >> 5, w0 = warp * WT;
        const int sh = (int)(p0 % V);  // misalignment of the tile in both buffers
        if (tid == 0) {
            const int nv = (sh + cnt + V - 1) / V;
            bulk_wait_read<0>();  // the previous tile's bulk store has left shared memory
            mbar_arrive_expect(bar, (uint32_t)nv * 16u);
            bulk_load(sb, src + (p0 - sh), (uint32_t)nv * 16u, bar);
        }
        const bool ok = mbar_wait(bar, phase, spin);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) bulk_drain<1>(err, bar, 1u, phase);
            return false;
        }
        phase ^= 1u;
        if (warp < C::NW && w0 < span) {
            // striped reads: which keys a lane starts with does not matter
            // once the warp's run is sorted
            T v[VT];
#pragma unroll
            for (int k = 0; k < VT; ++k) {
                const int i = w0 + k * 32 + lane;
                v[k] = (i < cnt) ? Traits<T>::flip(sb[sh + i], xin) : Traits<T>::max_item();
            }
            warp_sort<T, VT>(v, R0);
#pragma unroll
            for (int k = 0; k < VT; ++k) sa[pad<T>(w0 + lane * VT + k)] = v[k];
        }
        __syncthreads();
        if (span > R0) {
            const T* s0 = sa;
            T* s1 = sb;
            for (int w = R0; w < span; w <<= 1) {
                T* out = (2 * w >= span) ? s1 + sh : s1;  // the last round writes shifted
                if (w == R0)
                    merge_round_uniform<T, NTM, VT, false, PadIdx<T>>(s0, out, w, span, split);
                else
                    merge_round_uniform<T, NTM, VT, false, LinIdx>(s0, out, w, span, split);
                T* t = const_cast<T*>(s0);
                s0 = s1;
                s1 = t;
            }
            T* res = const_cast<T*>(s0);  // item i at res[sh + i]
            if (xout) {
                for (int i = tid; i < cnt; i += NTM) res[sh + i] = Traits<T>::flip(res[sh + i], xout);
            }
            fence_async_smem();
            __syncthreads();
            T* op = dst + (p0 - sh);  // 16-byte aligned
            const int x0 = sh ? V : 0;
            const int x1 = ((sh + cnt) / V) * V;
            if (x1 > x0) {
                if (tid == 0) {
                    bulk_store(op + x0, res + x0, (uint32_t)(x1 - x0) * (uint32_t)sizeof(T));
                    bulk_commit();
                }
                const int head = x0 - sh, tail = sh + cnt - x1;
                if (tid < head)
                    op[sh + tid] = res[sh + tid];
                else if (tid < head + tail)
                    op[x1 + tid - head] = res[x1 + tid - head];
            } else {
                for (int i = tid; i < cnt; i += NTM) op[sh + i] = res[sh + i];
            }
        } else {
            for (int i = tid; i < cnt; i += NTM) dst[p0 + i] = Traits<T>::flip(sa[pad<T>(i)], xout);
        }
        return true;
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
    __shared__ __align__(8) uint64_t bar;
    const uint32_t total = st.tot[0];
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    uint32_t phase = 0;
    for (uint32_t j = blockIdx.x; j < total; j += gridDim.x) {
        const uint32_t s = st.tileseg[j];
        const SegGeom<T> g(st.off, s, st.n);
        const uint32_t t = j - st.cnt[s];
        const uint64_t p0 = st.off[s] + (uint64_t)t * C::TILE;
        const int cnt = (int)min((uint64_t)C::TILE, g.len - (uint64_t)t * C::TILE);
        if (threadIdx.x == 32 && j + gridDim.x < total) {
            // this CTA's next tile into L2 while this one sorts: the whole
            // 16-byte chunks inside it (and inside the buffer)
            const uint32_t jn = j + gridDim.x, sn = st.tileseg[jn];
            const SegGeom<T> gn(st.off, sn, st.n);
            constexpr uint64_t IB = sizeof(T), TL = C::TILE;
            const uint64_t tn = jn - st.cnt[sn];
            const uint64_t items = gn.len > tn * TL ? gn.len - tn * TL : 0;
            const uint64_t b0 = (st.off[sn] + tn * TL) * IB;
            const uint64_t lim = (st.n * IB) & ~15ull;
            const uint64_t b1 = b0 + (items < TL ? items : TL) * IB;
            const uint64_t c0 = (b0 + 15) & ~15ull, c1 = (b1 < lim ? b1 : lim) & ~15ull;
            if (items > 0 && c1 > c0)
                bulk_prefetch_l2(reinterpret_cast<const char*>(d) + c0, (uint32_t)(c1 - c0));
        }
        if (!seg_tile_sort<T>(d, seg_buf<T>(g.levels, 0, d, tmp), p0, cnt, xmask, g.levels == 0 ? xmask : 0,
                              smem_raw, split, &bar, phase, st.err, st.spin))
            return;
        __syncthreads();
    }
    if (threadIdx.x == 0) bulk_wait_read<0>();
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

// What the merge kernel needs of one merge tile, recorded by the partition
// kernel: the pair's first item, the tile's output range within the pair, the
// A run length and four flags in its top bits.
struct SegTileRec {
    uint64_t base, d0, d1, la_flags;
    static constexpr uint64_t SRC_TMP = 1ull << 60, DST_TMP = 1ull << 61, LAST = 1ull << 62, PAIR_END = 1ull << 63;
    static constexpr uint64_t LA_MASK = (1ull << 60) - 1;
};

// 5. level l, partition: one thread per merge tile
template <class T>
__global__ void seg_part_kernel(SegState st, int l, const T* d, const T* tmp) {
    const uint32_t* pref = st.cnt + (size_t)(1 + l) * st.nseg;
    const uint32_t total = st.tot[1 + l];
    const uint64_t run = (uint64_t)SegCfg<T>::TILE << l;
    if (blockIdx.x == 0 && threadIdx.x == 0) st.claim[l] = 0;  // for this level's merge kernel
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < total;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = seg_of_job(pref, st.nseg, (uint32_t)j);
        const SegGeom<T> g(st.off, s, st.n);
        const SegPair p(g.len, run, j - pref[s], st.mtile);
        const uint64_t base = st.off[s] + p.pb;
        const T* A = seg_buf<const T>(g.levels, l, d, tmp) + base;
        st.splits[j] = global_merge_path_interp(A, (int64_t)p.la, A + p.la, (int64_t)p.lb, (int64_t)p.d0,
                                                st.n * sizeof(T) > (64ull << 20));
        uint64_t f = p.la;
        if (seg_buf<const T>(g.levels, l, d, tmp) == tmp) f |= SegTileRec::SRC_TMP;
        if (seg_buf<const T>(g.levels, l + 1, d, tmp) == tmp) f |= SegTileRec::DST_TMP;
        if ((uint32_t)l + 1 == g.levels) f |= SegTileRec::LAST;
        if (p.d1 == p.la + p.lb) f |= SegTileRec::PAIR_END;
        SegTileRec r;
        r.base = base;
        r.d0 = p.d0;
        r.d1 = p.d1;
        r.la_flags = f;
        st.rec[j] = r;
    }
}

// 6. level l, merge: persistent, double-buffered bulk copies, claimed tiles
// (the body of pair_merge_bulk_kernel). Segments start anywhere, so an output
// tile is generally not 16-byte aligned: the merged tile is written back into
// the stage shifted by the output's misalignment, the whole 16-byte chunks
// leave by one bulk store and single threads store the few items before and
// after them. Thread 0 refills the other stage only after the iteration's
// first barrier, when every thread is past the previous tile's stores from it.
struct SegBulkGeom {
    uint64_t job, obase;     // job >= total: none
    int as, na, bs, nb, sh;  // A at stage[as..), B at stage[bs..); output shift
    uint64_t flags;
};

// (The runs are always this sort's own tile-sorted or merged output; after an
// expired wait the merge kernels stop before they read any.)
template <class T>
__device__ __forceinline__ SegBulkGeom seg_bulk_issue(T* stage, const T* d, const T* tmp, uint64_t j,
                                                      const SegTileRec& r, int64_t s0, int64_t s1, uint64_t* bar) {
    constexpr int V = Vec<T>::N;
    const uint64_t la = r.la_flags & SegTileRec::LA_MASK;
    const int64_t a1 = (r.la_flags & SegTileRec::PAIR_END) ? (int64_t)la : s1;
    SegBulkGeom q;
    q.job = j;
    q.flags = r.la_flags;
    q.na = (int)(a1 - s0);
    q.nb = (int)(r.d1 - r.d0) - q.na;
    q.obase = r.base + r.d0;
    q.sh = (int)(q.obase % V);
    const T* src = (r.la_flags & SegTileRec::SRC_TMP) ? tmp : d;
    const uint64_t pa = r.base + (uint64_t)s0;
    const uint64_t pb = r.base + la + (r.d0 - (uint64_t)s0);
    const int a_lead = (int)(pa % V), b_lead = (int)(pb % V);
    const int nva = (a_lead + q.na + V - 1) / V, nvb = (b_lead + q.nb + V - 1) / V;
    q.as = a_lead;
    q.bs = nva * V + b_lead;
    mbar_arrive_expect(bar, (uint32_t)(nva + nvb) * 16u);
    if (nva) bulk_load(stage, src + (pa - a_lead), (uint32_t)nva * 16u, bar);
    if (nvb) bulk_load(stage + nva * V, src + (pb - b_lead), (uint32_t)nvb * 16u, bar);
    return q;
}

// Merge shapes of the level merges: 0 = the binary pass's first tile shape
// (P_*), 1 = its second (P2_*, twice the tile). Chosen per plan by the
// segmented tuning table (capi.cu), keyed by kind and mean segment length.
template <class T, int SH>
struct SegMergeCfg {
    using C = Config<T>;
    static constexpr int NT = SH ? C::P2_NT : C::P_NT;
    static constexpr int VT = SH ? C::P2_VT : C::P_VT;
    static constexpr int TILE = SH ? C::P2_TILE : C::P_TILE;
    static constexpr int MINB = SH ? C::P2_MINB : C::P_MINB;
    static constexpr bool STABLE = C::STABLE;
};
static_assert(2 * SegCfg<uint32_t>::TILE % Config<uint32_t>::P2_TILE == 0 &&
                  2 * SegCfg<uint64_t>::TILE % Config<uint64_t>::P2_TILE == 0 &&
                  2 * SegCfg<KV64>::TILE % Config<KV64>::P2_TILE == 0,
              "a merge tile never straddles two run pairs");
template <class T, int SH = 0>
using SegMergeShape = PairBulkShape<T, SegMergeCfg<T, SH>::NT, SegMergeCfg<T, SH>::VT, Config<T>::STABLE,
                                    SegMergeCfg<T, SH>::TILE>;

template <class T, int SH>
__global__ void __launch_bounds__(SegMergeCfg<T, SH>::NT, SegMergeCfg<T, SH>::MINB)
    seg_merge_kernel(SegState st, int l, T* d, T* tmp, uint64_t xmask) {
    using C = SegMergeCfg<T, SH>;
    using Sh = SegMergeShape<T, SH>;
    constexpr int V = Vec<T>::N;
    constexpr int VO = Block<T, C::VT, C::STABLE>::VO;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int split[Sh::In::SPLITS];
    __shared__ SegBulkGeom geom[2];
    __shared__ __align__(8) uint64_t bar[2];
    const int tid = threadIdx.x;
    const uint64_t total = st.tot[1 + l];
    const uint64_t G = gridDim.x;
    if (blockIdx.x >= total) return;
    // a wait of an earlier kernel expired: the runs are not sorted, stop here
    if (__syncthreads_or(tid == 0 && err_wait_set(st.err))) return;
    unsigned* claim = st.claim + l;
    auto stage = [&](int s) { return reinterpret_cast<T*>(smem_raw + (size_t)s * Sh::STAGE); };
    auto claim_next = [&] { return G + (uint64_t)atomicAdd(claim, 1u); };
    // thread 0's look-ahead: the next job (its record and splits) and the one after
    uint64_t nj = total, fj = total;
    SegTileRec nr{};
    int64_t n0 = 0, n1 = 0;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
        const uint64_t j0 = blockIdx.x;
        geom[0] = seg_bulk_issue<T>(stage(0), d, tmp, j0, st.rec[j0], st.splits[j0], st.splits[j0 + 1], &bar[0]);
        nj = claim_next();
        if (nj < total) {
            nr = st.rec[nj];
            n0 = st.splits[nj];
            n1 = st.splits[nj + 1];
            fj = claim_next();
        }
    }
    __syncthreads();
    uint32_t phase = 0;
    for (int s = 0;; s ^= 1) {
        const SegBulkGeom q = geom[s];
        if (q.job >= total) break;
        const bool ok = mbar_wait(&bar[s], (phase >> s) & 1u, st.spin);
        if (__syncthreads_or(!ok)) {
            // drain this stage's loads (no copy into the other stage is in
            // flight yet in this iteration)
            if (tid == 0) bulk_drain<2>(st.err, bar, 1u << s, phase);
            return;
        }
        phase ^= 1u << s;
        // every thread is past the previous tile's stores from the other
        // stage: thread 0 refills it with the next tile
        if (tid == 0) {
            if (nj < total) {
                bulk_wait_read<0>();
                geom[s ^ 1] = seg_bulk_issue<T>(stage(s ^ 1), d, tmp, nj, nr, n0, n1, &bar[s ^ 1]);
            } else {
                geom[s ^ 1].job = total;
            }
            nj = fj;
            if (nj < total) {
                nr = st.rec[nj];
                n0 = st.splits[nj];
                n1 = st.splits[nj + 1];
                fj = claim_next();
            }
        }
        T* buf = stage(s);
        const int tot = q.na + q.nb;
        const int nblk = (tot + VO - 1) / VO;
        if (tid < nblk) split[tid] = merge_path_ix<T, LinIdx>(buf, q.as, q.na, q.bs, q.nb, tid * VO);
        __syncthreads();
        T r[C::VT];
        const int diag = tid * VO;
        const int cnt = tid < nblk ? min(VO, tot - diag) : 0;
        if (tid < nblk) {
            const int sa = split[tid];
            const int ea = (tid + 1 < nblk) ? split[tid + 1] : q.na;
            merge_block_regs<T, C::VT, C::STABLE>(buf, q.as + sa, q.bs + (diag - sa), ea - sa, cnt, r);
        }
        __syncthreads();
        // stage index x holds output item x - sh, so x = 0 lies on a 16-byte
        // boundary of the output buffer
        const uint64_t xo = (q.flags & SegTileRec::LAST) ? xmask : 0;
        T* w = buf + q.sh + diag;
        if (cnt == VO) {
#pragma unroll
            for (int i = 0; i < VO; ++i) w[i] = Traits<T>::flip(r[i], xo);
        } else {
#pragma unroll
            for (int i = 0; i < VO; ++i)
                if (i < cnt) w[i] = Traits<T>::flip(r[i], xo);
        }
        fence_async_smem();
        __syncthreads();
        // whole 16-byte chunks [x0, x1) by one bulk store, the items before
        // and after them directly
        T* dst = (q.flags & SegTileRec::DST_TMP) ? tmp : d;
        T* op = dst + q.obase - q.sh;
        const int x0 = q.sh ? V : 0;
        const int x1 = ((q.sh + tot) / V) * V;
        if (x1 > x0) {
            if (tid == 0) {
                bulk_store(op + x0, buf + x0, (uint32_t)(x1 - x0) * (uint32_t)sizeof(T));
                bulk_commit();
            }
            const int head = x0 - q.sh, tail = q.sh + tot - x1;
            if (tid < head) op[q.sh + tid] = buf[q.sh + tid];
            else if (tid < head + tail) op[x1 + tid - head] = buf[x1 + tid - head];
        } else {
            for (int i = tid; i < tot; i += C::NT) op[q.sh + i] = buf[q.sh + i];
        }
    }
    if (tid == 0) bulk_wait_read<0>();
}

// ------------------------------------------------------------ scratch ----
template <class T>
inline uint64_t seg_tile_slots(uint64_t n, uint64_t nseg) {
    return n / Config<T>::P_TILE + nseg + 2;  // merge tiles of one level, upper bound (smaller shape)
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
    b += ((seg_tile_slots<T>(n, nseg) * sizeof(SegTileRec) + 255) & ~255ull);  // rec
    b += 256;                                                   // err
    b += ((q * 4 + 255) & ~255ull);                             // claim
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
    s.rec = reinterpret_cast<SegTileRec*>(take(seg_tile_slots<T>(n, nseg) * sizeof(SegTileRec)));
    s.err = reinterpret_cast<int*>(take(256));
    s.tileseg = reinterpret_cast<uint32_t*>(take(seg_tile_jobs<T>(n, nseg) * 4));
    s.claim = reinterpret_cast<unsigned*>(take(q * 4));
    s.spin = BULK_SPIN_LIMIT;
    s.mtile = Config<T>::P_TILE;
    return s;
}

}  // namespace origami
