// The plain-sort kernels:
//   K1 block_sort_kernel      - tile sort: registers (thread network) then
//                               merge-path rounds in shared memory
//   K4 pair_partition_kernel  - merge-path splitter search for one binary pass
//   K3 pair_merge_kernel      - one output tile of a binary pass, staged in
//                               shared memory and merged by merge path
//   K3 pair_merge_bulk_kernel - the same merge as a persistent kernel whose
//                               tiles move by double-buffered bulk copies
#pragma once
#include "bulk.cuh"
#include "common.cuh"
#include "kway_bulk.cuh"
#include "merge_core.cuh"
#include "warp_sort.cuh"

namespace origami {

// ---------------------------------------------------------------- K1 -----
// Sorts tiles of NT*VTS items. Restates the reference's phase 1 + phase 2
// (sorter.h:3831-3849: in-register networks, then binary merges up to the
// in-cache block size): each thread sorts VTS items in registers, then merge
// rounds in shared memory (merge_core.cuh, VTM-register blocks) double the run
// length until the tile (or the chunk) is sorted.
// `chunk` (power of two) caps the sorted run length for chunked sorts.
// xin/xout are the key masks applied on load / on store (sign flip for i64).
template <class T, int NT, int VTS, int VTM, bool STABLE>
struct BlockSortShape {
    static constexpr int TILE = NT * VTS;
    static constexpr int BUF = padded_items<T>(TILE + VTM + 1);  // items per buffer
    static constexpr int VO = Block<T, VTM, STABLE>::VO;
    static constexpr int SPLITS = TILE / VO + TILE / (2 * VTS) + 4;
    static constexpr size_t SMEM = 2 * (((size_t)BUF * sizeof(T) + 15) & ~(size_t)15);
};

// err (optional): the sort's error word, cleared by the first thread (the
// tile sort is the first kernel of a sort). samp / ssamp (optional): samples
// of the sorted tiles for a k-way pass that follows (kway_bulk.cuh).
template <class T, int NT, int VTS, int VTM, bool STABLE>
__global__ void __launch_bounds__(NT) block_sort_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                        uint64_t n, int chunk, uint64_t xin,
                                                        uint64_t xout, int* err = nullptr,
                                                        typename Traits<T>::Key* samp = nullptr,
                                                        typename Traits<T>::Key* ssamp = nullptr) {
    using Sh = BlockSortShape<T, NT, VTS, VTM, STABLE>;
    constexpr int TILE = Sh::TILE;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sa = reinterpret_cast<T*>(smem_raw);
    T* sb = reinterpret_cast<T*>(smem_raw + Sh::SMEM / 2);
    __shared__ int split[Sh::SPLITS];
    const int tid = threadIdx.x;
    if (err && blockIdx.x == 0 && tid == 0) *err = 0;
    const uint64_t base = (uint64_t)blockIdx.x * TILE;
    const int valid = (int)((n - base) < (uint64_t)TILE ? (n - base) : (uint64_t)TILE);

    // coalesced striped load; the tail of a partial tile is filled with the
    // largest item, which sorts after every real item (stably for key-value)
#pragma unroll
    for (int k = 0; k < VTS; ++k) {
        const int i = k * NT + tid;
        sa[pad<T>(i)] = (i < valid) ? Traits<T>::flip(in[base + i], xin) : Traits<T>::max_item();
    }
    __syncthreads();
    {
        T v[VTS];
#pragma unroll
        for (int k = 0; k < VTS; ++k) v[k] = sa[pad<T>(tid * VTS + k)];
        thread_sort<T, VTS, STABLE>(v, chunk);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < VTS; ++k) sa[pad<T>(tid * VTS + k)] = v[k];
    }
    __syncthreads();
    T* src = sa;
    if (VTS < TILE && VTS < chunk) {
        // first round reads the padded blocked layout, later rounds are unpadded
        merge_round_uniform<T, NT, VTM, STABLE, PadIdx<T>>(sa, sb, VTS, TILE, split);
        src = sb;
        T* dst = sa;
        for (int w = 2 * VTS; w < TILE && w < chunk; w <<= 1) {
            merge_round_uniform<T, NT, VTM, STABLE, LinIdx>(src, dst, w, TILE, split);
            T* t = src;
            src = dst;
            dst = t;
        }
#pragma unroll
        for (int k = 0; k < VTS; ++k) {
            const int i = k * NT + tid;
            if (i < valid) out[base + i] = Traits<T>::flip(src[i], xout);
        }
        if (samp) kb_emit_samples<T>(src, base, valid, samp, ssamp, NT);
    } else {
#pragma unroll
        for (int k = 0; k < VTS; ++k) {
            const int i = k * NT + tid;
            if (i < valid) out[base + i] = Traits<T>::flip(src[pad<T>(i)], xout);
        }
    }
}

// K1 for keys-only items: every one of NW warps sorts 32*VT keys entirely in
// registers (lane network + shuffle merges, warp_sort.cuh), then merge rounds
// in shared memory join the warps' runs into a tile of NW*32*VT keys. NWT >= NW
// warps share the merge rounds, so that every thread owns at most one merge
// block per round (NWT*32*(VT-1) >= tile).
template <class T, int NW, int VT, int NWT = NW>
struct WarpSortShape {
    static constexpr int NT = NW * 32;
    static constexpr int NTM = NWT * 32;
    static constexpr int TILE = NT * VT;
    static constexpr int WTILE = 32 * VT;
    static constexpr int BUF = padded_items<T>(TILE + VT + 1);
    static constexpr int VTM = VT;  // merge blocks of VT-1 outputs
    static constexpr size_t SMEM = 2 * (((size_t)BUF * sizeof(T) + 15) & ~(size_t)15);
};

// `ahead` > 0: the CTA first asks for the tile `ahead` places further on to be
// brought into L2 (the tile a CTA of the next wave will load), so that later
// CTAs find their keys in L2. err (optional): the sort's error word, cleared by
// the first thread. SAMPLES: also writes the samples of the sorted tiles to
// samp / ssamp for a k-way pass that follows (kway_bulk.cuh); a separate
// instantiation, so that the plain tile sort keeps its registers.
template <class T, int NW, int VT, int NWT = NW, int MINB = 1, bool SAMPLES = false, int RUN0 = 32 * VT>
__global__ void __launch_bounds__(NWT * 32, MINB) warp_block_sort_kernel(const T* __restrict__ in,
                                                                        T* __restrict__ out, uint64_t n,
                                                                        int chunk, uint64_t xin,
                                                                        uint64_t xout, uint32_t ahead = 0,
                                                                        int* err = nullptr,
                                                                        typename Traits<T>::Key* samp = nullptr,
                                                                        typename Traits<T>::Key* ssamp = nullptr) {
    using Sh = WarpSortShape<T, NW, VT, NWT>;
    static_assert(NWT >= NW, "the sorting warps take part in the merge rounds");
    constexpr int TILE = Sh::TILE, WT = Sh::WTILE;
    // runs the warps' register merges stop at; shared-memory rounds take over
    constexpr int R0 = RUN0 < WT ? RUN0 : WT;
    static_assert((R0 & (R0 - 1)) == 0 && R0 >= VT, "runs of a power of two, at least one lane's");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sa = reinterpret_cast<T*>(smem_raw);
    T* sb = reinterpret_cast<T*>(smem_raw + Sh::SMEM / 2);
    // blocks of a round: at most TILE / (VT - 1) plus one partial block per pair
    __shared__ int split[TILE / (VT - 1) + TILE / (2 * R0) + 4];
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const uint64_t base = (uint64_t)blockIdx.x * TILE;
    static_assert(VT % Vec<T>::N == 0, "lanes load whole vectors");
    const int valid = (int)((n - base) < (uint64_t)TILE ? (n - base) : (uint64_t)TILE);
    const int w0 = warp * WT;
    if (err && blockIdx.x == 0 && tid == 0) *err = 0;
    if (ahead && tid == 0) {
        const uint64_t pb = base + (uint64_t)ahead * TILE;
        if (pb + TILE <= n) bulk_prefetch_l2(in + pb, (uint32_t)(TILE * sizeof(T)));
    }

    // each lane loads VT keys with 16-byte vector loads; a partial tail is
    // filled with the largest key. When a chunk spans the warp's whole run the
    // lanes' keys may come from anywhere in it, so the loads are striped
    // (each instruction reads 512 contiguous bytes); smaller chunks need each
    // lane to hold its own VT consecutive keys (blocked).
    constexpr int V = Vec<T>::N;
    T v[VT];
    const bool sorter = warp < NW;
    if (sorter) {
        const bool striped = chunk >= WT;
#pragma unroll
        for (int j = 0; j < VT / V; ++j) {
            const int i0 = striped ? w0 + j * 32 * V + lane * V : w0 + lane * VT + j * V;
            const T* src = in + base + i0;
            if (i0 + V <= valid) {
                const uint4 q = *reinterpret_cast<const uint4*>(src);
                const T* e = reinterpret_cast<const T*>(&q);
#pragma unroll
                for (int k = 0; k < V; ++k) v[j * V + k] = Traits<T>::flip(e[k], xin);
            } else {
#pragma unroll
                for (int k = 0; k < V; ++k)
                    v[j * V + k] = (i0 + k < valid) ? Traits<T>::flip(src[k], xin) : Traits<T>::max_item();
            }
        }
        warp_sort<T, VT>(v, chunk < R0 ? chunk : R0);
    }
    if (R0 < TILE && R0 < chunk) {
        if (sorter) {
#pragma unroll
            for (int k = 0; k < VT; ++k) sa[pad<T>(w0 + lane * VT + k)] = v[k];
        }
        __syncthreads();
        merge_round_uniform<T, Sh::NTM, VT, false, PadIdx<T>>(sa, sb, R0, TILE, split);
        T* src = sb;
        T* dst = sa;
        for (int w = 2 * R0; w < TILE && w < chunk; w <<= 1) {
            merge_round_uniform<T, Sh::NTM, VT, false, LinIdx>(src, dst, w, TILE, split);
            T* t = src;
            src = dst;
            dst = t;
        }
        // coalesced 16-byte stores of the sorted tile
        const int nvec = valid / V;
        for (int i = tid; i < nvec; i += Sh::NTM) {
            const uint4 q = *reinterpret_cast<const uint4*>(src + (size_t)i * V);
            T e[V];
            const T* qe = reinterpret_cast<const T*>(&q);
#pragma unroll
            for (int k = 0; k < V; ++k) e[k] = Traits<T>::flip(qe[k], xout);
            *reinterpret_cast<uint4*>(out + base + (size_t)i * V) = *reinterpret_cast<const uint4*>(e);
        }
        for (int i = nvec * V + tid; i < valid; i += Sh::NTM) out[base + i] = Traits<T>::flip(src[i], xout);
        if constexpr (SAMPLES) kb_emit_samples<T>(src, base, valid, samp, ssamp, Sh::NTM);
    } else if (sorter) {
        // runs end at the warp (or chunk) size: each lane stores its own keys
        const int i0 = w0 + lane * VT;
        T* dp = out + base + i0;
#pragma unroll
        for (int j = 0; j < VT / V; ++j) {
            if (i0 + (j + 1) * V <= valid) {
                T e[V];
#pragma unroll
                for (int k = 0; k < V; ++k) e[k] = Traits<T>::flip(v[j * V + k], xout);
                *reinterpret_cast<uint4*>(dp + j * V) = *reinterpret_cast<const uint4*>(e);
            } else {
#pragma unroll
                for (int k = 0; k < V; ++k)
                    if (i0 + j * V + k < valid) dp[j * V + k] = Traits<T>::flip(v[j * V + k], xout);
            }
        }
    }
}

// Geometry of one binary pass: runs of `run` items (the last one may be short)
// are merged pairwise (2p, 2p+1) into runs of 2*run. Output tiles of `tile`
// items never straddle a pair because 2*run is a multiple of tile.
struct PairGeom {
    uint64_t pbase, la, lb;
    __device__ __forceinline__ PairGeom(uint64_t o, uint64_t n, uint64_t run) {
        pbase = (o / (2 * run)) * (2 * run);
        const uint64_t rest = n - pbase;
        la = rest < run ? rest : run;
        lb = (rest - la) < run ? (rest - la) : run;
    }
};

// ---------------------------------------------------------------- K4 -----
// One thread per output-tile boundary: the merge-path split (items taken from
// the left run) at the tile's first output: a few interpolation probes, then
// binary search (common.cuh). (Searches with more probes per step, by one
// thread or a whole warp, issue more random loads and measured slower.)
// splits has num_tiles+1 entries.
template <class T>
__global__ void pair_partition_kernel(const T* __restrict__ src, uint64_t n, uint64_t run, int tile,
                                      uint64_t num_tiles, int64_t* __restrict__ splits,
                                      unsigned* __restrict__ claim) {
    grid_dep_launch();  // the merge kernel may take its place on the SMs early
    grid_dep_wait();    // the previous pass's merge has finished (and read splits)
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0 && claim) *claim = 0;  // tile counter of the merge kernel that follows
    if (t > num_tiles) return;
    const uint64_t o = t * (uint64_t)tile < n ? t * (uint64_t)tile : n;
    if (o >= n) {
        splits[t] = 0;
        return;
    }
    const PairGeom g(o, n, run);
    const T* A = src + g.pbase;
    const bool interp = n * sizeof(T) > (64ull << 20);  // arrays larger than about half of L2
    splits[t] = global_merge_path_interp(A, (int64_t)g.la, A + g.la, (int64_t)g.lb, (int64_t)(o - g.pbase), interp);
}

// ---------------------------------------------------------------- K3 -----
// Restates one level of the reference's binary merge (merger.h:4079-4218,
// mergebl2_*) for one tile of output: the tile's slices of both runs arrive
// in shared memory by cp.async, one merge round (merge_core.cuh) merges them
// and the tile is written back coalesced.
template <class T, int NT, int VT, bool STABLE, int TILE>
struct PairShape {
    // input: A part and B part each padded to whole 16-byte vectors (+ read
    // slack); the merged tile is written back over the same buffer
    static constexpr int V = Vec<T>::N;
    static constexpr int IN_CAP = TILE + 4 * V + VT + 4;
    static constexpr size_t IN_BYTES = (((size_t)IN_CAP * sizeof(T)) + 15) & ~(size_t)15;
    static constexpr size_t SMEM = IN_BYTES;
    static constexpr int SPLITS = TILE / Block<T, VT, STABLE>::VO + 4;
    static_assert(NT * Block<T, VT, STABLE>::VO >= TILE, "one merge block per thread");
};

template <class T, int NT, int VT, bool STABLE, int TILE, int MINB = 1>
__global__ void __launch_bounds__(NT, MINB) pair_merge_kernel(const T* __restrict__ src, T* __restrict__ dst,
                                                        uint64_t n, uint64_t run,
                                                        const int64_t* __restrict__ splits,
                                                        uint64_t xout, int* err) {
    using Sh = PairShape<T, NT, VT, STABLE, TILE>;
    constexpr int V = Sh::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sin = reinterpret_cast<T*>(smem_raw);
    __shared__ int split[Sh::SPLITS];
    const int tid = threadIdx.x;
    const uint64_t t = blockIdx.x;
    const uint64_t o = t * TILE;
    const PairGeom g(o, n, run);
    const uint64_t d0 = o - g.pbase;
    const uint64_t pair_end = g.la + g.lb;
    const uint64_t d1 = (d0 + TILE) < pair_end ? (d0 + TILE) : pair_end;
    if (__syncthreads_or(tid == 0 && err_wait_set(err))) return;  // an earlier pass gave up
    const int64_t a0 = splits[t];
    const int64_t a1 = (o + TILE < g.pbase + pair_end) ? splits[t + 1] : (int64_t)g.la;
    const int total = (int)(d1 - d0);
    bool bad;
    const int na = tile_split(a0, a1, (int64_t)d0, total, (int64_t)g.la, (int64_t)g.lb, &bad);
    if (bad && tid == 0) err_first(err, ERR_BAD_RUNS);
    const int nb = total - na;
    const uint64_t pa = g.pbase + (uint64_t)a0;
    const uint64_t pb = g.pbase + g.la + (d0 - (uint64_t)a0);
    // A staged at sin[0..], B at the next vector boundary after A's vectors
    const int a_lead = stage_vec<T, NT>(sin, src, pa, na);
    const int b_base = ((a_lead + na + V - 1) / V) * V;
    const int b_lead = stage_vec<T, NT>(sin + b_base, src, pb, nb);
    cp_async_commit_all();
    cp_async_wait_all();
    __syncthreads();
    merge_pair_round_inplace<T, NT, VT, STABLE>(sin, a_lead, na, b_base + b_lead, nb, split);
    const T* sout = sin;
    // output tile starts 16-byte aligned (o is a multiple of TILE)
    T* out = dst + o;
    const int nvec = total / V;
    for (int i = tid; i < nvec; i += NT) {
        T tmp[V];
#pragma unroll
        for (int k = 0; k < V; ++k) tmp[k] = Traits<T>::flip(sout[i * V + k], xout);
        *reinterpret_cast<uint4*>(out + (size_t)i * V) = *reinterpret_cast<const uint4*>(tmp);
    }
    for (int i = nvec * V + tid; i < total; i += NT) out[i] = Traits<T>::flip(sout[i], xout);
}

// ------------------------------------------------------- K3, persistent ---
// The same binary-pass merge as pair_merge_kernel, as a persistent kernel
// whose tiles move by bulk copies (cp.async.bulk, bulk.cuh). Each CTA holds
// two stages: while it merges the tile in one, the next tile's slices of both
// runs are already on their way into the other, and a merged tile leaves
// shared memory by one bulk store. Thread 0 issues every copy.
//
// Tiles are claimed, not assigned: a CTA starts with tile blockIdx.x and then
// takes the next unclaimed tile from a counter (gridDim.x + atomicAdd), so CTAs
// that became resident late (another kernel held the SMs) simply merge fewer
// tiles. The claim for a tile is made two tiles ahead of its merge and its
// split values are loaded one tile ahead, so neither latency is waited for.
// *claim must be 0 at launch (pair_partition_kernel resets it).
struct BulkTileGeom {
    uint64_t tile;       // output tile; >= num_tiles: none (the CTA is done)
    int as, na, bs, nb;  // A at stage[as .. as+na), B at stage[bs .. bs+nb)
};

template <class T, int NT, int VT, bool STABLE, int TILE>
struct PairBulkShape {
    using In = PairShape<T, NT, VT, STABLE, TILE>;
    static constexpr size_t STAGE = (In::IN_BYTES + 127) & ~(size_t)127;
    static constexpr size_t SMEM = 2 * STAGE;
};

// Geometry of output tile t, and the bulk loads of its slices into `stage`.
// Splits that are inconsistent (runs that are not sorted) are clamped into
// the runs and reported in *err (ERR_BAD_RUNS).
template <class T, int TILE>
__device__ __forceinline__ BulkTileGeom pair_bulk_issue(T* stage, const T* src, uint64_t n, uint64_t run,
                                                        uint64_t t, int64_t s0, int64_t s1, uint64_t* bar, int* err) {
    constexpr int V = Vec<T>::N;
    const uint64_t o = t * TILE;
    const PairGeom g(o, n, run);
    const uint64_t d0 = o - g.pbase;
    const uint64_t pair_end = g.la + g.lb;
    const uint64_t d1 = (d0 + TILE) < pair_end ? (d0 + TILE) : pair_end;
    const int64_t a1 = (o + TILE < g.pbase + pair_end) ? s1 : (int64_t)g.la;
    BulkTileGeom q;
    q.tile = t;
    bool bad;
    q.na = tile_split(s0, a1, (int64_t)d0, (int)(d1 - d0), (int64_t)g.la, (int64_t)g.lb, &bad);
    if (bad) err_first(err, ERR_BAD_RUNS);
    q.nb = (int)(d1 - d0) - q.na;
    const uint64_t pa = g.pbase + (uint64_t)s0;
    const uint64_t pb = g.pbase + g.la + (d0 - (uint64_t)s0);
    // the enclosing 16-byte vectors of each slice (never outside them)
    const int a_lead = (int)(pa % V), b_lead = (int)(pb % V);
    const int nva = (a_lead + q.na + V - 1) / V, nvb = (b_lead + q.nb + V - 1) / V;
    q.as = a_lead;
    q.bs = nva * V + b_lead;
    mbar_arrive_expect(bar, (uint32_t)(nva + nvb) * 16u);
    if (nva) bulk_load(stage, src + (pa - a_lead), (uint32_t)nva * 16u, bar);
    if (nvb) bulk_load(stage + nva * V, src + (pb - b_lead), (uint32_t)nvb * 16u, bar);
    return q;
}

template <class T, int NT, int VT, bool STABLE, int TILE, int MINB = 1>
__global__ void __launch_bounds__(NT, MINB)
    pair_merge_bulk_kernel(const T* __restrict__ src, T* __restrict__ dst, uint64_t n, uint64_t run,
                           const int64_t* __restrict__ splits, uint64_t num_tiles, uint64_t xout,
                           unsigned* __restrict__ claim, unsigned max_tiles, int* err,
                           uint32_t spin = BULK_SPIN_LIMIT) {
    using Sh = PairBulkShape<T, NT, VT, STABLE, TILE>;
    constexpr int V = Vec<T>::N;
    constexpr int VO = Block<T, VT, STABLE>::VO;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int split[Sh::In::SPLITS];
    __shared__ BulkTileGeom geom[2];
    __shared__ __align__(8) uint64_t bar[2];
    const int tid = threadIdx.x;
    const uint64_t G = gridDim.x;
    if (blockIdx.x >= num_tiles) return;
    auto stage = [&](int s) { return reinterpret_cast<T*>(smem_raw + (size_t)s * Sh::STAGE); };
    unsigned claimed = 1;  // tiles this CTA took (thread 0), at most max_tiles
    auto claim_next = [&]() -> uint64_t {
        if (claimed >= max_tiles) return num_tiles;
        ++claimed;
        return G + (uint64_t)atomicAdd(claim, 1u);
    };
    // thread 0's look-ahead: the next tile (with its splits) and the one after
    uint64_t nt = num_tiles, ft = num_tiles;
    int64_t n0 = 0, n1 = 0;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
    }
    // launched as a dependent of the partition kernel: wait for its splits and
    // counter. (The kernel does not release its own dependents early: the next
    // partition launches as the CTAs exit. Releasing them at the start, so that
    // they take SM slots while this grid still merges, made a 1 GiB sort 25 %
    // slower.)
    grid_dep_wait();
    // an earlier pass gave up on a wait: its output is not sorted, stop here
    if (__syncthreads_or(tid == 0 && err_wait_set(err))) return;
    if (tid == 0) {
        const uint64_t t0 = blockIdx.x;
        geom[0] = pair_bulk_issue<T, TILE>(stage(0), src, n, run, t0, splits[t0], splits[t0 + 1], &bar[0], err);
        nt = claim_next();
        if (nt < num_tiles) {
            n0 = splits[nt];
            n1 = splits[nt + 1];
            ft = claim_next();
        }
    }
    __syncthreads();
    uint32_t phase = 0;  // bit s: parity of stage s's next completion
    for (int s = 0;; s ^= 1) {
        // geom[s] was written before the previous iteration's barriers
        const BulkTileGeom q = geom[s];
        if (q.tile >= num_tiles) break;
        if (tid == 0) {
            if (nt < num_tiles) {
                bulk_wait_read<0>();  // the other stage's last store has left shared memory
                geom[s ^ 1] = pair_bulk_issue<T, TILE>(stage(s ^ 1), src, n, run, nt, n0, n1, &bar[s ^ 1], err);
            } else {
                geom[s ^ 1].tile = num_tiles;
            }
            nt = ft;
            if (nt < num_tiles) {
                n0 = splits[nt];
                n1 = splits[nt + 1];
                ft = claim_next();
            }
        }
        const bool ok = mbar_wait(&bar[s], (phase >> s) & 1u, spin);
        if (__syncthreads_or(!ok)) {
            // drain this stage's loads and the other stage's (if issued)
            // before shared memory goes
            if (tid == 0)
                bulk_drain<2>(err, bar, (1u << s) | (geom[s ^ 1].tile < num_tiles ? 1u << (s ^ 1) : 0u), phase);
            return;
        }
        phase ^= 1u << s;
        T* buf = stage(s);
        const int total = q.na + q.nb;
        // one merge round, outputs kept in registers until every thread has
        // read its inputs, then written back over the stage
        const int nblk = (total + VO - 1) / VO;
        if (tid < nblk) split[tid] = merge_path_ix<T, LinIdx>(buf, q.as, q.na, q.bs, q.nb, tid * VO);
        __syncthreads();
        T r[VT];
        const int diag = tid * VO;
        const int cnt = tid < nblk ? min(VO, total - diag) : 0;
        if (tid < nblk) {
            const int sa = split[tid];
            const int ea = (tid + 1 < nblk) ? split[tid + 1] : q.na;
            merge_block_regs<T, VT, STABLE>(buf, q.as + sa, q.bs + (diag - sa), ea - sa, cnt, r);
        }
        __syncthreads();
        if (cnt == VO) {
#pragma unroll
            for (int i = 0; i < VO; ++i) buf[diag + i] = Traits<T>::flip(r[i], xout);
        } else {
#pragma unroll
            for (int i = 0; i < VO; ++i)
                if (i < cnt) buf[diag + i] = Traits<T>::flip(r[i], xout);
        }
        fence_async_smem();
        __syncthreads();
        // output tile starts 16-byte aligned (a multiple of TILE)
        T* out = dst + q.tile * TILE;
        const int nvec = total / V;
        if (tid == 0 && nvec) {
            bulk_store(out, buf, (uint32_t)nvec * 16u);
            bulk_commit();
        }
        // a ragged end (the array's last tile only, so no later tile refills
        // this stage) is stored item by item
        for (int i = nvec * V + tid; i < total; i += NT) out[i] = buf[i];
    }
    if (tid == 0) bulk_wait_read<0>();
}

}  // namespace origami
