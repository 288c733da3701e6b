// Sampled k-way merge pass: the GPU form of the reference's cache-resident
// merge tree (merge_tree.h: Merge4Way nodes, MergeTreeEven/Odd, used by
// sort_single_thread's phase 3 when min_k > 2, sorter.h:3871-3913) with its
// parallel partitioner (Partition.h:118-166) replaced by sample cuts.
//
// One pass merges groups of F (4, 8 or 16) consecutive sorted runs of R items.
// Work is cut without re-reading the runs:
//
//  samples        - the kernel that wrote the runs also wrote every S-th key
//                   (sample i = key of item (i+1)*S-1, one array for the whole
//                   input) and every SS-th sample (super-samples);
//  ranges (K4)    - for groups with more than KB_RANGE_SS super-samples,
//                   kway_split_kernel computes the exact split of every
//                   run's super-samples at evenly spaced super-sample ranks;
//  tiles (K4)     - kb_cut_kernel, one CTA per range: the range boundaries
//                   are concrete super-samples, refined to exact sample
//                   positions by one short search per run in the sample
//                   array; the range's samples are merged in shared memory and
//                   every M-th merged sample becomes a tile cut. A cut is a
//                   concrete item (the sample), stored with the number of
//                   samples of every run at or before it, so its exact item
//                   position in each run lies inside one S-item block;
//  merge (K3)     - kb_merge_kernel, persistent with claimed tiles: for each
//                   run the tile's samples plus the S-item block at either end
//                   arrive by cp.async.bulk (the 16-byte chunks enclosing
//                   them) into one of two stages while the other stage merges;
//                   one search per run inside each boundary block, in shared
//                   memory, gives the exact slices (the same search on the same
//                   block in the tile on either side of a cut, so neighbouring
//                   tiles agree). A tile therefore holds at most (M + F) * S
//                   items under any key distribution (every run contributes its
//                   samples in the tile plus one partial block), and no kernel
//                   reads the runs outside the merge itself;
//                   log2(F) rounds of merge path merge
//                   the slices in place (every thread keeps its output block
//                   in registers until all have read their inputs); the tile
//                   leaves by one bulk store of its whole 16-byte chunks plus
//                   single-thread stores of the ragged ends, and its samples
//                   for the next pass are written on the way.
//
// One HBM read and write of the items covers log2(F) merge levels.
//
// Ties: items are ordered by (key, run, position), which makes the merge stable
// across runs (key-value items keep their input order on equal keys) and gives
// every item exactly one place; samples are ordered the same way.
#pragma once
#include "bulk.cuh"
#include "common.cuh"
#include "kway.cuh"
#include "merge_core.cuh"

namespace origami {

// Per item type: sample stride S (items), merged samples per tile M (a tile
// holds M*S items nominally, at most (M + 16) * S), merge threads NT, merge
// registers VT (keys: blocks of VT-1 outputs, bitonic; key-value: serial
// blocks of VT), resident CTAs per SM the merge kernel is built for.
template <class T>
struct KbCfg;
template <>
struct KbCfg<uint32_t> {
    static constexpr int S = 64, M = 48, NT = 160, VT = 32, MINB = 6;
};
template <>
struct KbCfg<uint64_t> {
    static constexpr int S = 32, M = 48, NT = 160, VT = 16, MINB = 5;
};
template <>
struct KbCfg<KV64> {
    static constexpr int S = 16, M = 64, NT = 128, VT = 11, MINB = 4;
};
constexpr int KB_SS = 64;        // samples per super-sample
constexpr int KB_RANGE_SS = 32;  // super-samples per range (nominal) when a group is split
constexpr int KB_CUT_NT = 256;   // threads of the cut kernel

template <class T>
struct KbShape {
    using C = KbCfg<T>;
    using K = typename Traits<T>::Key;
    using E = SampleE<K>;
    static constexpr bool STABLE = Traits<T>::kStable;
    static constexpr int V = Vec<T>::N;
    static constexpr int TMAX = (C::M + KWAY_MAX) * C::S;  // items in a tile at most
    static constexpr int VO = Block<T, C::VT, STABLE>::VO;
    // each slice adds at most 2*(V-1) items of chunk padding; the final round
    // writes at an offset below V; merge blocks read up to VT items past a list
    static constexpr int CAP = TMAX + KWAY_MAX * 2 * V + 2 * V + C::VT + 2;
    static constexpr size_t STAGE = ((size_t)CAP * sizeof(T) + 127) & ~(size_t)127;
    static constexpr size_t SMEM = 2 * STAGE;
    static constexpr int MAXBLK = TMAX / VO + KWAY_MAX / 2 + 1;
    static_assert(C::NT >= MAXBLK, "every thread owns at most one merge block per round");
    // samples of one range at most: (super-samples in the range + one per run) * SS
    static constexpr int RANGE_SMAX = (KB_RANGE_SS + KWAY_MAX) * KB_SS;
    static constexpr int TPR = RANGE_SMAX / C::M + 2;  // tile slots per range
    // cut kernel shared memory: two sample buffers, then the per-tile tables
    static constexpr int EVT = 7;  // sample merge: serial blocks of 7
    static constexpr size_t SBUF = ((size_t)(RANGE_SMAX + EVT + 2) * sizeof(E) + 15) & ~(size_t)15;
    static constexpr size_t CUT_SMEM = 2 * SBUF + (size_t)(TPR + 1) * KWAY_MAX * 4;
    static constexpr int CUT_MAXBLK = RANGE_SMAX / EVT + KWAY_MAX + 2;
};

// Ranges per group of a pass: 1 when the group's samples fit one cut CTA.
template <class T>
inline int kb_ranges_per_group(uint64_t run, int fan) {
    const uint64_t g0 = run * (uint64_t)fan / ((uint64_t)KbCfg<T>::S * KB_SS);  // super-samples of a full group
    return g0 <= (uint64_t)KB_RANGE_SS ? 1 : (int)((g0 + KB_RANGE_SS - 1) / KB_RANGE_SS);
}

// The runs of group g: run k = [base + k*run, base + k*run + len(k)).
struct KbGroup {
    uint64_t base, run, n;
    __device__ __forceinline__ KbGroup(uint64_t g, uint64_t n_, uint64_t run_, int fan)
        : base(g * run_ * (uint64_t)fan), run(run_), n(n_) {}
    __device__ __forceinline__ uint64_t start(int k) const { return base + (uint64_t)k * run; }
    __device__ __forceinline__ uint64_t len(int k) const {
        const uint64_t s = start(k);
        return s >= n ? 0 : (n - s < run ? n - s : run);
    }
};

// Number of items of run `a` in [lo, hi) that precede a cut item of key y from
// run jy (items of earlier runs precede on equal keys, later ones follow):
// binary search, lo + count returned.
template <class T, class K>
__device__ __forceinline__ uint64_t kb_refine(const T* a, uint64_t lo, uint64_t hi, K y, bool earlier) {
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        const K v = Traits<T>::key(a[mid]);
        if (earlier ? (v <= y) : (v < y))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Samples of a sorted tile of `valid` items held in shared memory (`tile`,
// unpadded) whose first item is global item `base` (a multiple of S): called
// by the tile sort, every thread of the CTA (nthr of them).
// (A tile holds a whole number of super-samples: base is a multiple of S*SS.)
template <class T>
__device__ __forceinline__ void kb_emit_samples(const T* tile, uint64_t base, int valid,
                                                typename Traits<T>::Key* samp, typename Traits<T>::Key* ssamp,
                                                int nthr) {
    constexpr int S = KbCfg<T>::S;
    typename Traits<T>::Key* sp = samp + base / S;
    typename Traits<T>::Key* ssp = ssamp + base / (S * KB_SS);
    for (int j = threadIdx.x; j < valid / S; j += nthr) {
        const auto k = Traits<T>::key(tile[j * S + S - 1]);
        sp[j] = k;
        if ((j & (KB_SS - 1)) == KB_SS - 1) ssp[j / KB_SS] = k;
    }
}

// Samples of the items written by a kernel that does not produce them itself:
// samp[i] = key of src[(i+1)*S - 1] for i < n/S, and every SS-th of them into
// ssamp (strided reads, about one 32-byte sector per S items).
template <class T>
__global__ void kb_gather_samples_kernel(const T* __restrict__ src, uint64_t n, typename Traits<T>::Key* samp,
                                         typename Traits<T>::Key* ssamp) {
    constexpr int S = KbCfg<T>::S;
    const uint64_t ns = n / S;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (uint64_t)gridDim.x * blockDim.x) {
        const auto k = Traits<T>::key(src[(i + 1) * S - 1]);
        samp[i] = k;
        if (i % KB_SS == KB_SS - 1) ssamp[i / KB_SS] = k;
    }
}

// ------------------------------------------------------------- K4: cuts ---
// Cut table of the ranges of a pass: for range r, cuts c = 0 .. ntiles[r]
// (c = 0 is the range's start; tile c lies between cuts c and c+1):
//   q[r][c][k]  samples of run k at or before the cut (uint32)
//   key[r][c]   the cut item's key (a sample of run run[r][c])
//   run[r][c]   that run; -1: the group's start (all q = 0), -2: the group's
//               end (every run to its last item)
struct KbCuts {
    uint32_t* q;
    void* key;
    int* run;
};

// One CTA per range (blockIdx.x = g * rpg + b): writes the range's cut table,
// and appends its tiles (as slots r * TPR + c) to the pass's tile list
// tiles[0 .. *ntiles) (*ntiles is 0 at launch). bnd0 (rpg > 1):
// kway_split_kernel's super-sample counts per range boundary,
// [g * (rpg+1) + b][KWAY_MAX]. The first CTA resets the merge kernel's claim
// counter.
template <class T>
__global__ void __launch_bounds__(KB_CUT_NT) kb_cut_kernel(const typename Traits<T>::Key* __restrict__ samp,
                                                          uint64_t n, uint64_t run, int fan, int rpg,
                                                          const int64_t* __restrict__ bnd0, KbCuts cuts,
                                                          uint32_t* __restrict__ tiles, unsigned* __restrict__ ntiles,
                                                          unsigned* __restrict__ claim, int* __restrict__ err) {
    using Sh = KbShape<T>;
    using K = typename Sh::K;
    using E = typename Sh::E;
    constexpr int S = KbCfg<T>::S, M = KbCfg<T>::M, NT = KB_CUT_NT, TPR = Sh::TPR;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    E* sA = reinterpret_cast<E*>(smem_raw);
    E* sB = reinterpret_cast<E*>(smem_raw + Sh::SBUF);
    uint32_t* hist = reinterpret_cast<uint32_t*>(smem_raw + 2 * Sh::SBUF);  // [TPR+1][KWAY_MAX]
    __shared__ int off[KWAY_MAX + 1];
    __shared__ int mblk[Sh::CUT_MAXBLK];
    __shared__ uint64_t qs[2][KWAY_MAX];  // sample co-ranks of the range's start / end cut
    __shared__ uint64_t rns[KWAY_MAX];
    __shared__ K cy[2];                   // keys of the start / end cut items
    __shared__ int cj[2];                 // their runs (-1: group start / group end)
    __shared__ int cnt_all;
    __shared__ unsigned tbase;
    const int tid = threadIdx.x;
    const uint64_t bid = blockIdx.x;
    const uint64_t g = bid / (uint64_t)rpg;
    const int b = (int)(bid % (uint64_t)rpg);
    const KbGroup grp(g, n, run, fan);
    if (bid == 0 && tid == 0) *claim = 0;
    // a wait of an earlier kernel expired: the runs are not sorted, no tiles
    if (__syncthreads_or(tid == 0 && err_wait_set(err))) return;
    if (tid < KWAY_MAX) rns[tid] = (tid < fan ? grp.len(tid) : 0) / S;
    __syncthreads();
    const uint64_t sbase = grp.base / S;  // group's first sample (runs start at multiples of S)
    const uint64_t rs = run / S;          // samples per full run

    // --- range boundaries: sample co-ranks of the start (e = 0) and end (e = 1) cut
    for (int e = 0; e < 2; ++e) {
        const int bb = b + e;
        const bool group_start = bb == 0, group_end = bb == rpg;
        if (tid < 32) {
            // the cut is the largest of the runs' last super-samples before it,
            // by (key, run); lane k looks at run k
            const int k = tid;
            K key = 0;
            bool has = false;
            uint64_t q0 = 0;
            if (!group_start && !group_end && k < fan) {
                q0 = (uint64_t)bnd0[(g * (uint64_t)(rpg + 1) + bb) * KWAY_MAX + k];
                if (q0 > 0) {
                    has = true;
                    key = samp[sbase + (uint64_t)k * rs + q0 * KB_SS - 1];
                }
            }
            // lexicographic max over lanes (key, run)
            K bk = key;
            int bj = has ? k : -1;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const K ok = __shfl_xor_sync(0xFFFFFFFFu, bk, o);
                const int oj = __shfl_xor_sync(0xFFFFFFFFu, bj, o);
                if (oj >= 0 && (bj < 0 || ok > bk || (ok == bk && oj > bj))) {
                    bk = ok;
                    bj = oj;
                }
            }
            if (k == 0) {
                cy[e] = bk;
                cj[e] = group_end ? -2 : bj;  // -1: nothing before the cut (group start)
            }
            if (k < KWAY_MAX) {
                uint64_t v;
                if (group_end || k >= fan) {
                    v = k < fan ? rns[k] : 0;
                } else if (bj < 0) {
                    v = 0;
                } else if (k == bj) {
                    v = q0 * KB_SS;
                } else {
                    // window of run k's samples: one super-block
                    const uint64_t lo = q0 * KB_SS;
                    const uint64_t hi = min(lo + KB_SS - 1, rns[k]);
                    v = kb_refine<K, K>(samp + sbase + (uint64_t)k * rs, lo, hi, bk, k < bj);
                }
                qs[e][k] = v;
            }
        }
        __syncthreads();
    }
    // --- the range's samples, tagged (index in range << 4 | run). For sorted
    // runs the end cut never precedes the start cut and a range holds at most
    // RANGE_SMAX samples; otherwise the range is reported and left empty.
    if (tid == 0) {
        uint64_t o = 0;
        bool bad = false;
        for (int k = 0; k < KWAY_MAX; ++k) {
            if (qs[1][k] < qs[0][k]) {
                bad = true;
                qs[1][k] = qs[0][k];
            }
            o += qs[1][k] - qs[0][k];
        }
        if (bad || o > (uint64_t)Sh::RANGE_SMAX) {
            err_first(err, ERR_BAD_RUNS);
            for (int k = 0; k < KWAY_MAX; ++k) qs[1][k] = qs[0][k];
        }
        int c = 0;
        for (int k = 0; k < KWAY_MAX; ++k) {
            off[k] = c;
            c += (int)(qs[1][k] - qs[0][k]);
        }
        off[KWAY_MAX] = c;
        cnt_all = c;
    }
    __syncthreads();
    const int cnt = cnt_all;
    // one flat pass over the range's samples: item x belongs to the run k with
    // off[k] <= x < off[k+1] (all loads independent)
#pragma unroll 4
    for (int x = tid; x < cnt; x += NT) {
        int k = 0;
#pragma unroll
        for (int q = 1; q < KWAY_MAX; ++q) k += (off[q] <= x) ? 1 : 0;
        const int i = x - off[k];
        E e;
        e.key = samp[sbase + (uint64_t)k * rs + qs[0][k] + (uint64_t)i];
        e.tag = ((uint32_t)i << 4) | (uint32_t)k;
        sA[x] = e;
    }
    __syncthreads();
    E* merged = sA;
    if (cnt > 0) merged = merge_lists<E, NT, Sh::EVT, KWAY_MAX / 2, true>(sA, sB, off, fan, mblk);

    // --- tile cuts at merged positions M-1, 2M-1, ... and the range end
    const bool last_range = (b == rpg - 1);
    const int nfull = cnt / M;
    const int nt = nfull + ((last_range || cnt % M) ? 1 : 0);  // tiles of this range
    if (tid == 0) tbase = atomicAdd(ntiles, (unsigned)nt);
    for (int q = tid; q < (nt + 1) * KWAY_MAX; q += NT) hist[q] = 0;
    __syncthreads();
    for (int c = tid; c < nt; c += NT) tiles[tbase + c] = (uint32_t)(bid * TPR + (uint64_t)c);
    for (int x = tid; x < cnt; x += NT) atomicAdd(&hist[(x / M) * KWAY_MAX + (merged[x].tag & 15)], 1u);
    __syncthreads();
    // inclusive prefix over tiles: hist[t][k] = run-k samples at merged positions <= end of tile t
    if (tid < KWAY_MAX) {
        uint32_t acc = 0;
        for (int t = 0; t < nt; ++t) {
            acc += hist[t * KWAY_MAX + tid];
            hist[t * KWAY_MAX + tid] = acc;
        }
    }
    __syncthreads();
    const uint64_t row = bid * (uint64_t)(TPR + 1);
    for (int q = tid; q < (nt + 1) * KWAY_MAX; q += NT) {
        const int c = q / KWAY_MAX, k = q % KWAY_MAX;
        uint64_t v = 0;
        if (k >= fan) {
            v = 0;
        } else if (c == 0) {
            v = qs[0][k];
        } else if (c == nt && last_range) {
            v = rns[k];
        } else {
            v = qs[0][k] + hist[(c - 1) * KWAY_MAX + k];  // run-k samples up to the cut
        }
        cuts.q[row * KWAY_MAX + q] = (uint32_t)v;
    }
    for (int c = tid; c <= nt; c += NT) {
        K y = 0;
        int j;
        if (c == 0) {
            y = cy[0];
            j = cj[0];
        } else if (c == nt && last_range) {
            j = -2;
        } else {
            const E e = merged[(c == nt) ? cnt - 1 : c * M - 1];  // the cut sample
            y = e.key;
            j = (int)(e.tag & 15);
        }
        static_cast<K*>(cuts.key)[row + c] = y;
        cuts.run[row + c] = j;
    }
}

// ------------------------------------------------------------ K3: merge ---
// F-way merge of the lists of one tile in place: list k at buf[lst[k] ..
// lst[k] + len[k]) (geometry in shared memory, ping-ponged between rounds in
// geo[2][2][KWAY_MAX]); round r merges lists (2p, 2p+1) into a list at the
// first one's place; the last round writes the result to buf[out0 ..] through
// the item transform xo. Each thread owns at most one output block per round.
template <class T, int NT, int VT, bool STABLE>
__device__ __forceinline__ void kb_merge_tile(T* buf, int (*geo)[2][KWAY_MAX], int fan, int out0, uint64_t xo,
                                             int* split) {
    constexpr int VO = Block<T, VT, STABLE>::VO;
    const int tid = threadIdx.x;
    int cur = 0;
    for (int nl = fan; nl > 1; nl >>= 1) {
        const int* lst = geo[cur][0];
        const int* len = geo[cur][1];
        const int npairs = nl >> 1;
        const bool last = npairs == 1;
        // the pair (and block within it) this thread merges
        int p = -1, first = 0, nbp = 0, acc = 0;
#pragma unroll
        for (int q = 0; q < KWAY_MAX / 2; ++q) {
            if (q < npairs) {
                const int nb = (len[2 * q] + len[2 * q + 1] + VO - 1) / VO;
                if (tid >= acc && tid < acc + nb) {
                    p = q;
                    first = acc;
                    nbp = nb;
                }
                acc += nb;
            }
        }
        int a0 = 0, la = 0, b0 = 0, lb = 0, diag = 0;
        T r[VT];
        int cnt = 0;
        if (p >= 0) {
            a0 = lst[2 * p];
            la = len[2 * p];
            b0 = lst[2 * p + 1];
            lb = len[2 * p + 1];
            diag = (tid - first) * VO;
            cnt = min(VO, la + lb - diag);
        }
        // the block's end split comes from the next block's search
        if (p >= 0) split[tid] = merge_path_ix<T, LinIdx>(buf, a0, la, b0, lb, diag);
        __syncthreads();
        if (p >= 0) {
            const int sa = split[tid];
            const int ea = (tid - first + 1 < nbp) ? split[tid + 1] : la;
            merge_block_regs<T, VT, STABLE>(buf, a0 + sa, b0 + (diag - sa), ea - sa, cnt, r);
        }
        // next round's geometry (the other buffer; nothing reads it this round)
        if (tid < npairs) {
            geo[cur ^ 1][0][tid] = geo[cur][0][2 * tid];
            geo[cur ^ 1][1][tid] = geo[cur][1][2 * tid] + geo[cur][1][2 * tid + 1];
        }
        __syncthreads();
        if (p >= 0) {
            T* w = buf + (last ? out0 : a0) + diag;
            const uint64_t x = last ? xo : 0;
            if (x) {
#pragma unroll
                for (int i = 0; i < VO; ++i) r[i] = Traits<T>::flip(r[i], x);
            }
            if (cnt == VO) {
#pragma unroll
                for (int i = 0; i < VO; ++i) w[i] = r[i];
            } else {
#pragma unroll
                for (int i = 0; i < VO; ++i)
                    if (i < cnt) w[i] = r[i];
            }
        }
        __syncthreads();
        cur ^= 1;
    }
}

// A tile staged in shared memory (written by warp 0).
struct KbTileGeom {
    uint64_t slot;  // ~0: none (the CTA is done)
    uint64_t g;     // its group
    uint64_t o;     // first output item (after the boundary search)
    int total;      // items (after the boundary search)
};

// Per-run state of a staged tile (lane k of warp 0 keeps run k's).
struct KbSlice {
    uint64_t a;  // first staged item, offset in the run
    int lst;     // its stage index
    int len;     // staged items
    int dq;      // samples of the run in the tile: its end block starts at dq * S
};

// Persistent merge of every tile of the pass: tiles[0 .. *ntiles) (slots
// range * TPR + c, listed by the cut kernels). A CTA starts with tile
// blockIdx.x and claims later ones from *claim (reset by the cut kernel).
// Warp 0 stages the tiles: lane k handles run k, lane 0 the claims and the
// barrier; once a tile has landed it finds the exact slice of each run by one
// search in the block at each end. ntiles_next (may be null): the next pass's
// tile counter, reset here. samp_out / ssamp_out (may be null): samples of the
// output for the next pass.
template <class T>
__global__ void __launch_bounds__(KbCfg<T>::NT, KbCfg<T>::MINB)
    kb_merge_kernel(const T* __restrict__ src, T* __restrict__ dst, uint64_t n, uint64_t run, int fan, int rpg,
                    KbCuts cuts, const uint32_t* __restrict__ tiles, const unsigned* __restrict__ ntiles,
                    unsigned* __restrict__ ntiles_next, uint64_t xout, typename Traits<T>::Key* __restrict__ samp_out,
                    typename Traits<T>::Key* __restrict__ ssamp_out, unsigned* __restrict__ claim, int* err,
                    uint32_t spin) {
    using Sh = KbShape<T>;
    using C = KbCfg<T>;
    using K = typename Sh::K;
    constexpr int V = Sh::V, S = C::S, TPR = Sh::TPR, NT = C::NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int split[Sh::MAXBLK + 1];
    __shared__ int geo[2][2][2][KWAY_MAX];  // [stage][ping-pong][start, len][list]
    __shared__ KbTileGeom tg[2];
    __shared__ KbSlice sl[2][KWAY_MAX];
    __shared__ K cutk[2][2];                // [stage][start / end cut]: key
    __shared__ int cutj[2][2];              // run of the cut item (-1 group start, -2 group end)
    __shared__ __align__(8) uint64_t bar[2];
    const int tid = threadIdx.x, lane = tid & 31;
    const uint64_t G = gridDim.x;
    const K* ckey = static_cast<const K*>(cuts.key);
    auto stage = [&](int s) { return reinterpret_cast<T*>(smem_raw + (size_t)s * Sh::STAGE); };
    // Warp 0 runs a three-step look-ahead over the pass's tile list, one step
    // per tile merged, so that no global load it makes is waited for:
    //   claim  a tile index (lane 0's atomic)       (cpend)
    //   load   its slot from the tile list        (mid, mslot)
    //   load   its cuts: lane k's sample counts of run k, the cut items (nslot, ...)
    // and the tile with loaded cuts is staged next.
    const uint64_t NTL = *ntiles;  // tiles of the pass (the cut kernels have finished)
    uint64_t cpend = NTL, mid = NTL;
    uint32_t mslot = 0;
    uint64_t nslot = ~0ull;  // slot staged next (~0: none)
    uint32_t qa = 0, qe = 0;
    K ya = 0, ye = 0;
    int ja = -1, je = -2;
    auto fetch = [&]() {  // the cuts of tile `mid` (its slot loaded last step)
        nslot = mid < NTL ? (uint64_t)mslot : ~0ull;
        if (mid < NTL) {
            const uint64_t row = (nslot / TPR) * (uint64_t)(TPR + 1) + nslot % TPR;  // cut c of the range
            if (lane < KWAY_MAX) {
                qa = cuts.q[row * KWAY_MAX + lane];
                qe = cuts.q[(row + 1) * KWAY_MAX + lane];
            }
            ya = ckey[row];
            ye = ckey[row + 1];
            ja = cuts.run[row];
            je = cuts.run[row + 1];
        }
    };
    auto step = [&]() {  // warp 0: advance the look-ahead by one tile
        fetch();
        mid = __shfl_sync(0xFFFFFFFFu, cpend, 0);  // the claim made one step ago
        if (mid < NTL) mslot = tiles[mid];
        if (lane == 0) cpend = mid < NTL ? G + (uint64_t)atomicAdd(claim, 1u) : NTL;
    };
    // warp 0: stage the fetched tile into stage s (barrier bar[s]): for run k
    // the items from the block of cut c (its start, or the run's start at a
    // group start) to the end of the block of cut c+1 (or the run's end)
    auto issue = [&](int s) {
        const bool any = nslot != ~0ull;
        const uint64_t g = nslot / TPR / (uint64_t)rpg;
        const bool mine = lane < fan && any;
        const uint64_t rs = g * run * (uint64_t)fan + (uint64_t)lane * run;  // run start
        const uint64_t rl = mine ? (rs >= n ? 0 : (n - rs < run ? n - rs : run)) : 0;
        const uint64_t a = (ja < 0) ? 0 : (uint64_t)qa * S;
        uint64_t e = (je == -2) ? rl : (uint64_t)qe * S + S - 1;
        e = e < rl ? e : rl;
        // staged slices of sorted runs lie in their runs and hold at most TMAX
        // items in all; anything else (runs that are not sorted) is reported
        // and the tile is left out
        const bool inside = !mine || (a <= e && e - a <= (uint64_t)Sh::TMAX && qe >= qa);
        int tl = (inside && mine) ? (int)(e - a) : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tl += __shfl_xor_sync(0xFFFFFFFFu, tl, o);
        const bool bad = __any_sync(0xFFFFFFFFu, !inside) || tl > Sh::TMAX;
        if (bad && lane == 0) err_first(err, ERR_BAD_RUNS);
        const int len = (mine && !bad) ? (int)(e - a) : 0;
        const uint64_t abs = rs + a;
        const int lead = len > 0 ? (int)(abs % V) : 0;
        const int nv = len > 0 ? (lead + len + V - 1) / V : 0;
        // exclusive prefix of the slices' vectors over the lanes
        int pre = nv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int x = __shfl_up_sync(0xFFFFFFFFu, pre, o);
            if (lane >= o) pre += x;
        }
        const int total_v = __shfl_sync(0xFFFFFFFFu, pre, 31);
        const int voff = pre - nv;
        if (lane < KWAY_MAX) {
            KbSlice v;
            v.a = mine ? a : 0;
            v.lst = voff * V + lead;
            v.len = len;
            v.dq = (mine && !bad) ? (int)(qe - qa) : 0;
            sl[s][lane] = v;
        }
        if (lane == 0) {
            tg[s].slot = nslot;
            tg[s].g = g;
            cutk[s][0] = ya;
            cutk[s][1] = ye;
            cutj[s][0] = bad ? -1 : ja;
            cutj[s][1] = bad ? -2 : je;
            if (any) mbar_arrive_expect(&bar[s], (uint32_t)total_v * 16u);
        }
        __syncwarp();
        if (any && nv > 0) bulk_load(stage(s) + voff * V, src + (abs - lead), (uint32_t)nv * 16u, &bar[s]);
    };
    // warp 0, after stage s has landed: exact slices. Run k starts after the
    // items of its first block that precede the start cut and ends after the
    // items of its last block that precede the end cut (items of earlier runs
    // precede an equal key, later ones follow; the cut's own run is exact).
    auto bounds = [&](int s) {
        const T* buf = stage(s);
        int b = 0, e = 0;
        uint64_t a = 0;
        if (lane < fan) {
            const KbSlice v = sl[s][lane];
            const int j0 = cutj[s][0], j1 = cutj[s][1];
            const T* p = buf + v.lst;
            if (j0 >= 0 && lane != j0) b = (int)kb_refine<T, K>(p, 0, (uint64_t)min(S - 1, v.len), cutk[s][0], lane < j0);
            if (j1 == -2 || v.len == 0) {
                e = v.len;
            } else {
                const int base = min(v.dq * S, v.len);
                e = (lane == j1) ? base
                                 : (int)kb_refine<T, K>(p, base, (uint64_t)min(base + S - 1, v.len), cutk[s][1],
                                                        lane < j1);
            }
            if (e < b) {  // cannot happen for sorted runs
                err_first(err, ERR_BAD_RUNS);
                e = b;
            }
            a = v.a + (uint64_t)b;
            geo[s][0][0][lane] = v.lst + b;
            geo[s][0][1][lane] = e - b;
        } else if (lane < KWAY_MAX) {
            geo[s][0][0][lane] = 0;
            geo[s][0][1][lane] = 0;
        }
        int tot = e - b;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            tot += __shfl_xor_sync(0xFFFFFFFFu, tot, o);
            a += __shfl_xor_sync(0xFFFFFFFFu, a, o);
        }
        if (lane == 0) {
            tg[s].o = tg[s].g * run * (uint64_t)fan + a;
            tg[s].total = tot;
        }
    };

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
    }
    // the next pass's cut kernel counts its tiles here
    if (blockIdx.x == 0 && tid == 0 && ntiles_next) *ntiles_next = 0;
    // a wait of an earlier kernel expired: the runs are not sorted, stop here
    if (__syncthreads_or(tid == 0 && err_wait_set(err))) return;
    if (blockIdx.x >= NTL) return;
    if (tid < 32) {
        // prime the look-ahead: this CTA's first tile is tile blockIdx.x
        mid = blockIdx.x;
        mslot = tiles[mid];
        if (lane == 0) cpend = G + (uint64_t)atomicAdd(claim, 1u);
        step();  // cuts of the first tile; slot of the second
        issue(0);
        step();  // cuts of the second tile; slot of the third
    }
    __syncthreads();
    uint32_t phase = 0;  // bit s: parity of stage s's next completion
    for (int s = 0;; s ^= 1) {
        if (tg[s].slot == ~0ull) break;
        // warp 0 stages the next tile into the other stage (its previous bulk
        // store has left shared memory), then advances the look-ahead
        if (tid < 32) {
            if (lane == 0) bulk_wait_read<0>();
            __syncwarp();
            issue(s ^ 1);
            step();
        }
        const bool ok = mbar_wait(&bar[s], (phase >> s) & 1u, spin);
        if (__syncthreads_or(!ok)) {
            if (tid == 0)
                bulk_drain<2>(err, bar, (1u << s) | (tg[s ^ 1].slot != ~0ull ? 1u << (s ^ 1) : 0u), phase);
            return;
        }
        phase ^= 1u << s;
        if (tid < 32) bounds(s);
        __syncthreads();
        const KbTileGeom q = tg[s];
        T* buf = stage(s);
        const int sh = (int)(q.o % V);  // stage index x holds output item q.o + x - sh
        kb_merge_tile<T, NT, C::VT, Sh::STABLE>(buf, geo[s], fan, sh, xout, split);
        fence_async_smem();
        __syncthreads();
        // whole 16-byte chunks [x0, x1) of the output by one bulk store, the
        // items before and after them by single threads
        T* op = dst + q.o - sh;
        const int x0 = sh ? V : 0;
        const int x1 = ((sh + q.total) / V) * V;
        if (x1 > x0) {
            if (tid == 0) {
                bulk_store(op + x0, buf + x0, (uint32_t)(x1 - x0) * (uint32_t)sizeof(T));
                bulk_commit();
            }
            const int head = x0 - sh, tail = sh + q.total - x1;
            if (tid < head)
                op[sh + tid] = buf[sh + tid];
            else if (tid < head + tail)
                op[x1 + tid - head] = buf[x1 + tid - head];
        } else {
            for (int i = tid; i < q.total; i += NT) op[sh + i] = buf[sh + i];
        }
        // the next pass's samples: output items p with p % S == S - 1
        if (samp_out) {
            const uint64_t p0 = q.o + (uint64_t)((S - 1) - (int)(q.o % S));
            for (uint64_t p = p0 + (uint64_t)tid * S; p < q.o + (uint64_t)q.total; p += (uint64_t)NT * S) {
                const K k = Traits<T>::key(buf[sh + (int)(p - q.o)]) ^ (K)xout;
                samp_out[p / S] = k;
                if ((p / S) % KB_SS == KB_SS - 1) ssamp_out[p / S / KB_SS] = k;
            }
        }
        __syncthreads();  // every thread is done reading this stage before it is refilled
    }
    if (tid == 0) bulk_wait_read<0>();
}

}  // namespace origami
