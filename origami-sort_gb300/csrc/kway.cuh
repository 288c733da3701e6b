// k-way merge passes (fan-in F <= 16): the GPU form of the reference's
// cache-resident merge tree (merge_tree.h: Merge4Way nodes, MergeTreeEven/Odd)
// and its parallel partitioner (Partition.h:118-166).
//
// One pass merges groups of F consecutive sorted runs. Work is cut in two
// levels, both exact and skew-proof:
//  * ranges  - kway_split_kernel (K4) computes, for evenly spaced output ranks
//              of a group, the exact split of every run (merge path in k
//              dimensions: all runs bisected together, see below);
//  * tiles   - inside a range, range_merge_kernel (K3) takes every S-th item of
//              each run as a sample, merges the samples in shared memory and
//              cuts the range at every m-th merged sample. A cut at a concrete
//              item is exact by construction (its split in run j is one short
//              binary search in an S-item block) and bounds every tile to at
//              most (m + F) * S items, whatever the key distribution.
// Each tile's F slices are staged in shared memory and merged by log2(F)
// rounds of merge path, so one HBM read + write covers log2(F) merge levels.
//
// Ties: items are ordered by (key, run index, position), which makes the merge
// stable across runs and gives every item exactly one place.
#pragma once
#include "bulk.cuh"
#include "common.cuh"
#include "merge_core.cuh"

namespace origami {

constexpr int KWAY_MAX = 16;

// ------------------------------------------------------------ samples ----
template <class K>
struct SampleE {
    K key;
    uint32_t tag;  // (index in run) << 4 | run
};
template <class K>
__device__ __forceinline__ bool less(const SampleE<K>& a, const SampleE<K>& b) {
    return a.key < b.key;
}

// Asynchronous global -> shared copy of one item (cp.async; no register staging).
template <class T>
__device__ __forceinline__ void cp_async_item(T* smem, const T* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (sizeof(T) == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(sizeof(T)));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// ------------------------------------------------------- K4: ranges ------
// Exact split of a group of runs at output rank r: for every run i the number
// s_i of its items among the r smallest of the group. One 256-thread block per
// split; thread (j, i) = (tid / 16, tid % 16).
//
// All runs are bisected together. Each round every run j with an open window
// [lo_j, hi_j) offers its middle item x_j as a probe; lane (j, i) counts the
// items of run i that precede x_j, clamped to run i's window (one binary search
// in the window). The clamped counts sum to less than r exactly when x_j is
// among the r smallest, which moves every window: lo_i up to the count under a
// probe on the left, hi_i down to the count under a probe on the right. Run
// j's own window at least halves each round, so the loop ends after at most
// ~log2(run) + 1 rounds with lo_i == hi_i == s_i for all i.
struct SplitGeom {
    uint64_t base, G;
    int nr;
    __device__ __forceinline__ SplitGeom(uint64_t g, uint64_t n, uint64_t run, int F) {
        base = g * run * (uint64_t)F;
        const uint64_t rest = n - base;
        G = rest < run * (uint64_t)F ? rest : run * (uint64_t)F;
        nr = (int)((G + run - 1) / run);
    }
    __device__ __forceinline__ uint64_t len(int i, uint64_t run) const {
        const uint64_t s = (uint64_t)i * run;
        return (i < nr) ? ((G - s) < run ? (G - s) : run) : 0;
    }
};

// Where the sorted lists of merge group g live. Sort passes merge groups of F
// consecutive runs of one array (RunLists); the merge-tree entry point merges
// up to KWAY_MAX independent streams as one group (StreamLists). A group gives
// list(i) / len(i) for its lists (len 0 past the last) and out_base(), the
// group's first output position.
template <class T>
struct RunGroup {
    const T* src;
    uint64_t base, G, run;
    int nr;
    __device__ __forceinline__ const T* list(int i) const { return src + base + (uint64_t)i * run; }
    __device__ __forceinline__ uint64_t len(int i) const {
        const uint64_t s = (uint64_t)i * run;
        return (i < nr) ? ((G - s) < run ? (G - s) : run) : 0;
    }
    __device__ __forceinline__ uint64_t out_base() const { return base; }
};

template <class T>
struct RunLists {
    const T* src;
    uint64_t n, run;
    int F;
    __device__ __forceinline__ RunGroup<T> group(uint64_t g) const {
        const SplitGeom geo(g, n, run, F);
        return RunGroup<T>{src, geo.base, geo.G, run, geo.nr};
    }
};

template <class T>
struct StreamLists {
    const T* ptr[KWAY_MAX];
    uint64_t cnt[KWAY_MAX];
    uint64_t G;  // sum of cnt
    int nr;      // streams in use
    __device__ __forceinline__ const StreamLists& group(uint64_t) const { return *this; }
    __device__ __forceinline__ const T* list(int i) const { return ptr[i]; }
    __device__ __forceinline__ uint64_t len(int i) const { return i < nr ? cnt[i] : 0; }
    __device__ __forceinline__ uint64_t out_base() const { return 0; }
};

// Keys as compared: xin flips the sign bit of signed keys read straight from a
// caller's buffer (0 for data the pipeline has already flipped).
template <class T>
__device__ __forceinline__ typename Traits<T>::Key ckey(const T& v, uint64_t xin) {
    return Traits<T>::key(v) ^ (typename Traits<T>::Key)xin;
}

template <class T, class Lists>
__global__ void __launch_bounds__(256) kway_split_kernel(const Lists lists, int rpg, uint64_t xin,
                                                         int64_t* __restrict__ bnd,
                                                         int* __restrict__ err) {
    using K = typename Traits<T>::Key;
    __shared__ int64_t lo[KWAY_MAX], hi[KWAY_MAX];
    __shared__ unsigned long long nlo[KWAY_MAX], nhi[KWAY_MAX];
    __shared__ int open;
    const int tid = threadIdx.x;
    const uint64_t g = blockIdx.x / (uint64_t)(rpg + 1);
    const int b = (int)(blockIdx.x % (uint64_t)(rpg + 1));
    const auto& geo = lists.group(g);
    const uint64_t r = (uint64_t)(((unsigned __int128)b * geo.G) / (uint64_t)rpg);
    int64_t* out = bnd + (uint64_t)blockIdx.x * KWAY_MAX;
    if (tid < KWAY_MAX) {
        const int64_t L = (int64_t)geo.len(tid);
        const int64_t others = (int64_t)geo.G - L;
        lo[tid] = (int64_t)r - others > 0 ? (int64_t)r - others : 0;
        hi[tid] = (int64_t)r < L ? (int64_t)r : L;
    }
    __syncthreads();
    const int j = tid >> 4, i = tid & 15;
    const T* runj = geo.list(j);
    const T* runi = geo.list(i);
    for (int round = 0; round < 80; ++round) {
        if (tid == 0) {
            int o = 0;
            for (int q = 0; q < KWAY_MAX; ++q) o |= (lo[q] < hi[q]);
            open = o;
        }
        if (tid < KWAY_MAX) {
            nlo[tid] = (unsigned long long)lo[tid];
            nhi[tid] = (unsigned long long)hi[tid];
        }
        __syncthreads();
        if (!open) break;
        const int64_t loj = lo[j], hij = hi[j];
        const bool probe = (j < geo.nr) && (loj < hij);
        const int64_t pj = loj + (hij - loj) / 2;
        K xk = 0;
        if (probe && i == j) xk = ckey(runj[pj], xin);
        xk = __shfl_sync(0xFFFFFFFFu, xk, (tid & 16) | j);
        int64_t c = 0;
        if (probe && i < geo.nr) {
            if (i == j) {
                c = pj;
            } else {
                int64_t a = lo[i], e = hi[i];
                const bool le = i < j;  // earlier runs precede on equal keys
                while (a < e) {
                    const int64_t mid = (a + e) >> 1;
                    const K v = ckey(runi[mid], xin);
                    if (le ? (v <= xk) : (v < xk))
                        a = mid + 1;
                    else
                        e = mid;
                }
                c = a;
            }
        }
        // sum over i within the 16-lane group
        int64_t sum = c;
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
        if (probe && i < geo.nr) {
            if ((uint64_t)sum < r)
                atomicMax(&nlo[i], (unsigned long long)(i == j ? pj + 1 : c));
            else
                atomicMin(&nhi[i], (unsigned long long)(i == j ? pj : c));
        }
        __syncthreads();
        if (tid < KWAY_MAX) {
            lo[tid] = (int64_t)nlo[tid];
            hi[tid] = (int64_t)nhi[tid];
        }
        __syncthreads();
        if (round == 79 && tid == 0) err_first(err, ERR_BAD_RUNS);  // sorted runs: windows halve, never 80 rounds
    }
    if (tid < KWAY_MAX) out[tid] = lo[tid];
}

// ------------------------------------------------------- K3: ranges ------
// Per item type: threads, items per thread per merge round, sample stride S,
// tile capacity TMAX (tiles hold at most (M + F) * S <= TMAX items, nominal
// M * S) and the exact range size RANGE produced by K4.
template <class T>
struct KwayCfg;
// NT threads; VT registers per merge block (blocks of VT-1 outputs for keys,
// VT for key-value); sample stride S; tile capacity TMAX (tiles hold at most
// (M + 16) * S items, nominal M * S with M = TMAX / S - 16); exact range size
// RANGE produced by K4.
template <>
struct KwayCfg<uint32_t> {
    static constexpr int NT = 256, VT = 32, S = 32, TMAX = 8704;
    static constexpr int RANGE = 1 << 17;
    static constexpr bool STABLE = false;
};
template <>
struct KwayCfg<uint64_t> {
    static constexpr int NT = 256, VT = 16, S = 32, TMAX = 4096;
    static constexpr int RANGE = 1 << 16;
    static constexpr bool STABLE = false;
};
template <>
struct KwayCfg<KV64> {
    static constexpr int NT = 256, VT = 7, S = 16, TMAX = 1792;
    static constexpr int RANGE = 1 << 15;
    static constexpr bool STABLE = true;
};

// Shared memory: three unpadded tile buffers (the tile being merged, the next
// one arriving by cp.async, and a merge scratch), then the per-range tables.
// While the range's samples are merged the three buffers serve as two halves
// of the sample ping-pong.
template <class T, class C = KwayCfg<T>>
struct KwayLayout {
    using K = typename Traits<T>::Key;
    using E = SampleE<K>;
    static constexpr int EVT = 7;  // sample merge: serial blocks of 7
    static constexpr int CAP_ITEMS = C::TMAX + C::VT + 2;  // per buffer, with read slack
    static constexpr size_t BUF_BYTES = ((size_t)CAP_ITEMS * sizeof(T) + 15) & ~(size_t)15;
    static constexpr size_t SBUF_BYTES = (3 * BUF_BYTES / 2) & ~(size_t)15;
    static constexpr int SCAP = (int)(SBUF_BYTES / sizeof(E)) - EVT - 2;
    static constexpr int M = C::TMAX / C::S - KWAY_MAX;  // merged samples per tile
    static constexpr int MAXTILES = C::RANGE / (M * C::S) + 2;
    static constexpr size_t TAB_BYTES =
        (size_t)(MAXTILES + 1) * KWAY_MAX * 4 * 2 + (size_t)(MAXTILES + 1) * (KWAY_MAX + 1) * 4;
    static constexpr size_t SMEM = 3 * BUF_BYTES + TAB_BYTES + 64;
    static constexpr int VO = Block<T, C::VT, C::STABLE>::VO;
    static constexpr int MAXBLK_T = C::TMAX / VO + KWAY_MAX + 2;
    static constexpr int MAXBLK_S = (C::RANGE / C::S) / EVT + KWAY_MAX + 2;
    static constexpr int MAXBLK = MAXBLK_T > MAXBLK_S ? MAXBLK_T : MAXBLK_S;
    static_assert(C::RANGE / C::S <= SCAP, "range samples must fit the sample buffers");
};

// Phase hook of range_merge_kernel: the default does nothing and compiles away;
// a measurement harness can pass a type that records clock64() per phase.
struct NoProbe {
    __device__ __forceinline__ void mark(int) {}
};

// One CTA per range. groups mode (bnd == nullptr): the range is a whole group.
// xin: sign flip applied to items as they are read (signed keys straight from a
// caller's buffer); xout: flip applied as they are written.
// block0 offsets the block index, so that a pass can be launched in slices of
// consecutive ranges.
// Runs that are not sorted (the caller's streams) can give inconsistent
// bounds and cuts: every range and tile is then clamped into its runs and the
// shared-memory capacities, err (optional) receives ERR_BAD_RUNS, and nothing
// is read or written out of bounds.
template <class T, class Lists, class C = KwayCfg<T>, class Probe = NoProbe>
__global__ void __launch_bounds__(C::NT) range_merge_kernel(
    const Lists lists, T* __restrict__ dst, int rpg, const int64_t* __restrict__ bnd, uint64_t xin,
    uint64_t xout, uint32_t block0 = 0, Probe probe = Probe(), int* err = nullptr) {
    static_assert(C::STABLE || !Traits<T>::kStable, "key-value items need the stable merge");
    using Lay = KwayLayout<T, C>;
    using K = typename Traits<T>::Key;
    using E = SampleE<K>;
    constexpr int NT = C::NT, VT = C::VT, S = C::S, M = Lay::M;
    (void)VT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto buf = [&](int i) { return reinterpret_cast<T*>(smem_raw + (size_t)i * Lay::BUF_BYTES); };
    uint32_t* sp = reinterpret_cast<uint32_t*>(smem_raw + 3 * Lay::BUF_BYTES);  // [MAXTILES+1][16]
    uint32_t* hist = sp + (Lay::MAXTILES + 1) * KWAY_MAX;                       // [MAXTILES+1][16]
    int* toff = reinterpret_cast<int*>(hist + (Lay::MAXTILES + 1) * KWAY_MAX);  // [MAXTILES+1][17]
    __shared__ int off[KWAY_MAX + 1];
    __shared__ int mblk[Lay::MAXBLK];  // merge-round block splits
    __shared__ const T* lo[KWAY_MAX];  // first item of each list's slice of this range
    __shared__ int64_t skip[KWAY_MAX];  // items of each list before the range
    __shared__ uint32_t len[KWAY_MAX];
    __shared__ uint64_t out_base;
    const int tid = threadIdx.x;

    // --- range geometry
    const uint64_t bid = (uint64_t)blockIdx.x + block0;
    const uint64_t g = bnd ? bid / (uint64_t)rpg : bid;
    const int rb = bnd ? (int)(bid % (uint64_t)rpg) : 0;
    const auto& geo = lists.group(g);
    if (tid < KWAY_MAX) {
        const uint64_t L = geo.len(tid);
        int64_t a = 0, e = (int64_t)L;
        if (bnd) {
            const int64_t* bb = bnd + ((uint64_t)g * (rpg + 1) + rb) * KWAY_MAX;
            a = bb[tid];
            e = bb[KWAY_MAX + tid];
        }
        // bounds of sorted runs always hold this
        if (a < 0 || a > (int64_t)L || e < a || e > (int64_t)L) {
            if (err) err_first(err, ERR_BAD_RUNS);
            a = a < 0 ? 0 : (a > (int64_t)L ? (int64_t)L : a);
            e = e < a ? a : (e > (int64_t)L ? (int64_t)L : e);
        }
        lo[tid] = geo.list(tid) + a;
        skip[tid] = a;
        len[tid] = (uint32_t)(e - a);
    }
    __syncthreads();
    if (tid == 0) {
        uint64_t ob = geo.out_base();
        for (int q = 0; q < KWAY_MAX; ++q) ob += (uint64_t)skip[q];
        out_base = ob;
        int o = 0;
        for (int q = 0; q < KWAY_MAX; ++q) {
            off[q] = o;
            o += (int)(len[q] / S);
        }
        off[KWAY_MAX] = o;
        if (o > Lay::SCAP) {  // a range of sorted runs never holds more samples
            if (err) err_first(err, ERR_BAD_RUNS);
            for (int q = 0; q < KWAY_MAX; ++q) {
                off[q] = 0;
                len[q] = 0;
            }
            off[KWAY_MAX] = 0;
        }
    }
    __syncthreads();
    const int nsamp = off[KWAY_MAX];
    const int nl = (geo.nr <= 1) ? 1 : (geo.nr <= 2 ? 2 : (geo.nr <= 4 ? 4 : (geo.nr <= 8 ? 8 : 16)));

    probe.mark(0);
    // --- fine samples: the last item of every full S-block of every run
    E* sA = reinterpret_cast<E*>(smem_raw);
    E* sB = reinterpret_cast<E*>(smem_raw + Lay::SBUF_BYTES);
    for (int q = 0; q < geo.nr; ++q) {
        const int c = off[q + 1] - off[q];
        const T* rp = lo[q];
        const int o0 = off[q];
        for (int k = tid; k < c; k += NT) {
            E e;
            e.key = ckey(rp[(uint64_t)(k + 1) * S - 1], xin);
            e.tag = ((uint32_t)k << 4) | (uint32_t)q;
            sA[o0 + k] = e;
        }
    }
    __syncthreads();  // runs beyond nr hold no samples, so off[nr..16] == nsamp
    probe.mark(1);
    E* merged = sA;
    if (nl > 1 && nsamp > 0) merged = merge_lists<E, NT, Lay::EVT, KWAY_MAX / 2, true>(sA, sB, off, nl, mblk);

    probe.mark(2);
    // --- tile cuts at merged samples M-1, 2M-1, ...
    const int nt = nsamp / M + 1;
    for (int q = tid; q < (nt + 1) * KWAY_MAX; q += NT) hist[q] = 0;
    __syncthreads();
    for (int q = tid; q < nsamp; q += NT) atomicAdd(&hist[(q / M) * KWAY_MAX + (merged[q].tag & 15)], 1u);
    __syncthreads();
    // exclusive prefix over tiles: hist[b][j] = run-j samples at merged positions < b*M
    if (tid < KWAY_MAX) {
        uint32_t acc = 0;
        for (int b = 0; b < nt; ++b) {
            const uint32_t h = hist[b * KWAY_MAX + tid];
            hist[b * KWAY_MAX + tid] = acc;
            acc += h;
        }
        hist[nt * KWAY_MAX + tid] = acc;
    }
    __syncthreads();
    probe.mark(3);
    // sp[b][j] = items of run j (relative to lo[j]) that precede cut b
    for (int q = tid; q < (nt + 1) * KWAY_MAX; q += NT) {
        const int b = q / KWAY_MAX, j = q % KWAY_MAX;
        uint32_t v;
        if (b == 0) {
            v = 0;
        } else if (b == nt || j >= geo.nr) {
            v = (j < geo.nr) ? len[j] : 0;
        } else {
            const E gs = merged[b * M - 1];
            const int gi = (int)(gs.tag & 15);
            const uint32_t pj = hist[b * KWAY_MAX + j];
            if (j == gi) {
                v = pj * S;
            } else {
                uint32_t a = pj * S;
                uint32_t e = min(a + (uint32_t)(S - 1), len[j]);
                const T* rp = lo[j];
                const bool le = j < gi;  // earlier runs precede on equal keys
                while (a < e) {
                    const uint32_t mid = (a + e) >> 1;
                    const K kv = ckey(rp[mid], xin);
                    if (le ? (kv <= gs.key) : (kv < gs.key))
                        a = mid + 1;
                    else
                        e = mid;
                }
                v = a;
            }
        }
        sp[q] = v;
    }
    __syncthreads();
    // cuts of sorted runs only move forward; make sure of it
    if (tid < KWAY_MAX) {
        for (int b = 1; b <= nt; ++b) {
            uint32_t& v = sp[b * KWAY_MAX + tid];
            if (v < sp[(b - 1) * KWAY_MAX + tid]) {
                v = sp[(b - 1) * KWAY_MAX + tid];
                if (err) err_first(err, ERR_BAD_RUNS);
            }
        }
    }
    __syncthreads();
    // per-tile list offsets: toff[t][q] = items of tile t taken from runs < q;
    // a tile larger than the buffers (runs that are not sorted) is left out
    for (int t = tid; t < nt; t += NT) {
        int o = 0;
        for (int q = 0; q < KWAY_MAX; ++q) {
            toff[t * (KWAY_MAX + 1) + q] = o;
            o += (int)(sp[(t + 1) * KWAY_MAX + q] - sp[t * KWAY_MAX + q]);
        }
        toff[t * (KWAY_MAX + 1) + KWAY_MAX] = o;
        if (o > C::TMAX) {
            if (err) err_first(err, ERR_BAD_RUNS);
            for (int q = 0; q <= KWAY_MAX; ++q) toff[t * (KWAY_MAX + 1) + q] = 0;
        }
    }
    __syncthreads();

    probe.mark(4);
    // --- tiles: cp.async prefetch of tile t+1 overlaps the merge of tile t
    auto issue = [&](int t, T* b) {
        const int* to = toff + t * (KWAY_MAX + 1);
        for (int q = 0; q < geo.nr; ++q) {
            const int o0 = to[q];
            const int l = (to[KWAY_MAX] == 0) ? 0 : to[q + 1] - o0;
            const T* rp = lo[q] + sp[t * KWAY_MAX + q];
            for (int k = tid; k < l; k += NT) cp_async_item(&b[o0 + k], rp + k);
        }
        cp_async_commit();
    };
    issue(0, buf(0));
    int cur = 0;
    for (int t = 0; t < nt; ++t) {
        const int nxt = cur == 0 ? 1 : 0;
        if (t + 1 < nt)
            issue(t + 1, buf(nxt));
        else
            cp_async_commit();
        probe.mark(5);
        cp_async_wait<1>();
        __syncthreads();
        probe.mark(6);
        const int* to = toff + t * (KWAY_MAX + 1);
        const int tot = to[KWAY_MAX];
        if (xin) {  // flip signed keys of the arrived tile in place
            T* tb = buf(cur);
            for (int k = tid; k < tot; k += NT) tb[k] = Traits<T>::flip(tb[k], xin);
            __syncthreads();
        }
        T* res = buf(cur);
        if (nl > 1)
            res = merge_lists<T, NT, C::VT, KWAY_MAX / 2, C::STABLE>(buf(cur), buf(2), to, nl, mblk);
        probe.mark(7);
        uint64_t ob = out_base;
        for (int q = 0; q < KWAY_MAX; ++q) ob += sp[t * KWAY_MAX + q];
        T* op = dst + ob;
        for (int k = tid; k < tot; k += NT) op[k] = Traits<T>::flip(res[k], xout);
        __syncthreads();
        probe.mark(8);
        cur = nxt;
    }
    cp_async_wait<0>();
}

}  // namespace origami
