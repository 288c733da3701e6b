/* Origami oracle: scalar C restatement of the reference CPU mergesort.
 *
 * TEST INFRASTRUCTURE ONLY. The checker used by tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline leg; never linked into the GPU library.
 * Pinned against the unmodified reference (oracle/_ref) and the committed
 * golden fixtures (tests/golden) by tests/test_oracle.py.
 *
 * Every routine below cites the reference routine it restates
 * (paths relative to the reference project root).
 */
#define _GNU_SOURCE
#include "origami_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- engines --
 * std::mt19937 and std::mt19937_64 with their default seeds (5489), restated
 * from the published Mersenne Twister definitions (Matsumoto & Nishimura 1998;
 * Nishimura 2000 for the 64-bit variant). writer.h:50-71 default-constructs both. */
typedef struct { uint32_t mt[624]; int i; } mt32_t;
static void mt32_seed(mt32_t* s, uint32_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 624; i++) s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->i = 624;
}
static uint32_t mt32_next(mt32_t* s) {
    if (s->i >= 624) {
        for (int k = 0; k < 624; k++) {
            uint32_t y = (s->mt[k] & 0x80000000u) | (s->mt[(k + 1) % 624] & 0x7fffffffu);
            s->mt[k] = s->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        s->i = 0;
    }
    uint32_t y = s->mt[s->i++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}
typedef struct { uint64_t mt[312]; int i; } mt64_t;
static void mt64_seed(mt64_t* s, uint64_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 312; i++)
        s->mt[i] = 6364136223846793005ull * (s->mt[i - 1] ^ (s->mt[i - 1] >> 62)) + (uint64_t)i;
    s->i = 312;
}
static uint64_t mt64_next(mt64_t* s) {
    if (s->i >= 312) {
        for (int k = 0; k < 312; k++) {
            uint64_t y = (s->mt[k] & 0xFFFFFFFF80000000ull) | (s->mt[(k + 1) % 312] & 0x7FFFFFFFull);
            s->mt[k] = s->mt[(k + 156) % 312] ^ (y >> 1) ^ ((y & 1ull) ? 0xB5026F5AA96619E9ull : 0ull);
        }
        s->i = 0;
    }
    uint64_t y = s->mt[s->i++];
    y ^= (y >> 29) & 0x5555555555555555ull;
    y ^= (y << 17) & 0x71D67FFFEDA60000ull;
    y ^= (y << 37) & 0xFFF7EEE000000000ull;
    y ^= y >> 43;
    return y;
}
/* std::uniform_int_distribution<int64_t>() over [0, INT64_MAX] driven by
 * mt19937_64, as libstdc++ (GCC 13) computes it: the range 2^63 is reached by
 * the multiply-high downscaling step, which for this range is exactly x >> 1
 * and never rejects. writer.h:52-65 default-constructs the distribution. */
static int64_t dist_i64_nonneg(mt64_t* g) { return (int64_t)(mt64_next(g) >> 1); }

/* ------------------------------------------------------------ kind table -- */
typedef struct { int64_t key; int64_t value; } kv_t;    /* KeyValue<i64,i64>, packed 16 B */
typedef struct { uint64_t key; uint64_t value; } kvu_t; /* unsigned-key variant */

unsigned orc_item_bytes(int kind) {
    switch (kind) {
        case ORC_U32: return 4;
        case ORC_U64: case ORC_I64: return 8;
        default: return 16;
    }
}
/* config.h:27-84 (REG_TYPE 0): _P1_N is 8 for 32- and 64-bit keys, 16 for 64+64;
 * config.h:265: _P2_N = (L2_BYTES >> 1) / sizeof(Item) with L2_BYTES = 1 MiB. */
uint64_t orc_p1_n(int kind) { return orc_item_bytes(kind) == 16 ? 16 : 8; }
uint64_t orc_p2_n(int kind) { return (uint64_t)(1u << 19) / orc_item_bytes(kind); }

/* ------------------------------------------------- per-type instantiation --
 * ORC_DEFINE(SFX, T, LESS) emits the whole pipeline for item type T ordered by
 * the strict weak order LESS(a,b) (key-only for KV items). */

#define ORC_DEFINE(SFX, T, LESS)                                                                      \
    /* phase1_sort, scalar path (sorter.h:3636-3828 with Reg == Item): sorts each                  \
     * block of P1_N items with a compare-exchange network. Restated with                          \
     * Batcher's odd-even merge network over the block (a power of two). */                        \
    static inline void cx_##SFX(T* a, uint64_t i, uint64_t j) {                                    \
        T x = a[i], y = a[j];                                                                       \
        int sw = LESS(y, x);                                                                        \
        a[i] = sw ? y : x;                                                                          \
        a[j] = sw ? x : y;                                                                          \
    }                                                                                               \
    static void network_sort_##SFX(T* a, uint64_t n) {                                             \
        if ((n & (n - 1)) != 0) { /* ragged tail block: insertion sort */                           \
            for (uint64_t i = 1; i < n; i++) {                                                      \
                T v = a[i];                                                                         \
                uint64_t j = i;                                                                     \
                while (j > 0 && LESS(v, a[j - 1])) { a[j] = a[j - 1]; j--; }                        \
                a[j] = v;                                                                           \
            }                                                                                       \
            return;                                                                                 \
        }                                                                                           \
        for (uint64_t p = 1; p < n; p <<= 1)                                                        \
            for (uint64_t k = p; k >= 1; k >>= 1)                                                   \
                for (uint64_t j = k % p; j + k < n; j += 2 * k)                                     \
                    for (uint64_t i = 0; i < k && i + j + k < n; i++)                               \
                        if ((i + j) / (2 * p) == (i + j + k) / (2 * p)) cx_##SFX(a, i + j, i + j + k); \
    }                                                                                               \
                                                                                                    \
    /* mergebl2_scalar (merger.h:46-236): branchless two-way merge. The next item                   \
     * is taken from A while A's head does not exceed B's head (the reference                      \
     * compares *loadFrom <= *opposite, merger.h:80), selected without a branch. */                 \
    static void merge2_##SFX(const T* A, uint64_t la, const T* B, uint64_t lb, T* C) {              \
        uint64_t i = 0, j = 0, k = 0;                                                               \
        while (i < la && j < lb) {                                                                  \
            int takeB = LESS(B[j], A[i]);                                                           \
            C[k++] = takeB ? B[j] : A[i];                                                           \
            j += (uint64_t)takeB;                                                                   \
            i += (uint64_t)(1 - takeB);                                                             \
        }                                                                                           \
        while (i < la) C[k++] = A[i++];                                                             \
        while (j < lb) C[k++] = B[j++];                                                             \
    }                                                                                               \
                                                                                                    \
    /* origami_merger::merge (merger.h:4079-4218): one level, every adjacent pair                   \
     * of merge_start-runs merged into dst; a ragged tail run is carried over. */                  \
    static void merge_level_##SFX(const T* src, T* dst, uint64_t n, uint64_t run) {                 \
        for (uint64_t base = 0; base < n; base += 2 * run) {                                        \
            uint64_t la = n - base < run ? n - base : run;                                          \
            uint64_t rest = n - base - la;                                                          \
            uint64_t lb = rest < run ? rest : run;                                                  \
            merge2_##SFX(src + base, la, src + base + la, lb, dst + base);                          \
        }                                                                                           \
    }                                                                                               \
    /* merge_series (merger.h:4220-4228), applied chunk by chunk of sort_n. */                      \
    static T* merge_series_##SFX(T* src, T* dst, uint64_t n, uint64_t merge_start,                  \
                                 uint64_t sort_n) {                                                 \
        while (merge_start < sort_n) {                                                              \
            for (uint64_t c = 0; c < n; c += sort_n) {                                              \
                uint64_t m = n - c < sort_n ? n - c : sort_n;                                       \
                merge_level_##SFX(src + c, dst + c, m, merge_start);                                \
            }                                                                                       \
            merge_start <<= 1;                                                                      \
            T* t = dst; dst = src; src = t;                                                         \
        }                                                                                           \
        return src;                                                                                 \
    }                                                                                               \
                                                                                                    \
    /* MergeTree::merge (merge_tree.h:2792-3010, 3410-3735): WAY-way merge. The                     \
     * reference builds it from 4-way nodes with small buffers; the result is the                  \
     * k-way merge, restated with a tournament over stream heads (ties: lower                      \
     * stream first). */                                                                            \
    static void kway_##SFX(T** X, T** endX, T* C, unsigned way) {                                   \
        T* cur[4096];                                                                               \
        unsigned tree[8192];                                                                        \
        unsigned leaves = 1;                                                                        \
        while (leaves < way) leaves <<= 1;                                                          \
        for (unsigned s = 0; s < way; s++) cur[s] = X[s];                                           \
        /* winner tree over stream ids; id >= way means "no stream" */                              \
        for (unsigned l = 0; l < leaves; l++) tree[leaves + l] = l;                                 \
        for (unsigned v = leaves - 1; v >= 1; v--) {                                                \
            unsigned a = tree[2 * v], b = tree[2 * v + 1];                                          \
            int aok = a < way && cur[a] < endX[a], bok = b < way && cur[b] < endX[b];               \
            tree[v] = (!bok || (aok && !LESS(*cur[b], *cur[a]))) ? a : b;                           \
        }                                                                                           \
        for (;;) {                                                                                  \
            unsigned w = tree[1];                                                                   \
            if (!(w < way && cur[w] < endX[w])) break;                                              \
            *C++ = *cur[w]++;                                                                       \
            for (unsigned v = (leaves + w) >> 1; v >= 1; v >>= 1) {                                 \
                unsigned a = tree[2 * v], b = tree[2 * v + 1];                                      \
                int aok = a < way && cur[a] < endX[a], bok = b < way && cur[b] < endX[b];           \
                tree[v] = (!bok || (aok && !LESS(*cur[b], *cur[a]))) ? a : b;                       \
            }                                                                                       \
        }                                                                                           \
    }                                                                                               \
                                                                                                    \
    /* phase2_sort (sorter.h:3831-3849): phase1 over a block in place, then binary                  \
     * merges from P1_N up to sort_size into the ping-pong pair (block, tmp). */                    \
    static T* phase2_##SFX(T* d, T* tmp, uint64_t n, uint64_t p1, uint64_t sort_size) {             \
        for (uint64_t i = 0; i < n; i += p1) network_sort_##SFX(d + i, n - i < p1 ? n - i : p1);    \
        return merge_series_##SFX(d, tmp, n, p1, sort_size);                                        \
    }                                                                                               \
                                                                                                    \
    /* sort_single_thread (sorter.h:3851-3915). */                                                  \
    static T* sort_st_##SFX(T* d, T* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,              \
                            uint64_t p1n, uint64_t p2n) {                                           \
        if (sort_n >= n) {                                                                          \
            uint64_t pw = 1;                                                                        \
            while (pw < n) pw <<= 1;                                                                \
            sort_n = pw;                                                                            \
        }                                                                                           \
        uint64_t p1 = p1n < sort_n ? p1n : sort_n;                                                  \
        uint64_t Y = p2n, Ysort = Y < sort_n ? Y : sort_n;                                          \
        T* o = d;                                                                                   \
        for (uint64_t b = 0; b < n; b += Y) {                                                       \
            uint64_t m = n - b < Y ? n - b : Y;                                                     \
            T* r = phase2_##SFX(d + b, tmp + b, m, p1, Ysort);                                      \
            if (b == 0) o = (r == d + b) ? d : tmp;                                                 \
        }                                                                                           \
        if (n == 0) return d;                                                                       \
        if (sort_n <= Y) return o;                                                                  \
        T* src = o;                                                                                 \
        T* dst = (o == d) ? tmp : d;                                                                \
        if (min_k <= 2) return merge_series_##SFX(src, dst, n, Y, sort_n);                          \
        /* min_k-way merge-tree rounds (sorter.h:3875-3911) */                                      \
        unsigned levels = 0, kp = 0;                                                                \
        for (uint64_t s = Y; s < sort_n; s <<= 1) levels++;                                         \
        while ((1u << (kp + 1)) <= min_k) kp++;                                                     \
        uint64_t prev = Y;                                                                          \
        T* X[4096];                                                                                 \
        T* endX[4096];                                                                              \
        while (levels > 0) {                                                                        \
            /* sorter.h:3887: a round merges 2^kp runs unless fewer than 2*kp                       \
             * levels remain, then all remaining levels go in one round. */                        \
            unsigned wp = (levels < 2 * kp) ? levels : kp;                                          \
            uint64_t merged = prev << wp;                                                           \
            for (uint64_t g = 0; g < n; g += merged) {                                              \
                unsigned w = 0;                                                                     \
                for (uint64_t s = g; s < n && s < g + merged; s += prev, w++) {                     \
                    X[w] = src + s;                                                                 \
                    endX[w] = src + (n - s < prev ? n : s + prev);                                  \
                }                                                                                   \
                kway_##SFX(X, endX, dst + g, w);                                                    \
            }                                                                                       \
            prev = merged;                                                                          \
            levels -= wp;                                                                           \
            T* t = src; src = dst; dst = t;                                                         \
        }                                                                                           \
        return src;                                                                                 \
    }                                                                                               \
                                                                                                    \
    /* Partition_Ptrs (Partition.h:118-166): lower the stream holding the largest                   \
     * left-boundary item and raise the one holding the smallest right-boundary                    \
     * item, halving the step each time, until every left item precedes every                      \
     * right item. The sum of S is invariant. Windows [lo, hi] keep the proven                     \
     * bounds; ties are ordered by stream index. */                                                 \
    static void partition_##SFX(T** L, T** R, T** S, uint64_t K) {                                  \
        int64_t lo[4096], hi[4096];                                                                 \
        for (uint64_t k = 0; k < K; k++) { lo[k] = 0; hi[k] = R[k] - L[k]; }                        \
        for (;;) {                                                                                  \
            int64_t smax = -1, smin = -1;                                                           \
            for (uint64_t k = 0; k < K; k++) {                                                      \
                if (S[k] > L[k]) {                                                                  \
                    T x = S[k][-1];                                                                 \
                    if (smax < 0 || !LESS(x, *(S[smax] - 1))) smax = (int64_t)k;                    \
                }                                                                                   \
                if (S[k] < R[k]) {                                                                  \
                    T x = S[k][0];                                                                  \
                    if (smin < 0 || LESS(x, *S[smin])) smin = (int64_t)k;                           \
                }                                                                                   \
            }                                                                                       \
            if (smax < 0 || smin < 0) break;                                                        \
            T lm = *(S[smax] - 1), rm = *S[smin];                                                   \
            /* (key, stream) order: done when lmax precedes rmin */                                \
            if (LESS(lm, rm) || (!LESS(rm, lm) && smax <= smin)) break;                             \
            int64_t pmax = S[smax] - L[smax], pmin = S[smin] - L[smin];                             \
            hi[smax] = pmax - 1;                                                                    \
            lo[smin] = pmin + 1;                                                                    \
            int64_t dmax = (pmax - lo[smax] + 1) / 2, dmin = (hi[smin] - pmin + 1) / 2;             \
            int64_t dl = dmax < dmin ? dmax : dmin;                                                 \
            if (dl < 1) dl = 1;                                                                     \
            S[smax] -= dl;                                                                          \
            S[smin] += dl;                                                                          \
        }                                                                                           \
    }

#define LESS_SCALAR(a, b) ((a) < (b))
#define LESS_KEY(a, b) ((a).key < (b).key)
ORC_DEFINE(u32, uint32_t, LESS_SCALAR)
ORC_DEFINE(u64, uint64_t, LESS_SCALAR)
ORC_DEFINE(i64, int64_t, LESS_SCALAR)
ORC_DEFINE(kv, kv_t, LESS_KEY)
ORC_DEFINE(kvu, kvu_t, LESS_KEY)

#define DISPATCH(kind, CALL_U32, CALL_U64, CALL_I64, CALL_KV, CALL_KVU) \
    switch (kind) {                                                     \
        case ORC_U32: CALL_U32; break;                                  \
        case ORC_U64: CALL_U64; break;                                  \
        case ORC_I64: CALL_I64; break;                                  \
        case ORC_KV: CALL_KV; break;                                    \
        default: CALL_KVU; break;                                       \
    }

void* orc_sort_single_thread(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n,
                             unsigned min_k) {
    return orc_sort_single_thread_p(kind, d, tmp, n, sort_n, min_k, orc_p1_n(kind), orc_p2_n(kind));
}

void* orc_sort_single_thread_p(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n,
                               unsigned min_k, uint64_t p1, uint64_t p2) {
    if (sort_n == 0) sort_n = n;
    void* r = d;
    DISPATCH(kind, r = sort_st_u32(d, tmp, n, sort_n, min_k, p1, p2),
             r = sort_st_u64(d, tmp, n, sort_n, min_k, p1, p2),
             r = sort_st_i64(d, tmp, n, sort_n, min_k, p1, p2),
             r = sort_st_kv(d, tmp, n, sort_n, min_k, p1, p2),
             r = sort_st_kvu(d, tmp, n, sort_n, min_k, p1, p2))
    return r;
}

void* orc_merge_series(int kind, void* src, void* dst, uint64_t n, uint64_t merge_start,
                       uint64_t sort_n) {
    void* r = src;
    DISPATCH(kind, r = merge_series_u32(src, dst, n, merge_start, sort_n),
             r = merge_series_u64(src, dst, n, merge_start, sort_n),
             r = merge_series_i64(src, dst, n, merge_start, sort_n),
             r = merge_series_kv(src, dst, n, merge_start, sort_n),
             r = merge_series_kvu(src, dst, n, merge_start, sort_n))
    return r;
}

void orc_kway_merge(int kind, void** X, void** endX, void* C, unsigned way) {
    DISPATCH(kind, kway_u32((uint32_t**)X, (uint32_t**)endX, C, way),
             kway_u64((uint64_t**)X, (uint64_t**)endX, C, way),
             kway_i64((int64_t**)X, (int64_t**)endX, C, way),
             kway_kv((kv_t**)X, (kv_t**)endX, C, way), kway_kvu((kvu_t**)X, (kvu_t**)endX, C, way))
}

void orc_partition_ptrs(int kind, void** L, void** R, void** S, uint64_t K) {
    DISPATCH(kind, partition_u32((uint32_t**)L, (uint32_t**)R, (uint32_t**)S, K),
             partition_u64((uint64_t**)L, (uint64_t**)R, (uint64_t**)S, K),
             partition_i64((int64_t**)L, (int64_t**)R, (int64_t**)S, K),
             partition_kv((kv_t**)L, (kv_t**)R, (kv_t**)S, K),
             partition_kvu((kvu_t**)L, (kvu_t**)R, (kvu_t**)S, K))
}

/* ------------------------------------------------------- multi-thread ------
 * sort_multi_thread (sorter.h:4194-4287) with its worker (sorter.h:3961-4192):
 *  phase 1-2: P2_N blocks claimed from a shared counter (sorter.h:3982-4001);
 *  phase 3:   min_k-way merge rounds until M = max(min_k, n_threads) streams
 *             remain (sorter.h:4004-4083), groups claimed from a counter;
 *  phase 4:   Partition_Ptrs splits the M streams into n_threads*16 ranges of
 *             equal output size (sorter.h:4104-4134); each is M-way merged
 *             (sorter.h:4146-4190). */
typedef struct {
    int kind;
    unsigned char* src;
    unsigned char* dst;
    uint64_t n, item, p1, y, ysort;
    uint64_t prev, merged;   /* phase 3 round */
    unsigned way;
    uint64_t nparts, per_part; /* phase 4 */
    unsigned M;
    uint64_t stream_len;
    long long next;         /* shared job counter */
    unsigned char* first_res; /* phase 1-2 result of block 0 */
    int phase;
} mt_ctx;

static void* mt_worker(void* arg) {
    mt_ctx* c = (mt_ctx*)arg;
    const uint64_t s = c->item;
    for (;;) {
        long long j = __atomic_fetch_add(&c->next, 1, __ATOMIC_SEQ_CST);
        if (c->phase == 0) {
            uint64_t b = (uint64_t)j * c->y;
            if (b >= c->n) break;
            uint64_t m = c->n - b < c->y ? c->n - b : c->y;
            void* d = c->src + b * s;
            void* t = c->dst + b * s;
            void* r = NULL;
            DISPATCH(c->kind, r = phase2_u32(d, t, m, c->p1, c->ysort),
                     r = phase2_u64(d, t, m, c->p1, c->ysort), r = phase2_i64(d, t, m, c->p1, c->ysort),
                     r = phase2_kv(d, t, m, c->p1, c->ysort), r = phase2_kvu(d, t, m, c->p1, c->ysort))
            if (b == 0) c->first_res = (r == d) ? c->src : c->dst;
        } else if (c->phase == 1) {
            uint64_t g = (uint64_t)j * c->merged;
            if (g >= c->n) break;
            void* X[4096];
            void* endX[4096];
            unsigned w = 0;
            for (uint64_t st = g; st < c->n && st < g + c->merged; st += c->prev, w++) {
                X[w] = c->src + st * s;
                endX[w] = c->src + (c->n - st < c->prev ? c->n : st + c->prev) * s;
            }
            orc_kway_merge(c->kind, X, endX, c->dst + g * s, w);
        } else {
            uint64_t p = (uint64_t)j;
            if (p >= c->nparts) break;
            void* L[4096];
            void* R[4096];
            void* S0[4096];
            void* S1[4096];
            for (int e = 0; e < 2; e++) {
                uint64_t target = (p + (uint64_t)e) * c->per_part;
                if (target > c->n) target = c->n;
                void** S = e ? S1 : S0;
                uint64_t assigned = 0;
                for (unsigned k = 0; k < c->M; k++) {
                    uint64_t a = k * c->stream_len;
                    uint64_t b = a + c->stream_len < c->n ? a + c->stream_len : c->n;
                    if (a > c->n) a = c->n;
                    L[k] = c->src + a * s;
                    R[k] = c->src + b * s;
                    /* proportional initial guess (sorter.h:4110, 4129) */
                    uint64_t len = b - a;
                    uint64_t g = c->n ? (uint64_t)((__uint128_t)len * target / c->n) : 0;
                    S[k] = c->src + (a + g) * s;
                    assigned += g;
                }
                /* hand the rounding remainder to streams with room */
                for (unsigned k = 0; assigned < target && k < c->M; k++) {
                    uint64_t room = (uint64_t)((unsigned char*)R[k] - (unsigned char*)S[k]) / s;
                    uint64_t add = target - assigned < room ? target - assigned : room;
                    S[k] = (unsigned char*)S[k] + add * s;
                    assigned += add;
                }
                orc_partition_ptrs(c->kind, L, R, S, c->M);
            }
            uint64_t out0 = p * c->per_part;
            orc_kway_merge(c->kind, S0, S1, c->dst + out0 * s, c->M);
        }
    }
    return NULL;
}

static void mt_run(mt_ctx* c, unsigned nt) {
    pthread_t th[256];
    c->next = 0;
    if (nt > 256) nt = 256;
    for (unsigned t = 0; t < nt; t++) pthread_create(&th[t], NULL, mt_worker, c);
    for (unsigned t = 0; t < nt; t++) pthread_join(th[t], NULL);
}

void* orc_sort_multi_thread(int kind, void* d, void* out, uint64_t n, unsigned n_threads,
                            unsigned min_k) {
    if (n_threads <= 1 || n < 2 * orc_p2_n(kind))
        return orc_sort_single_thread(kind, d, out, n, n, min_k < 2 ? 2 : min_k);
    if (min_k < 2) min_k = 2;
    mt_ctx c;
    memset(&c, 0, sizeof c);
    c.kind = kind;
    c.item = orc_item_bytes(kind);
    c.n = n;
    c.p1 = orc_p1_n(kind);
    c.y = orc_p2_n(kind);
    c.ysort = c.y;
    /* phase 1-2 */
    c.src = (unsigned char*)d;
    c.dst = (unsigned char*)out;
    c.phase = 0;
    mt_run(&c, n_threads);
    unsigned char* src = c.first_res;
    unsigned char* dst = (src == (unsigned char*)d) ? (unsigned char*)out : (unsigned char*)d;
    /* phase 3: rounds until at most M streams remain */
    unsigned M = min_k > n_threads ? min_k : n_threads;
    unsigned mp = 0;
    while ((1u << (mp + 1)) <= M) mp++;
    M = 1u << mp;
    unsigned kp = 0;
    while ((1u << (kp + 1)) <= min_k) kp++;
    uint64_t prev = c.y;
    uint64_t streams = (n + prev - 1) / prev;
    while (streams > M) {
        unsigned levels = 0;
        for (uint64_t t = streams; t > M; t = (t + 1) / 2) levels++;
        unsigned wp = (levels < 2 * kp) ? levels : kp;
        c.prev = prev;
        c.merged = prev << wp;
        c.src = src;
        c.dst = dst;
        c.phase = 1;
        mt_run(&c, n_threads);
        prev = c.merged;
        streams = (n + prev - 1) / prev;
        unsigned char* t = src; src = dst; dst = t;
    }
    if (streams == 1) return src;
    /* phase 4 */
    c.M = (unsigned)streams;
    c.stream_len = prev;
    c.nparts = (uint64_t)n_threads * 16;
    c.per_part = (n + c.nparts - 1) / c.nparts;
    c.src = src;
    c.dst = dst;
    c.phase = 2;
    mt_run(&c, n_threads);
    return dst;
}

/* ------------------------------------------------------------ generators --
 * datagen::Writer<Item> (writer.h:25-244). Values are written in the item's
 * own type: u32 keys keep the low 32 bits like the reference's implicit casts. */
static void put(int kind, void* a, uint64_t i, uint64_t x, int kv_value_plus1) {
    switch (kind) {
        case ORC_U32: ((uint32_t*)a)[i] = (uint32_t)x; break;
        case ORC_U64: ((uint64_t*)a)[i] = x; break;
        case ORC_I64: ((int64_t*)a)[i] = (int64_t)x; break;
        case ORC_KV: ((kv_t*)a)[i].key = (int64_t)x; ((kv_t*)a)[i].value = (int64_t)(x + (uint64_t)kv_value_plus1); break;
        default: ((kvu_t*)a)[i].key = x; ((kvu_t*)a)[i].value = x + (uint64_t)kv_value_plus1; break;
    }
}

/* random_writer (writer.h:49-72) */
static void gen_random(int kind, void* a, uint64_t n) {
    if (kind == ORC_U32) {
        mt32_t g;
        mt32_seed(&g, 5489u);
        for (uint64_t i = 0; i < n; i++) ((uint32_t*)a)[i] = mt32_next(&g);
        return;
    }
    mt64_t g;
    mt64_seed(&g, 5489u);
    if (kind == ORC_U64) { /* uniform_int_distribution<uint64_t>(): full range = raw output */
        for (uint64_t i = 0; i < n; i++) ((uint64_t*)a)[i] = mt64_next(&g);
        return;
    }
    for (uint64_t i = 0; i < n; i++) put(kind, a, i, (uint64_t)dist_i64_nonneg(&g), 1);
}

static int cmp_asc(int kind, const void* x, const void* y) {
    switch (kind) {
        case ORC_U32: { uint32_t a = *(const uint32_t*)x, b = *(const uint32_t*)y; return (a > b) - (a < b); }
        case ORC_U64: { uint64_t a = *(const uint64_t*)x, b = *(const uint64_t*)y; return (a > b) - (a < b); }
        case ORC_I64: { int64_t a = *(const int64_t*)x, b = *(const int64_t*)y; return (a > b) - (a < b); }
        case ORC_KV: { int64_t a = ((const kv_t*)x)->key, b = ((const kv_t*)y)->key; return (a > b) - (a < b); }
        default: { uint64_t a = ((const kvu_t*)x)->key, b = ((const kvu_t*)y)->key; return (a > b) - (a < b); }
    }
}
static int g_sort_kind;
static int cmp_up(const void* x, const void* y) { return cmp_asc(g_sort_kind, x, y); }
static int cmp_down(const void* x, const void* y) { return cmp_asc(g_sort_kind, y, x); }

void orc_generate(int kind, void* a, uint64_t n, int type) {
    const unsigned s = orc_item_bytes(kind);
    switch (type) {
        case ORC_SAME: { /* all_same (writer.h:143-157) */
            mt64_t g;
            mt64_seed(&g, 5489u);
            uint64_t x = (uint64_t)dist_i64_nonneg(&g);
            for (uint64_t i = 0; i < n; i++) put(kind, a, i, x, 1);
            break;
        }
        case ORC_SORTED_SEQ: /* sorted (writer.h:159-162) */
        case ORC_REV_SORTED_SEQ: /* reverse_sorted (writer.h:164-167) */
            gen_random(kind, a, n);
            g_sort_kind = kind;
            qsort(a, n, s, type == ORC_SORTED_SEQ ? cmp_up : cmp_down);
            break;
        case ORC_ALMOST_SORTED: /* almost_sorted (writer.h:169-179) */
            gen_random(kind, a, n);
            for (uint64_t i = 0; i < n; i += 7) {
                if (kind == ORC_U32) ((uint32_t*)a)[i] = 0xFFFFFFFFu;
                else if (kind == ORC_I64) ((int64_t*)a)[i] = INT64_MAX;
                else if (kind == ORC_U64) ((uint64_t*)a)[i] = INT64_MAX;
                else if (kind == ORC_KV) ((kv_t*)a)[i].key = INT64_MAX;
                else ((kvu_t*)a)[i].key = INT64_MAX;
            }
            break;
        case ORC_PARETO_NONUNIFORM:
        case ORC_PARETO_B2B:
        case ORC_PARETO_SHUFF: { /* pareto_writer (writer.h:74-139) */
            const uint64_t A = 6364136223846793005ull, C = 1442695040888963407ull;
            uint64_t x = 1, y = 889;
            const double beta = 7;
            for (uint64_t i = 0; i < n;) {
                x = x * A + C;
                y = y * A + C;
                double u = (double)y / ((double)(1ull << 63) * 2);
                double fd = ceil(beta * (1 / (1 - u) - 1));
                uint64_t f = (uint64_t)(fd < 100000 ? fd : 100000);
                if (type == ORC_PARETO_NONUNIFORM) {
                    put(kind, a, i++, f, 1);
                } else if (i + f < n) {
                    for (uint64_t j = 0; j < f; j++) put(kind, a, i + j, x, 1);
                    i += f;
                } else if (i + 10 >= n) {
                    for (; i < n; ++i) put(kind, a, i, x, 1);
                }
            }
            if (type == ORC_PARETO_SHUFF) { /* fixed-seed Fisher-Yates in place of random_device */
                mt32_t g;
                mt32_seed(&g, 5489u);
                unsigned char tmp[16];
                for (uint64_t i = n; i > 1; i--) {
                    uint64_t j = (((uint64_t)mt32_next(&g) << 32) | mt32_next(&g)) % i;
                    memcpy(tmp, (unsigned char*)a + (i - 1) * s, s);
                    memcpy((unsigned char*)a + (i - 1) * s, (unsigned char*)a + j * s, s);
                    memcpy((unsigned char*)a + j * s, tmp, s);
                }
            }
            break;
        }
        case ORC_FIB_SEQ: { /* fibonacci (writer.h:181-220) */
            uint64_t fa = 0, fb = 1, fc;
            if (n > 0) put(kind, a, 0, 0, 1);
            if (n > 1) put(kind, a, 1, 1, 1);
            uint64_t i = 2;
            while (i < n) {
                fc = fa + fb;
                if (fc < fb) {
                    fa = 0;
                    fb = 1;
                    put(kind, a, i++, 0, 1);
                    if (i < n) put(kind, a, i++, 1, 1);
                } else {
                    fa = fb;
                    fb = fc;
                    put(kind, a, i++, fb, 1);
                }
            }
            break;
        }
        default: /* ORC_MT */
            gen_random(kind, a, n);
            break;
    }
}

/* ------------------------------------------------------------- checkers --
 * sort_correctness_checker (utils.h:38-47) over the whole array or per chunk. */
int orc_is_sorted(int kind, const void* a, uint64_t n) {
    const unsigned s = orc_item_bytes(kind);
    for (uint64_t i = 1; i < n; i++)
        if (cmp_asc(kind, (const unsigned char*)a + i * s, (const unsigned char*)a + (i - 1) * s) < 0)
            return 0;
    return 1;
}
int orc_chunks_sorted(int kind, const void* a, uint64_t n, uint64_t sort_n) {
    const unsigned s = orc_item_bytes(kind);
    if (sort_n == 0) sort_n = n;
    for (uint64_t c = 0; c < n; c += sort_n)
        if (!orc_is_sorted(kind, (const unsigned char*)a + c * s, n - c < sort_n ? n - c : sort_n)) return 0;
    return 1;
}
