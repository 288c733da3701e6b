/* Origami oracle: a scalar C restatement of the reference CPU mergesort
 * (arif-arman/origami-sort, the Origami headers), used ONLY as test infrastructure:
 * the checker in tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py. Nothing on the GPU product path links or calls it.
 *
 * Parity status: pinned. tests/test_oracle.py checks every function here against
 * the unmodified reference (compiled by oracle/Makefile into oracle/_ref/) and
 * against the committed fixtures in tests/golden/ that the reference produced.
 *
 * Item kinds (same numbering as the GPU C-ABI, include/origami_gpu.h):
 *   0 ORC_U32  uint32_t keys                      (reference KEY_TYPE 0, `ui`)
 *   1 ORC_U64  uint64_t keys, unsigned order      (API superset; i64 via k ^ 2^63)
 *   2 ORC_I64  int64_t keys, signed order         (reference KEY_TYPE 1, `i64`)
 *   3 ORC_KV   {int64 key; int64 value} 16 B      (reference KEY_TYPE 2, KeyValue<i64,i64>)
 *   4 ORC_KVU  {uint64 key; uint64 value} 16 B    (API superset, unsigned key order)
 * KV items compare by key only, like KeyValue::operator< (commons.h:57-59).
 */
#ifndef ORIGAMI_ORACLE_H
#define ORIGAMI_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_U32 = 0, ORC_U64 = 1, ORC_I64 = 2, ORC_KV = 3, ORC_KVU = 4 };

/* writer.h:27-35 distribution ids */
enum {
    ORC_MT = 1, ORC_SAME = 2, ORC_SORTED_SEQ = 3, ORC_REV_SORTED_SEQ = 4, ORC_ALMOST_SORTED = 5,
    ORC_PARETO_NONUNIFORM = 6, ORC_PARETO_B2B = 7, ORC_PARETO_SHUFF = 8, ORC_FIB_SEQ = 9
};

unsigned orc_item_bytes(int kind);
/* Phase sizes of the reference's scalar build (config.h:27-84 with REG_TYPE 0):
 * P1_N = in-register sort size, P2_N = in-cache block = (L2_BYTES/2)/sizeof(Item). */
uint64_t orc_p1_n(int kind);
uint64_t orc_p2_n(int kind);

/* datagen::Writer<Item>::generate (writer.h:222-242), default-seeded engines as
 * the reference uses them. PARETO_SHUFF shuffles with a fixed-seed mt19937 here
 * (the reference seeds it from std::random_device, writer.h:131-136). */
void orc_generate(int kind, void* a, uint64_t n, int type);

/* origami_sorter::sort_single_thread (sorter.h:3851-3915). Sorts [d, d+n) in
 * independent chunks of sort_n items (sort_n >= n: one full sort) using the
 * phase1 -> phase2 (in-cache binary merges) -> phase3 (binary merges when
 * min_k == 2, else min_k-way merge rounds) pipeline. Returns d or tmp, whichever
 * holds the result, by the same rule as the reference. Any n is accepted (the
 * reference needs n to be a multiple of P2_N); sort_n must be a power of two or
 * >= n. */
void* orc_sort_single_thread(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n,
                             unsigned min_k);

/* Same pipeline with explicit phase sizes, so the result-buffer rule of any
 * reference build (its _P1_N and _P2_N, config.h) can be reproduced. */
void* orc_sort_single_thread_p(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n,
                               unsigned min_k, uint64_t p1_n, uint64_t p2_n);

/* origami_sorter::sort_multi_thread (sorter.h:4194-4287) restated with POSIX
 * threads: phase 1-2 blocks in parallel, phase 3 k-way rounds in parallel, phase
 * 4 Partition_Ptrs splitting into n_threads*16 ranges merged in parallel.
 * Returns d or out. */
void* orc_sort_multi_thread(int kind, void* d, void* out, uint64_t n, unsigned n_threads,
                            unsigned min_k);

/* origami_merger::merge_series (merger.h:4220-4228): binary merge levels from
 * runs of merge_start items up to runs of sort_n, ping-ponging src/dst; returns
 * the buffer holding the result. */
void* orc_merge_series(int kind, void* src, void* dst, uint64_t n, uint64_t merge_start,
                       uint64_t sort_n);

/* MergeTree::merge(X, endX, C, n, ...) (merge_tree.h:2792, 3410): WAY-way merge
 * of the sorted streams [X[i], endX[i]) into C. Ties go to the lower stream. */
void orc_kway_merge(int kind, void** X, void** endX, void* C, unsigned way);

/* partition_templated::Partition_Ptrs (Partition.h:118-166). S holds initial
 * guesses on entry and the splitters on return. Ties between equal keys of
 * different streams are broken by stream index, which keeps the loop exact when
 * keys repeat (the reference compares keys only). */
void orc_partition_ptrs(int kind, void** L, void** R, void** S, uint64_t K);

/* Checkers (utils.h:29-58 and the KV multiset rule): 1 = pass, 0 = fail. */
int orc_is_sorted(int kind, const void* a, uint64_t n);
int orc_chunks_sorted(int kind, const void* a, uint64_t n, uint64_t sort_n);

#ifdef __cplusplus
}
#endif
#endif
