// Test infrastructure: a thin C wrapper around the UNMODIFIED Origami reference
// (compiled from its own headers in place, one shared library per
// REG_TYPE x KEY_TYPE variant by oracle/Makefile). Only the tests, the golden
// fixture generator and bench.py's CPU-baseline leg load the result; nothing on
// the GPU product path does.
//
// Entry points wrap, one to one:
//   ref_generate            -> datagen::Writer<Item>::generate       (writer.h:222-242)
//   ref_sort_single_thread  -> origami_sorter::sort_single_thread    (sorter.h:3851-3915)
//   ref_sort_multi_thread   -> origami_sorter::sort_multi_thread     (sorter.h:4194-4287)
//   ref_phase2_sort         -> origami_sorter::phase2_sort           (sorter.h:3831-3849)
//   ref_partition_ptrs      -> partition_templated::Partition_Ptrs   (Partition.h:118-166)
#include "commons.h"
#include "writer.h"
#include "utils.h"
#include "merge_utils.h"
#include "sorter.h"

using Item = Itemtype;
using Reg = Regtype;

extern "C" {

int ref_reg_type() { return REG_TYPE; }
int ref_key_type() { return KEY_TYPE; }
unsigned ref_item_bytes() { return (unsigned)sizeof(Item); }
unsigned long long ref_p1_n() { return _P1_N; }
unsigned long long ref_p2_n() { return _P2_N; }

void ref_generate(void* a, unsigned long long n, int type) {
    datagen::Writer<Item> w;
    w.generate((Item*)a, n, type);
}

// Returns the buffer (d or tmp) that holds the sorted output, as the reference does.
void* ref_sort_single_thread(void* d, void* tmp, unsigned long long n, unsigned long long sort_n,
                             unsigned min_k, void* interim) {
    Item* dd = (Item*)d;
    return origami_sorter::sort_single_thread<Item, Reg>(dd, (Item*)tmp, dd + n, sort_n, min_k,
                                                         (Item*)interim);
}

void* ref_sort_multi_thread(void* d, void* out, unsigned long long n, unsigned n_threads,
                            unsigned n_cores, unsigned min_k, void* kway_buf) {
    return origami_sorter::sort_multi_thread<Item, Reg>((Item*)d, (Item*)out, n, n_threads, n_cores,
                                                        min_k, (Item*)kway_buf);
}

void* ref_phase2_sort(void* d, void* tmp, unsigned long long n, unsigned long long sort_n) {
    Item* dd = (Item*)d;
    return origami_sorter::phase2_sort<Item, Reg, _P1_NREG, _P1_N, _P1_SWITCH, _P2_MERGE_UNROLL,
                                       _P2_MERGE_NREG_1x, _P2_MERGE_NREG_2x, _P2_MERGE_NREG_3x>(
        dd, (Item*)tmp, dd + n, sort_n);
}

// L, R, S are arrays of K element pointers; S holds the initial guesses on entry
// and the splitters on return.
void ref_partition_ptrs(void** L, void** R, void** S, unsigned long long K) {
    partition_templated::Partition_Ptrs<Item>((Item**)L, (Item**)R, (Item**)S, K);
}

}  // extern "C"
