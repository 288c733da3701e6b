/*
 * origami_gpu.h - C ABI of the GB300 (sm_103a) Origami mergesort.
 *
 * Drop-in for the CPU sort entry points of arif-arman/origami-sort. Every call
 * takes plain pointers and sizes; nothing here needs CUDA or torch headers
 * (streams are passed as `void*`, meaning a cudaStream_t; NULL = the legacy
 * default stream).
 *
 * Item kinds:
 *   u32   uint32_t keys                                    (reference `ui`, KEY_TYPE 0)
 *   u64   uint64_t keys, unsigned order                    (superset of the reference)
 *   i64   int64_t keys, signed order                       (reference `i64`, KEY_TYPE 1)
 *   kv64  {int64_t key; int64_t value;}, 16 B, by key      (reference KeyValue<i64,i64>, KEY_TYPE 2)
 *   kvu64 {uint64_t key; uint64_t value;}, 16 B, by key    (superset of the reference)
 * Key-value sorts are stable: equal keys keep their input order.
 *
 * Result-buffer convention (reference sorter.h:3852,3914): the sorted output
 * lands in one of the two caller buffers and *result says which. By default it
 * is `d`; ORIGAMI_FLAG_RESULT_IN_TMP asks for `tmp`.
 *
 * Return value: ORIGAMI_OK (0) or a negative ORIGAMI_ERR_* code; the message is
 * kept per thread and returned by origami_last_error(). No call ever exits the
 * process (the reference does: commons.h:103-104).
 */
#ifndef ORIGAMI_GPU_H
#define ORIGAMI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORIGAMI_GPU_VERSION 100

/* status codes */
#define ORIGAMI_OK 0
#define ORIGAMI_ERR_INVALID (-1)   /* null pointer, bad size, bad sort_n, overlapping buffers */
#define ORIGAMI_ERR_ALIGN (-2)     /* pointer not aligned to the item size */
#define ORIGAMI_ERR_OOM (-3)       /* device memory exhausted / over the arena budget */
#define ORIGAMI_ERR_CUDA (-4)      /* a CUDA runtime call failed */
#define ORIGAMI_ERR_TIMEOUT (-5)   /* a bounded device wait gave up */
#define ORIGAMI_ERR_DTYPE (-6)     /* unknown item kind */
#define ORIGAMI_ERR_NO_DEVICE (-7) /* no usable CUDA device */
#define ORIGAMI_ERR_BUSY (-8)      /* queue full / admission refused */
#define ORIGAMI_ERR_CANCELLED (-9) /* request cancelled before it ran */

/* item kinds (same numbering as the oracle) */
#define ORIGAMI_U32 0
#define ORIGAMI_U64 1
#define ORIGAMI_I64 2
#define ORIGAMI_KV64 3
#define ORIGAMI_KVU64 4

/* flags */
#define ORIGAMI_FLAG_RESULT_IN_TMP 0x1 /* leave the sorted output in tmp instead of d */
#define ORIGAMI_FLAG_SYNC 0x2          /* _device calls: synchronize the stream before returning */

int origami_version(void);
const char* origami_last_error(void);
unsigned origami_item_bytes(int kind);

/*
 * Plain sort: the drop-in for origami_sorter::sort_single_thread
 * (reference sorter.h:3851-3915) and sort_multi_thread (sorter.h:4194-4287).
 *
 *   d, tmp   two buffers of n items each. Host pointers (pageable or pinned)
 *            that the GPU can address (pinned memory; pageable memory on hosts
 *            whose GPU reads the host's page tables, such as Grace) are
 *            streamed: a large sort arrives in chunks that sort while the next
 *            ones land, and its last pass writes the result into the host
 *            buffer. Other host pointers are staged through the library's
 *            device arena. Device pointers are sorted in place with no copies.
 *            tmp may be NULL: device scratch is then taken from the arena.
 *   n        item count (any n >= 0)
 *   sort_n   chunk size: the array is sorted in independent chunks of sort_n
 *            items (the reference's "sort_n" / chunked sort,
 *            bench_sort_phases.cpp:1307-1425). 0 or >= n means one full sort.
 *            Otherwise it must be a power of two.
 *   min_k    merge fan-in of each HBM pass (the reference's min_k, sorter.h:3875):
 *            2 = binary merge passes, 4/8/16 = k-way passes. 0 picks the tuned value.
 *   result   receives d or tmp.
 * The call returns after the result is in place (host) or is enqueued on the
 * default stream (device pointers; add ORIGAMI_FLAG_SYNC to wait).
 * Errors found on the device are reported by the calls that wait for the sort
 * (host buffers, and device buffers with ORIGAMI_FLAG_SYNC): ORIGAMI_ERR_TIMEOUT
 * when a merge kernel's bounded wait for a bulk copy expired (the output is then
 * incomplete). The reference has no such error (ReportError, commons.h:103-104,
 * prints and exits).
 */
int origami_sort_u32(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k, int flags,
                     void** result);
int origami_sort_u64(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k, int flags,
                     void** result);
int origami_sort_i64(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k, int flags,
                     void** result);
int origami_sort_kv64(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k, int flags,
                      void** result);
int origami_sort_kvu64(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k, int flags,
                       void** result);

/* Device-pointer form on an explicit stream: zero-copy, asynchronous. */
int origami_sort_u32_device(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                            int flags, void** result, void* stream);
int origami_sort_u64_device(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                            int flags, void** result, void* stream);
int origami_sort_i64_device(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                            int flags, void** result, void* stream);
int origami_sort_kv64_device(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                             int flags, void** result, void* stream);
int origami_sort_kvu64_device(void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                              int flags, void** result, void* stream);

/* Kind-generic forms of the two calls above. */
int origami_sort(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                 int flags, void** result);
int origami_sort_device(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n, unsigned min_k,
                        int flags, void** result, void* stream);

/*
 * origami_merger::merge_series (reference merger.h:4220-4228): binary merge
 * levels over device buffers, from sorted runs of merge_start items up to runs
 * of sort_n items (both powers of two, merge_start < sort_n), ping-ponging
 * src/dst. *result receives src or dst, whichever holds the output.
 */
int origami_merge_series_device(int kind, void* src, void* dst, uint64_t n, uint64_t merge_start,
                                uint64_t sort_n, void** result, void* stream);

/*
 * Batched segmented sort (no single counterpart in the reference: it extends
 * the chunked sort of bench_sort_phases.cpp:1307-1425 to arbitrary, uneven
 * chunks). Segment s is items [offsets[s], offsets[s+1]) of d; every segment
 * is sorted independently and in place (the result is in d; tmp is scratch of
 * n items). All segments go through the same short launch sequence, planned
 * on the device (no host synchronisation, so it can be captured in a CUDA
 * graph): one tile-sort launch for every segment's tiles (a short segment is
 * one tile, sorted in registers and shared memory), then for each merge level
 * a partition and a persistent merge launch over the segments still merging.
 * Key-value segments are sorted stably.
 *   _device: d, tmp, offsets are device memory, d and tmp 16-byte aligned,
 *            offsets[nseg] == n, asynchronous on `stream`
 *            (ORIGAMI_FLAG_SYNC waits and reports device-side errors:
 *            ORIGAMI_ERR_INVALID for decreasing offsets, ORIGAMI_ERR_TIMEOUT
 *            if a bounded wait ran out).
 *   host:    d and offsets are host memory (offsets[0] == 0, n = offsets[nseg]);
 *            returns when d holds the result.
 */
int origami_sort_segmented_device(int kind, void* d, void* tmp, const uint64_t* offsets,
                                  uint64_t nseg, uint64_t n, int flags, void* stream);
int origami_sort_segmented(int kind, void* d, const uint64_t* offsets, uint64_t nseg, int flags);

/*
 * Segmented-sort plan (no counterpart in the reference): the launch sequence
 * of origami_sort_segmented_device over FIXED device buffers d, tmp, offsets,
 * recorded once into a CUDA graph with its own scratch. Each launch replays it
 * on `stream` (no allocation, one graph launch); refill d between launches.
 * status() waits for the stream and reports the last replay's device-side
 * errors like ORIGAMI_FLAG_SYNC does. Same argument rules as the _device call;
 * n and nseg must be > 0. Create the plan outside any other stream capture.
 */
typedef struct origami_seg_plan origami_seg_plan;
int origami_seg_plan_create(int kind, void* d, void* tmp, const uint64_t* offsets, uint64_t nseg,
                            uint64_t n, origami_seg_plan** out);
int origami_seg_plan_launch(origami_seg_plan* p, void* stream);
int origami_seg_plan_status(origami_seg_plan* p, void* stream);
uint64_t origami_seg_plan_kernels(const origami_seg_plan* p); /* kernels per replay */
int origami_seg_plan_destroy(origami_seg_plan* p);

/*
 * MergeTree::merge(X, endX, C, n, ...) (reference merge_tree.h:2792, 3410):
 * way-way merge of the sorted device streams [X[i], endX[i]) into C (any way;
 * up to 16 streams take one HBM pass, more take one pass per factor of 16).
 * X and endX are HOST arrays of `way` device pointers; C receives all items
 * (the reference aligns C down to its register block first; here C is used
 * as given). Streams must be aligned to the item size (16 bytes for key-value
 * items) and must not overlap C. Ties go to the lower stream, so the merge is
 * stable across streams. Asynchronous on `stream`.
 */
int origami_merge_tree_device(int kind, void* const* X, void* const* endX, void* C, unsigned way,
                              void* stream);

/*
 * partition_templated::Partition_Ptrs (reference Partition.h:118-166) as a
 * merge-path splitter search: for the K sorted device streams
 * [L[i], R[i]) and each requested output rank ranks[j] (host array, count
 * n_ranks), writes split offsets splits[j*K + i] (host array) such that taking
 * the first splits[j*K+i] items of every stream gives exactly the ranks[j]
 * smallest items, ties ordered by stream. K <= 1024. Waits for `stream`.
 * Partition_Ptrs(L, R, S, K) is this call with one rank: the sum of the
 * caller's initial S[k] - L[k]; the reference then moves S to the same split
 * whenever the keys at the boundary are distinct.
 */
int origami_partition_device(int kind, void* const* L, void* const* R, unsigned K,
                             const uint64_t* ranks, uint64_t n_ranks, uint64_t* splits,
                             void* stream);

/*
 * Launch accounting and profiling. Every kernel the library launches is
 * counted. While profiling is enabled launches are also bracketed by two CUDA
 * events on their own stream: every launch for on = 1, every on-th launch of
 * each kernel for on > 1 (the events sit between kernels that otherwise
 * overlap their start-up with their predecessor's end, so timing fewer of them
 * disturbs the timeline less); 0 disables. origami_profile_report() waits for
 * the events and writes one "kernel,launches,timed_ms,timed" line per kernel
 * into buf: all launches since enabling, and the total device milliseconds of
 * the `timed` launches among them (returns the length, or a negative status).
 * Enabling (or disabling) clears earlier records.
 */
int origami_profile_enable(int on);
int origami_profile_report(char* buf, uint64_t cap);
uint64_t origami_launch_count(void);

/*
 * Bound of every device-side wait (no counterpart in the reference, whose
 * sorts never wait on a device): the polls a merge kernel makes on a bulk copy's
 * mbarrier before it gives up, drains its own copies, records the expiry in the
 * sort's error word and returns, so that a stalled copy ends the kernel instead
 * of hanging the GPU. Default 2^20 polls. Read when a sort is launched (a
 * segmented plan keeps the value it was created with). 0 makes every first
 * wait expire: that is how the tests exercise the expiry path.
 */
uint32_t origami_get_wait_limit(void);
int origami_set_wait_limit(uint32_t polls);

/*
 * Allocation-free sort (no counterpart in the reference, which never needs
 * device memory). For callers that cannot allocate device memory during the
 * call: code running while another allocator holds the GPU's free memory, code
 * in a latency-critical loop that must not let an allocation stall the
 * device, runtimes that forbid the CUDA allocator. The regular entry points
 * take splitter scratch from the library's arena; this one uses a fixed
 * array of ORIGAMI_NOALLOC_SPLIT_SLOTS 8-byte slots (4 MiB) compiled into the
 * library's device image, held on every GPU that loads the library until the
 * process exits.
 *   - d and tmp: device buffers of n items, both required, 16-byte aligned;
 *     same result-buffer convention and flags as origami_sort_device.
 *   - n must not exceed origami_noalloc_max_items(kind) (ORIGAMI_ERR_INVALID
 *     otherwise); binary merge passes are used (min_k = 2).
 *   - The first call on a device looks up the array's device address; make
 *     that first call before any stream capture begins.
 *   - All calls share the one array: calls whose work overlaps on the GPU race
 *     and must be serialized by the caller.
 *   - With ORIGAMI_FLAG_SYNC the call also reads the sort's device error word
 *     (ORIGAMI_ERR_TIMEOUT when a merge kernel's bounded wait expired).
 */
#define ORIGAMI_NOALLOC_SPLIT_SLOTS 524288
uint64_t origami_noalloc_max_items(int kind);
int origami_sort_noalloc_device(int kind, void* d, void* tmp, uint64_t n, uint64_t sort_n,
                                int flags, void** result, void* stream);

/*
 * Serving loop (no counterpart in the reference, whose callers sort one array
 * per call). A server owns one worker thread that runs continuous batching and
 * two helper threads:
 *   - submit() queues a request: sort the `n` items of `kind` at `in` into
 *     `out` (out == in or NULL: in place; otherwise the two must not overlap).
 *     Each may be host pageable, host pinned or device memory, with any
 *     alignment; n = 0 completes at once. Both buffers must stay valid, and
 *     `out` untouched, until wait() returns for the request.
 *   - Requests are admitted in arrival order while the HBM budget allows and
 *     fewer than max_inflight batches are on the GPU. The oldest request that
 *     does not fit waits for running batches to return memory.
 *   - Device memory comes from the server's arena: slabs held until the server
 *     is destroyed, carved into blocks per batch; after warm-up no request
 *     allocates device memory.
 *   - A request of 2^24 items or more whose buffers the device can address
 *     (pinned or device memory; pageable memory on hosts whose GPU reads the
 *     host's page tables), 16-byte aligned, is a batch of its own: a helper
 *     thread runs the pipelined single-array sort on it (its chunks copied in
 *     while earlier chunks sort, its output copied out while later slices
 *     merge). Smaller requests of one kind are coalesced into one batched
 *     segmented sort (at most max_batch_items items unless one request is
 *     larger), each batch on its own stream, so new batches overlap running
 *     ones; pageable outputs are copied out by a helper thread.
 *   - Results are identical to sorting each request alone (key-value requests
 *     stably).
 * Errors: ORIGAMI_ERR_OOM at submit for a request that can never fit the
 * budget; ORIGAMI_ERR_BUSY when max_queue requests are pending (or, from
 * cancel, when the request was already admitted); ORIGAMI_ERR_TIMEOUT from
 * wait() when timeout_ms (< 0: no limit) passes first; ORIGAMI_ERR_CANCELLED
 * from wait() for a cancelled request; a failed batch's status (OOM when the
 * device could not supply the budgeted memory) from wait() for each of its
 * requests. wait() collects a finished request: its id is unknown afterwards.
 * Zero arguments to create() select the defaults: 120 GiB budget, 6 batches in
 * flight, 2^28 items per batch, 2^20 pending requests. destroy() cancels what
 * is pending, waits for the batches in flight and frees the server and its
 * arena; no other call on it may be in progress.
 */
typedef struct origami_server origami_server;

typedef struct origami_server_stats {
    uint64_t submitted, completed, failed, cancelled; /* requests since create/reset */
    uint64_t keys;                                    /* items of completed requests */
    uint64_t batches;                                 /* segmented launches */
    uint64_t pending;                                 /* requests waiting now */
    uint64_t bytes_reserved, peak_bytes_reserved;     /* against the HBM budget */
    uint64_t max_concurrent_batches;                  /* most batches in flight at once */
    double p50_ms, p99_ms, max_ms;                    /* latency, submission to completion */
    double keys_per_s; /* keys / (last completion - first submission) */
    uint64_t pipe_batches;              /* large requests run as the pipelined sort (in batches) */
    uint64_t arena_bytes, arena_grows;  /* the server's device arena: bytes held, slab allocations */
} origami_server_stats;

int origami_serve_create(origami_server** out, uint64_t hbm_budget_bytes, int max_inflight,
                          uint64_t max_batch_items, uint64_t max_queue);
int origami_serve_submit(origami_server* s, int kind, const void* in, void* out, uint64_t n,
                          uint64_t* id);
int origami_serve_wait(origami_server* s, uint64_t id, int64_t timeout_ms);
int origami_serve_cancel(origami_server* s, uint64_t id);
int origami_serve_get_stats(origami_server* s, origami_server_stats* out);
int origami_serve_reset_stats(origami_server* s);
int origami_serve_destroy(origami_server* s);

/*
 * Device-side input generator for the reference's Writer distributions
 * (writer.h:27-35; no device counterpart there): fills the device buffer d
 * with n items of `kind`, dist 1..9 = uniform, all same, sorted, reverse
 * sorted, almost sorted (every 7th item at the maximum), Pareto keys, Pareto
 * back to back, Pareto shuffled, Fibonacci. Distributions 2, 6, 7 and 9 are
 * the reference's exact sequences; 1, 3, 4, 5 draw from a counter-based
 * generator seeded by `seed` (the reference's std::mt19937 stream is
 * sequential) with the reference's value ranges; 8 shuffles 7 with `seed`.
 * Key-value items get value = key + 1. Asynchronous on `stream`.
 */
int origami_generate_device(int kind, void* d, uint64_t n, int dist, uint64_t seed, void* stream);

/*
 * Autotuning (no counterpart in the reference, whose tuning is compile-time
 * config.h constants and the bench_sort_phases switch-point sweeps). Every
 * sort with min_k = 0 takes its pass shape from a table indexed by item kind
 * and size class floor(log2 n): the merge fan-in (2 = binary passes, 4/8/16 =
 * k-way passes) and, for binary passes, one of four merge shapes: 0 (the
 * default) and 1 are two tile shapes (threads, items per thread, tile) of the
 * persistent bulk-copy merge kernel where the item kind has one, 2 is shape 0
 * as one tile per CTA, which interleaves better with sorts running on other
 * streams, 3 is shape 0's tile with half the items per thread. The table
 * starts from built-in entries measured on a GB300 (16-way passes for some
 * sizes about as large as L2, other binary shapes for others; binary passes
 * with shape 0 elsewhere). min_k = 2 keeps the table's merge shape with
 * binary passes; larger min_k forces that fan-in.
 *   origami_autotune   times every shape on n generated device items and stores
 *                      the fastest for n's size class; `report` (may be NULL)
 *                      receives one "fan= variant= ms=" line per shape.
 *   get / set          read or write one entry.
 *   save / load        the entries other than binary passes with shape 0 as
 *                      "kind class fan variant"
 *                      lines, and the segmented table's (below) as
 *                      "seg kind class shape" lines. The file named by
 *                      ORIGAMI_TUNING, if set, is loaded at first use.
 */
int origami_autotune(int kind, uint64_t n, char* report, uint64_t cap);
int origami_tuning_get(int kind, uint64_t n, int* fan, int* variant);
int origami_tuning_set(int kind, uint64_t n, int fan, int variant);
int origami_tuning_save(const char* path);
int origami_tuning_load(const char* path);

/*
 * Segmented-sort tuning (no counterpart in the reference; its analogue is the
 * compile-time config.h tables and the bench_sort_phases sweeps). The level
 * merges of a batched segmented sort use one of two merge shapes: 0 (the
 * default) is the binary pass's first tile shape, 1 its second (twice the tile,
 * more threads). The table is keyed by item kind and the size class
 * floor(log2(n / nseg)) of the mean segment length; every segmented launch
 * (origami_sort_segmented*, origami_seg_plan_create, the serving loop's
 * batches) takes its shape from it.
 *   origami_autotune_segmented  times both shapes on the caller's own device
 *                      segments (d is left holding its input), stores the
 *                      faster; `report` (may be NULL) gets "shape= ms=" lines.
 *   get / set          read or write one entry (shape 0 or 1).
 */
int origami_autotune_segmented(int kind, void* d, void* tmp, const uint64_t* offsets, uint64_t nseg, uint64_t n,
                               char* report, uint64_t cap);
int origami_seg_tuning_get(int kind, uint64_t n, uint64_t nseg, int* shape);
int origami_seg_tuning_set(int kind, uint64_t n, uint64_t nseg, int shape);

/* Device arena used by the host-pointer calls and by the serving loop. */
int origami_arena_reserve(uint64_t bytes);  /* pre-grow the pool */
int origami_arena_trim(void);               /* return cached memory to the driver */
uint64_t origami_arena_bytes_in_use(void);

#ifdef __cplusplus
}
#endif
#endif /* ORIGAMI_GPU_H */
