// Serving loop: continuous batching of sort requests.
//
// Clients submit requests (an input and an output buffer, which may be the
// same; host pageable, host pinned or device memory; any kind, any length) and
// wait for the sorted output. One worker thread owns admission and the device
// side; two helper threads run what would block it:
//  * admission: pending requests are taken in arrival order while the HBM
//    budget allows and fewer than `max_inflight` batches are on the device. The
//    oldest request that does not fit waits until running batches return
//    memory; nothing overtakes it.
//  * arena: batches take their device memory from the server's arena, slabs
//    of device memory held for the server's lifetime and carved into blocks
//    (best fit, neighbours merged on release). After warm-up no request
//    allocates or frees device memory.
//  * large requests (PIPE_MIN items or more, buffers the device can address):
//    each is a batch of its own, run by a helper thread as the pipelined
//    single-array sort: its input arrives in chunks that sort while the next
//    chunks are in flight, and the final k-way pass sends finished output
//    slices back while later slices merge, so its copies overlap its sort.
//  * coalescing: smaller requests of one kind and of comparable size (within a
//    factor SIZE_RATIO of the batch's first) form a batch: their items are
//    copied back to back into one arena block and sorted by one segmented
//    launch, each request a segment, on the batch's own stream, so new batches
//    overlap the batches already running.
//  * completion: results are copied back into the requests' own buffers
//    (pinned and device buffers on the batch's stream; pageable ones by a
//    helper thread, so the worker never waits on a copy). A host function on
//    the stream, or the helper, marks the batch finished and wakes the
//    worker, which returns its memory and releases the waiting clients.
// Latency is per request, from submission to the moment its batch finished.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/origami_gpu.h"
#include "dispatch.h"

namespace {

using Clock = std::chrono::steady_clock;
using origami::SegPlan;

enum ReqState { PENDING = 0, RUNNING = 1, DONE = 2, CANCELLED = 3, FAILED = 4 };
enum MemKind { MEM_PAGEABLE = 0, MEM_PINNED = 1, MEM_DEVICE = 2 };

struct Request {
    uint64_t id = 0;
    int kind = 0;
    const void* in = nullptr;
    void* out = nullptr;
    uint64_t n = 0;
    int mem_out = MEM_PAGEABLE;
    int state = PENDING;
    int status = ORIGAMI_OK;
    Clock::time_point t_submit, t_done;
};

// Largest size ratio between requests of one batch (the first and each other).
constexpr uint64_t SIZE_RATIO = 64;
// Requests of at least this many items take the pipelined single-array sort:
// from 2^24 items on it runs chunked, its copies on the copy engines (smaller
// sorts of host buffers would read and write the host inside their kernels,
// holding the SMs for the whole transfer while other batches wait).
constexpr uint64_t PIPE_MIN = 1ull << 24;
constexpr int HELPERS = 2;

// The server's device arena: slabs of device memory kept until the server is
// destroyed (or trimmed when nothing is in flight), carved into 256-byte
// aligned blocks by best fit; a released block merges with free neighbours of
// the same slab.
class Arena {
    struct Slab {
        char* base;
        uint64_t size;
    };
    std::vector<Slab> slabs_;
    std::map<char*, uint64_t> free_;  // free ranges: start -> bytes
    uint64_t reserved_ = 0, grows_ = 0;
    cudaStream_t st_ = nullptr;  // slab allocations (stream-ordered: no device-wide synchronization)

    const Slab* slab_of(const char* p) const {
        for (const Slab& s : slabs_)
            if (p >= s.base && p < s.base + s.size) return &s;
        return nullptr;
    }

  public:
    ~Arena() {
        trim(true);
        if (st_) cudaStreamDestroy(st_);
    }
    uint64_t reserved() const { return reserved_; }
    uint64_t grows() const { return grows_; }
    // A block of `bytes`, growing by a new slab (at least `slab_min` bytes, and
    // half of what is reserved, so that growth is rare) while the slabs stay
    // within `cap` bytes; nullptr when neither works.
    char* alloc(uint64_t bytes, uint64_t cap, uint64_t slab_min) {
        bytes = (bytes + 255) & ~255ull;
        auto best = free_.end();
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= bytes && (best == free_.end() || it->second < best->second)) best = it;
        if (best == free_.end()) {
            uint64_t sz = std::max(std::max(bytes, slab_min), reserved_ / 2);
            sz = (sz + (2ull << 20) - 1) & ~((2ull << 20) - 1);
            if (reserved_ + sz > cap) sz = bytes;
            if (reserved_ + sz > cap) return nullptr;
            if (!st_) cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking);
            char* p = nullptr;
            if (cudaMallocAsync(reinterpret_cast<void**>(&p), sz, st_) != cudaSuccess ||
                cudaStreamSynchronize(st_) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
            slabs_.push_back({p, sz});
            reserved_ += sz;
            ++grows_;
            best = free_.emplace(p, sz).first;
        }
        char* p = best->first;
        const uint64_t left = best->second - bytes;
        free_.erase(best);
        if (left) free_.emplace(p + bytes, left);
        return p;
    }
    void release(char* p, uint64_t bytes) {
        bytes = (bytes + 255) & ~255ull;
        const Slab* s = slab_of(p);
        auto next = free_.lower_bound(p);
        if (next != free_.end() && next->first == p + bytes && slab_of(next->first) == s) {
            bytes += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == p && slab_of(prev->first) == s) {
                prev->second += bytes;
                return;
            }
        }
        free_.emplace(p, bytes);
    }
    // Returns the slabs that hold no block (all of them with `all`) to the device.
    void trim(bool all = false) {
        for (size_t i = 0; i < slabs_.size();) {
            auto it = free_.find(slabs_[i].base);
            const bool empty = it != free_.end() && it->second == slabs_[i].size;
            if (empty || all) {
                if (it != free_.end()) free_.erase(it);
                cudaFreeAsync(slabs_[i].base, st_);
                reserved_ -= slabs_[i].size;
                slabs_.erase(slabs_.begin() + (long)i);
            } else {
                ++i;
            }
        }
        if (all) free_.clear();
        if (st_) cudaStreamSynchronize(st_);
    }
};

uint64_t item_bytes(int kind) { return kind == ORIGAMI_U32 ? 4u : (kind <= ORIGAMI_I64 ? 8u : 16u); }
uint64_t r256(uint64_t b) { return (b + 255) & ~255ull; }

// Arena block of one batch: d | tmp | offsets | scratch, each 256-byte aligned.
struct Layout {
    uint64_t tmp, off, scratch, total;
    SegPlan plan;
};
Layout layout(int kind, uint64_t items, uint64_t nseg) {
    Layout l;
    l.plan = origami::seg_plan(kind, items, nseg);
    const uint64_t data = r256(items * item_bytes(kind));
    l.tmp = data;
    l.off = 2 * data;
    l.scratch = l.off + r256((nseg + 1) * 8);
    l.total = l.scratch + r256(l.plan.scratch_bytes);
    return l;
}

int mem_kind(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return MEM_PAGEABLE;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return MEM_DEVICE;
    if (a.type == cudaMemoryTypeHost) return MEM_PINNED;
    return MEM_PAGEABLE;
}

}  // namespace

struct origami_server;

namespace {
struct Batch {
    origami_server* srv = nullptr;
    int kind = 0;
    bool pipe = false;  // one large request, sorted by a helper thread
    std::vector<std::shared_ptr<Request>> reqs;
    std::vector<uint64_t> off;
    Layout lay{};
    uint64_t bytes = 0;  // arena block size (reserved against the budget)
    cudaStream_t stream = nullptr;
    char* block = nullptr;
    int* herr = nullptr;  // pinned copy of the device error word
    int status = ORIGAMI_OK;
    std::atomic<bool> finished{false};
    bool copied = false;     // pageable outputs have been copied out (or there are none)
    bool abandoned = false;  // its stream failed before the completion marker ran
    Clock::time_point t_end;
};
}  // namespace

struct origami_server {
    uint64_t budget = 0;
    int max_inflight = 0;
    uint64_t max_batch_items = 0;
    uint64_t max_queue = 0;
    int device = 0;
    bool ats = false;  // the device reads pageable host memory through the host's page tables

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    uint64_t gen = 0;  // bumped by every submission and every finished batch
    std::deque<std::shared_ptr<Request>> pending;
    std::map<uint64_t, std::shared_ptr<Request>> reqs;  // until the client's wait() collects them
    uint64_t in_use = 0, peak_in_use = 0;
    bool stop = false;
    uint64_t next_id = 0;

    // statistics since creation or the last reset (under mu)
    std::vector<double> lat_ms;
    uint64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, keys = 0, batches = 0, pipe_batches = 0;
    uint64_t max_concurrent = 0;
    bool have_first = false;
    Clock::time_point t_first, t_last;

    // worker state; `inflight` changes only with mu held
    std::vector<std::unique_ptr<Batch>> inflight;
    std::vector<cudaStream_t> streams;
    std::vector<int*> err_words;
    std::vector<std::unique_ptr<Batch>> abandoned;  // kept: a late marker may still touch them
    Arena arena;  // used by the worker thread only
    std::atomic<uint64_t> arena_reserved{0}, arena_grows{0};  // its figures, for get_stats
    std::thread worker;

    // helper threads: large requests and pageable copies (tasks under mu)
    std::deque<std::function<void()>> tasks;
    std::condition_variable cv_task;
    int idle_helpers = 0;
    bool helpers_stop = false;
    std::vector<std::thread> helpers;

    uint64_t need(int kind, uint64_t items, uint64_t nseg) const { return layout(kind, items, nseg).total; }

    // Large requests whose buffers the device can address, 16-byte aligned,
    // take the pipelined sort.
    bool pipe_ok(const Request& r) const {
        if (r.n < PIPE_MIN) return false;
        auto addressable = [&](const void* p) {
            const int m = mem_kind(p);
            return (m != MEM_PAGEABLE || ats) && (((uintptr_t)p) & 15) == 0;
        };
        return addressable(r.in) && addressable(r.out);
    }
    uint64_t need_of(const Request& r) const {
        return pipe_ok(r) ? origami::host_pipe_bytes(r.kind, r.n) : need(r.kind, r.n, 1);
    }

    static void CUDART_CB on_done(void* p) {
        auto* b = static_cast<Batch*>(p);
        b->t_end = Clock::now();
        {
            std::lock_guard<std::mutex> lk(b->srv->mu);
            b->finished.store(true);
            ++b->srv->gen;
        }
        b->srv->cv_work.notify_one();
    }

    // Marks a batch finished from a helper thread.
    void helper_done(Batch& b) {
        {
            std::lock_guard<std::mutex> lk(mu);
            if (b.t_end == Clock::time_point()) b.t_end = Clock::now();
            b.finished.store(true);
            ++gen;
        }
        cv_work.notify_one();
    }

    void post(std::function<void()> f) {  // mu held
        tasks.push_back(std::move(f));
        cv_task.notify_one();
    }

    void helper_loop() {
        cudaSetDevice(device);
        cudaStream_t st = nullptr;
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
            ++idle_helpers;
            cv_task.wait(lk, [&] { return !tasks.empty() || helpers_stop; });
            --idle_helpers;
            if (tasks.empty()) break;  // stopping
            auto f = std::move(tasks.front());
            tasks.pop_front();
            lk.unlock();
            // a pipelined sort runs on this thread's own streams
            cur_stream = st;
            f();
            lk.lock();
        }
        lk.unlock();
        cudaStreamDestroy(st);
    }
    static thread_local cudaStream_t cur_stream;

    // Takes the next batch from the pending queue (mu held): the oldest
    // request decides. A large request is a batch of its own once a helper is
    // free; otherwise requests of its kind and comparable size follow it into a
    // segmented batch. Returns null when nothing can be admitted now.
    std::unique_ptr<Batch> admit() {
        while (!pending.empty() && pending.front()->state == CANCELLED) pending.pop_front();
        if (pending.empty()) return nullptr;
        auto b = std::make_unique<Batch>();
        b->srv = this;
        b->kind = -1;
        uint64_t items = 0;
        bool head = true;
        for (auto it = pending.begin(); it != pending.end();) {
            auto r = *it;
            if (r->state == CANCELLED) {
                it = pending.erase(it);
                continue;
            }
            const bool big = pipe_ok(*r);
            if (big) {
                if (!b->reqs.empty()) {  // a segmented batch is being formed: not for it
                    ++it;
                    continue;
                }
                const uint64_t nb = origami::host_pipe_bytes(r->kind, r->n);
                if (in_use + nb > budget) {
                    if (head) return nullptr;  // the oldest waits for memory; nothing overtakes it
                    ++it;
                    continue;
                }
                if (idle_helpers - (int)tasks.size() <= 0) {  // no helper free: let later requests go
                    head = false;
                    ++it;
                    continue;
                }
                b->kind = r->kind;
                b->pipe = true;
                b->bytes = nb;
                r->state = RUNNING;
                b->reqs.push_back(r);
                pending.erase(it);
                break;
            }
            if (b->kind >= 0 && r->kind != b->kind) {
                head = false;
                ++it;
                continue;
            }
            if (!b->reqs.empty() && items + r->n > max_batch_items) break;
            // requests of very different sizes go to different batches: a
            // small request batched with a huge one would wait for all of it
            if (!b->reqs.empty()) {
                const uint64_t h = b->reqs.front()->n, m = r->n;
                if (m > SIZE_RATIO * h + 1024 || h > SIZE_RATIO * m + 1024) break;
            }
            // the oldest request waits for memory rather than being overtaken,
            // so a large request is never starved by a stream of small ones
            if (in_use + need(r->kind, items + r->n, b->reqs.size() + 1) > budget) {
                if (b->reqs.empty() && !head) {
                    ++it;
                    continue;
                }
                break;
            }
            head = false;
            b->kind = r->kind;
            items += r->n;
            r->state = RUNNING;
            b->reqs.push_back(r);
            it = pending.erase(it);
        }
        if (b->reqs.empty()) return nullptr;
        if (!b->pipe) {
            b->off.assign(b->reqs.size() + 1, 0);
            for (size_t i = 0; i < b->reqs.size(); ++i) b->off[i + 1] = b->off[i] + b->reqs[i]->n;
            b->lay = layout(b->kind, items, b->reqs.size());
            b->bytes = b->lay.total;
        }
        b->copied = true;
        for (auto& r : b->reqs)
            if (!b->pipe && r->mem_out == MEM_PAGEABLE) b->copied = false;
        in_use += b->bytes;
        peak_in_use = std::max(peak_in_use, in_use);
        ++batches;
        if (b->pipe) ++pipe_batches;
        return b;
    }

    // Its arena block (worker thread, mu not held); false when the arena
    // cannot supply it now.
    bool take_block(Batch& b) {
        b.block = arena.alloc(b.bytes, budget, std::min<uint64_t>(budget, 1ull << 30));
        arena_reserved.store(arena.reserved());
        arena_grows.store(arena.grows());
        return b.block != nullptr;
    }

    // Enqueues a segmented batch's copies, sort and completion marker (mu not
    // held). A large request goes to a helper thread instead.
    void launch(Batch& b) {
        if (b.pipe) {
            Batch* pb = &b;
            std::lock_guard<std::mutex> lk(mu);
            post([this, pb] {
                const Request& r = *pb->reqs[0];
                pb->status = origami::host_pipe_sort(pb->kind, r.in, r.out, r.n, pb->block, cur_stream);
                pb->t_end = Clock::now();
                helper_done(*pb);
            });
            return;
        }
        if (streams.empty()) {
            cudaStream_t s = nullptr;
            cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
            streams.push_back(s);
        }
        b.stream = streams.back();
        streams.pop_back();
        if (err_words.empty()) {
            int* w = nullptr;
            if (cudaHostAlloc(&w, sizeof(int), cudaHostAllocDefault) != cudaSuccess) w = nullptr;
            err_words.push_back(w);
        }
        b.herr = err_words.back();
        err_words.pop_back();
        if (b.herr) *b.herr = 0;

        const uint64_t ib = item_bytes(b.kind);
        const uint64_t items = b.off.back();
        const uint64_t nseg = b.reqs.size();
        cudaError_t e = b.herr ? cudaSuccess : cudaErrorMemoryAllocation;
        char* d = b.block;
        uint64_t* doff = reinterpret_cast<uint64_t*>(d + b.lay.off);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(doff, b.off.data(), (nseg + 1) * 8, cudaMemcpyHostToDevice, b.stream);
        for (uint64_t i = 0; e == cudaSuccess && i < nseg; ++i) {
            const Request& r = *b.reqs[i];
            e = cudaMemcpyAsync(d + b.off[i] * ib, r.in, r.n * ib, cudaMemcpyDefault, b.stream);
        }
        if (e == cudaSuccess)
            e = origami::seg_launch(b.kind, d, d + b.lay.tmp, doff, nseg, items, d + b.lay.scratch, b.lay.plan,
                                    b.stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b.herr, d + b.lay.scratch + b.lay.plan.err_offset, sizeof(int),
                                cudaMemcpyDeviceToHost, b.stream);
        // pinned and device destinations are written on the stream; pageable
        // ones by a helper once the batch has finished, so this thread never
        // blocks on a running sort
        for (uint64_t i = 0; e == cudaSuccess && i < nseg; ++i) {
            const Request& r = *b.reqs[i];
            if (r.mem_out != MEM_PAGEABLE)
                e = cudaMemcpyAsync(r.out, d + b.off[i] * ib, r.n * ib, cudaMemcpyDefault, b.stream);
        }
        if (e != cudaSuccess) b.status = e == cudaErrorMemoryAllocation ? ORIGAMI_ERR_OOM : ORIGAMI_ERR_CUDA;
        if (cudaLaunchHostFunc(b.stream, on_done, &b) != cudaSuccess) {
            cudaStreamSynchronize(b.stream);
            if (b.status == ORIGAMI_OK) b.status = ORIGAMI_ERR_CUDA;
            b.t_end = Clock::now();
            std::lock_guard<std::mutex> lk(mu);
            b.finished.store(true);
            ++gen;
        }
    }

    // A finished segmented batch with pageable outputs: a helper copies them
    // out (mu held); the batch finishes again when it is done.
    void post_copy_out(Batch& b) {
        b.copied = true;
        b.finished.store(false);
        Batch* pb = &b;
        post([this, pb] {
            const uint64_t ib = item_bytes(pb->kind);
            for (size_t i = 0; i < pb->reqs.size() && pb->status == ORIGAMI_OK; ++i) {
                const Request& r = *pb->reqs[i];
                if (r.mem_out != MEM_PAGEABLE) continue;
                cudaError_t e = cudaMemcpyAsync(r.out, pb->block + pb->off[i] * ib, r.n * ib, cudaMemcpyDeviceToHost,
                                                pb->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(pb->stream);
                if (e != cudaSuccess) pb->status = ORIGAMI_ERR_CUDA;
            }
            pb->t_end = Clock::now();
            helper_done(*pb);
        });
    }

    // Reads the device error word and returns the batch's memory (mu not held).
    void retire(Batch& b) {
        if (!b.pipe && b.status == ORIGAMI_OK && b.herr && *b.herr != 0)
            b.status = origami::err_word_timeout(*b.herr) ? ORIGAMI_ERR_TIMEOUT : ORIGAMI_ERR_INVALID;
        if (b.abandoned) return;  // the stream is broken: keep its memory and stream out of reuse
        if (b.block) arena.release(b.block, b.bytes);
        if (b.stream) streams.push_back(b.stream);
        if (b.herr) err_words.push_back(b.herr);
    }

    void run() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        uint64_t seen = ~0ull;
        while (true) {
            // finished batches: pageable outputs still to copy go to a helper,
            // the others are retired
            std::vector<std::unique_ptr<Batch>> fin;
            for (size_t i = 0; i < inflight.size();) {
                Batch& b = *inflight[i];
                if (b.finished.load()) {
                    if (!b.copied && !b.abandoned && b.status == ORIGAMI_OK &&
                        !(b.herr && *b.herr != 0)) {
                        post_copy_out(b);
                        ++i;
                        continue;
                    }
                    fin.push_back(std::move(inflight[i]));
                    inflight.erase(inflight.begin() + (long)i);
                } else {
                    ++i;
                }
            }
            if (!fin.empty()) {
                lk.unlock();
                for (auto& b : fin) retire(*b);
                lk.lock();
                for (auto& b : fin) {
                    in_use -= b->bytes;
                    for (auto& r : b->reqs) {
                        r->state = b->status == ORIGAMI_OK ? DONE : FAILED;
                        r->status = b->status;
                        r->t_done = b->t_end;
                        lat_ms.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
                        if (b->status == ORIGAMI_OK) {
                            ++completed;
                            keys += r->n;
                        } else {
                            ++failed;
                        }
                    }
                    if (b->t_end > t_last) t_last = b->t_end;
                    if (b->abandoned) abandoned.push_back(std::move(b));
                }
                cv_done.notify_all();
            }
            // admit and launch
            std::vector<std::unique_ptr<Batch>> adm;
            while ((int)(inflight.size() + adm.size()) < max_inflight) {
                auto b = admit();
                if (!b) break;
                adm.push_back(std::move(b));
            }
            if (!adm.empty()) {
                lk.unlock();
                std::vector<std::unique_ptr<Batch>> back;  // no arena block now: back to the queue
                for (auto& b : adm) {
                    if (!take_block(*b)) {
                        if (inflight.empty() && adm.size() == 1) arena.trim();
                        if (!take_block(*b)) {
                            back.push_back(std::move(b));
                            continue;
                        }
                    }
                    launch(*b);
                }
                lk.lock();
                for (auto& b : adm)
                    if (b) inflight.push_back(std::move(b));
                for (auto it = back.rbegin(); it != back.rend(); ++it) {
                    Batch& b = **it;
                    in_use -= b.bytes;
                    --batches;
                    if (b.pipe) --pipe_batches;
                    if (inflight.empty()) {
                        // nothing will return memory: the request cannot be served
                        for (auto& r : b.reqs) {
                            r->state = FAILED;
                            r->status = ORIGAMI_ERR_OOM;
                            r->t_done = Clock::now();
                            ++failed;
                        }
                        cv_done.notify_all();
                        continue;
                    }
                    for (auto r = b.reqs.rbegin(); r != b.reqs.rend(); ++r) {
                        (*r)->state = PENDING;
                        pending.push_front(*r);
                    }
                }
                max_concurrent = std::max<uint64_t>(max_concurrent, inflight.size());
                if (back.empty()) continue;
            }
            if (!fin.empty()) continue;
            if (stop && inflight.empty()) break;  // destroy() cancelled everything pending
            // sleep until a submission or a finished batch; the timeout is a
            // backstop that also notices streams that failed
            if (gen == seen) {
                cv_work.wait_for(lk, std::chrono::milliseconds(2), [&] { return gen != seen || stop; });
                if (gen == seen && !inflight.empty()) {
                    for (auto& b : inflight) {
                        if (b->pipe || !b->stream || b->finished.load()) continue;
                        const cudaError_t q = cudaStreamQuery(b->stream);
                        if (q != cudaSuccess && q != cudaErrorNotReady && !b->finished.load()) {
                            b->abandoned = true;
                            b->status = ORIGAMI_ERR_CUDA;
                            b->t_end = Clock::now();
                            b->finished.store(true);
                            ++gen;
                        }
                    }
                }
            }
            seen = gen;
        }
        // no batch is in flight: stop the helpers
        helpers_stop = true;
        cv_task.notify_all();
        lk.unlock();
        for (auto& h : helpers) h.join();
        for (cudaStream_t s : streams) cudaStreamDestroy(s);
        for (int* w : err_words)
            if (w) cudaFreeHost(w);
        streams.clear();
        err_words.clear();
        arena.trim(true);
    }
};

thread_local cudaStream_t origami_server::cur_stream = nullptr;

extern "C" {

int origami_serve_create(origami_server** out, uint64_t hbm_budget_bytes, int max_inflight,
                          uint64_t max_batch_items, uint64_t max_queue) {
    if (!out) return origami::api_fail(ORIGAMI_ERR_INVALID, "out is NULL");
    *out = nullptr;
    const int rc = origami::arena_init();
    if (rc != ORIGAMI_OK) return rc;
    auto* s = new origami_server();
    s->budget = hbm_budget_bytes ? hbm_budget_bytes : (120ull << 30);
    s->max_inflight = max_inflight > 0 ? max_inflight : 6;
    s->max_batch_items = max_batch_items ? max_batch_items : (1ull << 28);
    s->max_queue = max_queue ? max_queue : (1ull << 20);
    cudaGetDevice(&s->device);
    int pageable = 0, host_tables = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, s->device);
    cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, s->device);
    s->ats = pageable && host_tables;
    for (int i = 0; i < HELPERS; ++i) s->helpers.emplace_back([s] { s->helper_loop(); });
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return ORIGAMI_OK;
}

int origami_serve_submit(origami_server* s, int kind, const void* in, void* out, uint64_t n,
                          uint64_t* id) {
    if (!s || !id) return origami::api_fail(ORIGAMI_ERR_INVALID, "server and id are required");
    *id = 0;
    if (kind < ORIGAMI_U32 || kind > ORIGAMI_KVU64) return origami::api_fail(ORIGAMI_ERR_DTYPE, "unknown item kind");
    if (!out) out = const_cast<void*>(in);
    if (n > 0 && !in) return origami::api_fail(ORIGAMI_ERR_INVALID, "input is NULL");
    if (n > (1ull << 36)) return origami::api_fail(ORIGAMI_ERR_INVALID, "request is too large");
    if (n > 0 && out != in) {
        const char* a = static_cast<const char*>(in);
        const char* c = static_cast<const char*>(out);
        const uint64_t bytes = n * item_bytes(kind);
        if (a < c + bytes && c < a + bytes)
            return origami::api_fail(ORIGAMI_ERR_INVALID, "input and output overlap without being the same buffer");
    }
    auto r = std::make_shared<Request>();
    r->kind = kind;
    r->in = in;
    r->out = out;
    r->n = n;
    r->mem_out = n ? mem_kind(out) : MEM_PAGEABLE;
    r->t_submit = Clock::now();
    const uint64_t alone = n ? s->need_of(*r) : 0;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return origami::api_fail(ORIGAMI_ERR_CANCELLED, "server is shutting down");
    if (alone > s->budget) return origami::api_fail(ORIGAMI_ERR_OOM, "request exceeds the HBM budget");
    if (s->pending.size() >= s->max_queue) return origami::api_fail(ORIGAMI_ERR_BUSY, "request queue is full");
    r->id = ++s->next_id;
    ++s->submitted;
    if (!s->have_first) {
        s->have_first = true;
        s->t_first = r->t_submit;
    }
    s->reqs[r->id] = r;
    *id = r->id;
    if (n == 0) {
        r->state = DONE;
        r->t_done = r->t_submit;
        s->lat_ms.push_back(0.0);
        ++s->completed;
        s->cv_done.notify_all();
        return ORIGAMI_OK;
    }
    s->pending.push_back(r);
    ++s->gen;
    s->cv_work.notify_one();
    return ORIGAMI_OK;
}

int origami_serve_wait(origami_server* s, uint64_t id, int64_t timeout_ms) {
    if (!s) return origami::api_fail(ORIGAMI_ERR_INVALID, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return origami::api_fail(ORIGAMI_ERR_INVALID, "unknown request id");
    auto r = it->second;
    auto ready = [&] { return r->state >= DONE; };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return origami::api_fail(ORIGAMI_ERR_TIMEOUT, "request not finished yet");
    }
    s->reqs.erase(r->id);
    if (r->state == CANCELLED) return origami::api_fail(ORIGAMI_ERR_CANCELLED, "request was cancelled");
    if (r->status != ORIGAMI_OK) return origami::api_fail(r->status, "the request's batch failed");
    return ORIGAMI_OK;
}

int origami_serve_cancel(origami_server* s, uint64_t id) {
    if (!s) return origami::api_fail(ORIGAMI_ERR_INVALID, "server is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return origami::api_fail(ORIGAMI_ERR_INVALID, "unknown request id");
    if (it->second->state != PENDING) return origami::api_fail(ORIGAMI_ERR_BUSY, "request already admitted");
    it->second->state = CANCELLED;
    ++s->cancelled;
    s->cv_done.notify_all();
    return ORIGAMI_OK;
}

int origami_serve_get_stats(origami_server* s, origami_server_stats* out) {
    if (!s || !out) return origami::api_fail(ORIGAMI_ERR_INVALID, "server and out are required");
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> l = s->lat_ms;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
        if (l.empty()) return 0.0;
        const size_t i = (size_t)(q * (double)(l.size() - 1) + 0.5);
        return l[std::min(i, l.size() - 1)];
    };
    std::memset(out, 0, sizeof *out);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->cancelled = s->cancelled;
    out->keys = s->keys;
    out->batches = s->batches;
    out->pending = s->pending.size();
    out->bytes_reserved = s->in_use;
    out->peak_bytes_reserved = s->peak_in_use;
    out->max_concurrent_batches = s->max_concurrent;
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->max_ms = l.empty() ? 0.0 : l.back();
    const double sec = s->have_first ? std::chrono::duration<double>(s->t_last - s->t_first).count() : 0.0;
    out->keys_per_s = sec > 0 ? (double)s->keys / sec : 0.0;
    out->pipe_batches = s->pipe_batches;
    out->arena_bytes = s->arena_reserved.load();
    out->arena_grows = s->arena_grows.load();
    return ORIGAMI_OK;
}

int origami_serve_reset_stats(origami_server* s) {
    if (!s) return origami::api_fail(ORIGAMI_ERR_INVALID, "server is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat_ms.clear();
    s->submitted = s->completed = s->failed = s->cancelled = s->keys = s->batches = s->pipe_batches = 0;
    s->max_concurrent = s->inflight.size();
    s->peak_in_use = s->in_use;
    s->have_first = false;
    s->t_last = Clock::time_point();
    return ORIGAMI_OK;
}

int origami_serve_destroy(origami_server* s) {
    if (!s) return origami::api_fail(ORIGAMI_ERR_INVALID, "server is NULL");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto& r : s->pending)
            if (r->state == PENDING) {
                r->state = CANCELLED;
                ++s->cancelled;
            }
        s->pending.clear();
        s->stop = true;
        ++s->gen;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    s->worker.join();
    delete s;
    return ORIGAMI_OK;
}

}  // extern "C"
