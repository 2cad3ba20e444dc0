// fz_server.cu -- a request loop that compresses and decompresses fields as they
// arrive, with continuous batching under an HBM budget.
//
// The server owns
//   * a device pool of `hbm_budget` bytes (one allocation, first-fit free list with
//     coalescing) from which each admitted request takes its input and output buffers;
//   * `slots` execution slots, each a CUDA stream with its own workspace (scan state),
//     a pinned 128-byte readback buffer and an event.
// Requests wait in a queue (admission: see admit()).  Host-buffer requests (pinned ones let
// the copies overlap) are staged through pool buffers; device-resident requests (FZ_REQUEST_DEVICE) run on
// the caller's device buffers and only count their bytes against the pool.
// Worker threads (up to kWorkers, each owning every kWorkers-th slot) retire requests
// whose work has finished and admit queued requests while a slot is free and the pool
// can hold their buffers; the CUDA calls that issue a request (launches, copies) run
// outside the server's lock, so several requests are issued at once.
// fz_server_poll never blocks: it hands out the completions.  Requests on different
// slots overlap on the device (copies on the copy engines, kernels side by side), so
// work that arrives while others run starts as soon as memory and a slot free up.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/fz.h"
#include "fz_internal.h"
#include "fz_workspace.h"

using namespace fz;

namespace {

// First-fit allocator over [0, size) with 256-byte granules; frees coalesce.
class Pool {
public:
    explicit Pool(uint64_t size) { free_[0] = size; }
    bool alloc(uint64_t bytes, uint64_t* off)
    {
        bytes = (bytes + 255) & ~uint64_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off              = it->first;
            const uint64_t rest = it->second - bytes, at = it->first + bytes;
            free_.erase(it);
            if (rest) free_[at] = rest;
            used_ += bytes;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes)
    {
        bytes = (bytes + 255) & ~uint64_t(255);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t used() const { return used_; }

private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t                     used_ = 0;
};

// WaitInHeader: a device-resident decompression waits for its stream header (64 B);
// WaitHeader: a compression waits for its output header (stream length).
enum class Phase { Idle, WaitInHeader, WaitHeader, WaitDone };

struct Slot {
    cudaStream_t  stream = nullptr;
    fz_workspace* ws     = nullptr;
    uint8_t*      h_buf  = nullptr;  // pinned: header (64 B) + status word
    uint32_t*     d_mirror = nullptr;  // device: header + status of a compression (one copy home)
    cudaEvent_t   ev     = nullptr;
    Phase         phase  = Phase::Idle;
    fz_request    req{};
    fz_header     hdr{};  // copy of req.header (req.header points at it while it runs)
    uint64_t      src_off = 0, src_bytes = 0, dst_off = 0, dst_bytes = 0;
    uint64_t      result  = 0;
    fz_status     status  = FZ_SUCCESS;
};

uint64_t max_stream_bytes(uint64_t n, fz_dims d, fz_mode m)
{
    uint64_t b = 0;
    return fz_max_compressed_bytes(n, d, m, &b) == FZ_SUCCESS ? b : 0;
}

// Admission: a request may start ahead of earlier queued ones that are waiting for pool
// memory, within the first kAdmitWindow queue entries (so a small request is not held
// behind a large one that does not fit yet).  Measured on the host-buffer trace of the
// mixed batch (2000 req/s, 8 slots): splitting host copies into 8 MiB pieces, or capping
// the requests with large copies running at once, lengthened the tails and cut the
// saturated throughput (198 -> 121-162 GB/s), so copies go out whole and nothing is capped.
constexpr uint32_t kAdmitWindow = 64;

}  // namespace

// A queued request with its own copy of the caller's header (if any).
struct Queued {
    fz_request r;  // r.header is null here; has_header says whether h holds a copy
    fz_header  h;
    bool       has_header;
};

constexpr uint32_t kWorkers = 8;  // issuing threads (at most one per slot)

struct fz_server {
    uint8_t*                   d_pool = nullptr;
    Pool*                      pool   = nullptr;
    uint64_t                   budget = 0, max_n = 0;
    int                        device = 0;
    std::vector<Slot>          slots;  // slot i belongs to worker i % workers.size()
    // guarded by mu: queue, done, pool, running
    std::mutex                 mu;
    std::condition_variable    cv;     // new requests, shutdown
    std::deque<Queued>         queue;
    std::deque<fz_completion>  done;   // finished but not yet handed out
    std::atomic<uint32_t>      ndone{0};  // done.size(), read without the lock by poll
    uint32_t                   running = 0;
    std::atomic<bool>          stop{false};
    std::vector<std::thread>   workers;
};

namespace {

bool is_device(const fz_request& r) { return (r.flags & FZ_REQUEST_DEVICE) != 0; }

// Pool bytes a request holds while it runs: its staging buffers, or for a device-resident
// request the size of its own input and output.
bool request_bytes(const fz_request& r, uint64_t* src, uint64_t* dst)
{
    if (r.dir == FZ_COMPRESS) {
        *src = 4 * r.n;
        *dst = is_device(r) ? r.dst_capacity : max_stream_bytes(r.n, r.dims, r.mode);
        return *dst != 0;
    }
    *src = r.src_bytes;
    if (is_device(r)) {
        *dst = r.dst_capacity;
        return true;
    }
    fz_header h;
    std::memcpy(&h, r.src, sizeof(h));
    *dst = 4 * h.n;
    return true;
}

// Hands a slot's request back (pool bytes released, completion queued).  Called by the
// slot's worker.
void finish(fz_server* S, Slot& sl, fz_status st, uint64_t result)
{
    std::lock_guard<std::mutex> lk(S->mu);
    S->pool->release(sl.src_off, sl.src_bytes);
    S->pool->release(sl.dst_off, sl.dst_bytes);
    S->done.push_back(fz_completion{sl.req.id, st, result});
    S->ndone.store((uint32_t)S->done.size(), std::memory_order_release);
    --S->running;
    sl.phase = Phase::Idle;
}

// Decompression of a stream whose header is known, into the slot's output buffer, then
// the status word (and for host requests the copy out).
fz_status issue_decompress(fz_server* S, Slot& sl, const fz_header& h)
{
    const bool  dev   = is_device(sl.req);
    const void* d_src = dev ? sl.req.src : S->d_pool + sl.src_off;
    float*      d_dst = reinterpret_cast<float*>(dev ? sl.req.dst : S->d_pool + sl.dst_off);
    if (4 * h.n > sl.req.dst_capacity) return FZ_OUT_OF_SPACE;
    fz_status st = fz_decompress(sl.ws, d_src, sl.req.src_bytes, &h, d_dst, h.n, reinterpret_cast<fz_stream_t>(sl.stream));
    if (st == FZ_SUCCESS && !dev &&
        cudaMemcpyAsync(sl.req.dst, d_dst, 4 * h.n, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess)
        st = FZ_FAIL_GPU_MEMCPY;
    if (st == FZ_SUCCESS && cudaMemcpyAsync(sl.h_buf + 64, sl.ws->status, 4, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess)
        st = FZ_FAIL_GPU_MEMCPY;
    if (st == FZ_SUCCESS && cudaEventRecord(sl.ev, sl.stream) != cudaSuccess) st = FZ_FAIL_GPU_ILLEGAL_ACCESS;
    sl.result = h.n;
    sl.phase  = Phase::WaitDone;
    return st;
}

// Enqueues a request's copies and kernels on a free slot.
void issue(fz_server* S, Slot& sl, const fz_request& r, uint64_t src_off, uint64_t src_b, uint64_t dst_off,
           uint64_t dst_b)
{
    sl.req = r, sl.src_off = src_off, sl.src_bytes = src_b, sl.dst_off = dst_off, sl.dst_bytes = dst_b;
    const bool  dev   = is_device(r);
    uint8_t*    d_src = dev ? (uint8_t*)r.src : S->d_pool + src_off;
    uint8_t*    d_dst = dev ? (uint8_t*)r.dst : S->d_pool + dst_off;
    fz_stream_t hs    = reinterpret_cast<fz_stream_t>(sl.stream);
    fz_status   st    = FZ_SUCCESS;
    if (!dev && cudaMemcpyAsync(d_src, r.src, src_b, cudaMemcpyHostToDevice, sl.stream) != cudaSuccess)
        st = FZ_FAIL_GPU_MEMCPY;
    if (r.dir == FZ_COMPRESS) {
        if (st == FZ_SUCCESS)
            st = compress_impl(sl.ws, reinterpret_cast<const float*>(d_src), r.n, r.dims, r.eb, r.eb_mode, r.mode,
                               d_dst, dev ? r.dst_capacity : dst_b, nullptr, hs, sl.d_mirror);
        // header and status come back first, in one copy of the mirror; the stream's
        // length follows from nnz
        if (st == FZ_SUCCESS && cudaMemcpyAsync(sl.h_buf, sl.d_mirror, 68, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess)
            st = FZ_FAIL_GPU_MEMCPY;
        if (st == FZ_SUCCESS && cudaEventRecord(sl.ev, sl.stream) != cudaSuccess) st = FZ_FAIL_GPU_ILLEGAL_ACCESS;
        sl.phase = Phase::WaitHeader;
    } else if (dev && sl.req.header) {
        if (st == FZ_SUCCESS) st = issue_decompress(S, sl, sl.hdr);
    } else if (dev) {
        // the header lives on the device: fetch it first (fz_server_poll never blocks)
        if (cudaMemcpyAsync(sl.h_buf, d_src, 64, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess) st = FZ_FAIL_GPU_MEMCPY;
        if (st == FZ_SUCCESS && cudaEventRecord(sl.ev, sl.stream) != cudaSuccess) st = FZ_FAIL_GPU_ILLEGAL_ACCESS;
        sl.phase = Phase::WaitInHeader;
    } else {
        fz_header h;
        std::memcpy(&h, r.src, sizeof(h));
        if (st == FZ_SUCCESS) st = issue_decompress(S, sl, h);
    }
    if (st != FZ_SUCCESS) {
        cudaStreamSynchronize(sl.stream);
        finish(S, sl, st, 0);
    }
}

// The request's status from the word copied home; a set word is cleared on the device
// (it is sticky in the workspace) so the slot's next request starts clean.
fz_status status_word(const Slot& sl)
{
    uint32_t w;
    std::memcpy(&w, sl.h_buf + 64, 4);
    if (w) {
        cudaMemsetAsync(sl.ws->status, 0, 4, sl.stream);
        cudaStreamSynchronize(sl.stream);
    }
    if (w & kStatusTimeout) return FZ_TIMEOUT;
    if (w & kStatusNonfinite) return FZ_NONFINITE_INPUT;
    if (w & kStatusCorrupt) return FZ_CORRUPT_STREAM;
    return FZ_SUCCESS;
}

// A busy slot whose current phase has finished moves on: a device stream's header has
// arrived (issue its decompression), a compressed stream's header has arrived (copy the
// stream home, or finish a device request), or the request is done.  Returns true when
// the slot changed state.
bool retire(fz_server* S, Slot& sl)
{
    const cudaError_t q = cudaEventQuery(sl.ev);
    if (q == cudaErrorNotReady) return false;
    if (q != cudaSuccess) {
        finish(S, sl, FZ_FAIL_GPU_ILLEGAL_ACCESS, 0);
        return true;
    }
    if (sl.phase == Phase::WaitInHeader) {
        fz_header h;
        std::memcpy(&h, sl.h_buf, sizeof(h));
        const fz_status st = issue_decompress(S, sl, h);
        if (st != FZ_SUCCESS) {
            cudaStreamSynchronize(sl.stream);
            finish(S, sl, st, 0);
        }
        return true;
    }
    if (sl.phase == Phase::WaitHeader) {
        fz_header h;
        std::memcpy(&h, sl.h_buf, sizeof(h));
        uint64_t  bytes = 0;
        fz_status st    = status_word(sl);
        if (st == FZ_SUCCESS) st = fz_stream_bytes(&h, &bytes);
        if (st == FZ_SUCCESS && bytes > sl.req.dst_capacity) st = FZ_OUT_OF_SPACE;
        if (st != FZ_SUCCESS || is_device(sl.req)) {  // a device result is in place already
            finish(S, sl, st, st == FZ_SUCCESS ? bytes : 0);
            return true;
        }
        if (cudaMemcpyAsync(sl.req.dst, S->d_pool + sl.dst_off, bytes, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess)
            st = FZ_FAIL_GPU_MEMCPY;
        if (st == FZ_SUCCESS && cudaEventRecord(sl.ev, sl.stream) != cudaSuccess) st = FZ_FAIL_GPU_ILLEGAL_ACCESS;
        if (st != FZ_SUCCESS) {
            finish(S, sl, st, 0);
            return true;
        }
        sl.result = bytes;
        sl.phase  = Phase::WaitDone;
        return true;
    }
    finish(S, sl, sl.req.dir == FZ_DECOMPRESS ? status_word(sl) : FZ_SUCCESS, sl.result);
    return true;
}

// Admits a queued request onto an idle slot: the first one among the first kAdmitWindow
// queue entries whose buffers the pool can hold; requests that can never run complete at
// once with an error.  The request is issued
// outside the lock.  Returns true when something was admitted or rejected.
bool admit(fz_server* S, Slot& sl)
{
    fz_request r;
    uint64_t   so = 0, sb = 0, dof = 0, db = 0;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        bool                        changed = false;
        uint32_t                    k       = 0;
        for (;;) {
            if (k >= S->queue.size() || k >= kAdmitWindow) return changed;
            const Queued& qf = S->queue[k];
            r                = qf.r;
            // a device-resident stream's element count is only known once its header is read
            // (fz_decompress checks it against the slot's workspace and dst_capacity then)
            const bool     dev_dec   = r.dir == FZ_DECOMPRESS && is_device(r);
            const uint64_t n         = r.dir == FZ_COMPRESS ? r.n
                                       : dev_dec            ? 0
                                                            : reinterpret_cast<const fz_header*>(r.src)->n;
            const bool     small_dst = r.dir == FZ_DECOMPRESS && 4 * n > r.dst_capacity;
            if (!request_bytes(r, &sb, &db) || n > S->max_n || small_dst || sb + db + 512 > S->budget) {
                S->done.push_back(fz_completion{r.id, n > S->max_n ? FZ_INVALID_ARG : FZ_OUT_OF_SPACE, 0});
                S->ndone.store((uint32_t)S->done.size(), std::memory_order_release);
                S->queue.erase(S->queue.begin() + k);  // can never run
                changed = true;
                continue;
            }
            if (!S->pool->alloc(sb, &so)) {  // it waits for memory to free up; a later one may fit
                ++k;
                continue;
            }
            if (!S->pool->alloc(db, &dof)) {
                S->pool->release(so, sb);
                ++k;
                continue;
            }
            sl.hdr = qf.h;
            if (qf.has_header) r.header = &sl.hdr;
            S->queue.erase(S->queue.begin() + k);
            ++S->running;
            break;
        }
    }
    issue(S, sl, r, so, sb, dof, db);
    return true;
}

void worker(fz_server* S, uint32_t first, uint32_t stride)
{
    cudaSetDevice(S->device);
    while (!S->stop.load(std::memory_order_relaxed)) {
        bool progress = false, busy = false;
        for (uint32_t i = first; i < S->slots.size(); i += stride) {
            Slot& sl = S->slots[i];
            if (sl.phase != Phase::Idle) progress |= retire(S, sl);
            if (sl.phase == Phase::Idle) progress |= admit(S, sl);
            busy |= sl.phase != Phase::Idle;
        }
        if (progress) continue;
        if (busy) {
            std::this_thread::yield();  // work in flight: look again soon
        } else {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv.wait_for(lk, std::chrono::milliseconds(1), [S] { return !S->queue.empty() || S->stop.load(); });
        }
    }
}

}  // namespace


extern "C" {

fz_status fz_server_create(uint64_t hbm_budget, uint32_t slots, uint64_t max_n, fz_server** out)
{
    if (!out || !hbm_budget || !slots || slots > 64 || !max_n) return FZ_INVALID_ARG;
    *out        = nullptr;
    fz_server* S = new (std::nothrow) fz_server();
    if (!S) return FZ_FAIL_GPU_MALLOC;
    S->budget = hbm_budget, S->max_n = max_n;
    if (cudaMalloc((void**)&S->d_pool, hbm_budget) != cudaSuccess) {
        delete S;
        return FZ_FAIL_GPU_OUT_OF_MEMORY;
    }
    S->pool = new Pool(hbm_budget);
    cudaGetDevice(&S->device);
    S->slots.resize(slots);
    for (Slot& sl : S->slots) {
        fz_status st = fz_workspace_create(max_n, &sl.ws);
        if (st == FZ_SUCCESS && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess)
            st = FZ_FAIL_GPU_ILLEGAL_ACCESS;
        if (st == FZ_SUCCESS && cudaMallocHost((void**)&sl.h_buf, 128) != cudaSuccess) st = FZ_FAIL_GPU_MALLOC;
        if (st == FZ_SUCCESS && cudaMalloc((void**)&sl.d_mirror, 128) != cudaSuccess) st = FZ_FAIL_GPU_MALLOC;
        if (st == FZ_SUCCESS && cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess)
            st = FZ_FAIL_GPU_ILLEGAL_ACCESS;
        if (st != FZ_SUCCESS) {
            fz_server_destroy(S);
            return st;
        }
    }
    const uint32_t nw = std::min(kWorkers, slots);
    for (uint32_t k = 0; k < nw; ++k) S->workers.emplace_back(worker, S, k, nw);
    *out = S;
    return FZ_SUCCESS;
}

fz_status fz_server_submit(fz_server* S, const fz_request* r)
{
    if (!S || !r || !r->src || !r->dst) return FZ_INVALID_ARG;
    if (r->dir != FZ_COMPRESS && r->dir != FZ_DECOMPRESS) return FZ_INVALID_ARG;
    if (r->dir == FZ_DECOMPRESS && r->src_bytes < FZ_HEADER_BYTES) return FZ_INVALID_ARG;
    Queued q{*r, {}, r->header != nullptr};
    if (q.has_header) q.h = *r->header;
    q.r.header = nullptr;  // re-pointed at the slot's copy when the request is issued
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->queue.push_back(q);
    }
    S->cv.notify_one();
    return FZ_SUCCESS;
}

fz_status fz_server_poll(fz_server* S, fz_completion* out, uint32_t max, uint32_t* count)
{
    if (!S || !count || (!out && max)) return FZ_INVALID_ARG;
    *count = 0;
    if (S->ndone.load(std::memory_order_acquire) == 0) return FZ_SUCCESS;  // nothing to hand out: no lock
    std::lock_guard<std::mutex> lk(S->mu);
    uint32_t                    k = 0;
    while (k < max && !S->done.empty()) {
        out[k++] = S->done.front();
        S->done.pop_front();
    }
    S->ndone.store((uint32_t)S->done.size(), std::memory_order_release);
    *count = k;
    return FZ_SUCCESS;
}

fz_status fz_server_pending(fz_server* S, uint32_t* queued, uint32_t* running, uint64_t* pool_used)
{
    if (!S) return FZ_INVALID_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    if (queued) *queued = (uint32_t)S->queue.size();
    if (running) *running = S->running;
    if (pool_used) *pool_used = S->pool->used();
    return FZ_SUCCESS;
}

fz_status fz_server_destroy(fz_server* S)
{
    if (!S) return FZ_INVALID_ARG;
    S->stop.store(true);
    S->cv.notify_all();
    for (std::thread& t : S->workers) t.join();
    for (Slot& sl : S->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.ws) fz_workspace_destroy(sl.ws);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.h_buf) cudaFreeHost(sl.h_buf);
        if (sl.d_mirror) cudaFree(sl.d_mirror);
        if (sl.ev) cudaEventDestroy(sl.ev);
    }
    cudaFree(S->d_pool);
    delete S->pool;
    delete S;
    return FZ_SUCCESS;
}

}  // extern "C"
