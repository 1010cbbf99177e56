// Request server: continuous batching of ray-query requests against
// device-resident DAGs (cbq_server_*).
//
//  - submit() queues a request (host rays in, host hits out) and returns a
//    ticket at once.
//  - A scheduler thread admits queued requests in FIFO order while the device
//    memory budget (a pool allocated once at creation) has room for their ray
//    and hit buffers and a launch slot is free.  Each admitted group becomes one
//    launch on the slot's stream: copies in, one persistent multi-volume
//    traversal (one job per request, each with its own query), copies out.
//    Groups are launched while earlier ones are still running, so requests that
//    arrive during a launch overlap it on the device.
//  - A completion thread waits for each launch's event, frees the requests'
//    memory and slot, records latency (submit -> results in host memory) and
//    wakes waiters.
// Nothing on the device waits on the host: every launch finishes on its own,
// and host waits are on CUDA events or condition variables.
#include "cbq_batch.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <exception>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

using namespace cbq;

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint64_t kAlign = 256;
constexpr size_t kInlineMaxInflight = 2;  // submit launches by itself below this many launches in flight
constexpr uint64_t kBytesPerRay = 16 + 16 + 12 + 12 + 12 + 4 + 4 + 1 + 1;  // rays in, all hit fields out

uint64_t align_up(uint64_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }

uint64_t request_bytes(uint64_t n) { return align_up(n * kBytesPerRay + 8 * kAlign); }

struct Request {
    uint64_t ticket = 0;
    cbq_request r{};
    uint64_t bytes = 0;      // pool bytes (0 for a direct request)
    uint64_t offset = 0;
    bool direct = false;     // served in place: the kernel reads and writes the caller's host buffers
    bool out_async = true;   // every hit buffer is page-locked (a copy into it does not block the host)
    const float* d_o = nullptr;
    const float* d_d = nullptr;
    cbq_hits d_hits{};
    Clock::time_point submitted;
    cbq_status status = CBQ_OK;
};

// The device address of host memory the GPU can use directly (page-locked and
// mapped, or managed), or nullptr when the buffer has to be staged.
const void* device_alias(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    if (a.type == cudaMemoryTypeManaged) return p;
    return nullptr;
}

// True when a device-to-host copy into `p` is asynchronous: page-locked or
// managed host memory (into pageable memory the copy blocks the calling thread).
bool copy_into_is_async(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type != cudaMemoryTypeUnregistered;
}

bool hits_copy_async(const cbq_hits& h)
{
    const void* fields[] = {h.hit, h.distance, h.material, h.position, h.normal, h.voxel, h.status};
    for (const void* f : fields)
        if (f && !copy_into_is_async(f)) return false;
    return true;
}

// Resolves every buffer of a request to a device alias; false if any needs staging.
bool resolve_direct(Request& rq)
{
    const cbq_request& r = rq.r;
    if (((uintptr_t)r.host_origin_tmax & 15u) || ((uintptr_t)r.host_direction & 15u)) return false;
    rq.d_o = (const float*)device_alias(r.host_origin_tmax);
    rq.d_d = (const float*)device_alias(r.host_direction);
    if (!rq.d_o || !rq.d_d) return false;
    const cbq_hits& h = r.host_hits;
    cbq_hits& d = rq.d_hits;
    struct F { void* host; void** dev; };
    const F fields[] = {{h.hit, (void**)&d.hit}, {h.distance, (void**)&d.distance}, {h.material, (void**)&d.material},
                        {h.position, (void**)&d.position}, {h.normal, (void**)&d.normal},
                        {h.voxel, (void**)&d.voxel}, {h.status, (void**)&d.status}};
    for (const F& f : fields) {
        *f.dev = nullptr;
        if (!f.host) continue;
        *f.dev = (void*)device_alias(f.host);
        if (!*f.dev) return false;
    }
    return true;
}

// First-fit allocator over [0, size).
class Pool {
public:
    void init(uint64_t size)
    {
        free_.clear();
        if (size) free_[0] = size;
    }
    bool alloc(uint64_t bytes, uint64_t* off)
    {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off = it->first;
            const uint64_t rest = it->second - bytes, start = it->first + bytes;
            free_.erase(it);
            if (rest) free_[start] = rest;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes)
    {
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }

private:
    std::map<uint64_t, uint64_t> free_;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    dev::JobDesc* h_table = nullptr;  // pinned
    dev::JobDesc* d_table = nullptr;
    uint64_t* d_counter = nullptr;
    std::vector<Request*> reqs;
};

double percentile(std::vector<double> v, double p)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double idx = p * (double)(v.size() - 1);
    const size_t lo = (size_t)idx;
    const size_t hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (v[hi] - v[lo]) * (idx - (double)lo);
}

}  // namespace

struct cbq_server {
    cbq_server_config cfg{};
    int device = 0;
    char* d_pool = nullptr;
    Pool pool;
    std::vector<Slot> slots;
    std::deque<int> free_slots;
    std::deque<int> inflight;
    std::deque<Request*> queue;
    std::map<uint64_t, cbq_status> finished;   // completed tickets not yet waited for
    std::map<uint64_t, int> live;              // tickets queued or in flight
    std::mutex mu;
    std::condition_variable cv_sched, cv_complete, cv_done;
    bool stopping = false;
    bool scheduler_done = false;
    int inline_pending = 0;   // launches being enqueued by submitting threads
    uint64_t next_ticket = 1;
    uint64_t completions = 0;  // generation count, bumped per finished launch
    std::thread scheduler, completer;
    // statistics
    std::vector<double> latencies_us;
    uint64_t submitted = 0, completed = 0, rays_completed = 0, launches = 0, launched_requests = 0;
    uint64_t direct_completed = 0;
    Clock::time_point first_submit, last_complete;
    bool have_first = false;

    void run_scheduler();
    void run_completer();
    cbq_status enqueue(Slot& s, const std::vector<Request*>& group);
    cbq_status copy_hits_back(const Request* rq, cudaStream_t stream) const;
    // Enqueues `group` on slot `si` (already taken) with `lk` released, then hands the
    // slot to the completion thread.  Called with `lk` held; returns with it held.
    void launch_group(int si, std::vector<Request*>& group, std::unique_lock<std::mutex>& lk);
};

void cbq_server::launch_group(int si, std::vector<Request*>& group, std::unique_lock<std::mutex>& lk)
{
    lk.unlock();
    int prev = device;
    cudaGetDevice(&prev);
    if (prev != device) cudaSetDevice(device);  // a submitting thread may have another device current
    const cbq_status st = enqueue(slots[si], group);
    if (st != CBQ_OK) {
        cudaGetLastError();
        for (Request* rq : group) rq->status = st;
        cudaEventRecord(slots[si].done, slots[si].stream);
    }
    if (prev != device) cudaSetDevice(prev);
    lk.lock();
    slots[si].reqs = group;
    inflight.push_back(si);
    launches++;
    launched_requests += group.size();
    cv_complete.notify_one();
}

cbq_status cbq_server::enqueue(Slot& s, const std::vector<Request*>& group)
{
    uint32_t njobs = 0;
    uint64_t total = 0;
    for (Request* rq : group) {
        const uint64_t n = rq->r.ray_count;
        if (rq->direct) {  // the kernel reads the rays and writes the hits in host memory itself
            dev::JobDesc jd;
            std::memset(&jd, 0, sizeof(jd));
            fill_job_volume(jd, rq->r.dag);
            jd.orig = (const float4*)rq->d_o;
            jd.dir = (const float4*)rq->d_d;
            const cbq_hits& dh = rq->d_hits;
            jd.out.hit = dh.hit;
            jd.out.distance = dh.distance;
            jd.out.material = dh.material;
            jd.out.position = dh.position;
            jd.out.normal = dh.normal;
            jd.out.voxel = dh.voxel;
            jd.out.status = dh.status;
            jd.count = n;
            jd.q.compute_surface = rq->r.query.compute_surface;
            jd.q.max_footprint = rq->r.query.max_footprint;
            jd.q.flags = rq->r.query.flags;
            if (!rq->r.dag->flat_ok) {
                cbq_rays rays{rq->d_o, rq->d_d};
                cbq_status st = cbq_intersect(rq->r.dag, &rays, n, &rq->r.query, &dh, (cbq_stream_t)s.stream);
                if (st != CBQ_OK) return st;
                continue;
            }
            jd.first = total;
            s.h_table[njobs++] = jd;
            total += n;
            continue;
        }
        char* p = d_pool + rq->offset;
        float* o = (float*)p;
        float* d = (float*)(p + n * 16);
        char* h = p + n * 32;
        dev::HitsOut out;
        out.position = (float*)h; h += align_up(n * 12);
        out.normal = (float*)h; h += align_up(n * 12);
        out.voxel = (int32_t*)h; h += align_up(n * 12);
        out.distance = (float*)h; h += align_up(n * 4);
        out.material = (uint32_t*)h; h += align_up(n * 4);
        out.hit = (uint8_t*)h; h += align_up(n);
        out.status = (uint8_t*)h;
        if (cudaMemcpyAsync(o, rq->r.host_origin_tmax, n * 16, cudaMemcpyHostToDevice, s.stream) != cudaSuccess ||
            cudaMemcpyAsync(d, rq->r.host_direction, n * 16, cudaMemcpyHostToDevice, s.stream) != cudaSuccess)
            return CBQ_ERR_CUDA;
        dev::JobDesc jd;
        std::memset(&jd, 0, sizeof(jd));
        fill_job_volume(jd, rq->r.dag);
        jd.orig = (const float4*)o;
        jd.dir = (const float4*)d;
        jd.out = out;
        jd.count = n;
        jd.q.compute_surface = rq->r.query.compute_surface;
        jd.q.max_footprint = rq->r.query.max_footprint;
        jd.q.flags = rq->r.query.flags;
        if (!rq->r.dag->flat_ok) {  // integer positions (far coordinates, huge stores): launched on its own
            cbq_rays rays{o, d};
            cbq_hits hits{out.hit, out.distance, out.material, out.position, out.normal, out.voxel, out.status};
            cbq_status st = cbq_intersect(rq->r.dag, &rays, n, &rq->r.query, &hits, (cbq_stream_t)s.stream);
            if (st != CBQ_OK) return st;
            continue;
        }
        jd.first = total;
        s.h_table[njobs++] = jd;
        total += n;
    }
    if (njobs) {
        if (cudaMemcpyAsync(s.d_table, s.h_table, njobs * sizeof(dev::JobDesc), cudaMemcpyHostToDevice, s.stream) !=
            cudaSuccess)
            return CBQ_ERR_CUDA;
        cbq_status st = launch_batch_kernel(s.d_table, njobs, total, s.d_counter, cfg.block, cfg.refill_min,
                                            kBatchStepsDefault, group[0]->r.dag->layout == CBQ_DAG_LAYOUT_COMPACT,
                                            device, s.stream);
        if (st != CBQ_OK) return st;
    }
    // Results back to page-locked host buffers; pageable ones are copied by the completion
    // thread once the launch is done, so that this thread never waits for the device.
    for (Request* rq : group) {
        if (rq->direct || !rq->out_async) continue;
        const cbq_status st = copy_hits_back(rq, s.stream);
        if (st != CBQ_OK) return st;
    }
    return cudaEventRecord(s.done, s.stream) == cudaSuccess ? CBQ_OK : CBQ_ERR_CUDA;
}

cbq_status cbq_server::copy_hits_back(const Request* rq, cudaStream_t stream) const
{
    const uint64_t n = rq->r.ray_count;
    char* h = d_pool + rq->offset + n * 32;
    const cbq_hits& hh = rq->r.host_hits;
    struct Copy { void* dst; size_t bytes; };
    const Copy copies[] = {{hh.position, n * 12}, {hh.normal, n * 12}, {hh.voxel, n * 12},
                           {hh.distance, n * 4}, {hh.material, n * 4}, {hh.hit, n}, {hh.status, n}};
    for (const Copy& c : copies) {
        if (c.dst && cudaMemcpyAsync(c.dst, h, c.bytes, cudaMemcpyDeviceToHost, stream) != cudaSuccess)
            return CBQ_ERR_CUDA;
        h += align_up(c.bytes);
    }
    return CBQ_OK;
}

void cbq_server::run_scheduler()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv_sched.wait(lk, [&] { return (!queue.empty() && !free_slots.empty()) || (stopping && queue.empty()); });
        if (queue.empty()) break;  // stopping, and nothing left to launch
        std::vector<Request*> group;
        uint64_t rays = 0;
        while (!queue.empty() && group.size() < (size_t)cfg.max_batch_requests) {
            Request* rq = queue.front();
            if (!group.empty() && rays + rq->r.ray_count > cfg.max_batch_rays) break;
            if (!group.empty() && rq->r.dag->layout != group[0]->r.dag->layout) break;  // one layout per launch
            uint64_t off = 0;
            if (rq->bytes && !pool.alloc(rq->bytes, &off)) break;  // FIFO: wait for memory rather than skip ahead
            rq->offset = off;
            group.push_back(rq);
            rays += rq->r.ray_count;
            queue.pop_front();
        }
        if (group.empty()) {
            const uint64_t gen = completions;
            cv_sched.wait(lk, [&] { return completions != gen; });
            continue;
        }
        const int si = free_slots.front();
        free_slots.pop_front();
        launch_group(si, group, lk);
    }
    scheduler_done = true;
    cv_complete.notify_all();
}

// Completes launches in whatever order they finish: a short launch that ends
// before a longer one issued earlier is not held behind it.  While launches
// are in flight this thread polls their events (and yields between rounds);
// with none in flight it sleeps on the condition variable.
void cbq_server::run_completer()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv_complete.wait(lk, [&] { return !inflight.empty() || (scheduler_done && inline_pending == 0); });
        if (inflight.empty()) break;  // scheduler finished and everything completed
        const std::vector<int> watch(inflight.begin(), inflight.end());
        lk.unlock();
        int si = -1;
        bool ok = true;
        for (unsigned spin = 0; si < 0; spin++) {
            for (int w : watch) {
                const cudaError_t e = cudaEventQuery(slots[w].done);
                if (e == cudaErrorNotReady) continue;
                si = w;
                ok = e == cudaSuccess;
                if (!ok) cudaGetLastError();
                break;
            }
            if (si >= 0) break;
            // Launches issued since `watch` was taken are picked up on the next round.
            if (spin % 64 == 63) {
                lk.lock();
                const bool grown = inflight.size() != watch.size();
                lk.unlock();
                if (grown) break;
            }
            std::this_thread::yield();
        }
        if (si < 0) {  // more launches in flight: watch them too
            lk.lock();
            continue;
        }
        if (ok) {  // hits for pageable buffers: copied now that the launch is done
            bool any = false;
            for (Request* rq : slots[si].reqs) {
                if (rq->direct || rq->out_async || rq->status != CBQ_OK) continue;
                any = true;
                if (copy_hits_back(rq, slots[si].stream) != CBQ_OK) rq->status = CBQ_ERR_CUDA;
            }
            if (any && cudaStreamSynchronize(slots[si].stream) != cudaSuccess) {
                cudaGetLastError();
                for (Request* rq : slots[si].reqs)
                    if (!rq->direct && !rq->out_async && rq->status == CBQ_OK) rq->status = CBQ_ERR_CUDA;
            }
        }
        const Clock::time_point now = Clock::now();
        lk.lock();
        inflight.erase(std::find(inflight.begin(), inflight.end(), si));
        for (Request* rq : slots[si].reqs) {
            if (!ok && rq->status == CBQ_OK) rq->status = CBQ_ERR_CUDA;
            latencies_us.push_back(std::chrono::duration<double, std::micro>(now - rq->submitted).count());
            if (rq->bytes) pool.release(rq->offset, rq->bytes);
            if (rq->direct) direct_completed++;
            finished[rq->ticket] = rq->status;
            live.erase(rq->ticket);
            completed++;
            rays_completed += rq->r.ray_count;
            delete rq;
        }
        slots[si].reqs.clear();
        free_slots.push_back(si);
        last_complete = now;
        completions++;
        cv_done.notify_all();
        cv_sched.notify_all();
    }
}

extern "C" {

cbq_status cbq_server_create(const cbq_server_config* cfg, cbq_server** out)
{
    if (!out) return CBQ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cbq_server* s = new (std::nothrow) cbq_server();
    if (!s) return CBQ_ERR_OUT_OF_MEMORY;
    cbq_server_config c{};
    if (cfg) c = *cfg;
    if (c.device_memory_budget == 0) c.device_memory_budget = 1ull << 30;
    if (c.max_inflight_launches <= 0) c.max_inflight_launches = 4;
    if (c.max_batch_requests <= 0) c.max_batch_requests = 256;
    if (c.max_batch_rays == 0) c.max_batch_rays = 4ull << 20;
    if (c.block <= 0) c.block = 128;
    if (c.refill_min == 0) c.refill_min = 8;
    if (c.block > 256 || (c.block % 32) || c.refill_min > 32 || c.max_inflight_launches > 64 ||
        c.max_batch_requests > 65536 || (c.flags & ~(uint32_t)CBQ_SERVER_IN_PLACE)) {
        delete s;
        return CBQ_ERR_INVALID_ARGUMENT;
    }
    s->cfg = c;
    if (cudaGetDevice(&s->device) != cudaSuccess) { delete s; return CBQ_ERR_CUDA; }
    if (cudaMalloc((void**)&s->d_pool, c.device_memory_budget) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    s->pool.init(c.device_memory_budget);
    s->slots.resize(c.max_inflight_launches);
    const size_t table = (size_t)c.max_batch_requests * sizeof(dev::JobDesc);
    bool ok = true;
    for (int i = 0; i < c.max_inflight_launches && ok; i++) {
        Slot& sl = s->slots[i];
        ok = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) == cudaSuccess &&
             cudaMallocHost((void**)&sl.h_table, table) == cudaSuccess &&
             cudaMalloc((void**)&sl.d_counter, 256 + table) == cudaSuccess;
        if (ok) sl.d_table = (dev::JobDesc*)((char*)sl.d_counter + 256);
        s->free_slots.push_back(i);
    }
    if (!ok) {
        cudaGetLastError();
        s->stopping = true;
        s->scheduler_done = true;
        cbq_server_destroy(s);
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    try {
        s->scheduler = std::thread([s] { s->run_scheduler(); });
        s->completer = std::thread([s] { s->run_completer(); });
    } catch (const std::exception&) {  // no thread: nothing may throw across the C ABI
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stopping = true;
        }
        cbq_server_destroy(s);
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    *out = s;
    return CBQ_OK;
}

cbq_status cbq_server_submit(cbq_server* s, const cbq_request* r, uint64_t* ticket)
{
    if (!s || !r || !ticket || !r->dag) return CBQ_ERR_INVALID_ARGUMENT;
    if (r->dag->device != s->device) return CBQ_ERR_INVALID_ARGUMENT;
    if (r->ray_count > 0 && (!r->host_origin_tmax || !r->host_direction)) return CBQ_ERR_INVALID_ARGUMENT;
    Request* rq = new (std::nothrow) Request();
    if (!rq) return CBQ_ERR_OUT_OF_MEMORY;
    rq->submitted = Clock::now();
    rq->r = *r;
    rq->direct = r->ray_count > 0 && (s->cfg.flags & CBQ_SERVER_IN_PLACE) && resolve_direct(*rq);
    rq->bytes = rq->direct ? 0 : request_bytes(r->ray_count);
    rq->out_async = rq->direct || hits_copy_async(r->host_hits);
    if (rq->bytes > s->cfg.device_memory_budget) {
        delete rq;
        return CBQ_ERR_CAPACITY;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stopping) { delete rq; return CBQ_ERR_SHUTDOWN; }
    rq->ticket = s->next_ticket++;
    *ticket = rq->ticket;
    s->submitted++;
    if (!s->have_first) { s->first_submit = rq->submitted; s->have_first = true; }
    if (r->ray_count == 0) {  // nothing to do
        s->finished[rq->ticket] = CBQ_OK;
        s->completed++;
        delete rq;
        s->cv_done.notify_all();
        return CBQ_OK;
    }
    s->live[rq->ticket] = 1;
    // A lightly loaded device (nothing queued, under two launches in flight), a slot and
    // memory free: launch from this thread, one thread hand-off fewer than through the
    // scheduler (arrival order is kept).  Under load, requests queue and leave in groups.
    uint64_t off = 0;
    if (s->queue.empty() && s->inflight.size() + s->inline_pending < kInlineMaxInflight &&
        !s->free_slots.empty() && (rq->bytes == 0 || s->pool.alloc(rq->bytes, &off))) {
        rq->offset = off;
        const int si = s->free_slots.front();
        s->free_slots.pop_front();
        s->inline_pending++;
        std::vector<Request*> group{rq};
        s->launch_group(si, group, lk);
        s->inline_pending--;
        s->cv_complete.notify_one();
        return CBQ_OK;
    }
    s->queue.push_back(rq);
    s->cv_sched.notify_one();
    return CBQ_OK;
}

cbq_status cbq_server_wait(cbq_server* s, uint64_t ticket, int64_t timeout_us)
{
    if (!s) return CBQ_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto ready = [&] { return s->finished.count(ticket) != 0 || s->live.count(ticket) == 0; };
    if (timeout_us < 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), ready)) {
        return CBQ_ERR_TIMEOUT;
    }
    auto it = s->finished.find(ticket);
    if (it == s->finished.end()) return CBQ_ERR_NOT_FOUND;
    const cbq_status st = it->second;
    s->finished.erase(it);
    return st;
}

cbq_status cbq_server_cancel(cbq_server* s, uint64_t ticket)
{
    if (!s) return CBQ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
        if ((*it)->ticket != ticket) continue;
        Request* rq = *it;
        s->queue.erase(it);
        s->live.erase(ticket);
        s->finished[ticket] = CBQ_ERR_CANCELLED;
        delete rq;
        s->cv_done.notify_all();
        return CBQ_OK;
    }
    if (s->live.count(ticket)) return CBQ_ERR_BUSY;  // already launched: it will complete
    return CBQ_ERR_NOT_FOUND;
}

cbq_status cbq_server_poll(cbq_server* s, uint64_t ticket, int32_t* done)
{
    if (!s || !done) return CBQ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->finished.count(ticket)) { *done = 1; return CBQ_OK; }
    if (s->live.count(ticket)) { *done = 0; return CBQ_OK; }
    return CBQ_ERR_NOT_FOUND;
}

cbq_status cbq_server_get_stats(cbq_server* s, cbq_server_stats* out)
{
    if (!s || !out) return CBQ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->rays_completed = s->rays_completed;
    out->launches = s->launches;
    out->mean_requests_per_launch = s->launches ? (double)s->launched_requests / (double)s->launches : 0.0;
    out->latency_p50_us = percentile(s->latencies_us, 0.50);
    out->latency_p99_us = percentile(s->latencies_us, 0.99);
    out->latency_max_us = s->latencies_us.empty() ? 0.0 : *std::max_element(s->latencies_us.begin(), s->latencies_us.end());
    double sum = 0;
    for (double v : s->latencies_us) sum += v;
    out->latency_mean_us = s->latencies_us.empty() ? 0.0 : sum / (double)s->latencies_us.size();
    out->direct_requests = s->direct_completed;
    out->queued = s->queue.size();
    out->inflight_launches = s->inflight.size();
    if (s->have_first && s->completed)
        out->busy_seconds = std::chrono::duration<double>(s->last_complete - s->first_submit).count();
    return CBQ_OK;
}

cbq_status cbq_server_reset_stats(cbq_server* s)
{
    if (!s) return CBQ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    s->latencies_us.clear();
    s->submitted = s->completed = s->rays_completed = s->launches = s->launched_requests = 0;
    s->direct_completed = 0;
    s->have_first = false;
    return CBQ_OK;
}

cbq_status cbq_server_destroy(cbq_server* s)
{
    if (!s) return CBQ_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_sched.notify_all();
    if (s->scheduler.joinable()) s->scheduler.join();  // drains the queue
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->scheduler_done = true;
    }
    s->cv_complete.notify_all();
    if (s->completer.joinable()) s->completer.join();  // waits for launches in flight
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.h_table) cudaFreeHost(sl.h_table);
        if (sl.d_counter) cudaFree(sl.d_counter);
    }
    if (s->d_pool) cudaFree(s->d_pool);
    for (Request* rq : s->queue) delete rq;
    delete s;
    return CBQ_OK;
}

cbq_status cbq_server_replay(cbq_server* s, const cbq_request* requests, const double* arrival_s, uint64_t count,
                             uint32_t max_outstanding, double* lateness_us, cbq_replay_result* result)
{
    if (!s || (count > 0 && (!requests || !arrival_s)) || max_outstanding == 0) return CBQ_ERR_INVALID_ARGUMENT;
    for (uint64_t k = 1; k < count; k++)
        if (!(arrival_s[k] >= arrival_s[k - 1])) return CBQ_ERR_INVALID_ARGUMENT;
    std::vector<uint64_t> tickets;
    std::vector<double> late, in_submit;
    try {
        tickets.assign(count, 0);
        late.assign(count, 0.0);
        in_submit.assign(count, 0.0);
    } catch (const std::exception&) {
        return CBQ_ERR_OUT_OF_MEMORY;
    }
    std::atomic<uint64_t> issued{0}, retired{0}, failed{0};
    std::atomic<bool> abort{false};
    // Waits for the requests in submission order; `retired` frees their buffers for reuse.
    std::thread waiter;
    auto wait_in_order = [&] {
        for (uint64_t k = 0; k < count; k++) {
            while (issued.load(std::memory_order_acquire) <= k) {
                if (abort.load(std::memory_order_acquire)) return;
                std::this_thread::yield();
            }
            if (cbq_server_wait(s, tickets[k], -1) != CBQ_OK) failed.fetch_add(1);
            retired.store(k + 1, std::memory_order_release);
        }
    };
    try {
        waiter = std::thread(wait_in_order);
    } catch (const std::exception&) {
        return CBQ_ERR_OUT_OF_MEMORY;  // nothing submitted yet
    }
    uint64_t backpressure = 0;
    cbq_status st = CBQ_OK;
    const Clock::time_point t0 = Clock::now();
    for (uint64_t k = 0; k < count; k++) {
        if (k >= max_outstanding && retired.load(std::memory_order_acquire) <= k - max_outstanding) {
            backpressure++;
            while (retired.load(std::memory_order_acquire) <= k - max_outstanding) std::this_thread::yield();
        }
        const Clock::time_point at =
            t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[k]));
        // Sleep while the arrival is far off, then spin for the last stretch.
        for (Clock::time_point now = Clock::now(); now < at; now = Clock::now()) {
            if (at - now > std::chrono::microseconds(300))
                std::this_thread::sleep_for(at - now - std::chrono::microseconds(200));
        }
        const Clock::time_point before = Clock::now();
        late[k] = std::chrono::duration<double, std::micro>(before - at).count();
        st = cbq_server_submit(s, &requests[k], &tickets[k]);
        in_submit[k] = std::chrono::duration<double, std::micro>(Clock::now() - before).count();
        if (st != CBQ_OK) break;
        issued.store(k + 1, std::memory_order_release);
    }
    if (st != CBQ_OK) abort.store(true, std::memory_order_release);
    waiter.join();
    const double wall = std::chrono::duration<double>(Clock::now() - t0).count();
    if (lateness_us)
        for (uint64_t k = 0; k < count; k++) lateness_us[k] = late[k];
    if (result) {
        std::memset(result, 0, sizeof(*result));
        result->wall_seconds = wall;
        result->submitted = issued.load();
        result->failed = failed.load();
        result->backpressure = backpressure;
        result->lateness_p50_us = percentile(late, 0.50);
        result->lateness_p99_us = percentile(late, 0.99);
        result->lateness_max_us = late.empty() ? 0.0 : *std::max_element(late.begin(), late.end());
        result->submit_p99_us = percentile(in_submit, 0.99);
        result->submit_max_us = in_submit.empty() ? 0.0 : *std::max_element(in_submit.begin(), in_submit.end());
    }
    return st;
}

}  // extern "C"
