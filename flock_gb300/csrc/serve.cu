// serve.cu -- the served form (flock_server_*): continuous batching on one
// GPU with admission by a device-memory budget.
//
// Requests are admitted in arrival order while the budgeted device arena has
// room for their resident state (costs, supplies/demands, the instance's
// working set, basis, duals and status).  Each admission group is uploaded on
// an upload stream and solved by one launch of the persistent batched kernel
// per size class, on an idle stream of a pool: a CTA takes one instance and
// runs it from the initial solution to the certificate with its tree in
// shared memory.  Launches overlap on the device, so a newly admitted
// request starts as soon as an SM has room, while earlier ones are still
// running.  A finished instance raises its own completion flag in
// host-mapped memory; a completer thread copies that instance's basis and
// status back, frees its region at once (backfilling the budget) and queues
// the result.  Instances above the largest staged size (m + n > 4096) run on
// the plain solver in a worker thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/flock.h"
#include "internal.h"

namespace flock {
void set_error(const std::string& s);
int validate_instance(const flock_instance* I);
ServeLayout serve_layout(int m, int n);
int serve_init();
int serve_launch(const BatchDesc* d_desc, int count, int maxV, int maxM, const flock_options& opt, int32_t* d_next,
                 cudaStream_t s);
void serve_collect(const Scalars& S, int V, const int32_t* out3, flock_flow* flows, flock_stats* st);
}  // namespace flock

namespace {

constexpr int kServeMaxV = 4096;     // largest m + n solved by the group kernels
constexpr int kSlots = 1 << 16;      // completion flags (requests in flight)
constexpr int kDescCap = 1 << 17;    // descriptor pool entries
// launch streams: enough that a new group nearly always finds an idle one
// (a group queued behind a long-running launch on a busy stream waits for it)
constexpr int kStreams = 64;
constexpr int kUrgentV = 512;        // size classes launched on the high-priority streams

using Clock = std::chrono::steady_clock;

// First-fit range allocator with coalescing.
class RangeAlloc {
    std::map<uint64_t, uint64_t> free_;   // offset -> size
 public:
    void reset(uint64_t cap) { free_.clear(); if (cap) free_[0] = cap; }
    bool alloc(uint64_t size, uint64_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < size) continue;
            *off = it->first;
            const uint64_t rest = it->second - size, noff = it->first + size;
            free_.erase(it);
            if (rest) free_[noff] = rest;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t size) {
        if (!size) return;
        auto it = free_.emplace(off, size).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
        }
    }
};

// Resident bytes of a request solved by the plain solver (its own buffers).
int64_t plain_bytes(int m, int n) {
    const int64_t ldc = (n + 3) & ~3;
    return 4 * (int64_t)m * ldc + 256 * (int64_t)(m + n) + 4096;
}

}  // namespace

struct flock_server {
    struct Req {
        uint64_t ticket = 0;
        int32_t m = 0, n = 0;
        std::vector<int32_t> s, d, c;
        Clock::time_point t_submit;
        int64_t bytes = 0;          // budget charge
        uint64_t off = 0;           // arena region (group kernels)
        int slot = -1;              // completion flag
        int group = -1;
        bool plain = false;
    };
    struct Done {
        flock_result res;
        std::vector<flock_flow> flows;
    };
    struct Group {
        uint64_t desc_off = 0;
        int count = 0, remaining = 0;
        cudaEvent_t ev = nullptr;
        bool live = false;
    };

    flock_server_config cfg;
    std::mutex mu;
    std::condition_variable cv;        // dispatcher, plain worker
    std::condition_variable cv_done;   // drain
    std::deque<std::unique_ptr<Req>> pending;
    std::deque<std::unique_ptr<Req>> plain_queue;
    std::vector<std::unique_ptr<Req>> inflight;
    std::deque<Done> done;
    int64_t resident = 0;
    uint64_t next_ticket = 1;
    int64_t submitted = 0, finished = 0;
    bool stop = false;
    std::thread dispatcher, completer, plain_worker;

    // device state (created by the dispatcher on first use)
    bool dev_ready = false;
    int dev_error = FLOCK_OK;
    uint8_t* arena = nullptr;
    uint64_t arena_cap = 0;
    RangeAlloc arena_alloc;
    flock::BatchDesc* d_desc = nullptr;
    int32_t* d_next = nullptr;
    RangeAlloc desc_alloc;
    int32_t* h_flags = nullptr;
    int32_t* d_flags = nullptr;
    std::vector<int> free_slots;
    std::vector<Group> groups;
    std::vector<int> free_groups;
    cudaStream_t up = nullptr, down = nullptr;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> stream_last;
    int rr = 0, rr_hi = 0;

    static int64_t request_bytes(int m, int n) {
        if (m + n > kServeMaxV) return plain_bytes(m, n);
        return (int64_t)flock::serve_layout(m, n).total;
    }

    int init_device() {
        cudaError_t e;
        size_t fr = 0, tot = 0;
        if ((e = cudaMemGetInfo(&fr, &tot)) != cudaSuccess) return fail(e, "cudaMemGetInfo");
        arena_cap = (uint64_t)std::min<int64_t>(cfg.memory_budget_bytes, (int64_t)(fr / 10 * 9));
        arena_cap &= ~uint64_t(255);
        if (arena_cap < 256) arena_cap = 256;
        if ((e = cudaMalloc(&arena, arena_cap)) != cudaSuccess) return fail(e, "arena");
        arena_alloc.reset(arena_cap);
        if ((e = cudaMalloc(&d_desc, sizeof(flock::BatchDesc) * kDescCap)) != cudaSuccess) return fail(e, "descriptors");
        if ((e = cudaMalloc(&d_next, sizeof(int32_t) * kDescCap)) != cudaSuccess) return fail(e, "counters");
        desc_alloc.reset(kDescCap);
        if ((e = cudaHostAlloc(&h_flags, sizeof(int32_t) * kSlots, cudaHostAllocMapped)) != cudaSuccess)
            return fail(e, "completion flags");
        memset(h_flags, 0, sizeof(int32_t) * kSlots);
        if ((e = cudaHostGetDevicePointer((void**)&d_flags, h_flags, 0)) != cudaSuccess) return fail(e, "flag mapping");
        free_slots.resize(kSlots);
        for (int k = 0; k < kSlots; k++) free_slots[k] = kSlots - 1 - k;
        if ((e = cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
        if ((e = cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
        const int ns = std::max(kStreams, cfg.max_inflight_batches);
        streams.resize(ns);
        stream_last.assign(ns, nullptr);
        // the first half of the pool at the highest priority, for the size
        // classes up to kUrgentV: their blocks are scheduled ahead of the
        // larger classes' waiting blocks, so short requests do not queue
        // behind long ones
        int lo_pri = 0, hi_pri = 0;
        if ((e = cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri)) != cudaSuccess) return fail(e, "stream priorities");
        for (int k = 0; k < ns; k++)
            if ((e = cudaStreamCreateWithPriority(&streams[k], cudaStreamNonBlocking, k < ns / 2 ? hi_pri : lo_pri)) !=
                cudaSuccess)
                return fail(e, "stream");
        const int rc = flock::serve_init();
        if (rc) return rc;
        dev_ready = true;
        return FLOCK_OK;
    }

    int fail(cudaError_t e, const char* what) {
        flock::set_error(std::string("served form: ") + what + ": " + cudaGetErrorString(e));
        return FLOCK_ERR_CUDA;
    }

    // An idle stream of the pool half for the launch's priority (urgent: the
    // first half) whose last launch finished, else the half's next one.
    int pick_stream(bool urgent) {
        const int half = (int)streams.size() / 2;
        const int base = urgent ? 0 : half, cnt = urgent ? half : (int)streams.size() - half;
        int& r = urgent ? rr_hi : rr;
        for (int k = 0; k < cnt; k++) {
            const int s = base + (r + k) % cnt;
            if (!stream_last[s] || cudaEventQuery(stream_last[s]) == cudaSuccess) { r = s - base + 1; return s; }
        }
        const int s = base + r % cnt;
        r = s - base + 1;
        return s;
    }

    // Deliver a result (lock held).
    void deliver(Req& r, Done&& d) {
        d.res.ticket = r.ticket;
        d.res.latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - r.t_submit).count();
        d.res.stats.ms_total = d.res.latency_ms;
        done.push_back(std::move(d));
        resident -= r.bytes;
        finished++;
        cv.notify_all();
        cv_done.notify_all();
    }

    void fail_requests(std::vector<std::unique_ptr<Req>>& rs, int rc) {
        std::lock_guard<std::mutex> lk(mu);
        for (auto& r : rs) {
            Done d;
            memset(&d.res, 0, sizeof(d.res));
            d.res.status = rc;
            if (r->slot >= 0) free_slots.push_back(r->slot);
            if (!r->plain && r->bytes && dev_ready) arena_alloc.release(r->off, (uint64_t)r->bytes);
            deliver(*r, std::move(d));
        }
        rs.clear();
    }

    // Upload one size class of an admission group and launch it.
    int launch_group(std::vector<Req*>& g) {
        int maxV = 0, maxM = 0;
        for (Req* r : g) { maxV = std::max(maxV, r->m + r->n); maxM = std::max(maxM, r->m); }
        uint64_t doff = 0;
        int gid = -1;
        {
            std::lock_guard<std::mutex> lk(mu);
            if (!desc_alloc.alloc(g.size(), &doff)) { flock::set_error("served form: descriptor pool full"); return FLOCK_ERR_CAPACITY; }
            if (free_groups.empty()) { groups.emplace_back(); gid = (int)groups.size() - 1; }
            else { gid = free_groups.back(); free_groups.pop_back(); }
        }
        Group& G = groups[gid];
        cudaError_t e;
        if (!G.ev && (e = cudaEventCreateWithFlags(&G.ev, cudaEventDisableTiming)) != cudaSuccess) return fail(e, "event");
        std::vector<flock::BatchDesc> hd(g.size());
        for (size_t k = 0; k < g.size(); k++) {
            Req& r = *g[k];
            const flock::ServeLayout L = flock::serve_layout(r.m, r.n);
            uint8_t* base = arena + r.off;
            flock::BatchDesc& d = hd[k];
            d.m = r.m; d.n = r.n; d.ldc = (r.n + 3) & ~3; d.index = (int)k;
            d.cost = (const int32_t*)(base + L.cost);
            d.sd = (const int32_t*)(base + L.sd);
            d.ws = base + L.ws;
            d.out = (int32_t*)(base + L.out);
            d.bfs = (int32_t*)(base + L.bfs);
            d.pot = (int64_t*)(base + L.pot);
            d.sc = (flock::Scalars*)(base + L.sc);
            d.done = d_flags + r.slot;
            ((volatile int32_t*)h_flags)[r.slot] = 0;
            r.group = gid;
            if ((e = cudaMemcpy2DAsync(base + L.cost, (size_t)d.ldc * 4, r.c.data(), (size_t)r.n * 4, (size_t)r.n * 4, r.m,
                                       cudaMemcpyHostToDevice, up)) != cudaSuccess) return fail(e, "cost upload");
            if ((e = cudaMemcpyAsync(base + L.sd, r.s.data(), (size_t)r.m * 4, cudaMemcpyHostToDevice, up)) != cudaSuccess)
                return fail(e, "supply upload");
            if ((e = cudaMemcpyAsync(base + L.sd + (size_t)r.m * 4, r.d.data(), (size_t)r.n * 4, cudaMemcpyHostToDevice,
                                     up)) != cudaSuccess) return fail(e, "demand upload");
        }
        if ((e = cudaMemcpyAsync(d_desc + doff, hd.data(), hd.size() * sizeof(flock::BatchDesc), cudaMemcpyHostToDevice,
                                 up)) != cudaSuccess) return fail(e, "descriptor upload");
        if ((e = cudaMemsetAsync(d_next + doff, 0, sizeof(int32_t), up)) != cudaSuccess) return fail(e, "counter reset");
        if ((e = cudaEventRecord(G.ev, up)) != cudaSuccess) return fail(e, "event");
        const int s = pick_stream(maxV <= kUrgentV);
        if ((e = cudaStreamWaitEvent(streams[s], G.ev, 0)) != cudaSuccess) return fail(e, "stream wait");
        const int rc = flock::serve_launch(d_desc + doff, (int)g.size(), maxV, maxM, cfg.options, d_next + doff, streams[s]);
        if (rc) return rc;
        if ((e = cudaEventRecord(G.ev, streams[s])) != cudaSuccess) return fail(e, "event");
        stream_last[s] = G.ev;
        std::lock_guard<std::mutex> lk(mu);
        G.desc_off = doff;
        G.count = G.remaining = (int)g.size();
        G.live = true;
        return FLOCK_OK;
    }

    void dispatch_loop() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return stop || !pending.empty(); });
            if (stop && pending.empty()) return;
            if (!dev_ready && !dev_error) {
                lk.unlock();
                const int rc = init_device();
                lk.lock();
                if (rc) dev_error = rc;
            }
            // admit in arrival order while the budget and the arena have room
            std::vector<std::unique_ptr<Req>> take;
            while (!pending.empty() && (int)take.size() < cfg.max_batch) {
                Req& r = *pending.front();
                if (dev_error && !r.plain) { take.push_back(std::move(pending.front())); pending.pop_front(); continue; }
                if (resident + r.bytes > cfg.memory_budget_bytes) break;
                if (r.plain) {
                    resident += r.bytes;
                    plain_queue.push_back(std::move(pending.front()));
                    pending.pop_front();
                    cv.notify_all();
                    continue;
                }
                if (free_slots.empty() || !arena_alloc.alloc((uint64_t)r.bytes, &r.off)) break;
                r.slot = free_slots.back();
                free_slots.pop_back();
                resident += r.bytes;
                take.push_back(std::move(pending.front()));
                pending.pop_front();
            }
            if (take.empty()) {
                // nothing fits: wait for a retirement (or new arrivals)
                cv.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
            if (dev_error) { const int rc = dev_error; lk.unlock(); fail_requests(take, rc); lk.lock(); continue; }
            lk.unlock();
            // size classes: a launch's shared memory and block size follow its largest instance
            std::sort(take.begin(), take.end(), [](const std::unique_ptr<Req>& a, const std::unique_ptr<Req>& b) {
                return a->m + a->n < b->m + b->n;
            });
            static const int edges[] = {128, 512, 1024, 2048, 2944, kServeMaxV};
            size_t i0 = 0;
            int rc = FLOCK_OK;
            for (int e = 0; e < 6 && i0 < take.size() && !rc; e++) {
                std::vector<Req*> g;
                size_t i1 = i0;
                while (i1 < take.size() && take[i1]->m + take[i1]->n <= edges[e]) g.push_back(take[i1++].get());
                if (!g.empty()) rc = launch_group(g);
                i0 = i1;
            }
            lk.lock();
            if (rc) {
                lk.unlock();
                fail_requests(take, rc);
                lk.lock();
                continue;
            }
            for (auto& r : take) inflight.push_back(std::move(r));
        }
    }

    void complete_loop() {
        std::vector<std::unique_ptr<Req>> fin;
        std::vector<std::vector<int32_t>> outs;
        std::vector<flock::Scalars> scs;
        for (;;) {
            {
                std::lock_guard<std::mutex> lk(mu);
                if (stop && inflight.empty()) return;
                for (size_t k = 0; k < inflight.size();) {
                    if (((volatile int32_t*)h_flags)[inflight[k]->slot]) {
                        fin.push_back(std::move(inflight[k]));
                        inflight[k] = std::move(inflight.back());
                        inflight.pop_back();
                    } else {
                        k++;
                    }
                }
                // groups whose launch has finished give back descriptors and counters
                for (size_t gi = 0; gi < groups.size(); gi++) {
                    Group& G = groups[gi];
                    if (G.live && G.remaining == 0 && cudaEventQuery(G.ev) == cudaSuccess) {
                        desc_alloc.release(G.desc_off, (uint64_t)G.count);
                        G.live = false;
                        free_groups.push_back((int)gi);
                    }
                }
            }
            if (fin.empty()) {
                std::this_thread::sleep_for(std::chrono::microseconds(50));
                continue;
            }
            outs.resize(fin.size());
            scs.resize(fin.size());
            int rc = FLOCK_OK;
            for (size_t k = 0; k < fin.size() && !rc; k++) {
                Req& r = *fin[k];
                const flock::ServeLayout L = flock::serve_layout(r.m, r.n);
                const int V = r.m + r.n;
                outs[k].resize((size_t)3 * (V - 1));
                if (V > 1 && cudaMemcpyAsync(outs[k].data(), arena + r.off + L.out, outs[k].size() * 4,
                                             cudaMemcpyDeviceToHost, down) != cudaSuccess) rc = FLOCK_ERR_CUDA;
                if (cudaMemcpyAsync(&scs[k], arena + r.off + L.sc, sizeof(flock::Scalars), cudaMemcpyDeviceToHost,
                                    down) != cudaSuccess) rc = FLOCK_ERR_CUDA;
            }
            if (!rc && cudaStreamSynchronize(down) != cudaSuccess) rc = FLOCK_ERR_CUDA;
            std::lock_guard<std::mutex> lk(mu);
            for (size_t k = 0; k < fin.size(); k++) {
                Req& r = *fin[k];
                Done d;
                memset(&d.res, 0, sizeof(d.res));
                if (rc) {
                    d.res.status = rc;
                } else {
                    d.flows.assign((size_t)r.m + r.n - 1, flock_flow{0, 0, 0});
                    flock::serve_collect(scs[k], r.m + r.n, outs[k].data(), d.flows.data(), &d.res.stats);
                    d.res.status = d.res.stats.status ? FLOCK_ERR_NOT_OPTIMAL : FLOCK_OK;
                }
                arena_alloc.release(r.off, (uint64_t)r.bytes);
                free_slots.push_back(r.slot);
                if (r.group >= 0) groups[r.group].remaining--;
                deliver(r, std::move(d));
            }
            fin.clear();
        }
    }

    void plain_loop() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return stop || !plain_queue.empty(); });
            if (plain_queue.empty()) { if (stop) return; continue; }
            std::unique_ptr<Req> r = std::move(plain_queue.front());
            plain_queue.pop_front();
            lk.unlock();
            flock_instance inst{r->m, r->n, r->s.data(), r->d.data(), r->c.data()};
            Done d;
            memset(&d.res, 0, sizeof(d.res));
            d.flows.assign((size_t)r->m + r->n - 1, flock_flow{0, 0, 0});
            const int rc = flock_solve(&inst, &cfg.options, d.flows.data(), nullptr, nullptr, &d.res.stats);
            d.res.status = rc;
            lk.lock();
            deliver(*r, std::move(d));
        }
    }

    void release_device() {
        for (auto& st : streams) if (st) cudaStreamDestroy(st);
        if (up) cudaStreamDestroy(up);
        if (down) cudaStreamDestroy(down);
        for (auto& G : groups) if (G.ev) cudaEventDestroy(G.ev);
        if (h_flags) cudaFreeHost(h_flags);
        if (d_next) cudaFree(d_next);
        if (d_desc) cudaFree(d_desc);
        if (arena) cudaFree(arena);
    }
};

extern "C" {

void flock_default_server_config(flock_server_config* cfg) {
    if (!cfg) return;
    cfg->memory_budget_bytes = (int64_t)40 << 30;
    cfg->max_inflight_batches = 16;
    cfg->max_batch = 512;
    flock_default_options(&cfg->options);
}

int64_t flock_server_request_bytes(int32_t m, int32_t n) {
    if (m < 1 || n < 1) return -1;
    return flock_server::request_bytes(m, n);
}

int flock_server_create(const flock_server_config* cfg, flock_server** out) {
    if (!out) return FLOCK_ERR_ARG;
    if (cfg && cfg->options.bfs_method == FLOCK_BFS_VOGEL_DEVICE) return FLOCK_ERR_ARG;   // plain solve only
    if (cfg && cfg->options.pivot_method == FLOCK_PIVOT_SS) return FLOCK_ERR_ARG;       // plain solve only
    flock_server* s = new flock_server();
    if (cfg) s->cfg = *cfg; else flock_default_server_config(&s->cfg);
    if (s->cfg.max_inflight_batches < 1) s->cfg.max_inflight_batches = 1;
    if (s->cfg.max_batch < 1) s->cfg.max_batch = 1;
    s->dispatcher = std::thread([s] { s->dispatch_loop(); });
    s->completer = std::thread([s] { s->complete_loop(); });
    s->plain_worker = std::thread([s] { s->plain_loop(); });
    *out = s;
    return FLOCK_OK;
}

int flock_server_submit(flock_server* s, const flock_instance* inst, uint64_t* ticket) {
    if (!s) return FLOCK_ERR_ARG;
    int rc = flock::validate_instance(inst);
    if (rc) return rc;
    auto r = std::make_unique<flock_server::Req>();
    r->m = inst->m; r->n = inst->n;
    r->plain = inst->m + inst->n > kServeMaxV;
    r->bytes = flock_server::request_bytes(inst->m, inst->n);
    if (r->bytes > s->cfg.memory_budget_bytes) { flock::set_error("request exceeds the memory budget"); return FLOCK_ERR_BUDGET; }
    r->s.assign(inst->supply, inst->supply + inst->m);
    r->d.assign(inst->demand, inst->demand + inst->n);
    r->c.assign(inst->cost, inst->cost + (size_t)inst->m * inst->n);
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    if (ticket) *ticket = r->ticket;
    s->pending.push_back(std::move(r));
    s->submitted++;
    s->cv.notify_all();
    return FLOCK_OK;
}

int flock_server_poll(flock_server* s, flock_result* results, flock_flow** flows_out, int32_t max, int32_t* count) {
    if (!s || !count || (max > 0 && !results)) return FLOCK_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    int k = 0;
    while (k < max && !s->done.empty()) {
        flock_server::Done& d = s->done.front();
        results[k] = d.res;
        if (flows_out && flows_out[k] && !d.flows.empty())
            memcpy(flows_out[k], d.flows.data(), d.flows.size() * sizeof(flock_flow));
        s->done.pop_front();
        k++;
    }
    *count = k;
    return FLOCK_OK;
}

int flock_server_drain(flock_server* s) {
    if (!s) return FLOCK_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [s] { return s->finished >= s->submitted; });
    return FLOCK_OK;
}

int flock_server_destroy(flock_server* s) {
    if (!s) return FLOCK_ERR_ARG;
    flock_server_drain(s);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->dispatcher.joinable()) s->dispatcher.join();
    if (s->completer.joinable()) s->completer.join();
    if (s->plain_worker.joinable()) s->plain_worker.join();
    if (s->dev_ready) {
        for (auto& st : s->streams) cudaStreamSynchronize(st);
        cudaStreamSynchronize(s->up);
        cudaStreamSynchronize(s->down);
        s->release_device();
    }
    delete s;
    return FLOCK_OK;
}

}  // extern "C"
