// host.cpp -- host-side parts of the C ABI: the .dat reader, the instance
// generators and the serving loop (continuous batching with admission by a
// device-memory budget).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/flock.h"

namespace flock {
void set_error(const std::string& s);
struct BatchRunner;
BatchRunner* batch_runner_new();
void batch_runner_free(BatchRunner* r);
int batch_runner_prepare(BatchRunner* r, int cnt, const flock_instance* insts, const flock_options* o);
int batch_runner_solve(BatchRunner* r);
void batch_runner_collect(BatchRunner* r, int k, flock_flow* flows, flock_stats* st);
}  // namespace flock

// ================================================================ reader ===
// Whitespace tokenizer over the whole file (src/instance.cpp:80-141 reads
// with operator>> the same way: m, n, m supplies, n demands, m*n costs).
namespace {

struct Tok {
    std::vector<char> buf;
    size_t p = 0;
    bool next(const char** s, size_t* len) {
        while (p < buf.size() && (buf[p] == ' ' || buf[p] == '\t' || buf[p] == '\n' || buf[p] == '\r')) p++;
        if (p >= buf.size()) return false;
        const size_t b = p;
        while (p < buf.size() && !(buf[p] == ' ' || buf[p] == '\t' || buf[p] == '\n' || buf[p] == '\r')) p++;
        *s = buf.data() + b;
        *len = p - b;
        return true;
    }
};

int load(const char* path, Tok& t) {
    if (!path) return FLOCK_ERR_ARG;
    FILE* f = fopen(path, "rb");
    if (!f) { flock::set_error(std::string("input file not found: ") + path); return FLOCK_ERR_FILE; }
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    t.buf.resize(sz > 0 ? (size_t)sz : 0);
    size_t got = sz > 0 ? fread(t.buf.data(), 1, (size_t)sz, f) : 0;
    fclose(f);
    if ((long)got != sz) { flock::set_error("short read"); return FLOCK_ERR_FILE; }
    return FLOCK_OK;
}

// integer token (supplies, demands, sizes)
bool parse_int(const char* s, size_t len, int64_t* out) {
    size_t i = 0;
    bool neg = false;
    if (i < len && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; i++; }
    if (i >= len) return false;
    int64_t v = 0;
    for (; i < len; i++) {
        if (s[i] < '0' || s[i] > '9') return false;
        v = v * 10 + (s[i] - '0');
        if (v > ((int64_t)1 << 40)) return false;
    }
    *out = neg ? -v : v;
    return true;
}

// decimal token -> exact integer value * 10^scale; returns false on bad text,
// sets *inexact when nonzero digits beyond `scale` exist.
bool parse_scaled(const char* s, size_t len, int scale, int64_t* out, bool* inexact, int* frac_digits) {
    size_t i = 0;
    bool neg = false;
    if (i < len && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; i++; }
    int64_t ip = 0;
    int nd = 0;
    for (; i < len && s[i] >= '0' && s[i] <= '9'; i++) { ip = ip * 10 + (s[i] - '0'); nd++; if (ip > ((int64_t)1 << 40)) return false; }
    int64_t fp = 0;
    int fd = 0, sig = 0;
    if (i < len && s[i] == '.') {
        i++;
        for (; i < len && s[i] >= '0' && s[i] <= '9'; i++) {
            fd++;
            if (s[i] != '0') sig = fd;
            if (fd <= scale) fp = fp * 10 + (s[i] - '0');
            else if (s[i] != '0') *inexact = true;
            nd++;
        }
    }
    if (i != len || nd == 0) return false;
    for (int k = std::min(fd, scale); k < scale; k++) fp *= 10;
    int64_t p10 = 1;
    for (int k = 0; k < scale; k++) p10 *= 10;
    int64_t v = ip * p10 + fp;
    *out = neg ? -v : v;
    if (frac_digits) *frac_digits = sig;
    return true;
}

}  // namespace

extern "C" {

int flock_dat_shape(const char* path, int32_t* m, int32_t* n) {
    Tok t;
    int rc = load(path, t);
    if (rc) return rc;
    const char* s; size_t l; int64_t a, b;
    if (!t.next(&s, &l) || !parse_int(s, l, &a)) return FLOCK_ERR_PARSE;
    if (!t.next(&s, &l) || !parse_int(s, l, &b)) return FLOCK_ERR_PARSE;
    if (a < 1 || b < 1 || a > (1 << 28) || b > (1 << 28)) return FLOCK_ERR_PARSE;
    if (m) *m = (int32_t)a;
    if (n) *n = (int32_t)b;
    return FLOCK_OK;
}

int flock_dat_scale(const char* path, int32_t* scale) {
    Tok t;
    int rc = load(path, t);
    if (rc) return rc;
    const char* s; size_t l; int64_t a, b, x;
    if (!t.next(&s, &l) || !parse_int(s, l, &a)) return FLOCK_ERR_PARSE;
    if (!t.next(&s, &l) || !parse_int(s, l, &b)) return FLOCK_ERR_PARSE;
    for (int64_t k = 0; k < a + b; k++) if (!t.next(&s, &l) || !parse_int(s, l, &x)) return FLOCK_ERR_PARSE;
    int best = 0;
    for (int64_t k = 0; k < a * b; k++) {
        bool inexact = false; int fd = 0; int64_t v;
        if (!t.next(&s, &l) || !parse_scaled(s, l, 0, &v, &inexact, &fd)) return FLOCK_ERR_PARSE;
        best = std::max(best, fd);
    }
    if (scale) *scale = best;
    return FLOCK_OK;
}

int flock_read_dat(const char* path, int32_t scale, int32_t m, int32_t n,
                   int32_t* supply, int32_t* demand, int32_t* cost) {
    if (!supply || !demand || !cost || scale < 0 || scale > 9) return FLOCK_ERR_ARG;
    Tok t;
    int rc = load(path, t);
    if (rc) return rc;
    const char* s; size_t l; int64_t a, b, x;
    if (!t.next(&s, &l) || !parse_int(s, l, &a)) return FLOCK_ERR_PARSE;
    if (!t.next(&s, &l) || !parse_int(s, l, &b)) return FLOCK_ERR_PARSE;
    if (a != m || b != n) { flock::set_error("shape mismatch"); return FLOCK_ERR_ARG; }
    for (int i = 0; i < m; i++) {
        if (!t.next(&s, &l) || !parse_int(s, l, &x) || x < INT32_MIN || x > INT32_MAX) return FLOCK_ERR_PARSE;
        supply[i] = (int32_t)x;
    }
    for (int j = 0; j < n; j++) {
        if (!t.next(&s, &l) || !parse_int(s, l, &x) || x < INT32_MIN || x > INT32_MAX) return FLOCK_ERR_PARSE;
        demand[j] = (int32_t)x;
    }
    const int64_t mn = (int64_t)m * n;
    for (int64_t k = 0; k < mn; k++) {
        bool inexact = false;
        if (!t.next(&s, &l) || !parse_scaled(s, l, scale, &x, &inexact, nullptr)) { flock::set_error("bad cost token"); return FLOCK_ERR_PARSE; }
        if (inexact) { flock::set_error("cost not integral at this decimal scale"); return FLOCK_ERR_INEXACT; }
        if (x > (1 << 30) || x < -(1 << 30)) { flock::set_error("cost out of range"); return FLOCK_ERR_RANGE; }
        cost[k] = (int32_t)x;
    }
    return FLOCK_OK;
}

// ============================================================= generator ===
// splitmix64 stream + Lemire's bounded integers: the same integers on every
// platform for a given seed.
namespace {
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    uint32_t bounded(uint32_t range) {   // uniform in [0, range)
        uint32_t x = (uint32_t)(next() >> 32);
        uint64_t mm = (uint64_t)x * range;
        uint32_t l = (uint32_t)mm;
        if (l < range) {
            const uint32_t t = (uint32_t)(-range) % range;
            while (l < t) { x = (uint32_t)(next() >> 32); mm = (uint64_t)x * range; l = (uint32_t)mm; }
        }
        return (uint32_t)(mm >> 32);
    }
    int32_t uniform(int32_t lo, int32_t hi) { return lo + (int32_t)bounded((uint32_t)(hi - lo + 1)); }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};
}  // namespace

int flock_generate(int32_t kind, uint64_t seed, int32_t m, int32_t n,
                   int32_t c_lo, int32_t c_hi, int32_t q_lo, int32_t q_hi,
                   int32_t* supply, int32_t* demand, int32_t* cost) {
    if (m < 1 || n < 1 || !supply || !demand || !cost || q_lo < 0 || q_hi < q_lo) return FLOCK_ERR_ARG;
    Rng r{seed};
    if (kind == 0) {
        if (c_hi < c_lo) return FLOCK_ERR_ARG;
        for (int64_t k = 0; k < (int64_t)m * n; k++) cost[k] = r.uniform(c_lo, c_hi);
    } else if (kind == 1) {
        std::vector<double> px(m), py(m), qx(n), qy(n);
        for (int i = 0; i < m; i++) { px[i] = 1000.0 * r.unit(); py[i] = 1000.0 * r.unit(); }
        for (int j = 0; j < n; j++) { qx[j] = 1000.0 * r.unit(); qy[j] = 1000.0 * r.unit(); }
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++) {
                const double dx = px[i] - qx[j], dy = py[i] - qy[j];
                const double sq = dx * dx;
                const double s2 = sq + dy * dy;   // separate statements: no contraction
                cost[(size_t)i * n + j] = (int32_t)std::round(std::sqrt(s2));
            }
    } else {
        return FLOCK_ERR_ARG;
    }
    int64_t S = 0, R = 0;
    for (int i = 0; i < m; i++) { supply[i] = r.uniform(q_lo, q_hi); S += supply[i]; }
    std::vector<int64_t> raw(n);
    for (int j = 0; j < n; j++) { raw[j] = r.uniform(q_lo, q_hi); R += raw[j]; }
    int64_t D = 0;
    for (int j = 0; j < n; j++) {
        const int64_t dj = R > 0 ? (raw[j] * S) / R : (j == n - 1 ? S : 0);
        demand[j] = (int32_t)dj;
        D += dj;
    }
    demand[n - 1] += (int32_t)(S - D);
    return FLOCK_OK;
}

int flock_generate_sizes(uint64_t seed, int32_t count, int32_t lo, int32_t hi, int32_t* ms, int32_t* ns) {
    if (count < 0 || lo < 1 || hi < lo || !ms || !ns) return FLOCK_ERR_ARG;
    Rng r{seed};
    const double a = std::log((double)lo), b = std::log((double)hi);
    for (int k = 0; k < count; k++) {
        const double um = a + (b - a) * r.unit();
        const double un = a + (b - a) * r.unit();
        ms[k] = (int32_t)std::min<double>(hi, std::max<double>(lo, std::round(std::exp(um))));
        ns[k] = (int32_t)std::min<double>(hi, std::max<double>(lo, std::round(std::exp(un))));
    }
    return FLOCK_OK;
}

}  // extern "C"

// ================================================================ server ===
// Requests are copied at submit.  A dispatcher thread admits waiting requests
// (FIFO) into free launch slots while the summed resident estimate stays
// within the budget.  Each slot has its own thread, batch runner and CUDA
// streams, so a slot solving one group of requests overlaps on the device
// with the other slots; requests arriving meanwhile are admitted into the
// next slot that frees up.
struct flock_server {
    struct Req {
        uint64_t ticket;
        int32_t m, n;
        std::vector<int32_t> s, d, c;
        int64_t bytes;
        std::chrono::steady_clock::time_point t_submit;
    };
    struct Done {
        flock_result res;
        std::vector<flock_flow> flows;
    };
    struct Slot {
        flock::BatchRunner* runner = nullptr;
        std::vector<Req> reqs;
        bool busy = false;      // assigned requests, running or about to run
        std::thread th;
    };
    flock_server_config cfg;
    std::mutex mu;
    std::condition_variable cv;        // dispatcher and slot threads wait here
    std::condition_variable cv_done;   // drain waits here
    std::deque<Req> pending;
    std::deque<Done> done;
    std::vector<Slot> slots;
    int64_t resident = 0;
    uint64_t next_ticket = 1;
    int64_t submitted = 0, finished = 0;
    bool stop = false;
    std::thread dispatcher;

    static int64_t estimate(int m, int n) {
        const int64_t ldc = (n + 3) & ~3;
        return 4 * (int64_t)m * ldc + 256 * (int64_t)(m + n) + 4096;
    }

    void slot_loop(int id) {
        Slot& sl = slots[id];
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return stop || (sl.busy && !sl.reqs.empty()); });
            if (!(sl.busy && !sl.reqs.empty())) { if (stop) return; continue; }
            std::vector<Req> reqs = std::move(sl.reqs);
            sl.reqs.clear();
            lk.unlock();
            std::vector<flock_instance> insts(reqs.size());
            for (size_t k = 0; k < reqs.size(); k++)
                insts[k] = {reqs[k].m, reqs[k].n, reqs[k].s.data(), reqs[k].d.data(), reqs[k].c.data()};
            int rc = flock::batch_runner_prepare(sl.runner, (int)insts.size(), insts.data(), &cfg.options);
            if (!rc) rc = flock::batch_runner_solve(sl.runner);
            const auto now = std::chrono::steady_clock::now();
            std::vector<Done> out(reqs.size());
            for (size_t k = 0; k < reqs.size(); k++) {
                Done& d = out[k];
                memset(&d.res, 0, sizeof(d.res));
                d.res.ticket = reqs[k].ticket;
                if (rc) {
                    d.res.status = rc;
                } else {
                    d.flows.assign((size_t)reqs[k].m + reqs[k].n - 1, flock_flow{0, 0, 0});
                    flock::batch_runner_collect(sl.runner, (int)k, d.flows.data(), &d.res.stats);
                    d.res.status = d.res.stats.status ? FLOCK_ERR_NOT_OPTIMAL : FLOCK_OK;
                }
                d.res.latency_ms = std::chrono::duration<double, std::milli>(now - reqs[k].t_submit).count();
                d.res.stats.ms_total = d.res.latency_ms;
            }
            lk.lock();
            for (auto& r : reqs) resident -= r.bytes;
            for (auto& d : out) done.push_back(std::move(d));
            finished += (int64_t)reqs.size();
            sl.busy = false;
            cv.notify_all();
            cv_done.notify_all();
        }
    }

    void dispatch_loop() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] {
                if (stop) return true;
                if (pending.empty()) return false;
                for (auto& sl : slots) if (!sl.busy) return true;
                return false;
            });
            if (stop) return;
            for (auto& sl : slots) {
                if (sl.busy || pending.empty()) continue;
                std::vector<Req> take;
                while (!pending.empty() && (int)take.size() < cfg.max_batch &&
                       resident + pending.front().bytes <= cfg.memory_budget_bytes) {
                    resident += pending.front().bytes;
                    take.push_back(std::move(pending.front()));
                    pending.pop_front();
                }
                if (take.empty()) break;    // the budget is full: wait for a slot to retire
                sl.reqs = std::move(take);
                sl.busy = true;
            }
            cv.notify_all();
            // nothing admitted (budget full): wait for a retirement
            cv.wait_for(lk, std::chrono::milliseconds(1));
        }
    }
};

extern "C" {

void flock_default_server_config(flock_server_config* cfg) {
    if (!cfg) return;
    cfg->memory_budget_bytes = (int64_t)40 << 30;
    cfg->max_inflight_batches = 4;
    cfg->max_batch = 512;
    flock_default_options(&cfg->options);
}

int flock_server_create(const flock_server_config* cfg, flock_server** out) {
    if (!out) return FLOCK_ERR_ARG;
    flock_server* s = new flock_server();
    if (cfg) s->cfg = *cfg; else flock_default_server_config(&s->cfg);
    if (s->cfg.max_inflight_batches < 1) s->cfg.max_inflight_batches = 1;
    if (s->cfg.max_batch < 1) s->cfg.max_batch = 1;
    s->slots.resize(s->cfg.max_inflight_batches);
    for (size_t k = 0; k < s->slots.size(); k++) {
        s->slots[k].runner = flock::batch_runner_new();
        s->slots[k].th = std::thread([s, k] { s->slot_loop((int)k); });
    }
    s->dispatcher = std::thread([s] { s->dispatch_loop(); });
    *out = s;
    return FLOCK_OK;
}

int flock_server_submit(flock_server* s, const flock_instance* inst, uint64_t* ticket) {
    if (!s || !inst || !inst->supply || !inst->demand || !inst->cost || inst->m < 1 || inst->n < 1) return FLOCK_ERR_ARG;
    flock_server::Req r;
    r.m = inst->m; r.n = inst->n;
    r.s.assign(inst->supply, inst->supply + inst->m);
    r.d.assign(inst->demand, inst->demand + inst->n);
    r.c.assign(inst->cost, inst->cost + (size_t)inst->m * inst->n);
    r.bytes = flock_server::estimate(inst->m, inst->n);
    if (r.bytes > s->cfg.memory_budget_bytes) { flock::set_error("request exceeds the memory budget"); return FLOCK_ERR_BUDGET; }
    r.t_submit = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    r.ticket = s->next_ticket++;
    if (ticket) *ticket = r.ticket;
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
    for (auto& sl : s->slots) if (sl.th.joinable()) sl.th.join();
    for (auto& sl : s->slots) flock::batch_runner_free(sl.runner);
    delete s;
    return FLOCK_OK;
}

}  // extern "C"
