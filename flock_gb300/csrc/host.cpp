// host.cpp -- host-side parts of the C ABI: the .dat reader and the instance
// generators.
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
