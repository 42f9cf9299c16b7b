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

// Reads the file (its first `limit` bytes when limit > 0).
int load(const char* path, Tok& t, long limit = 0) {
    if (!path) return FLOCK_ERR_ARG;
    FILE* f = fopen(path, "rb");
    if (!f) { flock::set_error(std::string("input file not found: ") + path); return FLOCK_ERR_FILE; }
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (limit > 0 && sz > limit) sz = limit;
    t.buf.resize(sz > 0 ? (size_t)sz : 0);
    size_t got = sz > 0 ? fread(t.buf.data(), 1, (size_t)sz, f) : 0;
    fclose(f);
    if ((long)got != sz) { flock::set_error("short read"); return FLOCK_ERR_FILE; }
    return FLOCK_OK;
}

inline bool is_space(char ch) { return ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r'; }

// The cost section in parallel.  The bytes from `from` on are cut into
// chunks at whitespace; each chunk's tokens are counted, a prefix sum gives
// each chunk its first token index, and every chunk parses its tokens into
// place.  Only the first `count` tokens are used (as the sequential reader,
// which stops after them); fewer is a parse error.  visit(k, s, len) handles
// token k and returns 0 or an error code; the error of the lowest token index
// wins, so the result equals a sequential left-to-right pass.
template <class F>
int parallel_tokens(const std::vector<char>& buf, size_t from, int64_t count, const F& visit) {
    const size_t end = buf.size();
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const size_t bytes = end > from ? end - from : 0;
    int T = (int)std::min<size_t>(std::min(hw, 64), std::max<size_t>(1, bytes / (1 << 20)));
    std::vector<size_t> cut(T + 1);
    cut[0] = from;
    cut[T] = end;
    for (int t = 1; t < T; t++) {
        size_t p = from + bytes * t / T;
        while (p < end && !is_space(buf[p])) p++;     // a chunk starts at whitespace
        cut[t] = std::max(p, cut[t - 1]);
    }
    std::vector<int64_t> cnt(T, 0);
    auto count_tokens = [&](int t) {
        int64_t c = 0;
        bool in = false;
        for (size_t p = cut[t]; p < cut[t + 1]; p++) {
            const bool sp = is_space(buf[p]);
            if (!sp && !in) c++;
            in = !sp;
        }
        cnt[t] = c;
    };
    std::vector<std::thread> th;
    for (int t = 1; t < T; t++) th.emplace_back(count_tokens, t);
    count_tokens(0);
    for (auto& x : th) x.join();
    th.clear();
    std::vector<int64_t> first(T + 1, 0);
    for (int t = 0; t < T; t++) first[t + 1] = first[t] + cnt[t];
    std::vector<int64_t> err_at(T, INT64_MAX);
    std::vector<int> err_rc(T, 0);
    auto parse_chunk = [&](int t) {
        int64_t k = first[t];
        size_t p = cut[t];
        while (p < cut[t + 1] && k < count) {
            while (p < cut[t + 1] && is_space(buf[p])) p++;
            if (p >= cut[t + 1]) break;
            const size_t b = p;
            while (p < cut[t + 1] && !is_space(buf[p])) p++;
            const int rc = visit(k, buf.data() + b, p - b);
            if (rc) { err_at[t] = k; err_rc[t] = rc; return; }
            k++;
        }
    };
    for (int t = 1; t < T; t++) th.emplace_back(parse_chunk, t);
    parse_chunk(0);
    for (auto& x : th) x.join();
    int64_t best = INT64_MAX;
    int rc = 0;
    for (int t = 0; t < T; t++) if (err_at[t] < best) { best = err_at[t]; rc = err_rc[t]; }
    if (!rc && first[T] < count) rc = FLOCK_ERR_PARSE;      // the file ends early
    return rc;
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
    int rc = load(path, t, 4096);
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
    std::atomic<int> best{0};
    rc = parallel_tokens(t.buf, t.p, a * b, [&](int64_t, const char* s2, size_t l2) {
        bool inexact = false; int fd = 0; int64_t v;
        if (!parse_scaled(s2, l2, 0, &v, &inexact, &fd)) return (int)FLOCK_ERR_PARSE;
        int cur = best.load(std::memory_order_relaxed);
        while (fd > cur && !best.compare_exchange_weak(cur, fd, std::memory_order_relaxed)) {}
        return 0;
    });
    if (rc) return rc;
    if (scale) *scale = best.load();
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
    rc = parallel_tokens(t.buf, t.p, mn, [&](int64_t k, const char* s2, size_t l2) {
        bool inexact = false;
        int64_t v;
        if (!parse_scaled(s2, l2, scale, &v, &inexact, nullptr)) return (int)FLOCK_ERR_PARSE;
        if (inexact) return (int)FLOCK_ERR_INEXACT;
        if (v > (1 << 30) || v < -(1 << 30)) return (int)FLOCK_ERR_RANGE;
        cost[k] = (int32_t)v;
        return 0;
    });
    if (rc == FLOCK_ERR_PARSE) flock::set_error("bad or missing cost token");
    if (rc == FLOCK_ERR_INEXACT) flock::set_error("cost not integral at this decimal scale");
    if (rc == FLOCK_ERR_RANGE) flock::set_error("cost out of range");
    return rc;
}

// ========================================================== binary file ===
// "FLKBIN01", int32 m, int32 n, then m supplies, n demands and m*n costs,
// int32 little-endian, costs row-major.
namespace {
const char kBinMagic[8] = {'F', 'L', 'K', 'B', 'I', 'N', '0', '1'};

bool little_endian() {
    const uint32_t one = 1;
    unsigned char b;
    memcpy(&b, &one, 1);
    return b == 1;
}

int bin_open(const char* path, FILE** f, int32_t* m, int32_t* n) {
    if (!path) return FLOCK_ERR_ARG;
    if (!little_endian()) { flock::set_error("binary instance files need a little-endian host"); return FLOCK_ERR_ARG; }
    *f = fopen(path, "rb");
    if (!*f) { flock::set_error(std::string("input file not found: ") + path); return FLOCK_ERR_FILE; }
    char magic[8];
    int32_t hdr[2];
    if (fread(magic, 1, 8, *f) != 8 || memcmp(magic, kBinMagic, 8) != 0 || fread(hdr, 4, 2, *f) != 2 ||
        hdr[0] < 1 || hdr[1] < 1 || hdr[0] > (1 << 28) || hdr[1] > (1 << 28)) {
        fclose(*f);
        flock::set_error("not a flock binary instance file");
        return FLOCK_ERR_PARSE;
    }
    fseek(*f, 0, SEEK_END);
    const int64_t want = 16 + 4 * ((int64_t)hdr[0] + hdr[1] + (int64_t)hdr[0] * hdr[1]);
    if ((int64_t)ftell(*f) != want) {
        fclose(*f);
        flock::set_error("binary instance file has the wrong size");
        return FLOCK_ERR_PARSE;
    }
    fseek(*f, 16, SEEK_SET);
    *m = hdr[0];
    *n = hdr[1];
    return FLOCK_OK;
}
}  // namespace

extern "C" {

// The reference's .dat layout, as in its data/ files: "m n", the supplies
// and then the demands on one line each with a tab after every value, then
// one cost per line.  A cost is written as cost / 10^decimal_scale in decimal
// with trailing zeros trimmed (at least one fractional digit when the scale
// is positive); reading the file back with the same scale gives the same
// integers.
int flock_write_dat(const char* path, const flock_instance* inst, int32_t decimal_scale) {
    if (!path || !inst || !inst->supply || !inst->demand || !inst->cost || inst->m < 1 || inst->n < 1 ||
        decimal_scale < 0 || decimal_scale > 9)
        return FLOCK_ERR_ARG;
    FILE* f = fopen(path, "wb");
    if (!f) { flock::set_error(std::string("cannot write: ") + path); return FLOCK_ERR_FILE; }
    int64_t p10 = 1;
    for (int k = 0; k < decimal_scale; k++) p10 *= 10;
    std::string buf;
    buf.reserve(1 << 20);
    bool ok = true;
    auto flush = [&] {
        if (!buf.empty() && fwrite(buf.data(), 1, buf.size(), f) != buf.size()) ok = false;
        buf.clear();
    };
    auto put_uint = [&](uint64_t u) {
        char t[24];
        int k = 0;
        do { t[k++] = (char)('0' + u % 10); u /= 10; } while (u);
        while (k) buf += t[--k];
    };
    auto put_int = [&](int64_t v) {
        if (v < 0) buf += '-';
        put_uint(v < 0 ? (uint64_t)(-v) : (uint64_t)v);
    };
    put_int(inst->m); buf += ' '; put_int(inst->n); buf += '\n';
    for (int i = 0; i < inst->m; i++) { put_int(inst->supply[i]); buf += '\t'; }
    buf += '\n';
    for (int j = 0; j < inst->n; j++) { put_int(inst->demand[j]); buf += '\t'; }
    buf += '\n';
    const size_t mn = (size_t)inst->m * inst->n;
    for (size_t x = 0; x < mn && ok; x++) {
        const int64_t v = inst->cost[x];
        const uint64_t u = v < 0 ? (uint64_t)(-v) : (uint64_t)v;
        if (v < 0) buf += '-';
        put_uint(u / (uint64_t)p10);
        if (decimal_scale > 0) {
            uint64_t frac = u % (uint64_t)p10;
            int digits = decimal_scale;
            while (digits > 1 && frac % 10 == 0) { frac /= 10; digits--; }
            buf += '.';
            char t[12];
            for (int k = digits - 1; k >= 0; k--) { t[k] = (char)('0' + frac % 10); frac /= 10; }
            buf.append(t, (size_t)digits);
        }
        buf += '\n';
        if (buf.size() > (1u << 20)) flush();
    }
    flush();
    if (fclose(f) != 0 || !ok) { flock::set_error(std::string("short write: ") + path); return FLOCK_ERR_FILE; }
    return FLOCK_OK;
}

int flock_write_bin(const char* path, const flock_instance* inst) {
    if (!path || !inst || !inst->supply || !inst->demand || !inst->cost || inst->m < 1 || inst->n < 1) return FLOCK_ERR_ARG;
    if (!little_endian()) { flock::set_error("binary instance files need a little-endian host"); return FLOCK_ERR_ARG; }
    FILE* f = fopen(path, "wb");
    if (!f) { flock::set_error(std::string("cannot write: ") + path); return FLOCK_ERR_FILE; }
    const int32_t hdr[2] = {inst->m, inst->n};
    const size_t mn = (size_t)inst->m * inst->n;
    const bool ok = fwrite(kBinMagic, 1, 8, f) == 8 && fwrite(hdr, 4, 2, f) == 2 &&
                    fwrite(inst->supply, 4, (size_t)inst->m, f) == (size_t)inst->m &&
                    fwrite(inst->demand, 4, (size_t)inst->n, f) == (size_t)inst->n && fwrite(inst->cost, 4, mn, f) == mn;
    if (fclose(f) != 0 || !ok) { flock::set_error(std::string("short write: ") + path); return FLOCK_ERR_FILE; }
    return FLOCK_OK;
}

int flock_bin_shape(const char* path, int32_t* m, int32_t* n) {
    FILE* f = nullptr;
    int32_t a = 0, b = 0;
    const int rc = bin_open(path, &f, &a, &b);
    if (rc) return rc;
    fclose(f);
    if (m) *m = a;
    if (n) *n = b;
    return FLOCK_OK;
}

int flock_read_bin(const char* path, int32_t m, int32_t n, int32_t* supply, int32_t* demand, int32_t* cost) {
    if (!supply || !demand || !cost) return FLOCK_ERR_ARG;
    FILE* f = nullptr;
    int32_t a = 0, b = 0;
    int rc = bin_open(path, &f, &a, &b);
    if (rc) return rc;
    if (a != m || b != n) { fclose(f); flock::set_error("shape mismatch"); return FLOCK_ERR_ARG; }
    const size_t mn = (size_t)m * n;
    const bool ok = fread(supply, 4, (size_t)m, f) == (size_t)m && fread(demand, 4, (size_t)n, f) == (size_t)n &&
                    fread(cost, 4, mn, f) == mn;
    fclose(f);
    if (!ok) { flock::set_error("short read"); return FLOCK_ERR_FILE; }
    return FLOCK_OK;
}

}  // extern "C"

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
