// bsg_io.cpp -- the reference's file formats, parsed and written in parallel.
//
// Input (blackscholes.c:695-739): a count read with "%i", then per option
// "%f %f %f %f %f %f %c %f %f" = s strike r divq v t OptionType divs DGrefval.
// Output (blackscholes.c:923-947): "%i\n" then "%.18f\n" per price.
//
// The parser converts every float to the value glibc's scanf "%f" (strtof,
// round to nearest) gives, so arrays are bit-identical to the reference's:
// plain decimals of up to 19 significant digits take an exact fast path
// (below), everything else goes to strtof.  It splits the text at line
// starts and parses the chunks on nthreads threads;
// when a chunk does not hold whole 9-field records (a record spread over
// lines) it falls back to one sequential pass.  The writer formats "%.18f"
// exactly with integer arithmetic (round half to even, as glibc's printf
// does in the default rounding mode), in parallel, and falls back to
// snprintf for non-finite values and |x| >= 2^40.
#include "bsg.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

inline bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f';
}

struct Cursor {
    const char* p;
    const char* end;
};

inline void skip_ws(Cursor& c) {
    while (c.p < c.end && is_space(*c.p)) ++c.p;
}

// Exact decimal -> float fast path (Clinger's method).  For a token
// [+-]digits[.digits][(e|E)[+-]digits] with at most 19 significant digits,
// the value is m x 10^e10 with m an integer:
//  * m <= 2^24 and |e10| <= 10: m and 10^|e10| are exact floats, so one
//    correctly rounded float multiply or divide gives the correctly rounded
//    result;
//  * m <= 2^53 and |e10| <= 22: the same in double gives the correctly
//    rounded double d; rounding d to float is then correct unless d lies
//    exactly halfway between two floats (the decimal value may not), or d
//    is outside the normal float range: those go to strtof.
// Returns false (nothing consumed) when the token needs strtof.
const float kPow10f[11] = {1e0f, 1e1f, 1e2f, 1e3f, 1e4f, 1e5f, 1e6f, 1e7f, 1e8f, 1e9f, 1e10f};
const double kPow10d[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                            1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

inline bool is_digit(char ch) { return ch >= '0' && ch <= '9'; }

inline bool fast_float(const char* p, const char* end, float* out, const char** stop) {
    const char* q = p;
    bool neg = false;
    if (q < end && (*q == '+' || *q == '-')) neg = (*q++ == '-');
    uint64_t m = 0;
    int sig = 0, e10 = 0;
    bool any = false;
    while (q < end && is_digit(*q)) {
        any = true;
        if (m == 0 && *q == '0') { ++q; continue; }  // leading zeros
        if (++sig > 19) return false;
        m = m * 10 + (uint64_t)(*q++ - '0');
    }
    if (q < end && *q == '.') {
        ++q;
        while (q < end && is_digit(*q)) {
            any = true;
            --e10;
            if (m == 0 && *q == '0') { ++q; continue; }
            if (++sig > 19) return false;
            m = m * 10 + (uint64_t)(*q++ - '0');
        }
    }
    if (!any) return false;  // no digits (inf, nan, ".", hex, ...): strtof decides
    if (q < end && (*q == 'x' || *q == 'X')) return false;  // "0x..." hexadecimal
    if (q < end && (*q == 'e' || *q == 'E')) {
        const char* r = q + 1;
        bool eneg = false;
        if (r < end && (*r == '+' || *r == '-')) eneg = (*r++ == '-');
        if (r < end && is_digit(*r)) {  // else the 'e' is not part of the number
            int ex = 0;
            while (r < end && is_digit(*r)) {
                if (ex > 10000) return false;
                ex = ex * 10 + (*r++ - '0');
            }
            e10 += eneg ? -ex : ex;
            q = r;
        }
    }
    float v;
    if (m == 0) {
        v = 0.0f;
    } else if (m <= (1ull << 24) && e10 >= -10 && e10 <= 10) {
        v = (float)m;
        v = e10 >= 0 ? v * kPow10f[e10] : v / kPow10f[-e10];
    } else if (m <= (1ull << 53) && e10 >= -22 && e10 <= 22) {
        double d = (double)m;
        d = e10 >= 0 ? d * kPow10d[e10] : d / kPow10d[-e10];
        if (!(d >= (double)FLT_MIN && d <= (double)FLT_MAX)) return false;
        v = (float)d;
        if ((double)v != d) {  // inexact: a tie in double may not be one in decimal
            const float w = std::nextafter(v, (double)v < d ? FLT_MAX : 0.0f);
            if (d == ((double)v + (double)w) * 0.5) return false;
        }
    } else {
        return false;
    }
    *out = neg ? -v : v;
    *stop = q;
    return true;
}

// One "%f": the fast path, else strtof on the next token (the buffer is
// NUL-terminated).
inline bool read_float(Cursor& c, float* out) {
    skip_ws(c);
    if (c.p >= c.end) return false;
    const char* stop = nullptr;
    if (fast_float(c.p, c.end, out, &stop)) {
        c.p = stop;
        return true;
    }
    char* e = nullptr;
    const float v = std::strtof(c.p, &e);
    if (e == c.p) return false;
    *out = v;
    c.p = e;
    return true;
}

// " %c": the next non-space character.
inline bool read_char(Cursor& c, char* out) {
    skip_ws(c);
    if (c.p >= c.end) return false;
    *out = *c.p++;
    return true;
}

struct Rec {
    float s, k, r, v, t, dg;
    int32_t ot;
};

// Parses whole records from [p, end); returns false on a malformed record.
bool parse_records(const char* p, const char* end, std::vector<Rec>* out, bool stop_at_end) {
    Cursor c{p, end};
    for (;;) {
        skip_ws(c);
        if (c.p >= c.end) return true;
        Rec r;
        float divq, divs;
        char type;
        if (!read_float(c, &r.s) || !read_float(c, &r.k) || !read_float(c, &r.r) ||
            !read_float(c, &divq) || !read_float(c, &r.v) || !read_float(c, &r.t) ||
            !read_char(c, &type) || !read_float(c, &divs) || !read_float(c, &r.dg))
            return false;
        if (stop_at_end && c.p > c.end) return false;
        r.ot = (type == 'P') ? 1 : 0;  // blackscholes.c:760
        out->push_back(r);
    }
}

void free_book(bsg_book* b) {
    if (b && b->mem_) std::free(b->mem_);
    if (b) std::memset(b, 0, sizeof(*b));
}

bool alloc_book(bsg_book* b, size_t n) {
    std::memset(b, 0, sizeof(*b));
    const size_t al = (n + 63) / 64 * 64;
    void* m = nullptr;
    if (posix_memalign(&m, 256, 7 * al * sizeof(float) + 256) != 0) return false;
    float* f = static_cast<float*>(m);
    b->n = n;
    b->sptprice = f;
    b->strike = f + al;
    b->rate = f + 2 * al;
    b->volatility = f + 3 * al;
    b->otime = f + 4 * al;
    b->otype = reinterpret_cast<int32_t*>(f + 5 * al);
    b->dgrefval = f + 6 * al;
    b->mem_ = m;
    return true;
}

void store(bsg_book* b, size_t i, const Rec& r) {
    b->sptprice[i] = r.s;
    b->strike[i] = r.k;
    b->rate[i] = r.r;
    b->volatility[i] = r.v;
    b->otime[i] = r.t;
    b->otype[i] = r.ot;
    b->dgrefval[i] = r.dg;
}

// ---------------------------------------------------------------- "%.18f"
const uint64_t kPow10_18 = 1000000000000000000ull;

// Writes "%.18f" of x into buf (at least 64 bytes); returns the length.
int format_f18(float x, char* buf) {
    if (!std::isfinite(x) || std::fabs(x) >= 1099511627776.0f)  // 2^40
        return std::snprintf(buf, 64, "%.18f", (double)x);
    uint32_t bits;
    std::memcpy(&bits, &x, 4);
    const bool neg = bits >> 31;
    const uint32_t ex = (bits >> 23) & 0xff;
    uint32_t man = bits & 0x7fffff;
    int e;  // |x| = man * 2^e
    if (ex == 0) {
        e = -149;
    } else {
        man |= 0x800000;
        e = (int)ex - 150;
    }
    unsigned __int128 N;
    if (e >= 0) {
        N = (unsigned __int128)man << e;
        N *= kPow10_18;
    } else {
        const int s = -e;  // 1 .. 149
        const unsigned __int128 P = (unsigned __int128)man * kPow10_18;  // < 2^84
        if (s >= 100) {
            N = 0;  // P / 2^s < 2^-16 < 1/2
        } else {
            const unsigned __int128 q = P >> s;
            const unsigned __int128 r = P - (q << s);
            const unsigned __int128 half = (unsigned __int128)1 << (s - 1);
            N = q + ((r > half || (r == half && (q & 1))) ? 1 : 0);
        }
    }
    const uint64_t ip = (uint64_t)(N / kPow10_18);
    const uint64_t fp = (uint64_t)(N % kPow10_18);
    char* p = buf;
    if (neg) *p++ = '-';
    char tmp[24];
    int t = 0;
    uint64_t v = ip;
    do {
        tmp[t++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (t) *p++ = tmp[--t];
    *p++ = '.';
    v = fp;
    for (int i = 17; i >= 0; --i) {
        p[i] = (char)('0' + v % 10);
        v /= 10;
    }
    p += 18;
    return (int)(p - buf);
}

int clamp_threads(int nthreads, size_t work, size_t per_thread_min) {
    int hw = (int)std::thread::hardware_concurrency();
    if (hw < 1) hw = 1;
    int t = nthreads > 0 ? nthreads : hw;
    const size_t by_work = work / per_thread_min + 1;
    if ((size_t)t > by_work) t = (int)by_work;
    return t < 1 ? 1 : t;
}

}  // namespace

extern "C" {

int bsg_parse_parsec(const char* text, size_t len, int nthreads, bsg_book* out) {
    if (!text || !out) return BSG_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    // the buffer must end in a NUL for strtof; copy if it does not
    std::string own;
    if (len == 0 || text[len] != '\0') {
        own.assign(text, len);
        text = own.c_str();
    }
    const char* end = text + len;
    // count: "%i" (base prefixes as strtol with base 0)
    Cursor c{text, end};
    skip_ws(c);
    char* e = nullptr;
    errno = 0;
    const long long cnt = std::strtoll(c.p, &e, 0);
    if (e == c.p || errno || cnt < 0) return BSG_ERR_INVALID_ARG;
    const size_t n = (size_t)cnt;
    const char* body = e;
    if (!alloc_book(out, n)) return BSG_ERR_OUT_OF_MEMORY;
    if (n == 0) return BSG_OK;

    const int T = clamp_threads(nthreads, (size_t)(end - body), 1 << 20);
    std::vector<std::vector<Rec>> parts(T);
    std::vector<int> ok(T, 1);
    // chunk boundaries at line starts
    std::vector<const char*> cut(T + 1);
    cut[0] = body;
    cut[T] = end;
    for (int i = 1; i < T; ++i) {
        const char* q = body + (size_t)(end - body) * i / T;
        if (q < cut[i - 1]) q = cut[i - 1];
        while (q < end && *q != '\n') ++q;
        cut[i] = (q < end) ? q + 1 : end;
    }
    std::vector<std::thread> th;
    for (int i = 0; i < T; ++i)
        th.emplace_back([&, i] {
            parts[i].reserve(n / T + 16);
            ok[i] = parse_records(cut[i], cut[i + 1], &parts[i], true);
        });
    for (auto& t : th) t.join();
    bool all_ok = true;
    for (int i = 0; i < T; ++i) all_ok = all_ok && ok[i];
    size_t total = 0;
    for (auto& p : parts) total += p.size();
    if (!all_ok) {
        // records spread over lines (or a malformed one): one sequential pass
        parts.assign(1, {});
        parts[0].reserve(n);
        Cursor s{body, end};
        for (size_t i = 0; i < n; ++i) {
            Rec r;
            float divq, divs;
            char type;
            if (!read_float(s, &r.s) || !read_float(s, &r.k) || !read_float(s, &r.r) ||
                !read_float(s, &divq) || !read_float(s, &r.v) || !read_float(s, &r.t) ||
                !read_char(s, &type) || !read_float(s, &divs) || !read_float(s, &r.dg)) {
                free_book(out);
                return BSG_ERR_INVALID_ARG;  // "Unable to read from file"
            }
            r.ot = (type == 'P') ? 1 : 0;
            parts[0].push_back(r);
        }
        total = n;
    }
    if (total < n) {
        free_book(out);
        return BSG_ERR_INVALID_ARG;  // fewer records than the count
    }
    // the reference reads exactly n records and ignores anything after
    // them: each part is stored from its offset, the parts in parallel
    std::vector<size_t> at(parts.size() + 1, 0);
    for (size_t j = 0; j < parts.size(); ++j) at[j + 1] = at[j] + parts[j].size();
    std::vector<std::thread> st;
    for (size_t j = 0; j < parts.size(); ++j)
        st.emplace_back([&, j] {
            for (size_t k = 0; k < parts[j].size() && at[j] + k < n; ++k)
                store(out, at[j] + k, parts[j][k]);
        });
    for (auto& t : st) t.join();
    return BSG_OK;
}

int bsg_read_parsec(const char* path, int nthreads, bsg_book* out) {
    if (!path || !out) return BSG_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) return BSG_ERR_INVALID_ARG;
    struct stat sb;
    if (::fstat(fd, &sb) != 0 || sb.st_size < 0) {
        ::close(fd);
        return BSG_ERR_INVALID_ARG;
    }
    const size_t sz = (size_t)sb.st_size;
    // read in parallel, disjoint ranges with pread, into an uninitialised
    // buffer ended by a NUL (for the strtof fallback)
    std::unique_ptr<char[]> buf(new (std::nothrow) char[sz + 1]);
    if (!buf) {
        ::close(fd);
        return BSG_ERR_OUT_OF_MEMORY;
    }
    const int T = clamp_threads(nthreads, sz, 8 << 20);
    std::vector<int> ok(T, 1);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            size_t a = sz * t / T;
            const size_t b = sz * (t + 1) / T;
            while (a < b) {
                const ssize_t r = ::pread(fd, buf.get() + a, b - a, (off_t)a);
                if (r <= 0) {
                    if (r < 0 && errno == EINTR) continue;
                    ok[t] = 0;
                    return;
                }
                a += (size_t)r;
            }
        });
    for (auto& x : th) x.join();
    ::close(fd);
    for (int v : ok)
        if (!v) return BSG_ERR_INVALID_ARG;
    buf[sz] = '\0';
    return bsg_parse_parsec(buf.get(), sz, nthreads, out);
}

void bsg_book_free(bsg_book* b) { free_book(b); }

int bsg_format_prices(const float* prices, size_t n, int nthreads, char** text, size_t* len) {
    if ((!prices && n) || !text || !len) return BSG_ERR_INVALID_ARG;
    *text = nullptr;
    *len = 0;
    const int T = clamp_threads(nthreads, n, 1 << 16);
    std::vector<std::string> parts(T);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            const size_t a = n * t / T, b = n * (t + 1) / T;
            std::string& s = parts[t];
            s.resize((b - a) * 24 + 64);
            size_t w = 0;
            char tmp[80];
            for (size_t i = a; i < b; ++i) {
                const int k = format_f18(prices[i], tmp);
                if (w + (size_t)k + 1 > s.size()) s.resize(2 * s.size() + (size_t)k + 1);
                std::memcpy(&s[w], tmp, (size_t)k);
                w += (size_t)k;
                s[w++] = '\n';
            }
            s.resize(w);
        });
    for (auto& t : th) t.join();
    char head[32];
    const int hl = std::snprintf(head, sizeof head, "%i\n", (int)n);  // blackscholes.c:929
    size_t total = (size_t)hl;
    for (auto& p : parts) total += p.size();
    char* out = static_cast<char*>(std::malloc(total + 1));
    if (!out) return BSG_ERR_OUT_OF_MEMORY;
    std::memcpy(out, head, (size_t)hl);
    size_t w = (size_t)hl;
    for (auto& p : parts) {
        std::memcpy(out + w, p.data(), p.size());
        w += p.size();
    }
    out[w] = '\0';
    *text = out;
    *len = w;
    return BSG_OK;
}

void bsg_text_free(char* text) { std::free(text); }

int bsg_write_parsec_prices(const char* path, const float* prices, size_t n, int nthreads) {
    if (!path) return BSG_ERR_INVALID_ARG;
    char* text = nullptr;
    size_t len = 0;
    int st = bsg_format_prices(prices, n, nthreads, &text, &len);
    if (st) return st;
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        std::free(text);
        return BSG_ERR_INVALID_ARG;
    }
    const size_t w = std::fwrite(text, 1, len, f);
    std::free(text);
    if (std::fclose(f) != 0 || w != len) return BSG_ERR_INVALID_ARG;
    return BSG_OK;
}

int bsg_write_parsec_input(const char* path, const bsg_book* b, int nthreads) {
    if (!path || !b || (b->n && (!b->sptprice || !b->strike || !b->rate || !b->volatility ||
                                 !b->otime || !b->otype)))
        return BSG_ERR_INVALID_ARG;
    const size_t n = b->n;
    const int T = clamp_threads(nthreads, n, 1 << 15);
    std::vector<std::string> parts(T);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            const size_t a = n * t / T, e = n * (t + 1) / T;
            std::string& s = parts[t];
            s.reserve((e - a) * 96);
            char line[256];
            for (size_t i = a; i < e; ++i) {
                // %.9g round-trips every float exactly through "%f" parsing
                const int k = std::snprintf(
                    line, sizeof line, "%.9g %.9g %.9g 0 %.9g %.9g %c 0 %.17g\n",
                    (double)b->sptprice[i], (double)b->strike[i], (double)b->rate[i],
                    (double)b->volatility[i], (double)b->otime[i], b->otype[i] == 1 ? 'P' : 'C',
                    b->dgrefval ? (double)b->dgrefval[i] : 0.0);
                s.append(line, (size_t)k);
            }
        });
    for (auto& t : th) t.join();
    FILE* f = std::fopen(path, "wb");
    if (!f) return BSG_ERR_INVALID_ARG;
    bool ok = std::fprintf(f, "%i\n", (int)n) > 0;
    for (auto& p : parts) ok = ok && std::fwrite(p.data(), 1, p.size(), f) == p.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? BSG_OK : BSG_ERR_INVALID_ARG;
}

// Binary SoA: "BSGSOA01", uint64 n, then sptprice, strike, rate, volatility,
// otime (float32), otype (int32), dgrefval (float32), each n elements,
// little-endian as the machine writes them.
static const char kMagic[8] = {'B', 'S', 'G', 'S', 'O', 'A', '0', '1'};

int bsg_write_soa(const char* path, const bsg_book* b) {
    if (!path || !b) return BSG_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return BSG_ERR_INVALID_ARG;
    const uint64_t n = b->n;
    bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(&n, 8, 1, f) == 1;
    const void* arrs[7] = {b->sptprice, b->strike, b->rate, b->volatility, b->otime, b->otype,
                           b->dgrefval};
    for (int j = 0; j < 7 && ok; ++j) ok = n == 0 || std::fwrite(arrs[j], 4, n, f) == n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? BSG_OK : BSG_ERR_INVALID_ARG;
}

int bsg_read_soa(const char* path, bsg_book* out) {
    if (!path || !out) return BSG_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    FILE* f = std::fopen(path, "rb");
    if (!f) return BSG_ERR_INVALID_ARG;
    char m[8];
    uint64_t n = 0;
    if (std::fread(m, 1, 8, f) != 8 || std::memcmp(m, kMagic, 8) != 0 || std::fread(&n, 8, 1, f) != 1 ||
        n > ((uint64_t)1 << 36)) {
        std::fclose(f);
        return BSG_ERR_INVALID_ARG;
    }
    if (!alloc_book(out, (size_t)n)) {
        std::fclose(f);
        return BSG_ERR_OUT_OF_MEMORY;
    }
    void* arrs[7] = {out->sptprice, out->strike, out->rate, out->volatility, out->otime,
                     out->otype, out->dgrefval};
    bool ok = true;
    for (int j = 0; j < 7 && ok; ++j) ok = n == 0 || std::fread(arrs[j], 4, n, f) == n;
    std::fclose(f);
    if (!ok) {
        free_book(out);
        return BSG_ERR_INVALID_ARG;
    }
    return BSG_OK;
}

}  // extern "C"
