// Fast readers for the reference's input files, and a binary cache.
//
// The reference reads option and yield files with iostream extraction
// (common/Arrays.hpp:15-32: skip to '[', then "value ," pairs up to ']'), one
// value at a time; at 10^5-10^6 options the parse dominates a run's wall time.
// Here the file is read into memory once, the eight "[..]" bodies are located, and
// each body is split at commas into chunks that host threads parse in parallel with
// std::from_chars (correctly rounded, like strtod, so the doubles are the ones the
// reference's stream extraction produces).  Integer fields must hold integral
// values in range; option types must be 0 or 1 (common/Options.hpp:35-46).
//
// The binary cache is the SoA arrays as they are in memory: a 32-byte header
// ("HWTOPT1" magic, option count) followed by the eight arrays in field order, each
// padded to a multiple of 8 bytes.  Reading it is one fread per array.
#include <charconv>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hwtree.h"

namespace {

constexpr char kMagic[8] = {'H', 'W', 'T', 'O', 'P', 'T', '1', '\0'};
constexpr size_t kAlign = 64;
constexpr size_t kParallelBytes = 1 << 20;  // bodies shorter than this parse on one thread

size_t up(size_t v, size_t a) { return (v + a - 1) / a * a; }

void set_err(char *err, int len, const std::string &msg)
{
    if (err && len > 0) {
        std::snprintf(err, (size_t)len, "%s", msg.c_str());
    }
}

bool read_file(const char *path, std::string &buf)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (size < 0) {
        std::fclose(f);
        return false;
    }
    buf.resize((size_t)size);
    const size_t got = size > 0 ? std::fread(&buf[0], 1, (size_t)size, f) : 0;
    std::fclose(f);
    return got == (size_t)size;
}

// One "[..]" body: [begin, end) between the brackets.
struct Body {
    const char *begin = nullptr, *end = nullptr;
};

// Finds the next body at or after p; false if there is none.
bool next_body(const char *&p, const char *stop, Body &b)
{
    const char *o = (const char *)std::memchr(p, '[', (size_t)(stop - p));
    if (!o) return false;
    const char *c = (const char *)std::memchr(o + 1, ']', (size_t)(stop - o - 1));
    if (!c) return false;
    b.begin = o + 1;
    b.end = c;
    p = c + 1;
    return true;
}

size_t count_values(const Body &b)
{
    // values = commas + 1, unless the body is blank
    bool blank = true;
    for (const char *q = b.begin; q < b.end; ++q)
        if (*q != ' ' && *q != '\t' && *q != '\n' && *q != '\r') {
            blank = false;
            break;
        }
    if (blank) return 0;
    size_t n = 1;
    for (const char *q = b.begin; q < b.end; ++q) n += (*q == ',');
    return n;
}

inline const char *skip_ws(const char *q, const char *e)
{
    while (q < e && (*q == ' ' || *q == '\t' || *q == '\n' || *q == '\r' || *q == '+')) ++q;
    return q;
}

// Parses the comma-separated values of [begin, end) into out[0..]; returns the
// number parsed, or -1 - (index of the first bad value).
template <typename T>
long parse_range(const char *begin, const char *end, T *out, long first_index)
{
    long k = 0;
    const char *q = begin;
    while (q < end) {
        q = skip_ws(q, end);
        double v = 0.0;
        const auto r = std::from_chars(q, end, v);
        if (r.ec != std::errc()) return -1 - (first_index + k);
        q = skip_ws(r.ptr, end);
        if (q < end && *q != ',') return -1 - (first_index + k);
        if constexpr (std::is_same<T, double>::value) {
            out[k] = v;
        } else {
            const double lo = std::is_same<T, int8_t>::value ? -128.0 : 0.0;
            const double hi = std::is_same<T, int8_t>::value ? 127.0 : 65535.0;
            if (!(v >= lo && v <= hi) || v != (double)(long long)v) return -1 - (first_index + k);
            out[k] = (T)(long long)v;
        }
        ++k;
        if (q < end) ++q;  // the comma
    }
    return k;
}

// Parses one body of n values into out, split across threads for long bodies.
template <typename T>
long parse_body(const Body &b, size_t n, T *out)
{
    const size_t bytes = (size_t)(b.end - b.begin);
    unsigned threads = std::thread::hardware_concurrency();
    if (threads == 0) threads = 1;
    if (threads > 32) threads = 32;
    if (bytes < kParallelBytes || threads == 1) {
        const long k = parse_range<T>(b.begin, b.end, out, 0);
        return k < 0 ? k : (k == (long)n ? k : -1 - k);
    }
    // chunk boundaries just after commas; the value index of each chunk start
    std::vector<const char *> cut(threads + 1);
    cut[0] = b.begin;
    cut[threads] = b.end;
    for (unsigned t = 1; t < threads; ++t) {
        const char *q = b.begin + bytes * t / threads;
        if (q < cut[t - 1]) q = cut[t - 1];
        while (q < b.end && *q != ',') ++q;
        cut[t] = q < b.end ? q + 1 : b.end;
    }
    std::vector<size_t> start(threads + 1, 0);
    for (unsigned t = 0; t < threads; ++t) {
        size_t c = 0;
        for (const char *q = cut[t]; q < cut[t + 1]; ++q) c += (*q == ',');
        // a chunk ending right after a comma holds exactly `c` values
        start[t + 1] = start[t] + c;
    }
    // the last chunk's value has no trailing comma
    if (start[threads] + 1 != n) return -1 - (long)start[threads];
    std::vector<long> res(threads, 0);
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < threads; ++t) {
        pool.emplace_back([&, t]() {
            if (cut[t] == cut[t + 1]) return;
            res[t] = parse_range<T>(cut[t], cut[t + 1], out + start[t], (long)start[t]);
        });
    }
    for (auto &th : pool) th.join();
    for (unsigned t = 0; t < threads; ++t)
        if (res[t] < 0) return res[t];
    return (long)n;
}

// One allocation for the eight arrays of n options, 64-byte aligned pieces.
struct Layout {
    size_t off[8];
    size_t total;
};

Layout layout(size_t n)
{
    const size_t sz[8] = {8 * n, 8 * n, 8 * n, 2 * n, 2 * n, 8 * n, 8 * n, n};
    Layout l;
    size_t o = 0;
    for (int i = 0; i < 8; ++i) {
        l.off[i] = o;
        o = up(o + sz[i], kAlign);
    }
    l.total = o > 0 ? o : kAlign;
    return l;
}

bool alloc_options(size_t n, hwt_options *o)
{
    const Layout l = layout(n);
    char *base = (char *)std::aligned_alloc(kAlign, up(l.total, kAlign));
    if (!base) return false;
    o->n = (int32_t)n;
    o->strike = (const double *)(base + l.off[0]);
    o->bond_maturity = (const double *)(base + l.off[1]);
    o->option_maturity = (const double *)(base + l.off[2]);
    o->term_unit = (const uint16_t *)(base + l.off[3]);
    o->term_steps = (const uint16_t *)(base + l.off[4]);
    o->a = (const double *)(base + l.off[5]);
    o->sigma = (const double *)(base + l.off[6]);
    o->type = (const int8_t *)(base + l.off[7]);
    return true;
}

const char *kFieldName[8] = {"StrikePrices", "Maturities", "Lengths", "TermUnits", "TermStepCounts",
                             "ReversionRates", "Volatilities", "Types"};

int read_options_bin(const std::string &buf, hwt_options *out, char *err, int err_len)
{
    if (buf.size() < 32) {
        set_err(err, err_len, "binary options file is truncated");
        return HWT_EINVAL;
    }
    int64_t n = 0;
    std::memcpy(&n, buf.data() + 8, 8);
    if (n < 0 || n > INT32_MAX) {
        set_err(err, err_len, "binary options file has a bad option count");
        return HWT_EINVAL;
    }
    const size_t N = (size_t)n;
    const size_t sz[8] = {8 * N, 8 * N, 8 * N, 2 * N, 2 * N, 8 * N, 8 * N, N};
    size_t need = 32;
    for (size_t s : sz) need += up(s, 8);
    if (buf.size() != need) {
        set_err(err, err_len, "binary options file size does not match its option count");
        return HWT_EINVAL;
    }
    if (!alloc_options(N, out)) {
        set_err(err, err_len, "out of host memory");
        return HWT_ENOMEM;
    }
    void *dst[8] = {(void *)out->strike, (void *)out->bond_maturity, (void *)out->option_maturity,
                    (void *)out->term_unit, (void *)out->term_steps, (void *)out->a, (void *)out->sigma,
                    (void *)out->type};
    size_t pos = 32;
    for (int i = 0; i < 8; ++i) {
        std::memcpy(dst[i], buf.data() + pos, sz[i]);
        pos += up(sz[i], 8);
    }
    for (size_t i = 0; i < N; ++i)
        if (out->type[i] != 0 && out->type[i] != 1) {
            hwt_free_options(out);
            set_err(err, err_len, "invalid option type at index " + std::to_string(i));
            return HWT_EINVAL;
        }
    return HWT_OK;
}

}  // namespace

extern "C" {

int hwt_read_options(const char *path, hwt_options *out, char *err, int err_len)
{
    if (!path || !*path || !out) {
        set_err(err, err_len, "File not specified.");
        return HWT_EINVAL;
    }
    std::memset(out, 0, sizeof(*out));
    std::string buf;
    if (!read_file(path, buf)) {
        set_err(err, err_len, std::string("File '") + path + "' does not exist.");
        return HWT_EINVAL;
    }
    if (buf.size() >= 8 && std::memcmp(buf.data(), kMagic, 8) == 0) return read_options_bin(buf, out, err, err_len);

    const char *p = buf.data(), *stop = buf.data() + buf.size();
    Body body[8];
    for (int i = 0; i < 8; ++i) {
        if (!next_body(p, stop, body[i])) {
            set_err(err, err_len, std::string("File '") + path + "' holds " + std::to_string(i) +
                                      " arrays, expected 8.");
            return HWT_EINVAL;
        }
    }
    const size_t n = count_values(body[0]);
    for (int i = 1; i < 8; ++i)
        if (count_values(body[i]) != n) {
            set_err(err, err_len, std::string("array ") + kFieldName[i] + " has a different length from StrikePrices");
            return HWT_EINVAL;
        }
    if (n > (size_t)INT32_MAX) {
        set_err(err, err_len, "too many options");
        return HWT_EINVAL;
    }
    if (!alloc_options(n, out)) {
        set_err(err, err_len, "out of host memory");
        return HWT_ENOMEM;
    }
    long r[8];
    r[0] = parse_body<double>(body[0], n, (double *)out->strike);
    r[1] = parse_body<double>(body[1], n, (double *)out->bond_maturity);
    r[2] = parse_body<double>(body[2], n, (double *)out->option_maturity);
    r[3] = parse_body<uint16_t>(body[3], n, (uint16_t *)out->term_unit);
    r[4] = parse_body<uint16_t>(body[4], n, (uint16_t *)out->term_steps);
    r[5] = parse_body<double>(body[5], n, (double *)out->a);
    r[6] = parse_body<double>(body[6], n, (double *)out->sigma);
    r[7] = parse_body<int8_t>(body[7], n, (int8_t *)out->type);
    for (int i = 0; i < 8; ++i)
        if (r[i] < 0) {
            hwt_free_options(out);
            set_err(err, err_len, std::string("bad value in ") + kFieldName[i] + " at index " + std::to_string(-1 - r[i]));
            return HWT_EINVAL;
        }
    for (size_t i = 0; i < n; ++i)
        if (out->type[i] != 0 && out->type[i] != 1) {
            hwt_free_options(out);
            set_err(err, err_len, "Invalid OptionType read from stream (index " + std::to_string(i) + ").");
            return HWT_EINVAL;
        }
    return HWT_OK;
}

void hwt_free_options(hwt_options *o)
{
    if (!o) return;
    std::free((void *)o->strike);  // the eight arrays share the allocation that starts here
    std::memset(o, 0, sizeof(*o));
}

int hwt_write_options_bin(const char *path, const hwt_options *o)
{
    if (!path || !o || o->n < 0) return HWT_EINVAL;
    const size_t n = (size_t)o->n;
    if (n > 0 && (!o->strike || !o->bond_maturity || !o->option_maturity || !o->term_unit || !o->term_steps ||
                  !o->a || !o->sigma || !o->type))
        return HWT_EINVAL;
    FILE *f = std::fopen(path, "wb");
    if (!f) return HWT_EINVAL;
    char head[32] = {0};
    std::memcpy(head, kMagic, 8);
    const int64_t n64 = (int64_t)n;
    std::memcpy(head + 8, &n64, 8);
    bool ok = std::fwrite(head, 1, 32, f) == 32;
    const void *src[8] = {o->strike, o->bond_maturity, o->option_maturity, o->term_unit, o->term_steps, o->a,
                          o->sigma, o->type};
    const size_t sz[8] = {8 * n, 8 * n, 8 * n, 2 * n, 2 * n, 8 * n, 8 * n, n};
    static const char zeros[8] = {0};
    for (int i = 0; i < 8 && ok; ++i) {
        if (sz[i]) ok = std::fwrite(src[i], 1, sz[i], f) == sz[i];
        const size_t pad = up(sz[i], 8) - sz[i];
        if (ok && pad) ok = std::fwrite(zeros, 1, pad, f) == pad;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? HWT_OK : HWT_EINVAL;
}

int hwt_read_yield(const char *path, hwt_yield *out, char *err, int err_len)
{
    if (!path || !*path || !out) {
        set_err(err, err_len, "File not specified.");
        return HWT_EINVAL;
    }
    std::memset(out, 0, sizeof(*out));
    std::string buf;
    if (!read_file(path, buf)) {
        set_err(err, err_len, "File does not exist.");
        return HWT_EINVAL;
    }
    const char *p = buf.data(), *stop = buf.data() + buf.size();
    Body rates, days;
    if (!next_body(p, stop, rates) || !next_body(p, stop, days)) {
        set_err(err, err_len, "yield file holds fewer than 2 arrays");
        return HWT_EINVAL;
    }
    const size_t n = count_values(rates);
    if (count_values(days) != n || n == 0 || n > (size_t)INT32_MAX) {
        set_err(err, err_len, "yield arrays are empty or of different lengths");
        return HWT_EINVAL;
    }
    char *base = (char *)std::malloc(up(8 * n, 8) + 4 * n);
    if (!base) {
        set_err(err, err_len, "out of host memory");
        return HWT_ENOMEM;
    }
    double *r = (double *)base;
    int32_t *d = (int32_t *)(base + up(8 * n, 8));
    long k = parse_range<double>(rates.begin, rates.end, r, 0);
    std::vector<double> dd(n);
    long k2 = k == (long)n ? parse_range<double>(days.begin, days.end, dd.data(), 0) : -1;
    if (k != (long)n || k2 != (long)n) {
        std::free(base);
        set_err(err, err_len, "bad value in the yield file");
        return HWT_EINVAL;
    }
    for (size_t i = 0; i < n; ++i) {
        if (dd[i] != (double)(int32_t)dd[i]) {
            std::free(base);
            set_err(err, err_len, "yield day counts must be whole days");
            return HWT_EINVAL;
        }
        d[i] = (int32_t)dd[i];
    }
    out->n = (int32_t)n;
    out->rate = r;
    out->day = d;
    return HWT_OK;
}

void hwt_free_yield(hwt_yield *y)
{
    if (!y) return;
    std::free((void *)y->rate);  // rates and days share the allocation that starts here
    std::memset(y, 0, sizeof(*y));
}

}  // extern "C"
