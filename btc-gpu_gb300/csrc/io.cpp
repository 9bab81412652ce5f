// Text I/O, the train shuffle and the synthetic generator.
//
// read_entries follows main.cpp:47-99: a line is skipped when it is empty,
// starts with '#' or '%', or does not begin with three integers and a number
// (stream extraction semantics: leading whitespace skipped, extra fields
// ignored); coord_base is subtracted and out-of-range coordinates are an
// error.  The whole file is read at once and parsed without iostreams, in
// newline-aligned chunks on host threads for large files.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

#include "btc_gpu.h"
#include "common.h"

namespace btc {
namespace {

inline bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

// int extraction like std::istream >> int: optional sign, then digits
bool parse_int(const char*& p, const char* end, int32_t& out)
{
    while (p < end && is_ws(*p))
        p++;
    const char* q = p;
    bool neg = false;
    if (q < end && (*q == '+' || *q == '-')) {
        neg = *q == '-';
        q++;
    }
    if (q >= end || *q < '0' || *q > '9')
        return false;
    long long v = 0;
    bool overflow = false;
    while (q < end && *q >= '0' && *q <= '9') {
        v = v * 10 + (*q - '0');
        if (v > (long long)INT_MAX + 1)
            overflow = true, v = (long long)INT_MAX + 1;
        q++;
    }
    if (neg)
        v = -v;
    if (overflow || v > INT_MAX || v < INT_MIN)
        return false;  // the stream sets failbit on overflow
    out = (int32_t)v;
    p = q;
    return true;
}

// double extraction: the characters a number can hold, then strtod on them
bool parse_double(const char*& p, const char* end, double& out)
{
    while (p < end && is_ws(*p))
        p++;
    char buf[128];
    int n = 0;
    const char* q = p;
    auto put = [&](char c) {
        if (n < 127)
            buf[n++] = c;
    };
    if (q < end && (*q == '+' || *q == '-'))
        put(*q++);
    int digits = 0;
    while (q < end && *q >= '0' && *q <= '9')
        put(*q++), digits++;
    if (q < end && *q == '.') {
        put(*q++);
        while (q < end && *q >= '0' && *q <= '9')
            put(*q++), digits++;
    }
    if (digits == 0)
        return false;
    if (q < end && (*q == 'e' || *q == 'E')) {
        const char* r = q + 1;
        char sign = 0;
        if (r < end && (*r == '+' || *r == '-'))
            sign = *r++;
        if (r < end && *r >= '0' && *r <= '9') {
            put(*q);
            if (sign)
                put(sign);
            q = r;
            while (q < end && *q >= '0' && *q <= '9')
                put(*q++);
        } else {
            return false;  // a dangling exponent fails extraction
        }
    }
    buf[n] = 0;
    out = std::strtod(buf, nullptr);
    if (std::isinf(out))
        return false;  // overflow fails extraction; underflow is accepted
    p = q;
    return true;
}

// SplitMix64: counter-based, identical on every host
inline uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
inline uint64_t hash4(uint64_t seed, uint64_t a, uint64_t b, uint64_t c)
{
    return mix64(mix64(mix64(seed ^ mix64(a)) ^ b) ^ c);
}
inline double unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }
inline double normal(uint64_t h1, uint64_t h2)
{
    double u1 = unit(h1), u2 = unit(h2);
    if (u1 < 1e-300)
        u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

struct Zipf {
    std::vector<double> cdf;
    int n = 0;
    double s = 0;
    void init(int n_, double s_)
    {
        n = n_;
        s = s_;
        if (s <= 0)
            return;
        cdf.resize(n);
        double acc = 0;
        for (int i = 0; i < n; i++) {
            acc += std::pow((double)(i + 1), -s);
            cdf[i] = acc;
        }
        for (int i = 0; i < n; i++)
            cdf[i] /= acc;
    }
    int sample(double u) const
    {
        if (s <= 0)
            return std::min(n - 1, (int)(u * n));
        int k = (int)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        return std::min(k, n - 1);
    }
};

}  // namespace

double init_uniform(uint64_t seed, int mode, int64_t row, int col, double lo, double hi)
{
    return lo + (hi - lo) * unit(hash4(seed, (uint64_t)mode + 1, (uint64_t)row, (uint64_t)col));
}

}  // namespace btc

using namespace btc;

extern "C" {

void btc_free(void* p) { std::free(p); }

btc_status btc_read_entries(const char* path, int32_t coord_base, int32_t I, int32_t J, int32_t K,
                            int32_t** xyz, double** val, int64_t* n, int64_t* line_no)
{
    if (!path || !xyz || !val || !n)
        return BTC_ERR_ARG;
    *xyz = nullptr;
    *val = nullptr;
    *n = 0;
    if (line_no)
        *line_no = 0;
    FILE* f = std::fopen(path, "rb");
    if (!f)
        return BTC_ERR_IO;
    std::fseek(f, 0, SEEK_END);
    long long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<char> buf((size_t)std::max(0LL, size));
    if (size > 0 && std::fread(buf.data(), 1, (size_t)size, f) != (size_t)size) {
        std::fclose(f);
        return BTC_ERR_IO;
    }
    std::fclose(f);
    // Lines are parsed in chunks cut at newlines, one per thread; a chunk
    // stops at its first out-of-range line, the earliest such line in file
    // order is the error (as the serial scan would report it), and the
    // chunks' entries are concatenated in order.
    const char* begin = buf.data();
    const char* end = begin + buf.size();
    int T = size >= (64LL << 20) ? (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency())) : 1;
    std::vector<const char*> cut((size_t)T + 1, end);
    cut[0] = begin;
    for (int t = 1; t < T; t++) {
        const char* c = std::max(begin + (size_t)((long long)buf.size() * t / T), cut[(size_t)t - 1]);
        const char* nl = c < end ? (const char*)std::memchr(c, '\n', (size_t)(end - c)) : nullptr;
        cut[(size_t)t] = nl ? nl + 1 : end;
    }
    struct Part {
        std::vector<int32_t> cx;
        std::vector<double> cv;
        int64_t lines = 0, bad = 0;  // lines in the chunk; 1-based line of its first error, 0 if none
    };
    std::vector<Part> part((size_t)T);
    auto work = [&](int t) {
        Part& P = part[(size_t)t];
        const char* p = cut[(size_t)t];
        const char* e = cut[(size_t)t + 1];
        P.cx.reserve((size_t)((e - p) / 16) * 3);
        P.cv.reserve((size_t)((e - p) / 16));
        while (p < e) {
            const char* eol = (const char*)std::memchr(p, '\n', (size_t)(e - p));
            if (!eol)
                eol = e;
            P.lines++;
            const char* q = p;
            if (q < eol && *q != '#' && *q != '%') {
                int32_t x, y, z;
                double v;
                if (parse_int(q, eol, x) && parse_int(q, eol, y) && parse_int(q, eol, z) &&
                    parse_double(q, eol, v)) {
                    x -= coord_base;
                    y -= coord_base;
                    z -= coord_base;
                    if (x < 0 || x >= I || y < 0 || y >= J || z < 0 || z >= K) {
                        P.bad = P.lines;
                        return;
                    }
                    P.cx.push_back(x);
                    P.cx.push_back(y);
                    P.cx.push_back(z);
                    P.cv.push_back(v);
                }
            }
            p = eol + 1;
        }
    };
    {
        std::vector<std::thread> pool;
        for (int t = 1; t < T; t++)
            pool.emplace_back(work, t);
        work(0);
        for (auto& th : pool)
            th.join();
    }
    int64_t ln = 0, cnt = 0;
    for (const Part& P : part) {
        if (P.bad) {
            if (line_no)
                *line_no = ln + P.bad;
            return BTC_ERR_RANGE;
        }
        ln += P.lines;
        cnt += (int64_t)P.cv.size();
    }
    *xyz = (int32_t*)std::malloc(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(cnt, 1));
    *val = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(cnt, 1));
    if (!*xyz || !*val) {
        std::free(*xyz);
        std::free(*val);
        *xyz = nullptr;
        *val = nullptr;
        return BTC_ERR_ALLOC;
    }
    int64_t o = 0;
    for (const Part& P : part) {
        if (!P.cv.empty()) {
            std::memcpy(*xyz + 3 * o, P.cx.data(), sizeof(int32_t) * P.cx.size());
            std::memcpy(*val + o, P.cv.data(), sizeof(double) * P.cv.size());
        }
        o += (int64_t)P.cv.size();
    }
    *n = cnt;
    return BTC_OK;
}

}  // extern "C"

namespace {

// Binary cache of a parsed file: this header, then n x 3 int32 coordinates
// (base already subtracted) and n doubles, in host byte order.
struct CacheHdr {
    char magic[8];
    int32_t coord_base, I, J, K;
    int64_t n, src_size, src_mtime_ns;
};
constexpr char kCacheMagic[8] = {'B', 'T', 'C', 'C', 'O', 'O', '0', '1'};

bool source_stamp(const char* path, int64_t& size, int64_t& mtime_ns)
{
    struct stat st;
    if (stat(path, &st) != 0)
        return false;
    size = (int64_t)st.st_size;
    mtime_ns = (int64_t)st.st_mtim.tv_sec * 1000000000LL + (int64_t)st.st_mtim.tv_nsec;
    return true;
}

bool read_cache(const char* cache, const CacheHdr& want, int32_t** xyz, double** val, int64_t* n)
{
    FILE* f = std::fopen(cache, "rb");
    if (!f)
        return false;
    CacheHdr h;
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 && std::memcmp(h.magic, kCacheMagic, 8) == 0 &&
              h.coord_base == want.coord_base && h.I == want.I && h.J == want.J && h.K == want.K &&
              h.src_size == want.src_size && h.src_mtime_ns == want.src_mtime_ns && h.n >= 0;
    if (ok) {
        struct stat st;
        ok = fstat(fileno(f), &st) == 0 &&
             (int64_t)st.st_size == (int64_t)sizeof h + h.n * (int64_t)(3 * sizeof(int32_t) + sizeof(double));
    }
    int32_t* x = nullptr;
    double* v = nullptr;
    if (ok) {
        x = (int32_t*)std::malloc(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(h.n, 1));
        v = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(h.n, 1));
        ok = x && v && std::fread(x, sizeof(int32_t) * 3, (size_t)h.n, f) == (size_t)h.n &&
             std::fread(v, sizeof(double), (size_t)h.n, f) == (size_t)h.n;
        // the header cannot vouch for the payload (a damaged or edited file,
        // a stamp collision): coordinates are held to the ranges the text
        // parser enforces, and a cache that breaks them is parsed again
        for (int64_t i = 0; ok && i < h.n; i++)
            ok = (uint32_t)x[3 * i] < (uint32_t)want.I && (uint32_t)x[3 * i + 1] < (uint32_t)want.J &&
                 (uint32_t)x[3 * i + 2] < (uint32_t)want.K;
    }
    std::fclose(f);
    if (!ok) {
        std::free(x);
        std::free(v);
        return false;
    }
    *xyz = x;
    *val = v;
    *n = h.n;
    return true;
}

void write_cache(const char* cache, const CacheHdr& hdr, const int32_t* xyz, const double* val)
{
    std::string tmp = std::string(cache) + ".tmp." + std::to_string((long long)getpid());
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f)
        return;  // the cache is an optimisation: an unwritable location is no error
    bool ok = std::fwrite(&hdr, sizeof hdr, 1, f) == 1 &&
              std::fwrite(xyz, sizeof(int32_t) * 3, (size_t)hdr.n, f) == (size_t)hdr.n &&
              std::fwrite(val, sizeof(double), (size_t)hdr.n, f) == (size_t)hdr.n;
    ok = std::fclose(f) == 0 && ok;
    if (!ok || std::rename(tmp.c_str(), cache) != 0)
        std::remove(tmp.c_str());
}

}  // namespace

extern "C" {

btc_status btc_read_entries_cached(const char* path, const char* cache, int32_t coord_base, int32_t I, int32_t J,
                                   int32_t K, int32_t** xyz, double** val, int64_t* n, int64_t* line_no,
                                   int32_t* from_cache)
{
    if (!path || !cache || !xyz || !val || !n || !from_cache)
        return BTC_ERR_ARG;
    *from_cache = 0;
    CacheHdr hdr{};
    std::memcpy(hdr.magic, kCacheMagic, 8);
    hdr.coord_base = coord_base;
    hdr.I = I;
    hdr.J = J;
    hdr.K = K;
    const bool stamped = source_stamp(path, hdr.src_size, hdr.src_mtime_ns);
    if (stamped && read_cache(cache, hdr, xyz, val, n)) {
        if (line_no)
            *line_no = 0;
        *from_cache = 1;
        return BTC_OK;
    }
    btc_status st = btc_read_entries(path, coord_base, I, J, K, xyz, val, n, line_no);
    if (st == BTC_OK && stamped) {
        hdr.n = *n;
        write_cache(cache, hdr, *xyz, *val);
    }
    return st;
}

btc_status btc_shuffle_entries(int32_t* xyz, double* val, int64_t n, uint32_t seed)
{
    if (n < 0 || (n > 0 && (!xyz || !val)))
        return BTC_ERR_ARG;
    if (n <= 1)
        return BTC_OK;
    // permute indices with the same std::shuffle/mt19937 sequence the
    // reference applies to its vector<T_node>
    std::vector<int64_t> perm((size_t)n);
    for (int64_t i = 0; i < n; i++)
        perm[(size_t)i] = i;
    std::mt19937 rng(seed);
    std::shuffle(perm.begin(), perm.end(), rng);
    std::vector<int32_t> nx((size_t)n * 3);
    std::vector<double> nv((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        int64_t s = perm[(size_t)i];
        nx[3 * i] = xyz[3 * s];
        nx[3 * i + 1] = xyz[3 * s + 1];
        nx[3 * i + 2] = xyz[3 * s + 2];
        nv[i] = val[s];
    }
    std::memcpy(xyz, nx.data(), sizeof(int32_t) * 3 * (size_t)n);
    std::memcpy(val, nv.data(), sizeof(double) * (size_t)n);
    return BTC_OK;
}

btc_status btc_gen_tensor(const btc_gen_spec* sp, int32_t** txyz, double** tval, int64_t* ntr,
                          int32_t** sxyz, double** sval, int64_t* nte)
{
    if (!sp || !txyz || !tval || !ntr || !sxyz || !sval || !nte)
        return BTC_ERR_ARG;
    if (sp->I <= 0 || sp->J <= 0 || sp->K <= 0 || sp->nnz < 0)
        return BTC_ERR_ARG;
    const double cells = (double)sp->I * (double)sp->J * (double)sp->K;
    if ((double)sp->nnz > 0.5 * cells)
        return BTC_ERR_ARG;
    int threads = sp->threads > 0 ? sp->threads : (int)std::max(1u, std::thread::hardware_concurrency());
    Zipf z[3];
    const int dims[3] = {sp->I, sp->J, sp->K};
    for (int a = 0; a < 3; a++)
        z[a].init(dims[a], sp->zipf_s[a]);
    const uint64_t JK = (uint64_t)sp->J * (uint64_t)sp->K;
    // open-addressing set of cell keys; entries kept in first-draw order
    uint64_t cap = 1;
    while (cap < (uint64_t)sp->nnz * 2 + 16)
        cap <<= 1;
    std::vector<uint64_t> table(cap, ~0ULL);
    std::vector<uint64_t> keys;
    keys.reserve((size_t)sp->nnz);
    uint64_t drawn = 0;
    const uint64_t batch = 1 << 22;
    std::vector<uint64_t> cand(batch);
    while ((int64_t)keys.size() < sp->nnz) {
        std::atomic<uint64_t> next(0);
        auto work = [&]() {
            for (;;) {
                uint64_t b0 = next.fetch_add(65536);
                if (b0 >= batch)
                    break;
                uint64_t b1 = std::min(batch, b0 + 65536);
                for (uint64_t i = b0; i < b1; i++) {
                    uint64_t d = drawn + i;
                    uint64_t x = (uint64_t)z[0].sample(unit(hash4(sp->seed, 11, d, 0)));
                    uint64_t y = (uint64_t)z[1].sample(unit(hash4(sp->seed, 11, d, 1)));
                    uint64_t w = (uint64_t)z[2].sample(unit(hash4(sp->seed, 11, d, 2)));
                    cand[i] = x * JK + y * (uint64_t)sp->K + w;
                }
            }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < threads; t++)
            pool.emplace_back(work);
        work();
        for (auto& t : pool)
            t.join();
        for (uint64_t i = 0; i < batch && (int64_t)keys.size() < sp->nnz; i++) {
            uint64_t k = cand[i];
            uint64_t h = mix64(k) & (cap - 1);
            while (table[h] != ~0ULL && table[h] != k)
                h = (h + 1) & (cap - 1);
            if (table[h] == ~0ULL) {
                table[h] = k;
                keys.push_back(k);
            }
        }
        drawn += batch;
        if (drawn > (uint64_t)sp->nnz * 1000 + (1ULL << 26))
            return BTC_ERR_RANGE;  // distribution too concentrated for the requested count
    }
    std::vector<uint64_t>().swap(table);
    const int64_t n = (int64_t)keys.size();
    const int R = sp->gt_rank;
    // ground-truth factors
    std::vector<double> gt[3];
    for (int a = 0; a < 3 && R > 0; a++) {
        gt[a].resize((size_t)dims[a] * R);
        for (int64_t i = 0; i < (int64_t)dims[a] * R; i++)
            gt[a][(size_t)i] = sp->gt_std * normal(hash4(sp->seed, 21 + a, (uint64_t)i, 0),
                                                   hash4(sp->seed, 21 + a, (uint64_t)i, 1));
    }
    std::vector<int32_t> xyz((size_t)n * 3);
    std::vector<double> val((size_t)n);
    std::vector<uint8_t> is_train((size_t)n);
    {
        std::atomic<int64_t> next(0);
        auto work = [&]() {
            for (;;) {
                int64_t b0 = next.fetch_add(65536);
                if (b0 >= n)
                    break;
                int64_t b1 = std::min(n, b0 + 65536);
                for (int64_t i = b0; i < b1; i++) {
                    uint64_t k = keys[(size_t)i];
                    int32_t x = (int32_t)(k / JK), y = (int32_t)((k / (uint64_t)sp->K) % (uint64_t)sp->J),
                            w = (int32_t)(k % (uint64_t)sp->K);
                    xyz[3 * i] = x;
                    xyz[3 * i + 1] = y;
                    xyz[3 * i + 2] = w;
                    double v;
                    if (R > 0) {
                        v = 0;
                        for (int r = 0; r < R; r++)
                            v += gt[0][(size_t)x * R + r] * gt[1][(size_t)y * R + r] * gt[2][(size_t)w * R + r];
                        v += sp->noise_std * normal(hash4(sp->seed, 31, k, 0), hash4(sp->seed, 31, k, 1));
                    } else {
                        v = std::exp(normal(hash4(sp->seed, 32, k, 0), hash4(sp->seed, 32, k, 1)));
                    }
                    val[(size_t)i] = v;
                    is_train[(size_t)i] = unit(hash4(sp->seed, 41, k, 0)) < sp->train_frac;
                }
            }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < threads; t++)
            pool.emplace_back(work);
        work();
        for (auto& t : pool)
            t.join();
    }
    if (R <= 0 && n > 0) {  // log-normal values rescaled to [0, 1]
        double mx = 0;
        for (double v : val)
            mx = std::max(mx, v);
        for (double& v : val)
            v /= mx;
    }
    int64_t a = 0, b = 0;
    for (int64_t i = 0; i < n; i++)
        (is_train[(size_t)i] ? a : b)++;
    *txyz = (int32_t*)std::malloc(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(a, 1));
    *tval = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(a, 1));
    *sxyz = (int32_t*)std::malloc(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(b, 1));
    *sval = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(b, 1));
    if (!*txyz || !*tval || !*sxyz || !*sval)
        return BTC_ERR_ALLOC;
    int64_t ia = 0, ib = 0;
    for (int64_t i = 0; i < n; i++) {
        if (is_train[(size_t)i]) {
            std::memcpy(*txyz + 3 * ia, &xyz[3 * i], 12);
            (*tval)[ia++] = val[(size_t)i];
        } else {
            std::memcpy(*sxyz + 3 * ib, &xyz[3 * i], 12);
            (*sval)[ib++] = val[(size_t)i];
        }
    }
    *ntr = a;
    *nte = b;
    return BTC_OK;
}

}  // extern "C"
