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
        build_guide();
    }
    // guide[j] = first index whose cdf reaches j / G (G = 2^14, a table
    // small enough to stay in cache).  For u in [j / G, (j + 1) / G) --
    // j = floor(u * G) is exact, G being a power of two -- lower_bound(cdf, u)
    // lies in [guide[j], guide[j + 1]], so a binary search over that range
    // gives exactly lower_bound(cdf, u) (the guide-table inversion of Chen
    // and Asau, 1974).  Skewed distributions keep most searches in the head.
    static constexpr int G = 1 << 14;
    std::vector<int> guide;
    void build_guide()
    {
        if (s <= 0)
            return;
        guide.resize((size_t)G + 1);
        int k = 0;
        for (int j = 0; j <= G; j++) {
            const double t = (double)j / (double)G;
            while (k < n && cdf[(size_t)k] < t)
                k++;
            guide[(size_t)j] = k;
        }
    }
    int sample(double u) const
    {
        if (s <= 0)
            return std::min(n - 1, (int)(u * n));
        const size_t j = std::min((size_t)G - 1, (size_t)(u * (double)G));
        const int lo = guide[j], hi = std::min(n, guide[j + 1] + 1);
        const int k = (int)(std::lower_bound(cdf.begin() + lo, cdf.begin() + hi, u) - cdf.begin());
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

namespace {

// std::shuffle of the indices 0..n-1 with std::mt19937(seed), then the
// entries gathered in that order on host threads (every output slot is
// written once) and copied back.
template <typename Idx>
void shuffled_gather(int32_t* xyz, double* val, int64_t n, uint32_t seed)
{
    std::vector<Idx> perm((size_t)n);
    for (int64_t i = 0; i < n; i++)
        perm[(size_t)i] = (Idx)i;
    std::mt19937 rng(seed);
    std::shuffle(perm.begin(), perm.end(), rng);
    std::vector<int32_t> nx((size_t)n * 3);
    std::vector<double> nv((size_t)n);
    const int T = n >= (1 << 20) ? (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency())) : 1;
    auto gather = [&](int t) {
        for (int64_t i = n * t / T; i < n * (t + 1) / T; i++) {
            const int64_t s = (int64_t)perm[(size_t)i];
            nx[(size_t)(3 * i)] = xyz[3 * s];
            nx[(size_t)(3 * i + 1)] = xyz[3 * s + 1];
            nx[(size_t)(3 * i + 2)] = xyz[3 * s + 2];
            nv[(size_t)i] = val[s];
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++)
        pool.emplace_back(gather, t);
    gather(0);
    for (auto& th : pool)
        th.join();
    std::memcpy(xyz, nx.data(), sizeof(int32_t) * 3 * (size_t)n);
    std::memcpy(val, nv.data(), sizeof(double) * (size_t)n);
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
    // reference applies to its vector<T_node> (32-bit indices when they
    // suffice: the same permutation, half the memory traffic of its swaps)
    if (n <= INT32_MAX)
        shuffled_gather<int32_t>(xyz, val, n, seed);
    else
        shuffled_gather<int64_t>(xyz, val, n, seed);
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
    // The entries are the first nnz distinct cells in draw order (draw d
    // picks its three indices from hash(seed, d, axis)).  Draws are taken in
    // batches on host threads; each cell key goes to one of 4096 partitions
    // by its hash, and every partition, on its own thread, inserts its keys
    // into its own open-addressing set in draw order, marking the draws that
    // saw a cell first.  The marked draws, in order, are the entries: the
    // result does not depend on the thread count.  Many partitions keep each
    // set small enough to stay in cache while its keys are inserted.
    constexpr int P = 4096;
    struct PartSet {
        std::vector<uint64_t> t;
        uint64_t used = 0;
        bool insert(uint64_t k)
        {
            if (2 * (used + 1) > t.size()) {
                std::vector<uint64_t> old;
                old.swap(t);
                t.assign(std::max<size_t>(1024, old.size() * 2), ~0ULL);
                for (uint64_t v : old)
                    if (v != ~0ULL) {
                        uint64_t h = mix64(v) & (t.size() - 1);
                        while (t[h] != ~0ULL)
                            h = (h + 1) & (t.size() - 1);
                        t[h] = v;
                    }
            }
            uint64_t h = mix64(k) & (t.size() - 1);
            while (t[h] != ~0ULL) {
                if (t[h] == k)
                    return false;
                h = (h + 1) & (t.size() - 1);
            }
            t[h] = k;
            used++;
            return true;
        }
    };
    std::vector<PartSet> sets(P);
    {
        size_t per = 1024;
        while (per < (size_t)(2.5 * (double)sp->nnz / P))
            per <<= 1;
        for (auto& ps : sets)
            ps.t.assign(per, ~0ULL);
    }
    std::vector<uint64_t> keys;
    keys.reserve((size_t)sp->nnz);
    uint64_t drawn = 0;
    const uint64_t batch = (uint64_t)std::min<int64_t>(1LL << 24, std::max<int64_t>(1LL << 16, sp->nnz));
    std::vector<uint64_t> cand(batch);
    std::vector<uint16_t> part_of(batch);
    std::vector<uint8_t> first(batch);
    std::vector<uint32_t> by_part(batch);
    const int T = std::max(1, std::min(threads, 64));
    std::vector<uint32_t> cnt((size_t)T * P), pos((size_t)T * P);
    std::vector<uint32_t> part_off(P + 1);
    auto run = [&](int nt, const auto& fn) {
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; t++)
            pool.emplace_back(fn, t);
        fn(0);
        for (auto& th : pool)
            th.join();
    };
    while ((int64_t)keys.size() < sp->nnz) {
        // draws of this batch: keys and partitions; per-thread partition counts
        run(T, [&](int t) {
            const uint64_t lo = batch * (uint64_t)t / (uint64_t)T, hi = batch * (uint64_t)(t + 1) / (uint64_t)T;
            uint32_t* c = &cnt[(size_t)t * P];
            std::fill(c, c + P, 0u);
            for (uint64_t i = lo; i < hi; i++) {
                const uint64_t d = drawn + i;
                const uint64_t x = (uint64_t)z[0].sample(unit(hash4(sp->seed, 11, d, 0)));
                const uint64_t y = (uint64_t)z[1].sample(unit(hash4(sp->seed, 11, d, 1)));
                const uint64_t w = (uint64_t)z[2].sample(unit(hash4(sp->seed, 11, d, 2)));
                const uint64_t k = x * JK + y * (uint64_t)sp->K + w;
                cand[i] = k;
                const uint16_t q = (uint16_t)(mix64(k ^ 0x5851F42D4C957F2DULL) >> 52);
                part_of[i] = q;
                c[q]++;
            }
        });
        // draws grouped by partition, each partition's in draw order
        uint32_t o = 0;
        for (int q = 0; q < P; q++) {
            part_off[(size_t)q] = o;
            for (int t = 0; t < T; t++) {
                pos[(size_t)t * P + q] = o;
                o += cnt[(size_t)t * P + q];
            }
        }
        part_off[P] = o;
        run(T, [&](int t) {
            const uint64_t lo = batch * (uint64_t)t / (uint64_t)T, hi = batch * (uint64_t)(t + 1) / (uint64_t)T;
            uint32_t* ps = &pos[(size_t)t * P];
            for (uint64_t i = lo; i < hi; i++)
                by_part[ps[part_of[i]]++] = (uint32_t)i;
        });
        std::atomic<int> nextp(0);
        run(T, [&](int) {
            for (;;) {
                const int q = nextp.fetch_add(1);
                if (q >= P)
                    return;
                PartSet& S = sets[(size_t)q];
                for (uint32_t j = part_off[(size_t)q]; j < part_off[(size_t)q + 1]; j++) {
                    const uint32_t i = by_part[j];
                    first[i] = S.insert(cand[i]) ? 1 : 0;
                }
            }
        });
        // the batch's new cells, in draw order, up to nnz in all
        {
            std::vector<int64_t> nf((size_t)T + 1, 0);
            run(T, [&](int t) {
                const uint64_t lo = batch * (uint64_t)t / (uint64_t)T, hi = batch * (uint64_t)(t + 1) / (uint64_t)T;
                int64_t c = 0;
                for (uint64_t i = lo; i < hi; i++)
                    c += first[i];
                nf[(size_t)t + 1] = c;
            });
            for (int t = 0; t < T; t++)
                nf[(size_t)t + 1] += nf[(size_t)t];
            const size_t k0 = keys.size();
            const int64_t room = sp->nnz - (int64_t)k0;
            keys.resize(k0 + (size_t)std::min<int64_t>(room, nf[(size_t)T]));
            run(T, [&](int t) {
                const uint64_t lo = batch * (uint64_t)t / (uint64_t)T, hi = batch * (uint64_t)(t + 1) / (uint64_t)T;
                int64_t o = nf[(size_t)t];
                for (uint64_t i = lo; i < hi && o < room; i++)
                    if (first[i])
                        keys[k0 + (size_t)o++] = cand[i];
            });
        }
        drawn += batch;
        if (drawn > (uint64_t)sp->nnz * 1000 + (1ULL << 26))
            return BTC_ERR_RANGE;  // distribution too concentrated for the requested count
    }
    std::vector<PartSet>().swap(sets);
    const int64_t n = (int64_t)keys.size();
    const int R = sp->gt_rank;
    // ground-truth factors
    std::vector<double> gt[3];
    for (int a = 0; a < 3 && R > 0; a++) {
        const int64_t m = (int64_t)dims[a] * R;
        gt[a].resize((size_t)m);
        run(m >= (1 << 20) ? T : 1, [&](int t) {
            const int nt = m >= (1 << 20) ? T : 1;
            for (int64_t i = m * t / nt; i < m * (t + 1) / nt; i++)
                gt[a][(size_t)i] = sp->gt_std * normal(hash4(sp->seed, 21 + a, (uint64_t)i, 0),
                                                       hash4(sp->seed, 21 + a, (uint64_t)i, 1));
        });
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
    // train and test entries keep their order; ranges of entries are split
    // on threads, each writing at the offsets the ranges before it leave
    const int TS = n >= (1 << 20) ? T : 1;
    std::vector<int64_t> na((size_t)TS + 1, 0), nbv((size_t)TS + 1, 0);
    run(TS, [&](int t) {
        const int64_t lo = n * t / TS, hi = n * (t + 1) / TS;
        int64_t c = 0;
        for (int64_t i = lo; i < hi; i++)
            c += is_train[(size_t)i];
        na[(size_t)t + 1] = c;
        nbv[(size_t)t + 1] = (hi - lo) - c;
    });
    for (int t = 0; t < TS; t++) {
        na[(size_t)t + 1] += na[(size_t)t];
        nbv[(size_t)t + 1] += nbv[(size_t)t];
    }
    const int64_t a = na[(size_t)TS], b = nbv[(size_t)TS];
    *txyz = (int32_t*)std::malloc(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(a, 1));
    *tval = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(a, 1));
    *sxyz = (int32_t*)std::malloc(sizeof(int32_t) * 3 * (size_t)std::max<int64_t>(b, 1));
    *sval = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(b, 1));
    if (!*txyz || !*tval || !*sxyz || !*sval)
        return BTC_ERR_ALLOC;
    run(TS, [&](int t) {
        const int64_t lo = n * t / TS, hi = n * (t + 1) / TS;
        int64_t ia = na[(size_t)t], ib = nbv[(size_t)t];
        for (int64_t i = lo; i < hi; i++) {
            if (is_train[(size_t)i]) {
                std::memcpy(*txyz + 3 * ia, &xyz[3 * i], 12);
                (*tval)[ia++] = val[(size_t)i];
            } else {
                std::memcpy(*sxyz + 3 * ib, &xyz[3 * i], 12);
                (*sval)[ib++] = val[(size_t)i];
            }
        }
    });
    *ntr = a;
    *nte = b;
    return BTC_OK;
}

}  // extern "C"
