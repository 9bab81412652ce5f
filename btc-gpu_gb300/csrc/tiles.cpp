// Tile construction for the staged kernel (see tiles.h).
//
// A scheduled block's entries are taken in block order and cut into tiles
// when the tile reaches `wave` entries (the reference kernel's concurrency
// unit: one pass of thread_size threads over a slot, sgd_Kernel.cu:358-392),
// when one more entry would need more than `cap` distinct rows, or when it
// would put a row into the tile for the (repeat + 1)-th time.  Every entry of
// a tile reads the rows as they were when the tile started, so a row met c
// times in one tile takes c updates computed from one snapshot: a Jacobi
// step whose gain grows as lr * c * |other rows|^2, which diverged on skewed
// tensors (hot rows met hundreds of times per tile) once the factors had
// grown; the repeat bound keeps c small.  For each
// mode the tile's entries are counting-sorted by row (CSR) and every row's
// list is split into owner segments of at most `seg` entries; a segment is
// the unit one lane group reduces before a single shared-memory add.
#include "tiles.h"

#include <algorithm>
#include <cstring>
#include <thread>

namespace btc {
namespace {

// The tiles of blocks blk[0..nb), in that order, into `out` (offsets local
// to `out`); first[i] / count[i] receive block blk[i]'s first tile and tile
// count.
void build_range(const Schedule& s, const int32_t* xyz, const double* val, const int* dims, int cap, int wave,
                 int seg, int repeat, bool want64, const int* blk, size_t nb, TileSet& out, int* first, int* count)
{
    std::vector<int> stamp[3], loc[3];
    for (int a = 0; a < 3; a++) {
        stamp[a].assign((size_t)dims[a], -1);
        loc[a].assign((size_t)dims[a], 0);
    }
    int tile_id = 0;
    std::vector<int32_t> rows_m[3];
    std::vector<int32_t> uses_m[3];  // entries of the current tile per staged row
    struct Ent {
        int32_t e;
        uint16_t l[3];
    };
    std::vector<Ent> cur;
    std::vector<int> cnt, start;
    std::vector<uint16_t> order;

    auto close = [&]() {
        if (cur.empty())
            return;
        TileHdr h{};
        const int nx = (int)rows_m[0].size(), ny = (int)rows_m[1].size(), nz = (int)rows_m[2].size();
        h.roff = (long long)out.rows.size();
        h.eoff = (long long)out.ent.size();
        h.soff = (long long)out.segs.size();
        h.coff = (long long)out.csr.size();
        h.n = (int)cur.size();
        h.nrows = nx + ny + nz;
        h.nx = nx;
        h.ny = ny;
        for (int a = 0; a < 3; a++)
            out.rows.insert(out.rows.end(), rows_m[a].begin(), rows_m[a].end());
        const int base[3] = {0, nx, nx + ny};
        for (const Ent& q : cur) {
            float fv = (float)val[q.e];
            int bits;
            std::memcpy(&bits, &fv, 4);
            int4 v;
            v.x = (int)q.l[0] | ((int)(q.l[1] + base[1]) << 16);
            v.y = (int)(q.l[2] + base[2]);
            v.z = 0;
            v.w = bits;
            out.ent.push_back(v);
        }
        if (want64)
            for (const Ent& q : cur)
                out.val64.push_back(val[q.e]);
        const int nm[3] = {nx, ny, nz};
        for (int a = 0; a < 3; a++) {
            cnt.assign((size_t)nm[a] + 1, 0);
            for (const Ent& q : cur)
                cnt[q.l[a] + 1]++;
            for (int r = 0; r < nm[a]; r++)
                cnt[(size_t)r + 1] += cnt[(size_t)r];
            start.assign(cnt.begin(), cnt.end());
            order.assign(cur.size(), 0);
            for (size_t i = 0; i < cur.size(); i++)
                order[(size_t)start[cur[i].l[a]]++] = (uint16_t)i;
            out.csr.insert(out.csr.end(), order.begin(), order.end());
            for (int r = 0; r < nm[a]; r++) {
                for (int b = cnt[(size_t)r]; b < cnt[(size_t)r + 1]; b += seg) {
                    int c = std::min(seg, cnt[(size_t)r + 1] - b);
                    out.segs.push_back(make_int4(r + base[a], a, b, c));
                }
            }
        }
        while (out.csr.size() % 8)
            out.csr.push_back(0);
        h.nseg = (int)((long long)out.segs.size() - h.soff);
        out.max_rows = std::max(out.max_rows, h.nrows);
        out.max_n = std::max(out.max_n, h.n);
        out.tiles.push_back(h);
        cur.clear();
        for (int a = 0; a < 3; a++) {
            rows_m[a].clear();
            uses_m[a].clear();
        }
        tile_id++;
    };

    for (size_t i = 0; i < nb; i++) {
        const int b = blk[i];
        first[i] = (int)out.tiles.size();
        for (int32_t e : s.blocks[(size_t)b].ent) {
            const int32_t* c = xyz + 3 * (int64_t)e;
            int need = 0;
            bool full_row = false;
            for (int a = 0; a < 3; a++) {
                const bool in = stamp[a][(size_t)c[a]] == tile_id;
                need += !in;
                full_row |= in && uses_m[a][(size_t)loc[a][(size_t)c[a]]] >= repeat;
            }
            int nrows = (int)(rows_m[0].size() + rows_m[1].size() + rows_m[2].size());
            if (!cur.empty() && ((int)cur.size() >= wave || nrows + need > cap || full_row)) {
                close();
            }
            Ent q;
            q.e = e;
            for (int a = 0; a < 3; a++) {
                if (stamp[a][(size_t)c[a]] != tile_id) {
                    stamp[a][(size_t)c[a]] = tile_id;
                    loc[a][(size_t)c[a]] = (int)rows_m[a].size();
                    rows_m[a].push_back(c[a]);
                    uses_m[a].push_back(0);
                }
                q.l[a] = (uint16_t)loc[a][(size_t)c[a]];
                uses_m[a][(size_t)q.l[a]]++;
            }
            cur.push_back(q);
        }
        close();
        count[i] = (int)out.tiles.size() - first[i];
    }
}

}  // namespace

// Blocks are tiled independently (a tile never spans two blocks), so the
// blocks, in order of first use by the slots, are split into contiguous
// runs of about equal entry count, one per thread, and the runs' tile sets
// are concatenated in order with their offsets moved: the result does not
// depend on the thread count.
void build_tiles(const Schedule& s, const int32_t* xyz, const double* val, int I, int J, int K, int cap,
                 int wave, int seg, int repeat, bool want64, TileSet& out, int threads)
{
    out = TileSet();
    const int dims[3] = {I, J, K};
    out.block_tile0.assign(s.blocks.size(), -1);
    out.block_ntiles.assign(s.blocks.size(), 0);
    std::vector<int> order;
    std::vector<long long> ent_before(1, 0);
    {
        std::vector<char> seen(s.blocks.size(), 0);
        for (int b : s.slot_block)
            if (!seen[(size_t)b]) {
                seen[(size_t)b] = 1;
                order.push_back(b);
                ent_before.push_back(ent_before.back() + (long long)s.blocks[(size_t)b].ent.size());
            }
    }
    const long long total = ent_before.back();
    int T = std::max(1, std::min(threads, 64));
    if (total < (1LL << 20))
        T = 1;  // small inputs: one run
    std::vector<size_t> cut((size_t)T + 1, 0);
    for (int t = 1; t < T; t++)
        cut[(size_t)t] = (size_t)(std::lower_bound(ent_before.begin(), ent_before.end(), total * t / T) -
                                  ent_before.begin());
    cut[(size_t)T] = order.size();
    for (int t = 1; t <= T; t++)
        cut[(size_t)t] = std::max(cut[(size_t)t], cut[(size_t)t - 1]);
    std::vector<TileSet> part((size_t)T);
    std::vector<int> first(order.size()), count(order.size());
    auto work = [&](int t) {
        const size_t lo = cut[(size_t)t], hi = cut[(size_t)t + 1];
        build_range(s, xyz, val, dims, cap, wave, seg, std::max(1, repeat), want64, order.data() + lo, hi - lo,
                    part[(size_t)t],
                    first.data() + lo, count.data() + lo);
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++)
        pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool)
        th.join();
    for (int t = 0; t < T; t++) {
        int tile_base = 0;
        for (int u = 0; u < t; u++)
            tile_base += (int)part[(size_t)u].tiles.size();
        for (size_t i = cut[(size_t)t]; i < cut[(size_t)t + 1]; i++) {
            // a block without entries has no tiles and no first tile
            out.block_tile0[(size_t)order[i]] = count[i] > 0 ? tile_base + first[i] : -1;
            out.block_ntiles[(size_t)order[i]] = count[i];
        }
        out.max_rows = std::max(out.max_rows, part[(size_t)t].max_rows);
        out.max_n = std::max(out.max_n, part[(size_t)t].max_n);
    }
    if (T == 1) {  // one run: its offsets are already the final ones
        out.tiles.swap(part[0].tiles);
        out.ent.swap(part[0].ent);
        out.csr.swap(part[0].csr);
        out.segs.swap(part[0].segs);
        out.rows.swap(part[0].rows);
        out.val64.swap(part[0].val64);
        return;
    }
    // runs are copied into place in parallel, each run's offsets moved by the
    // sizes of the runs before it (every run's CSR length is a multiple of 8)
    struct Off {
        size_t t, e, c, s, r, v;
    };
    std::vector<Off> off((size_t)T + 1, Off{0, 0, 0, 0, 0, 0});
    for (int t = 0; t < T; t++) {
        const TileSet& p = part[(size_t)t];
        const Off& a = off[(size_t)t];
        off[(size_t)t + 1] = Off{a.t + p.tiles.size(), a.e + p.ent.size(), a.c + p.csr.size(),
                                 a.s + p.segs.size(), a.r + p.rows.size(), a.v + p.val64.size()};
    }
    const Off& all = off[(size_t)T];
    out.tiles.resize(all.t);
    out.ent.resize(all.e);
    out.csr.resize(all.c);
    out.segs.resize(all.s);
    out.rows.resize(all.r);
    out.val64.resize(all.v);
    auto place = [&](int t) {
        TileSet& p = part[(size_t)t];
        const Off& a = off[(size_t)t];
        for (size_t i = 0; i < p.tiles.size(); i++) {
            TileHdr h = p.tiles[i];
            h.eoff += (long long)a.e;
            h.roff += (long long)a.r;
            h.soff += (long long)a.s;
            h.coff += (long long)a.c;
            out.tiles[a.t + i] = h;
        }
        std::copy(p.ent.begin(), p.ent.end(), out.ent.begin() + (long long)a.e);
        std::copy(p.csr.begin(), p.csr.end(), out.csr.begin() + (long long)a.c);
        std::copy(p.segs.begin(), p.segs.end(), out.segs.begin() + (long long)a.s);
        std::copy(p.rows.begin(), p.rows.end(), out.rows.begin() + (long long)a.r);
        std::copy(p.val64.begin(), p.val64.end(), out.val64.begin() + (long long)a.v);
        p = TileSet();
    };
    pool.clear();
    for (int t = 1; t < T; t++)
        pool.emplace_back(place, t);
    place(0);
    for (auto& th : pool)
        th.join();
}

}  // namespace btc
