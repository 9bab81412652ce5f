// Tile construction for the staged kernel (see tiles.h).
//
// A scheduled block's entries are taken in block order and cut into tiles
// when the tile reaches `wave` entries (the reference kernel's concurrency
// unit: one pass of thread_size threads over a slot, sgd_Kernel.cu:358-392)
// or when one more entry would need more than `cap` distinct rows.  For each
// mode the tile's entries are counting-sorted by row (CSR) and every row's
// list is split into owner segments of at most `seg` entries; a segment is
// the unit one lane group reduces before a single shared-memory add.
#include "tiles.h"

#include <algorithm>
#include <cstring>

namespace btc {

void build_tiles(const Schedule& s, const int32_t* xyz, const double* val, int I, int J, int K, int cap,
                 int wave, int seg, bool want64, TileSet& out)
{
    out = TileSet();
    const int dims[3] = {I, J, K};
    std::vector<int> stamp[3], loc[3];
    for (int a = 0; a < 3; a++) {
        stamp[a].assign((size_t)dims[a], -1);
        loc[a].assign((size_t)dims[a], 0);
    }
    out.block_tile0.assign(s.blocks.size(), -1);
    out.block_ntiles.assign(s.blocks.size(), 0);
    int tile_id = 0;
    std::vector<int32_t> rows_m[3];
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
        for (int a = 0; a < 3; a++)
            rows_m[a].clear();
        tile_id++;
    };

    for (size_t k = 0; k < s.slot_block.size(); k++) {
        const int b = s.slot_block[k];
        if (out.block_tile0[(size_t)b] >= 0)
            continue;
        out.block_tile0[(size_t)b] = (int)out.tiles.size();
        for (int32_t e : s.blocks[(size_t)b].ent) {
            const int32_t* c = xyz + 3 * (int64_t)e;
            int need = 0;
            for (int a = 0; a < 3; a++)
                need += stamp[a][(size_t)c[a]] != tile_id;
            int nrows = (int)(rows_m[0].size() + rows_m[1].size() + rows_m[2].size());
            if (!cur.empty() && ((int)cur.size() >= wave || nrows + need > cap)) {
                close();
            }
            Ent q;
            q.e = e;
            for (int a = 0; a < 3; a++) {
                if (stamp[a][(size_t)c[a]] != tile_id) {
                    stamp[a][(size_t)c[a]] = tile_id;
                    loc[a][(size_t)c[a]] = (int)rows_m[a].size();
                    rows_m[a].push_back(c[a]);
                }
                q.l[a] = (uint16_t)loc[a][(size_t)c[a]];
            }
            cur.push_back(q);
        }
        close();
        out.block_ntiles[(size_t)b] = (int)out.tiles.size() - out.block_tile0[(size_t)b];
    }
}

}  // namespace btc
