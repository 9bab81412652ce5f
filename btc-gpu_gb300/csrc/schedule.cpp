// Host-side schedule builder (see schedule.h).
//
// Same results as the reference, different machinery:
//  * blocking (block.cu:154-401): the tree keeps integer prefix codes instead
//    of vector<bool> copies; each entry is routed by three float bucket codes
//    computed exactly as hx does (block.cu:38-50), including the split bit
//    taken at the GLOBAL level of the axis (block.cu:215-216, 285-286,
//    353-354) and the re-split of a full or empty child (block.cu:237-253);
//  * strata (block.cu:1024-1148): the reference's repeated greedy scans equal
//    a first-fit assignment of blocks in ascending id order (a block joins the
//    first stratum whose members it conflicts with on no axis), computed here
//    with 64-bin interval masks as a prefilter;
//  * padding (block.cu:545-565, 660-697): per group, candidates are scanned
//    in (nnz, id) order so the first zero-conflict candidate ends the scan;
//    groups are independent, so they are padded on several threads;
//  * coe weights (block.cu:470-513): union-find per axis inside each group.
#include "schedule.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <set>
#include <sstream>
#include <thread>

namespace btc {
namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Node {
    int32_t left = -1, right = -1, block = 0, h = 1;
    int32_t len[3] = {1, 1, 1};
    uint64_t code[3] = {0, 0, 0};
};

inline int axis_of_h(int h)
{
    int t = h % 3;
    return t == 1 ? 0 : (t == 2 ? 1 : 2);
}

// hx (block.cu:38-50): n_1 = (end+1)/2^(level-1) rounded to float, then
// floor(num / n_1) in float.
struct Axis {
    float n1[66];
    void init(int end)
    {
        for (int l = 1; l <= 65; l++)
            n1[l] = (float)((double)(end + 1) / std::ldexp(1.0, l - 1));
    }
    inline bool hx(int level, int num, int64_t& out) const
    {
        float q = (float)num / n1[level];
        float f = std::floor(q);
        if (!(f >= 0.0f) || f >= 2147483648.0f)
            return false;
        out = (int64_t)f;
        return true;
    }
};

inline uint64_t prefix_bits(int64_t n2, int g, int L)
{
    if (L <= 1)
        return 0;
    return ((uint64_t)n2 >> (g - L)) & ((1ULL << (L - 1)) - 1ULL);
}

inline uint64_t left_align(uint64_t code, int level)
{
    int m = level - 1;
    return m == 0 ? 0 : code << (64 - m);
}

inline uint64_t bin_mask(uint64_t lcode, int level)
{
    int m = level - 1;
    uint64_t first = lcode >> 58;
    if (m >= 6)
        return 1ULL << first;
    int count = 1 << (6 - m);
    uint64_t span = count == 64 ? ~0ULL : ((1ULL << count) - 1ULL);
    return span << first;
}

// find_conflict_x (block.cu:413-430) on left-aligned codes
inline bool axis_conflict(const BlockRec& a, const BlockRec& b, int ax)
{
    int m = std::min(a.level[ax], b.level[ax]) - 1;
    if (m == 0)
        return true;
    return ((a.lcode[ax] ^ b.lcode[ax]) >> (64 - m)) == 0;
}

void finish_block_codes(BlockRec& b)
{
    for (int a = 0; a < 3; a++) {
        b.lcode[a] = left_align(b.code[a], b.level[a]);
        b.bins[a] = bin_mask(b.lcode[a], b.level[a]);
    }
}

// Route one entry from `node` down to a leaf with bucket codes pc at global
// levels g (search_block, block.cu:64-88).
// The left child of a node split on axis a has len[a] + 1 and code[a] << 1
// (Create_Btree below), so each step reads the parent only.
inline int route(const std::vector<Node>& nodes, int node, const int64_t* pc, const int* g)
{
    for (;;) {
        const Node& P = nodes[(size_t)node];
        if (P.left < 0)
            return node;
        const int a = axis_of_h(P.h);
        node = prefix_bits(pc[a], g[a], P.len[a] + 1) == (P.code[a] << 1) ? P.left : P.right;
    }
}

// The tree for routing only, 16 bytes a node: a split node's children sit
// at left and left + 1 (both passes allocate them as a pair); a leaf has
// left = -1.  want / len: the left child's code and length on the split
// axis.
struct RNode {
    int32_t left = -1;
    uint8_t axis = 0, len = 0;
    uint16_t pad = 0;
    uint64_t want = 0;
};

inline RNode rnode_of(const Node& P)
{
    RNode r;
    if (P.left >= 0) {
        const int a = axis_of_h(P.h);
        r.left = P.left;
        r.axis = (uint8_t)a;
        r.len = (uint8_t)(P.len[a] + 1);
        r.want = P.code[a] << 1;
    }
    return r;
}

inline int route_fast(const RNode* rn, int node, const int64_t* pc, const int* g)
{
    for (;;) {
        const RNode& P = rn[node];
        if (P.left < 0)
            return node;
        node = prefix_bits(pc[P.axis], g[P.axis], P.len) == P.want ? P.left : P.left + 1;
    }
}

btc_status blocking(const int32_t* xyz, int64_t n, int I, int J, int K, int bs, int threads, Schedule& s)
{
    Axis ax[3];
    ax[0].init(I);
    ax[1].init(J);
    ax[2].init(K);
    int g[3] = {1, 1, 1};
    std::vector<Node> nodes(1);
    std::vector<BlockRec>& blocks = s.blocks;
    blocks.clear();
    blocks.reserve((size_t)std::max<int64_t>(16, n / std::max(1, bs) * 2));
    blocks.emplace_back();
    for (int a = 0; a < 3; a++) {
        blocks[0].level[a] = 1;
        blocks[0].code[a] = 0;
    }
    blocks[0].ent.reserve(bs);
    std::vector<int32_t> t1, t2;
    t1.reserve(bs + 1);
    t2.reserve(bs + 1);

    // Entries are routed in chunks on several threads against a snapshot of
    // the tree and of the global levels, then inserted in order.  Internal
    // nodes never change once split, so an entry whose snapshot leaf is still
    // a leaf has the route the reference would compute now; a leaf that split
    // since the snapshot is descended further, and a change of a global level
    // (which changes every bucket code) re-routes from the root.
    const int64_t CH = 1 << 16;
    // leaf_block: the block each entry's snapshot leaf held, for prefetching
    std::vector<int> leaf((size_t)std::min<int64_t>(n, CH)), leaf_block((size_t)std::min<int64_t>(n, CH));
    std::vector<int64_t> codes((size_t)std::min<int64_t>(n, CH) * 3);
    std::atomic<int> bad(0);
    for (int64_t base = 0; base < n; base += CH) {
        const int64_t cn = std::min<int64_t>(CH, n - base);
        const int g0[3] = {g[0], g[1], g[2]};
        {
            auto work = [&](int64_t lo, int64_t hi) {
                for (int64_t k = lo; k < hi; k++) {
                    const int32_t* p = xyz + 3 * (base + k);
                    int64_t* pc = &codes[(size_t)(3 * k)];
                    for (int a = 0; a < 3; a++)
                        if (!ax[a].hx(g0[a], p[a], pc[a])) {
                            bad = 1;
                            return;
                        }
                    leaf[(size_t)k] = route(nodes, 0, pc, g0);
                    leaf_block[(size_t)k] = nodes[(size_t)leaf[(size_t)k]].block;
                }
            };
            const int nt = std::max(1, std::min<int>(threads, (int)(cn / 4096) + 1));
            std::vector<std::thread> pool;
            for (int t = 1; t < nt; t++)
                pool.emplace_back(work, cn * t / nt, cn * (t + 1) / nt);
            work(0, cn / nt);
            for (auto& t : pool)
                t.join();
            if (bad)
                return BTC_ERR_RANGE;
        }
      for (int64_t k = 0; k < cn; k++) {
        // The appends land in scattered blocks: fetch ahead the record of the
        // block an entry 16 further was routed to and the tail of the entry
        // list 8 further (hints only; a block split since the snapshot
        // merely wastes the fetch).
        if (k + 16 < cn)
            __builtin_prefetch(&blocks[(size_t)leaf_block[(size_t)(k + 16)]]);
        if (k + 8 < cn) {
            const BlockRec& F = blocks[(size_t)leaf_block[(size_t)(k + 8)]];
            __builtin_prefetch(F.ent.data() + F.ent.size(), 1);
        }
        const int64_t i = base + k;
        const int32_t* p = xyz + 3 * i;
        int64_t pc[3];
        int node;
        if (g[0] == g0[0] && g[1] == g0[1] && g[2] == g0[2]) {
            pc[0] = codes[(size_t)(3 * k)];
            pc[1] = codes[(size_t)(3 * k + 1)];
            pc[2] = codes[(size_t)(3 * k + 2)];
            node = route(nodes, leaf[(size_t)k], pc, g);
        } else {
            for (int a = 0; a < 3; a++)
                if (!ax[a].hx(g[a], p[a], pc[a]))
                    return BTC_ERR_RANGE;
            node = route(nodes, 0, pc, g);
        }
        int id = nodes[node].block;
        if ((int)blocks[id].ent.size() < bs) {
            blocks[id].ent.push_back((int32_t)i);
            continue;
        }
        bool done = false;
        while (!done) {
            int a;
            {
                const BlockRec& B = blocks[id];
                if (B.level[0] == B.level[1] && B.level[1] == B.level[2])
                    a = 0;
                else if (B.level[1] < B.level[0])
                    a = 1;
                else if (B.level[2] < B.level[1])
                    a = 2;
                else
                    return BTC_ERR_STATE;
            }
            blocks[id].level[a]++;
            if (blocks[id].level[a] > g[a])
                g[a] = blocks[id].level[a];
            if (g[a] > 63)
                return BTC_ERR_RANGE;
            // Create_Btree (block.cu:90-152)
            int nb = (int)blocks.size();
            {
                int l = (int)nodes.size();
                nodes.resize(nodes.size() + 2);
                Node& P = nodes[node];
                int ta = axis_of_h(P.h);
                Node L = P, R = P;
                L.h = R.h = P.h + 1;
                L.left = L.right = R.left = R.right = -1;
                L.len[ta] = R.len[ta] = P.len[ta] + 1;
                L.code[ta] = P.code[ta] << 1;
                R.code[ta] = (P.code[ta] << 1) | 1ULL;
                L.block = id;
                R.block = nb;
                P.block = -1;
                P.left = l;
                P.right = l + 1;
                nodes[l] = L;
                nodes[l + 1] = R;
            }
            blocks.emplace_back();
            BlockRec& NB = blocks[nb];
            BlockRec& B = blocks[id];
            for (int q = 0; q < 3; q++) {
                NB.level[q] = B.level[q];
                NB.code[q] = B.code[q];
            }
            NB.code[a] = (B.code[a] << 1) | 1ULL;
            B.code[a] = B.code[a] << 1;
            t1.clear();
            t2.clear();
            // a split re-buckets the block's entries: their coordinates lie
            // scattered over the whole input, so they are fetched ahead
            for (size_t j = 0; j < B.ent.size(); j++) {
                if (j + 16 < B.ent.size())
                    __builtin_prefetch(xyz + 3 * (int64_t)B.ent[j + 16] + a);
                const int32_t e = B.ent[j];
                int64_t hv;
                if (!ax[a].hx(g[a], xyz[3 * (int64_t)e + a], hv))
                    return BTC_ERR_RANGE;
                ((hv & 1) == 0 ? t1 : t2).push_back(e);
            }
            int64_t hp;
            if (!ax[a].hx(g[a], p[a], hp))
                return BTC_ERR_RANGE;
            int bit = (int)(hp & 1);
            if ((int)t1.size() < bs && (int)t2.size() < bs) {
                done = true;
                (bit == 0 ? t1 : t2).push_back((int32_t)i);
                B.ent.assign(t1.begin(), t1.end());
                NB.ent.assign(t2.begin(), t2.end());
            } else if (bit == 0) {
                B.ent.assign(t1.begin(), t1.end());
                NB.ent.assign(t2.begin(), t2.end());
                node = nodes[node].left;
            } else {
                // the reference stores t1 then t2 into the NEW block; the old
                // block keeps its previous entries (block.cu:244-253)
                NB.ent.assign(t2.begin(), t2.end());
                id = nb;
                node = nodes[node].right;
            }
            if ((int)NB.ent.capacity() < bs)
                NB.ent.reserve(bs);
        }
      }
    }
    for (auto& b : blocks)
        finish_block_codes(b);
    for (int a = 0; a < 3; a++)
        s.global_levels[a] = g[a];
    return BTC_OK;
}

// The same blocking on host threads, bit-identical to blocking() above.
//
// Insertions interact in two ways only: through the leaf an entry lands in
// (a subtree's evolution depends only on the entries routed into it, in
// order, since internal nodes never change), and through the global levels
// (every bucket code, and the split bit, is taken at them).  So entries are
// processed in chunks: each chunk is routed against a snapshot of the tree,
// grouped by snapshot leaf, and every group replays its entries into its own
// subtree on a thread with the global levels held fixed.  A group stops at
// the first entry whose split would raise a global level (an "event"): the
// chunk is then replayed up to the earliest event, that entry is inserted
// alone (raising the level), and the next chunk starts after it.  New blocks
// receive their ids in the order the serial loop would allocate them: by
// entry, then by split within the entry's re-split loop.
namespace par {

struct LBlock {
    int32_t level[3];
    uint64_t code[3];
    std::vector<int32_t> ent;
};

struct Group {
    int32_t leaf = 0, b0 = 0;      // snapshot leaf (global node) and its block
    int32_t first = 0, count = 0;  // the group's entries in the chunk's grouped order
    int64_t event = -1;            // chunk index of the entry that would raise a global level
    bool bad = false;              // a bucket code out of range
    bool split = false;            // the leaf split inside the chunk
    int32_t napp = 0;              // entries appended to b0 (no split): app[first, first + napp)
    std::vector<Node> nodes;       // when split: local subtree, [0] = the leaf
    std::vector<LBlock> lb;        // when split: [0] = b0, then new blocks in creation order
    std::vector<uint64_t> log;     // (entry << 8 | split seq) of each new block lb[1..]
};

inline int choose_axis(const int32_t* lv)
{
    if (lv[0] == lv[1] && lv[1] == lv[2])
        return 0;
    if (lv[1] < lv[0])
        return 1;
    if (lv[2] < lv[1])
        return 2;
    return -1;
}

// Replays the group's entries (chunk indices ascending, below `limit`) into
// the subtree of its snapshot leaf with global levels g fixed.
void run_group(Group& G, const int32_t* pts, const int64_t* codes, int64_t base, int64_t limit, const int* g,
               int bs, const int32_t* xyz, const Axis* ax, const std::vector<Node>& gnodes,
               const std::vector<BlockRec>& blocks, int32_t* app)
{
    G.event = -1;
    G.bad = false;
    G.split = false;
    G.napp = 0;
    G.nodes.clear();
    G.lb.clear();
    G.log.clear();
    const std::vector<int32_t>& e0 = blocks[(size_t)G.b0].ent;
    std::vector<int32_t> t1, t2;
    for (int32_t q = 0; q < G.count; q++) {
        const int64_t k = pts[G.first + q];
        if (k >= limit)
            return;
        const int64_t i = base + k;
        const int64_t* pc = codes + 3 * k;
        int node = 0, id = 0;
        if (!G.split) {
            if ((int64_t)e0.size() + G.napp < bs) {
                app[G.first + G.napp++] = (int32_t)i;
                continue;
            }
            // the leaf's block is full: from here on the subtree is local
            G.split = true;
            G.nodes.push_back(gnodes[(size_t)G.leaf]);
            G.nodes[0].block = 0;
            LBlock b;
            const BlockRec& B0 = blocks[(size_t)G.b0];
            for (int a = 0; a < 3; a++) {
                b.level[a] = B0.level[a];
                b.code[a] = B0.code[a];
            }
            b.ent.reserve((size_t)bs + 1);
            b.ent.assign(e0.begin(), e0.end());
            b.ent.insert(b.ent.end(), app + G.first, app + G.first + G.napp);
            G.lb.push_back(std::move(b));
        } else {
            node = route(G.nodes, 0, pc, g);
            id = G.nodes[(size_t)node].block;
            if ((int)G.lb[(size_t)id].ent.size() < bs) {
                G.lb[(size_t)id].ent.push_back((int32_t)i);
                continue;
            }
        }
        const int32_t* p = xyz + 3 * i;
        int seq = 0;
        for (bool done = false; !done;) {
            const int a = choose_axis(G.lb[(size_t)id].level);
            if (a < 0 || G.lb[(size_t)id].level[a] + 1 > g[a]) {
                G.event = k;  // the serial pass takes this entry
                return;
            }
            G.lb[(size_t)id].level[a]++;
            const int nb = (int)G.lb.size();
            {
                const int l = (int)G.nodes.size();
                G.nodes.resize(G.nodes.size() + 2);
                Node& P = G.nodes[(size_t)node];
                const int ta = axis_of_h(P.h);
                Node L = P, R = P;
                L.h = R.h = P.h + 1;
                L.left = L.right = R.left = R.right = -1;
                L.len[ta] = R.len[ta] = P.len[ta] + 1;
                L.code[ta] = P.code[ta] << 1;
                R.code[ta] = (P.code[ta] << 1) | 1ULL;
                L.block = id;
                R.block = nb;
                P.block = -1;
                P.left = l;
                P.right = l + 1;
                G.nodes[(size_t)l] = L;
                G.nodes[(size_t)l + 1] = R;
            }
            G.lb.emplace_back();
            G.log.push_back(((uint64_t)k << 8) | (uint64_t)seq++);
            LBlock& NB = G.lb[(size_t)nb];
            LBlock& B = G.lb[(size_t)id];
            for (int q2 = 0; q2 < 3; q2++) {
                NB.level[q2] = B.level[q2];
                NB.code[q2] = B.code[q2];
            }
            NB.code[a] = (B.code[a] << 1) | 1ULL;
            B.code[a] = B.code[a] << 1;
            t1.clear();
            t2.clear();
            for (int32_t e : B.ent) {
                int64_t hv;
                if (!ax[a].hx(g[a], xyz[3 * (int64_t)e + a], hv)) {
                    G.bad = true;
                    return;
                }
                ((hv & 1) == 0 ? t1 : t2).push_back(e);
            }
            int64_t hp;
            if (!ax[a].hx(g[a], p[a], hp)) {
                G.bad = true;
                return;
            }
            const int bit = (int)(hp & 1);
            if ((int)t1.size() < bs && (int)t2.size() < bs) {
                done = true;
                (bit == 0 ? t1 : t2).push_back((int32_t)i);
                B.ent.assign(t1.begin(), t1.end());
                NB.ent.assign(t2.begin(), t2.end());
            } else if (bit == 0) {
                B.ent.assign(t1.begin(), t1.end());
                NB.ent.assign(t2.begin(), t2.end());
                node = G.nodes[(size_t)node].left;
            } else {
                // the old block keeps its entries (block.cu:244-253)
                NB.ent.assign(t2.begin(), t2.end());
                id = nb;
                node = G.nodes[(size_t)node].right;
            }
        }
    }
}

}  // namespace par

btc_status blocking_parallel(const int32_t* xyz, int64_t n, int I, int J, int K, int bs, int threads,
                             Schedule& s)
{
    using namespace par;
    Axis ax[3];
    ax[0].init(I);
    ax[1].init(J);
    ax[2].init(K);
    int g[3] = {1, 1, 1};
    std::vector<Node> nodes(1);
    std::vector<RNode> rnodes(1);
    std::vector<BlockRec>& blocks = s.blocks;
    blocks.clear();
    blocks.reserve((size_t)std::max<int64_t>(16, n / std::max(1, bs) * 2));
    blocks.emplace_back();
    for (int a = 0; a < 3; a++) {
        blocks[0].level[a] = 1;
        blocks[0].code[a] = 0;
    }
    const int T = std::max(1, std::min(threads, 64));
    const int64_t CH_MIN = 1 << 12, CH_MAX = 1 << 22;
    const int64_t cap = std::min<int64_t>(n, CH_MAX);
    std::vector<int64_t> codes((size_t)cap * 3);
    std::vector<int32_t> leaf((size_t)cap), pts((size_t)cap), app((size_t)cap);
    std::vector<int32_t> group_of_node;
    std::vector<std::vector<int32_t>> tcount, tfirst;  // per grouping thread: count per leaf, leaves first seen
    std::vector<Group> groups;
    std::vector<int32_t> order;  // groups by size, largest first
    std::vector<int32_t> t1, t2;

    // a pool that runs fn(t) for t in [0, T) and waits
    auto parallel = [&](int nt, const std::function<void(int)>& fn) {
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; t++)
            pool.emplace_back(fn, t);
        fn(0);
        for (auto& th : pool)
            th.join();
    };

    // the serial insertion of one entry from the root (blocking() above)
    auto insert_one = [&](int64_t i) -> btc_status {
        const int32_t* p = xyz + 3 * i;
        int64_t pc[3];
        for (int a = 0; a < 3; a++)
            if (!ax[a].hx(g[a], p[a], pc[a]))
                return BTC_ERR_RANGE;
        int node = route_fast(rnodes.data(), 0, pc, g);
        int id = nodes[(size_t)node].block;
        if ((int)blocks[(size_t)id].ent.size() < bs) {
            blocks[(size_t)id].ent.push_back((int32_t)i);
            return BTC_OK;
        }
        for (bool done = false; !done;) {
            const int a = choose_axis(blocks[(size_t)id].level);
            if (a < 0)
                return BTC_ERR_STATE;
            blocks[(size_t)id].level[a]++;
            if (blocks[(size_t)id].level[a] > g[a])
                g[a] = blocks[(size_t)id].level[a];
            if (g[a] > 63)
                return BTC_ERR_RANGE;
            const int nb = (int)blocks.size();
            {
                const int l = (int)nodes.size();
                nodes.resize(nodes.size() + 2);
                Node& P = nodes[(size_t)node];
                const int ta = axis_of_h(P.h);
                Node L = P, R = P;
                L.h = R.h = P.h + 1;
                L.left = L.right = R.left = R.right = -1;
                L.len[ta] = R.len[ta] = P.len[ta] + 1;
                L.code[ta] = P.code[ta] << 1;
                R.code[ta] = (P.code[ta] << 1) | 1ULL;
                L.block = id;
                R.block = nb;
                P.block = -1;
                P.left = l;
                P.right = l + 1;
                nodes[(size_t)l] = L;
                nodes[(size_t)l + 1] = R;
                rnodes.resize(nodes.size());
                rnodes[(size_t)node] = rnode_of(nodes[(size_t)node]);
                rnodes[(size_t)l] = RNode();
                rnodes[(size_t)l + 1] = RNode();
            }
            blocks.emplace_back();
            BlockRec& NB = blocks[(size_t)nb];
            BlockRec& B = blocks[(size_t)id];
            for (int q = 0; q < 3; q++) {
                NB.level[q] = B.level[q];
                NB.code[q] = B.code[q];
            }
            NB.code[a] = (B.code[a] << 1) | 1ULL;
            B.code[a] = B.code[a] << 1;
            t1.clear();
            t2.clear();
            for (int32_t e : B.ent) {
                int64_t hv;
                if (!ax[a].hx(g[a], xyz[3 * (int64_t)e + a], hv))
                    return BTC_ERR_RANGE;
                ((hv & 1) == 0 ? t1 : t2).push_back(e);
            }
            int64_t hp;
            if (!ax[a].hx(g[a], p[a], hp))
                return BTC_ERR_RANGE;
            const int bit = (int)(hp & 1);
            if ((int)t1.size() < bs && (int)t2.size() < bs) {
                done = true;
                (bit == 0 ? t1 : t2).push_back((int32_t)i);
                B.ent.assign(t1.begin(), t1.end());
                NB.ent.assign(t2.begin(), t2.end());
            } else if (bit == 0) {
                B.ent.assign(t1.begin(), t1.end());
                NB.ent.assign(t2.begin(), t2.end());
                node = nodes[(size_t)node].left;
            } else {
                NB.ent.assign(t2.begin(), t2.end());
                id = nb;
                node = nodes[(size_t)node].right;
            }
        }
        return BTC_OK;
    };

    int64_t ch = CH_MIN;
    for (int64_t base = 0; base < n;) {
        const int64_t cn = std::min(ch, n - base);
        // 1. bucket codes at the current global levels and snapshot leaves
        std::atomic<int> bad(0);
        {
            const int nt = std::max(1, std::min<int>(T, (int)(cn / 4096) + 1));
            parallel(nt, [&](int t) {
                const int64_t lo = cn * t / nt, hi = cn * (t + 1) / nt;
                for (int64_t k = lo; k < hi; k++) {
                    const int32_t* p = xyz + 3 * (base + k);
                    int64_t* pc = &codes[(size_t)(3 * k)];
                    for (int a = 0; a < 3; a++)
                        if (!ax[a].hx(g[a], p[a], pc[a])) {
                            bad = 1;
                            return;
                        }
                    leaf[(size_t)k] = route_fast(rnodes.data(), 0, pc, g);
                }
            });
        }
        if (bad)
            return BTC_ERR_RANGE;
        // 2. groups by snapshot leaf (numbered in order of first appearance
        //    in the chunk); each group's entries in chunk order.  Threads
        //    count their share of the chunk per leaf, then write their
        //    entries at the offsets the shares before them leave.
        if (group_of_node.size() < nodes.size())
            group_of_node.resize(nodes.size(), -1);
        const int ntg = std::max(1, std::min<int>(T, (int)(cn / 65536) + 1));
        if ((int)tcount.size() < ntg)
            tcount.resize((size_t)ntg);
        for (int t = 0; t < ntg; t++)
            if (tcount[(size_t)t].size() < nodes.size())
                tcount[(size_t)t].resize(nodes.size(), 0);
        tfirst.assign((size_t)ntg, std::vector<int32_t>());
        parallel(ntg, [&](int t) {
            const int64_t lo = cn * t / ntg, hi = cn * (t + 1) / ntg;
            std::vector<int32_t>& c = tcount[(size_t)t];
            for (int64_t k = lo; k < hi; k++) {
                const int32_t l = leaf[(size_t)k];
                if (c[(size_t)l]++ == 0)
                    tfirst[(size_t)t].push_back(l);
            }
        });
        int32_t ng = 0;
        for (int t = 0; t < ntg; t++)
            for (int32_t l : tfirst[(size_t)t]) {
                int32_t& q = group_of_node[(size_t)l];
                if (q >= 0)
                    continue;
                q = ng++;
                if ((int32_t)groups.size() < ng)
                    groups.emplace_back();
                Group& G = groups[(size_t)q];
                G.leaf = l;
                G.b0 = nodes[(size_t)l].block;
                G.count = 0;
            }
        {
            // per group, each thread's write offset; tcount becomes that offset
            int32_t o = 0;
            for (int32_t q = 0; q < ng; q++) {
                Group& G = groups[(size_t)q];
                G.first = o;
                for (int t = 0; t < ntg; t++) {
                    int32_t& c = tcount[(size_t)t][(size_t)G.leaf];
                    const int32_t k = c;
                    c = o;
                    o += k;
                }
                G.count = o - G.first;
            }
            parallel(ntg, [&](int t) {
                const int64_t lo = cn * t / ntg, hi = cn * (t + 1) / ntg;
                std::vector<int32_t>& c = tcount[(size_t)t];
                for (int64_t k = lo; k < hi; k++)
                    pts[(size_t)c[(size_t)leaf[(size_t)k]]++] = (int32_t)k;
            });
            for (int32_t q = 0; q < ng; q++) {
                group_of_node[(size_t)groups[(size_t)q].leaf] = -1;
                for (int t = 0; t < ntg; t++)
                    tcount[(size_t)t][(size_t)groups[(size_t)q].leaf] = 0;
            }
        }
        order.resize((size_t)ng);
        for (int32_t q = 0; q < ng; q++)
            order[(size_t)q] = q;
        std::sort(order.begin(), order.end(),
                  [&](int32_t a, int32_t b) { return groups[(size_t)a].count > groups[(size_t)b].count; });
        // 3. replay every group on the threads (twice when an event cuts the
        //    chunk short: the second pass stops before the earliest event)
        int64_t limit = cn, event = -1;
        for (int pass = 0; pass < 2; pass++) {
            std::atomic<int32_t> next(0);
            const int nt = std::max(1, std::min<int>(T, ng));
            parallel(nt, [&](int) {
                for (;;) {
                    const int32_t q = next.fetch_add(1);
                    if (q >= ng)
                        return;
                    run_group(groups[(size_t)order[(size_t)q]], pts.data(), codes.data(), base, limit, g, bs,
                              xyz, ax, nodes, blocks, app.data());
                }
            });
            event = -1;
            for (int32_t q = 0; q < ng; q++) {
                if (groups[(size_t)q].bad)
                    return BTC_ERR_RANGE;
                const int64_t e = groups[(size_t)q].event;
                if (e >= 0 && (event < 0 || e < event))
                    event = e;
            }
            if (event < 0)
                break;
            limit = event;  // replay up to the earliest event
        }
        if (event >= 0)
            return BTC_ERR_STATE;  // the second pass cannot meet an event
        // 4. commit: new block ids in serial allocation order, subtrees
        //    spliced under their leaves
        struct NewB {
            uint64_t key;
            int32_t group, local;
        };
        std::vector<NewB> nbs;
        std::vector<int32_t> node_off((size_t)ng + 1, 0);
        for (int32_t q = 0; q < ng; q++) {
            const Group& G = groups[(size_t)q];
            node_off[(size_t)q + 1] = node_off[(size_t)q] + (G.split ? (int32_t)G.nodes.size() - 1 : 0);
            if (G.split)
                for (size_t j = 0; j < G.log.size(); j++)
                    nbs.push_back(NewB{G.log[j], q, (int32_t)j + 1});
        }
        std::sort(nbs.begin(), nbs.end(), [](const NewB& a, const NewB& b) { return a.key < b.key; });
        const int32_t nb0 = (int32_t)blocks.size();
        std::vector<std::vector<int32_t>> lmap((size_t)ng);
        for (int32_t q = 0; q < ng; q++)
            if (groups[(size_t)q].split) {
                lmap[(size_t)q].assign(groups[(size_t)q].lb.size(), -1);
                lmap[(size_t)q][0] = groups[(size_t)q].b0;
            }
        for (size_t r = 0; r < nbs.size(); r++)
            lmap[(size_t)nbs[r].group][(size_t)nbs[r].local] = nb0 + (int32_t)r;
        blocks.resize(blocks.size() + nbs.size());
        const int32_t nn0 = (int32_t)nodes.size();
        nodes.resize(nodes.size() + (size_t)node_off[(size_t)ng]);
        rnodes.resize(nodes.size());
        {
            std::atomic<int32_t> next(0);
            const int nt = std::max(1, std::min<int>(T, ng / 64 + 1));
            parallel(nt, [&](int) {
                for (;;) {
                    const int32_t q = next.fetch_add(1);
                    if (q >= ng)
                        return;
                    Group& G = groups[(size_t)q];
                    if (!G.split) {
                        std::vector<int32_t>& e = blocks[(size_t)G.b0].ent;
                        e.insert(e.end(), app.data() + G.first, app.data() + G.first + G.napp);
                        continue;
                    }
                    const std::vector<int32_t>& m = lmap[(size_t)q];
                    for (size_t j = 0; j < G.lb.size(); j++) {
                        BlockRec& B = blocks[(size_t)m[j]];
                        for (int a = 0; a < 3; a++) {
                            B.level[a] = G.lb[j].level[a];
                            B.code[a] = G.lb[j].code[a];
                        }
                        B.ent.swap(G.lb[j].ent);
                        G.lb[j].ent.clear();
                    }
                    auto gnode = [&](int32_t l) { return l == 0 ? G.leaf : nn0 + node_off[(size_t)q] + l - 1; };
                    for (size_t j = 0; j < G.nodes.size(); j++) {
                        Node v = G.nodes[j];
                        if (v.left >= 0) {
                            v.left = gnode(v.left);
                            v.right = gnode(v.right);
                        }
                        if (v.block >= 0)
                            v.block = m[(size_t)v.block];
                        nodes[(size_t)gnode((int32_t)j)] = v;
                        rnodes[(size_t)gnode((int32_t)j)] = rnode_of(v);
                    }
                }
            });
        }
        if (limit < cn) {
            // the event entry, alone: it raises a global level
            btc_status rc = insert_one(base + limit);
            if (rc != BTC_OK)
                return rc;
            base += limit + 1;
            ch = std::max(CH_MIN, ch / 2);
        } else {
            base += cn;
            ch = std::min(CH_MAX, ch * 2);
        }
    }
    for (auto& b : blocks)
        finish_block_codes(b);
    for (int a = 0; a < 3; a++)
        s.global_levels[a] = g[a];
    return BTC_OK;
}

// search_parallel_block_Tree as first-fit in ascending block id.
//
// A block joins the lowest-numbered stratum none of whose members it meets
// on any axis (two blocks meet on an axis when their dyadic intervals
// nest).  On skewed inputs almost every refusal comes from the head of an
// axis: blocks that contain the same few hottest buckets all nest, so the
// scan would re-test them stratum by stratum.  Per axis the 64 finest
// buckets at the axis' global level ("hot buckets") are indexed by a binary
// tree of 127 ranges; each range keeps a bitset of the strata holding a
// member that covers one of its buckets.  A block covering hot buckets (an
// aligned range, one tree node) certainly meets every stratum in its node's
// bitset on that axis, so the scan skips those strata 64 at a time and runs
// the exact test only on the rest.  Skipping only what the exact test would
// refuse leaves the first fit unchanged.
void strata_first_fit(Schedule& s, int threads)
{
    (void)threads;
    const uint64_t FULL = 1ULL << 63;
    struct St {
        uint64_t bins[3] = {0, 0, 0};
        uint64_t used[3] = {0, 0, 0};
        std::vector<int32_t> mem;
    };
    std::vector<St> st;
    const auto& B = s.blocks;
    auto fits = [&](const St& S, const BlockRec& cb, const uint64_t* len) {
        if (FULL - S.used[0] < len[0] || FULL - S.used[1] < len[1] || FULL - S.used[2] < len[2])
            return false;
        for (int a = 0; a < 3; a++) {
            if ((S.bins[a] & cb.bins[a]) == 0)
                continue;
            for (int32_t m : S.mem)
                if (axis_conflict(B[m], cb, a))
                    return false;
        }
        return true;
    };
    // hot-bucket tree node of a block on axis a: 0 when it covers no hot
    // bucket, else the heap index (1 = all hot buckets) of its aligned range
    int hb[3], hlog[3];
    for (int a = 0; a < 3; a++) {
        const int g1 = s.global_levels[a] - 1;  // code bits at the global level
        hlog[a] = std::min(6, g1);
        hb[a] = 1 << hlog[a];
    }
    auto hot_node = [&](const BlockRec& b, int a) -> int {
        const int g1 = s.global_levels[a] - 1, m = b.level[a] - 1;
        // b covers the global-level buckets whose top m bits equal its code
        const int sh = g1 - m;
        if (sh >= 63)
            return 1;
        const uint64_t lo = b.code[a] << sh;
        if (lo >= (uint64_t)hb[a])
            return 0;
        const int t = std::min(sh, hlog[a]);  // log2 of the covered hot range
        return (int)((hb[a] + lo) >> t);
    };
    // bitsets over strata: per axis and tree node, and the closed strata
    std::vector<std::vector<uint64_t>> tb(3 * 128);
    std::vector<uint64_t> closed;
    size_t words = 0;
    auto grow = [&](size_t nst) {
        const size_t need = (nst + 63) / 64;
        if (need <= words)
            return;
        const size_t nw = std::max<size_t>(need, words * 2 + 16);
        for (auto& v : tb)
            if (!v.empty() || true)
                v.resize(nw, 0);
        closed.resize(nw, 0);
        words = nw;
    };
    auto set_bit = [](std::vector<uint64_t>& v, size_t i) { v[i >> 6] |= 1ULL << (i & 63); };
    // mark stratum k in every node whose range meets node u's: u, its
    // ancestors and its descendants
    auto mark = [&](int a, int u, size_t k) {
        for (int v = u; v >= 1; v >>= 1)
            set_bit(tb[(size_t)a * 128 + (size_t)v], k);
        int lo = u, hi = u;
        while ((lo << 1) < 2 * hb[a]) {
            lo <<= 1;
            hi = (hi << 1) | 1;
            for (int v = lo; v <= hi; v++)
                set_bit(tb[(size_t)a * 128 + (size_t)v], k);
        }
    };
    for (int32_t b = 0; b < (int32_t)B.size(); b++) {
        if (B[b].ent.empty())
            continue;
        const BlockRec& cb = B[b];
        uint64_t len[3];
        int node[3];
        for (int a = 0; a < 3; a++) {
            len[a] = 1ULL << (64 - cb.level[a]);
            node[a] = hot_node(cb, a);
        }
        const uint64_t* cx = node[0] ? tb[(size_t)node[0]].data() : nullptr;
        const uint64_t* cy = node[1] ? tb[128 + (size_t)node[1]].data() : nullptr;
        const uint64_t* cz = node[2] ? tb[256 + (size_t)node[2]].data() : nullptr;
        int32_t found = -1;
        const size_t nst = st.size();
        for (size_t w = 0; w * 64 < nst && found < 0; w++) {
            uint64_t busy = closed[w];
            if (cx)
                busy |= cx[w];
            if (cy)
                busy |= cy[w];
            if (cz)
                busy |= cz[w];
            uint64_t cand = ~busy;
            if ((w + 1) * 64 > nst)
                cand &= (1ULL << (nst - w * 64)) - 1ULL;
            while (cand) {
                const size_t k = w * 64 + (size_t)__builtin_ctzll(cand);
                cand &= cand - 1;
                if (fits(st[k], cb, len)) {
                    found = (int32_t)k;
                    break;
                }
            }
        }
        if (found < 0) {
            found = (int32_t)st.size();
            st.emplace_back();
            grow(st.size());
        }
        St& S = st[(size_t)found];
        S.mem.push_back(b);
        bool full = false;
        for (int a = 0; a < 3; a++) {
            S.bins[a] |= cb.bins[a];
            S.used[a] += len[a];
            full |= S.used[a] >= FULL;
            if (node[a])
                mark(a, node[a], (size_t)found);
        }
        if (full)
            set_bit(closed, (size_t)found);
    }
    s.strata_off.assign(1, 0);
    s.strata_ids.clear();
    s.max_parallel_cf = 0;
    for (auto& S : st) {
        s.strata_ids.insert(s.strata_ids.end(), S.mem.begin(), S.mem.end());
        s.strata_off.push_back((int32_t)s.strata_ids.size());
        s.max_parallel_cf = std::max<int32_t>(s.max_parallel_cf, (int32_t)S.mem.size());
    }
}

// update_conflict_weights (block.cu:470-513) for one group
void coe_weights(const std::vector<BlockRec>& B, const int32_t* ids, int n, double* coe)
{
    std::vector<int> par(n);
    std::vector<long long> sum(n);
    auto find = [&](int i) {
        while (par[i] != i) {
            par[i] = par[par[i]];
            i = par[i];
        }
        return i;
    };
    for (int a = 0; a < 3; a++) {
        for (int i = 0; i < n; i++) {
            par[i] = i;
            sum[i] = 0;
        }
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++)
                if (axis_conflict(B[ids[i]], B[ids[j]], a)) {
                    int ra = find(i), rb = find(j);
                    if (ra != rb)
                        par[rb] = ra;
                }
        for (int i = 0; i < n; i++) {
            int c = B[ids[i]].ent.empty() ? 1 : (int)B[ids[i]].ent.size();
            sum[find(i)] += c;
        }
        for (int i = 0; i < n; i++) {
            int c = B[ids[i]].ent.empty() ? 1 : (int)B[ids[i]].ent.size();
            int t = (int)sum[find(i)];
            coe[3 * i + a] = t > 0 ? (double)c / (double)t : 1.0;
        }
    }
}

// balance_parallel_sequences_for_gpu (block.cu:660-697) + the coe pass of
// Preproccess_list (block.cu:1157)
void balance(Schedule& s, int threads)
{
    const auto& B = s.blocks;
    const int target = s.target;
    std::vector<std::vector<int32_t>> groups;
    for (size_t st = 0; st + 1 < s.strata_off.size(); st++) {
        std::vector<int32_t> cur;
        for (int32_t k = s.strata_off[st]; k < s.strata_off[st + 1]; k++) {
            int32_t id = s.strata_ids[k];
            if (B[id].ent.empty())
                continue;
            cur.push_back(id);
            if ((int)cur.size() == target) {
                groups.push_back(cur);
                cur.clear();
            }
        }
        if (!cur.empty())
            groups.push_back(cur);
    }
    // candidates in (nnz, id) order: the first zero-score one is the answer
    std::vector<int32_t> order;
    for (int32_t i = 0; i < (int32_t)B.size(); i++)
        if (!B[i].ent.empty())
            order.push_back(i);
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return B[a].ent.size() < B[b].ent.size(); });

    std::atomic<size_t> next(0);
    auto worker = [&]() {
        for (;;) {
            size_t gi = next.fetch_add(1);
            if (gi >= groups.size())
                break;
            std::vector<int32_t>& G = groups[gi];
            while ((int)G.size() < target) {
                int best = -1, best_score = 0;
                for (int32_t c : order) {
                    bool member = false;
                    for (int32_t m : G)
                        if (m == c) {
                            member = true;
                            break;
                        }
                    if (member)
                        continue;
                    const BlockRec& cb = B[c];
                    int score = 0;
                    bool pruned = false;
                    for (int32_t m : G) {
                        const BlockRec& mb = B[m];
                        for (int a = 0; a < 3; a++)
                            if ((mb.bins[a] & cb.bins[a]) && axis_conflict(mb, cb, a))
                                score++;
                        if (best >= 0 && score >= best_score) {
                            pruned = true;
                            break;
                        }
                    }
                    if (pruned)
                        continue;
                    if (best < 0 || score < best_score) {
                        best = c;
                        best_score = score;
                        if (score == 0)
                            break;
                    }
                }
                if (best < 0)
                    break;
                G.push_back(best);
            }
        }
    };
    int nt = std::max(1, std::min<int>(threads, (int)groups.size()));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++)
        pool.emplace_back(worker);
    worker();
    for (auto& t : pool)
        t.join();

    s.group_off.assign(1, 0);
    s.slot_block.clear();
    s.max_parallel = 0;
    s.scheduled_updates = 0;
    for (auto& G : groups) {
        s.slot_block.insert(s.slot_block.end(), G.begin(), G.end());
        s.group_off.push_back((int32_t)s.slot_block.size());
        s.max_parallel = std::max<int32_t>(s.max_parallel, (int32_t)G.size());
        for (int32_t b : G)
            s.scheduled_updates += (int64_t)B[b].ent.size();
    }
    s.slot_coe.assign(3 * s.slot_block.size(), 1.0);
    for (size_t gi = 0; gi + 1 < s.group_off.size(); gi++) {
        int32_t o = s.group_off[gi];
        coe_weights(B, s.slot_block.data() + o, s.group_off[gi + 1] - o, s.slot_coe.data() + 3 * (size_t)o);
    }
}

}  // namespace

int32_t stratum_target(int32_t max_parallel, int32_t block_num, int32_t pss, int32_t resident)
{
    int32_t target;
    if (pss > 0) {
        target = pss;
    } else {
        target = max_parallel > 0 ? max_parallel : 1;
        if (resident > 0 && resident < target)
            target = resident;
        if (target < 1)
            target = 1;
        if (block_num > 0 && target > block_num)
            target = block_num;
    }
    if (target < 1)
        target = 1;
    if (block_num > 0 && target > block_num)
        target = block_num;
    return target;
}

btc_status build_schedule(const btc_config& cfg, const int32_t* xyz, int64_t n, int resident,
                          int threads, Schedule& s)
{
    if (n < 0 || n > 0x7fffffffLL || cfg.block_s <= 0 || cfg.I <= 0 || cfg.J <= 0 || cfg.K <= 0 ||
        cfg.parallel_sequence_size < 0)
        return BTC_ERR_ARG;
    for (int64_t i = 0; i < 3 * n; i++) {
        int d = (i % 3 == 0) ? cfg.I : (i % 3 == 1 ? cfg.J : cfg.K);
        if (xyz[i] < 0 || xyz[i] >= d)
            return BTC_ERR_RANGE;
    }
    s = Schedule();
    s.I = cfg.I;
    s.J = cfg.J;
    s.K = cfg.K;
    s.block_s = cfg.block_s;
    s.pss = cfg.parallel_sequence_size;
    s.train_nnz = n;
    double t0 = now_s();
    // one thread: the serial pass; several: the chunked pass (same result)
    btc_status rc = threads > 1 && n >= (1 << 16)
                        ? blocking_parallel(xyz, n, cfg.I, cfg.J, cfg.K, cfg.block_s, threads, s)
                        : blocking(xyz, n, cfg.I, cfg.J, cfg.K, cfg.block_s, threads, s);
    if (rc != BTC_OK)
        return rc;
    double t1 = now_s();
    strata_first_fit(s, threads);
    double t2 = now_s();
    s.target = stratum_target(s.max_parallel_cf, (int32_t)s.blocks.size(), s.pss, resident);
    balance(s, threads);
    double t3 = now_s();
    s.seconds[0] = t1 - t0;
    s.seconds[1] = t2 - t1;
    s.seconds[2] = t3 - t2;
    return BTC_OK;
}

namespace {
// axis_range_to_string (block.cu:787-820): double-width ranges for the report
std::string axis_range(const BlockRec& b, int a, int axis_size)
{
    std::ostringstream ss;
    if (axis_size <= 0)
        return "[]";
    int levels = b.level[a] - 1;
    if (levels <= 0 || levels >= 62) {
        ss << "[0," << axis_size - 1 << "]";
        return ss.str();
    }
    long long partitions = 1LL << levels;
    long long code = (long long)b.code[a];
    double width = (axis_size + 1.0) / partitions;
    int begin = (int)std::floor(code * width);
    int end = (int)std::floor((code + 1) * width) - 1;
    if (begin < 0)
        begin = 0;
    if (begin >= axis_size)
        begin = axis_size - 1;
    if (end < begin)
        end = begin;
    if (end >= axis_size)
        end = axis_size - 1;
    ss << "[" << begin << "," << end << "]";
    return ss.str();
}

std::string id_string(const BlockRec& b, int a)
{
    std::string r(1, '0');
    for (int k = b.level[a] - 2; k >= 0; k--)
        r += ((b.code[a] >> k) & 1ULL) ? '1' : '0';
    return r;
}

struct Stats {
    int count = 0, minv = 0, maxv = 0, scheduled = 0, unique = 0;
};

Stats stats_of(const std::vector<int32_t>& off, const std::vector<int32_t>& ids)
{
    Stats st;
    std::set<int32_t> u;
    for (size_t g = 0; g + 1 < off.size(); g++) {
        int sz = off[g + 1] - off[g];
        if (sz == 0)
            continue;
        st.count++;
        st.scheduled += sz;
        if (st.minv == 0 || sz < st.minv)
            st.minv = sz;
        st.maxv = std::max(st.maxv, sz);
        for (int k = off[g]; k < off[g + 1]; k++)
            u.insert(ids[k]);
    }
    st.unique = (int)u.size();
    return st;
}
}  // namespace

std::string report_text(const Schedule& s)
{
    std::ostringstream o;
    int ngroups = (int)s.group_off.size() - 1;
    int num_parallel = ngroups + 1;
    int non_empty = 0;
    for (const auto& b : s.blocks)
        non_empty += b.ent.empty() ? 0 : 1;
    Stats cf = stats_of(s.strata_off, s.strata_ids);
    Stats ac = stats_of(s.group_off, s.slot_block);
    o << "# block_s " << s.block_s << "\n";
    o << "# parallel_sequence_size " << (s.pss > 0 ? s.pss : 0) << " (0 means auto)\n";
    o << "# num_block_total " << s.blocks.size() << "\n";
    o << "# non_empty_blocks " << non_empty << "\n";
    o << "# num_parallel_nodes " << num_parallel << "\n";
    o << "# scheduled_blocks " << ac.scheduled << "\n";
    o << "# unique_scheduled_blocks " << ac.unique << "\n";
    o << "# max_sequence_size " << ac.maxv << "\n";
    o << "# target_gpu_blocks " << s.target << "\n";
    o << "# conflict_free_sequence_count " << cf.count << "\n";
    o << "# conflict_free_min_parallel_blocks " << cf.minv << "\n";
    o << "# conflict_free_max_parallel_blocks " << cf.maxv << "\n";
    o << "# conflict_free_scheduled_blocks " << cf.scheduled << "\n";
    o << "# conflict_free_unique_blocks " << cf.unique << "\n";
    o << "# after_conflict_sequence_count " << ac.count << "\n";
    o << "# after_conflict_min_parallel_blocks " << ac.minv << "\n";
    o << "# after_conflict_max_parallel_blocks " << ac.maxv << "\n";
    o << "# after_conflict_scheduled_blocks " << ac.scheduled << "\n";
    o << "# after_conflict_unique_blocks " << ac.unique << "\n";
    o << "\n";
    o << "[blocks]\n";
    o << "block_id nnz level_x level_y level_z x_id x_range y_id y_range z_id z_range\n";
    const int dims[3] = {s.I, s.J, s.K};
    for (size_t i = 0; i < s.blocks.size(); i++) {
        const BlockRec& b = s.blocks[i];
        if (b.ent.empty())
            continue;
        o << i << ' ' << b.ent.size() << ' ' << b.level[0] << ' ' << b.level[1] << ' ' << b.level[2];
        for (int a = 0; a < 3; a++)
            o << ' ' << id_string(b, a) << ' ' << axis_range(b, a, dims[a]);
        o << "\n";
    }
    o << "\n";
    o << "[parallel_sequences]\n";
    o << "sequence_id size total_nnz block_ids\n";
    int seq = 0;
    for (int g = 0; g < ngroups; g++) {
        int a = s.group_off[g], e = s.group_off[g + 1];
        if (a == e)
            continue;
        long long tot = 0;
        for (int k = a; k < e; k++)
            tot += (long long)s.blocks[s.slot_block[k]].ent.size();
        o << seq << ' ' << (e - a) << ' ' << (int)tot << ' ';
        for (int k = a; k < e; k++) {
            if (k > a)
                o << ',';
            o << s.slot_block[k];
        }
        o << "\n";
        seq++;
    }
    return o.str();
}

}  // namespace btc
