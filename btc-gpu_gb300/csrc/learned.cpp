// Learned blocking: a schedule that is not bound to reproduce the reference.
//
// The reference splits a full block at the midpoint of its code range on the
// axis its levels name next (block.cu:154-401), groups blocks into strata by
// first fit (block.cu:1024-1148) and pads every group to the GPU width with
// blocks that already run elsewhere (block.cu:660-697), so some blocks are
// updated several times per epoch.  This builder keeps the method -- a binary
// tree over the (i, j, k) index space whose leaves hold at most block_s
// entries, conflict-free groups of blocks -- and changes three things:
//
//  * split points: a node is split at the median coordinate of its entries on
//    the chosen axis, so both children hold about half the entries;
//  * split axes: with a cost model, the axis whose two children the model
//    predicts to be cheapest in total (block time as a function of block
//    features: entries, distinct rows per mode and the largest row share);
//    without one, the axes in turn (x, y, z by depth);
//  * packing: every block is scheduled exactly once per epoch (no padding);
//    blocks are taken in order of predicted cost, heaviest first, and each
//    joins the first recent group it meets on no axis (groups hold at most
//    `width` blocks), so the groups are conflict-free and every coe weight
//    is 1.
//
// The tree is built level by level on host threads; the entries of a node
// are a contiguous range of one index array, stably partitioned at each
// split, so a block's entries keep their input order.  Medians and, for
// nodes above 2^16 entries, the features are taken from an even sample of
// the node.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "schedule.h"

namespace btc {
namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void run_threads(int nt, const std::function<void(int)>& fn)
{
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++)
        pool.emplace_back(fn, t);
    fn(0);
    for (auto& th : pool)
        th.join();
}

struct Scratch {
    std::vector<int32_t> stamp[3], cnt[3];
    int32_t gen = 0;
    std::vector<int32_t> tmp;
    void init(const int* dims)
    {
        for (int a = 0; a < 3; a++) {
            stamp[a].assign((size_t)dims[a], 0);
            cnt[a].assign((size_t)dims[a], 0);
        }
    }
};

constexpr int64_t kExact = 1 << 16;  // nodes up to this size are measured exactly
constexpr int64_t kBig = 1 << 22;    // nodes from this size are partitioned by all threads

// Features of a block (or a candidate child) for the cost model, from n
// entries ent[0..n) that stand for n_true (an even sample of a large node):
// log entries, distinct rows per mode over entries, the largest row's share
// of the entries per mode, log staged rows, mean distinct share, fill.
void block_features(const int32_t* xyz, const int32_t* ent, int64_t n, int64_t n_true, int bs, Scratch& S,
                    float* f)
{
    // n entries read (ent[0..n)), standing for n_true entries
    if (++S.gen == 0x7fffffff) {
        for (int a = 0; a < 3; a++)
            std::fill(S.stamp[a].begin(), S.stamp[a].end(), 0);
        S.gen = 1;
    }
    int64_t d[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; i++) {
        const int32_t* c = xyz + 3 * (int64_t)ent[i];
        for (int a = 0; a < 3; a++) {
            int32_t& st = S.stamp[a][(size_t)c[a]];
            int32_t& ct = S.cnt[a][(size_t)c[a]];
            if (st != S.gen) {
                st = S.gen;
                ct = 0;
                d[a]++;
            }
            if (++ct > mx[a])
                mx[a] = ct;
        }
    }
    const double nn = (double)std::max<int64_t>(1, n);
    f[0] = (float)(std::log2(1.0 + (double)n_true) / 16.0);
    for (int a = 0; a < 3; a++) {
        f[1 + a] = (float)((double)d[a] / nn);
        f[4 + a] = (float)((double)mx[a] / nn);
    }
    f[7] = (float)(std::log2(1.0 + (double)(d[0] + d[1] + d[2]) * (double)n_true / nn) / 16.0);
    f[8] = (float)((double)(d[0] + d[1] + d[2]) / (3.0 * nn));
    f[9] = (float)std::min(1.0, (double)n_true / (double)std::max(1, bs));
}

}  // namespace

btc_status build_learned(const btc_config& cfg, const int32_t* xyz, int64_t n, int threads,
                         const std::function<bool(const float*, int64_t, float*)>& predict, Schedule& s)
{
    if (n < 0 || n > 0x7fffffffLL || cfg.block_s <= 0 || cfg.I <= 0 || cfg.J <= 0 || cfg.K <= 0)
        return BTC_ERR_ARG;
    const int dims[3] = {cfg.I, cfg.J, cfg.K};
    for (int64_t i = 0; i < n; i++)
        for (int a = 0; a < 3; a++)
            if (xyz[3 * i + a] < 0 || xyz[3 * i + a] >= dims[a])
                return BTC_ERR_RANGE;
    const int bs = cfg.block_s;
    const int T = std::max(1, std::min(threads, 64));
    s = Schedule();
    s.I = cfg.I;
    s.J = cfg.J;
    s.K = cfg.K;
    s.block_s = bs;
    s.pss = cfg.parallel_sequence_size;
    s.train_nnz = n;
    s.learned = true;
    const double t0 = now_s();

    struct KNode {
        int64_t b, e;     // entries ent[b, e)
        int32_t lo[3], hi[3];
        int depth;
        int level[3];
    };
    std::vector<int32_t> ent((size_t)n), tmp((size_t)n);
    for (int64_t i = 0; i < n; i++)
        ent[(size_t)i] = (int32_t)i;
    std::vector<Scratch> scr((size_t)T);
    for (auto& S : scr)
        S.init(dims);
    std::vector<KNode> cur, leaves;
    if (n > 0) {
        KNode r{};
        r.b = 0;
        r.e = n;
        for (int a = 0; a < 3; a++) {
            r.lo[a] = 0;
            r.hi[a] = dims[a];
            r.level[a] = 1;
        }
        cur.push_back(r);
    }
    constexpr int NF = 10;
    while (!cur.empty()) {
        // nodes that stay leaves
        std::vector<KNode> split;
        for (const KNode& k : cur)
            (k.e - k.b > bs ? split : leaves).push_back(k);
        if (split.empty())
            break;
        const size_t ns = split.size();
        // per node and axis: split coordinate (-1: the axis cannot split)
        // and the features of the two children
        std::vector<int32_t> cut(ns * 3, -1);
        std::vector<int64_t> nleft(ns * 3, 0);
        std::vector<float> feat(ns * 6 * NF, 0.f);
        std::atomic<size_t> next(0);
        const bool use_model = (bool)predict;
        run_threads(std::min<int>(T, (int)ns), [&](int t) {
            Scratch& S = scr[(size_t)t];
            std::vector<int32_t> vals, side;
            for (;;) {
                const size_t q = next.fetch_add(1);
                if (q >= ns)
                    return;
                const KNode& k = split[q];
                const int64_t m = k.e - k.b;
                const int64_t step = std::max<int64_t>(1, m / kExact);
                const int heur = k.depth % 3;
                for (int a = 0; a < 3; a++) {
                    if (!use_model && a != heur)
                        continue;
                    // median coordinate of the (sampled) entries on axis a
                    vals.clear();
                    for (int64_t i = k.b; i < k.e; i += step)
                        vals.push_back(xyz[3 * (int64_t)ent[(size_t)i] + a]);
                    const size_t mid = vals.size() / 2;
                    std::nth_element(vals.begin(), vals.begin() + (long)mid, vals.end());
                    int32_t c = vals[mid];
                    // entries below c go left; when that leaves the left side
                    // empty, the median value itself goes left too
                    int64_t lc = 0, le = 0;
                    for (int32_t v : vals) {
                        lc += v < c;
                        le += v <= c;
                    }
                    if (lc == 0)
                        c = c + 1, lc = le;
                    if (lc == 0 || lc == (int64_t)vals.size())
                        continue;  // one coordinate only: no split on this axis
                    cut[q * 3 + a] = c;
                    nleft[q * 3 + a] = lc * step;
                    if (!use_model)
                        continue;
                    // children's features
                    side.clear();
                    for (int64_t i = k.b; i < k.e; i += step)
                        if (xyz[3 * (int64_t)ent[(size_t)i] + a] < c)
                            side.push_back(ent[(size_t)i]);
                    const int64_t nl = (int64_t)side.size();
                    const int64_t nr_s = (int64_t)((k.e - k.b + step - 1) / step) - nl;
                    block_features(xyz, side.data(), nl, std::min<int64_t>(m, nl * step), bs, S,
                                   &feat[(q * 6 + (size_t)a * 2) * NF]);
                    side.clear();
                    for (int64_t i = k.b; i < k.e; i += step)
                        if (xyz[3 * (int64_t)ent[(size_t)i] + a] >= c)
                            side.push_back(ent[(size_t)i]);
                    block_features(xyz, side.data(), (int64_t)side.size(), std::min<int64_t>(m, nr_s * step), bs, S,
                                   &feat[(q * 6 + (size_t)a * 2 + 1) * NF]);
                }
            }
        });
        // the fallback: axes in turn, the next one that can split
        std::vector<int> axis(ns, -1);
        if (use_model) {
            std::vector<float> pred(ns * 6, 0.f);
            if (!predict(feat.data(), (int64_t)(ns * 6), pred.data()))
                return BTC_ERR_CUDA;
            for (size_t q = 0; q < ns; q++) {
                double best = 1e300;
                for (int a = 0; a < 3; a++) {
                    if (cut[q * 3 + a] < 0)
                        continue;
                    const double c = std::exp((double)pred[q * 6 + (size_t)a * 2]) +
                                     std::exp((double)pred[q * 6 + (size_t)a * 2 + 1]);
                    if (c < best) {
                        best = c;
                        axis[q] = a;
                    }
                }
            }
        } else {
            for (size_t q = 0; q < ns; q++) {
                const int heur = split[q].depth % 3;
                if (cut[q * 3 + heur] >= 0) {
                    axis[q] = heur;
                    continue;
                }
                // evaluate the other two axes now (rare: the turn's axis holds one coordinate)
                const KNode& k = split[q];
                for (int d = 1; d < 3 && axis[q] < 0; d++) {
                    const int a = (heur + d) % 3;
                    std::vector<int32_t> vals;
                    for (int64_t i = k.b; i < k.e; i++)
                        vals.push_back(xyz[3 * (int64_t)ent[(size_t)i] + a]);
                    const size_t mid = vals.size() / 2;
                    std::nth_element(vals.begin(), vals.begin() + (long)mid, vals.end());
                    int32_t c = vals[mid];
                    int64_t lc = 0, le = 0;
                    for (int32_t v : vals) {
                        lc += v < c;
                        le += v <= c;
                    }
                    if (lc == 0)
                        c = c + 1, lc = le;
                    if (lc > 0 && lc < (int64_t)vals.size()) {
                        cut[q * 3 + a] = c;
                        axis[q] = a;
                    }
                }
            }
        }
        // stable partition of every split node's range around its cut
        std::vector<KNode> nxt;
        nxt.reserve(ns * 2);
        std::vector<int64_t> lcount(ns, 0);
        // big nodes: every thread takes a share of the range, counts its
        // left entries, then writes both sides at offsets that keep order
        for (size_t q = 0; q < ns; q++) {
            const KNode& k = split[q];
            const int a = axis[q];
            if (a < 0 || k.e - k.b < kBig)
                continue;
            const int32_t c = cut[q * 3 + (size_t)a];
            const int64_t m = k.e - k.b;
            std::vector<int64_t> nl((size_t)T + 1, 0);
            run_threads(T, [&](int t) {
                int64_t v = 0;
                for (int64_t i = k.b + m * t / T; i < k.b + m * (t + 1) / T; i++)
                    v += xyz[3 * (int64_t)ent[(size_t)i] + a] < c;
                nl[(size_t)t + 1] = v;
            });
            for (int t = 0; t < T; t++)
                nl[(size_t)t + 1] += nl[(size_t)t];
            const int64_t left = nl[(size_t)T];
            run_threads(T, [&](int t) {
                const int64_t lo = k.b + m * t / T, hi = k.b + m * (t + 1) / T;
                int64_t ol = k.b + nl[(size_t)t], orr = k.b + left + (lo - k.b) - nl[(size_t)t];
                for (int64_t i = lo; i < hi; i++) {
                    const int32_t e = ent[(size_t)i];
                    if (xyz[3 * (int64_t)e + a] < c)
                        tmp[(size_t)ol++] = e;
                    else
                        tmp[(size_t)orr++] = e;
                }
            });
            run_threads(T, [&](int t) {
                const int64_t lo = k.b + m * t / T, hi = k.b + m * (t + 1) / T;
                std::memcpy(&ent[(size_t)lo], &tmp[(size_t)lo], sizeof(int32_t) * (size_t)(hi - lo));
            });
            lcount[q] = left;
        }
        next = 0;
        run_threads(std::min<int>(T, (int)ns), [&](int) {
            for (;;) {
                const size_t q = next.fetch_add(1);
                if (q >= ns)
                    return;
                const KNode& k = split[q];
                const int a = axis[q];
                if (a < 0 || k.e - k.b >= kBig)
                    continue;
                const int32_t c = cut[q * 3 + (size_t)a];
                int64_t o = k.b;
                for (int64_t i = k.b; i < k.e; i++)
                    if (xyz[3 * (int64_t)ent[(size_t)i] + a] < c)
                        tmp[(size_t)o++] = ent[(size_t)i];
                lcount[q] = o - k.b;
                for (int64_t i = k.b; i < k.e; i++)
                    if (xyz[3 * (int64_t)ent[(size_t)i] + a] >= c)
                        tmp[(size_t)o++] = ent[(size_t)i];
                std::memcpy(&ent[(size_t)k.b], &tmp[(size_t)k.b], sizeof(int32_t) * (size_t)(k.e - k.b));
            }
        });
        for (size_t q = 0; q < ns; q++) {
            const KNode& k = split[q];
            const int a = axis[q];
            if (a < 0) {  // identical coordinates on every axis cannot happen for distinct cells
                leaves.push_back(k);
                continue;
            }
            KNode L = k, R = k;
            L.e = R.b = k.b + lcount[q];
            L.hi[a] = R.lo[a] = cut[q * 3 + (size_t)a];
            L.depth = R.depth = k.depth + 1;
            L.level[a] = R.level[a] = k.level[a] + 1;
            nxt.push_back(L);
            nxt.push_back(R);
        }
        cur.swap(nxt);
    }
    // leaves in tree order -> blocks
    std::sort(leaves.begin(), leaves.end(), [](const KNode& a, const KNode& b) { return a.b < b.b; });
    const int64_t nb = (int64_t)leaves.size();
    s.blocks.resize((size_t)nb);
    for (int a = 0; a < 3; a++)
        s.global_levels[a] = 1;
    for (int64_t i = 0; i < nb; i++) {
        const KNode& k = leaves[(size_t)i];
        BlockRec& B = s.blocks[(size_t)i];
        B.ent.assign(ent.begin() + k.b, ent.begin() + k.e);
        for (int a = 0; a < 3; a++) {
            B.level[a] = k.level[a];
            B.code[a] = B.lcode[a] = B.bins[a] = 0;
            B.lo[a] = k.lo[a];
            B.hi[a] = k.hi[a];
            s.global_levels[a] = std::max(s.global_levels[a], k.level[a]);
        }
        B.boxed = true;
    }
    std::vector<int32_t>().swap(ent);
    std::vector<int32_t>().swap(tmp);
    const double t1 = now_s();

    // predicted cost of every block (entries when there is no model)
    std::vector<double> cost((size_t)nb, 0.0);
    if (predict && nb > 0) {
        std::vector<float> f((size_t)nb * NF);
        std::atomic<int64_t> next(0);
        run_threads(std::min<int>(T, (int)std::max<int64_t>(1, nb / 64)), [&](int t) {
            for (;;) {
                const int64_t i = next.fetch_add(1);
                if (i >= nb)
                    return;
                const auto& e = s.blocks[(size_t)i].ent;
                block_features(xyz, e.data(), (int64_t)e.size(), (int64_t)e.size(), bs, scr[(size_t)t],
                               &f[(size_t)i * NF]);
            }
        });
        std::vector<float> p((size_t)nb);
        if (!predict(f.data(), nb, p.data()))
            return BTC_ERR_CUDA;
        for (int64_t i = 0; i < nb; i++)
            cost[(size_t)i] = std::exp((double)p[(size_t)i]);
    } else {
        for (int64_t i = 0; i < nb; i++)
            cost[(size_t)i] = (double)s.blocks[(size_t)i].ent.size();
    }
    // packing: heaviest first, first fit among the most recent open groups
    const int width = cfg.parallel_sequence_size > 0 ? cfg.parallel_sequence_size : 8;
    std::vector<int32_t> order((size_t)nb);
    for (int64_t i = 0; i < nb; i++)
        order[(size_t)i] = (int32_t)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return cost[(size_t)a] > cost[(size_t)b]; });
    auto meets = [&](const BlockRec& a, const BlockRec& b) {
        for (int q = 0; q < 3; q++)
            if (a.lo[q] < b.hi[q] && b.lo[q] < a.hi[q])
                return true;
        return false;
    };
    constexpr size_t kWindow = 64;
    std::vector<std::vector<int32_t>> groups;
    std::vector<size_t> open;  // groups with room, oldest first
    for (int32_t b : order) {
        const BlockRec& cb = s.blocks[(size_t)b];
        int64_t found = -1;
        const size_t from = open.size() > kWindow ? open.size() - kWindow : 0;
        for (size_t k = from; k < open.size() && found < 0; k++) {
            bool ok = true;
            for (int32_t m : groups[open[k]])
                if (meets(s.blocks[(size_t)m], cb)) {
                    ok = false;
                    break;
                }
            if (ok)
                found = (int64_t)k;
        }
        if (found < 0) {
            groups.emplace_back();
            open.push_back(groups.size() - 1);
            found = (int64_t)open.size() - 1;
        }
        const size_t g = open[(size_t)found];
        groups[g].push_back(b);
        if ((int)groups[g].size() >= width)
            open.erase(open.begin() + found);
    }
    s.target = width;
    s.strata_off.assign(1, 0);
    s.strata_ids.clear();
    s.group_off.assign(1, 0);
    s.slot_block.clear();
    s.max_parallel = s.max_parallel_cf = 0;
    s.scheduled_updates = 0;
    for (auto& G : groups) {
        s.strata_ids.insert(s.strata_ids.end(), G.begin(), G.end());
        s.strata_off.push_back((int32_t)s.strata_ids.size());
        s.slot_block.insert(s.slot_block.end(), G.begin(), G.end());
        s.group_off.push_back((int32_t)s.slot_block.size());
        s.max_parallel = std::max<int32_t>(s.max_parallel, (int32_t)G.size());
        for (int32_t b : G)
            s.scheduled_updates += (int64_t)s.blocks[(size_t)b].ent.size();
    }
    s.max_parallel_cf = s.max_parallel;
    s.slot_coe.assign(3 * s.slot_block.size(), 1.0);  // conflict-free groups
    const double t2 = now_s();
    s.seconds[0] = t1 - t0;
    s.seconds[1] = t2 - t1;
    s.seconds[2] = 0;
    return BTC_OK;
}

void scheduled_block_features(const Schedule& s, const int32_t* xyz, int threads, std::vector<int32_t>& blocks,
                              std::vector<float>& feat)
{
    const int dims[3] = {s.I, s.J, s.K};
    std::vector<char> seen(s.blocks.size(), 0);
    blocks.clear();
    for (int32_t b : s.slot_block)
        if (!seen[(size_t)b]) {
            seen[(size_t)b] = 1;
            blocks.push_back(b);
        }
    const int T = std::max(1, std::min(threads, 64));
    std::vector<Scratch> scr((size_t)T);
    for (auto& S : scr)
        S.init(dims);
    feat.assign(blocks.size() * 10, 0.f);
    std::atomic<size_t> next(0);
    run_threads(std::min<int>(T, (int)std::max<size_t>(1, blocks.size() / 64)), [&](int t) {
        for (;;) {
            const size_t i = next.fetch_add(1);
            if (i >= blocks.size())
                return;
            const auto& e = s.blocks[(size_t)blocks[i]].ent;
            block_features(xyz, e.data(), (int64_t)e.size(), (int64_t)e.size(), s.block_s, scr[(size_t)t],
                           &feat[i * 10]);
        }
    });
}

}  // namespace btc
