// Host-side schedule of the GB300 CP-SGD path: adaptive binary-tree
// blocking, conflict-free strata, GPU balancing and coe weights.  Produces the
// same blocks, strata and slots as the reference's block_problem
// (block.cu:1233-1278) for the same input order.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "btc_gpu.h"

namespace btc {

struct BlockRec {
    int32_t level[3];
    uint64_t code[3];   // id positions 1..level-1, right-aligned, MSB first
    uint64_t lcode[3];  // the same bits left-aligned in 64 bits (for prefix tests)
    uint64_t bins[3];   // which of the 64 top-level intervals the block covers
    std::vector<int32_t> ent;  // entry indices in block order
    // learned schedules: the block's box [lo, hi) per axis (no codes)
    bool boxed = false;
    int32_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};

struct Schedule {
    int32_t I = 0, J = 0, K = 0, block_s = 0, pss = 0;
    int64_t train_nnz = 0;
    std::vector<BlockRec> blocks;
    // conflict-free strata (search_parallel_block_Tree's lists)
    std::vector<int32_t> strata_off, strata_ids;
    int32_t max_parallel_cf = 0;
    int32_t target = 1;
    // balanced groups (the GPU schedule) and per-slot weights
    std::vector<int32_t> group_off, slot_block;
    std::vector<double> slot_coe;  // 3 per slot
    int32_t max_parallel = 0;
    int32_t global_levels[3] = {1, 1, 1};
    double seconds[3] = {0, 0, 0};
    int64_t scheduled_updates = 0;
    bool learned = false;  // built by build_learned: boxes, no padding
};

// Builds the whole schedule.  Returns BTC_OK or an error status.
btc_status build_schedule(const btc_config& cfg, const int32_t* xyz, int64_t n, int resident,
                          int threads, Schedule& out);

// The auto stratum width (block.cu:577-619).
int32_t stratum_target(int32_t max_parallel, int32_t block_num, int32_t pss, int32_t resident);

// block_parallel.txt text (block.cu:822-925).
std::string report_text(const Schedule& s);

// The learned schedule (learned.cpp): median splits on the axis a cost model
// picks (`predict`: features -> log microseconds per block; empty = axes in
// turn), every block scheduled once, conflict-free groups heaviest first.
btc_status build_learned(const btc_config& cfg, const int32_t* xyz, int64_t n, int threads,
                         const std::function<bool(const float*, int64_t, float*)>& predict, Schedule& out);
// The 10 cost-model features of every scheduled block (first use order).
void scheduled_block_features(const Schedule& s, const int32_t* xyz, int threads, std::vector<int32_t>& blocks,
                              std::vector<float>& feat);

}  // namespace btc
