// C ABI of the GB300 CP-SGD path (include/btc_gpu.h): configuration, host
// schedule and the device context that replaces sgd_train's state.
//
// Device layout of one context (all in HBM, one allocation per array):
//   coo        int4 per scheduled entry: (x, y, z, float value bits), blocks
//              stored once, contiguously, in order of first use by the
//              schedule, so one epoch streams the array front to back
//   val64      FP64 value per entry (f64 contexts only)
//   slot_off / slot_nnz / slot_coe   per scheduled slot (a block may occupy
//              several slots: the reference pads strata with blocks already
//              scheduled elsewhere, block.cu:686-690)
//   items      (slot, first entry) work items of `chunk` entries, schedule order
//   A, B, C    factor rows, row stride Rp (rank rounded up to the kernel's
//              vector width, padding kept at zero)
//   eval_*     train and test entries for the metrics kernel
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <limits>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "btc_gpu.h"
#include "common.h"
#include "kernels.h"
#include "schedule.h"
#include "staged.h"
#include "tiles.h"

struct btc_schedule {
    btc::Schedule s;
};

struct btc_ctx {
    btc_config cfg{};
    int dtype = 0, mode = 0, R = 0, Rp = 0, esize = 4;
    int sms = 0, hw_grid = 0, hw_block = 256, chunk = 128, metric_grid = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int4* coo = nullptr;
    double* val64 = nullptr;
    long long* slot_off = nullptr;
    int* slot_nnz = nullptr;
    void* slot_coe = nullptr;
    int2* items = nullptr;
    long long nitems = 0;
    void* F[3] = {nullptr, nullptr, nullptr};
    int64_t rows[3] = {0, 0, 0};
    int4* eval_coo[2] = {nullptr, nullptr};
    double* eval_val[2] = {nullptr, nullptr};
    int64_t eval_n[2] = {0, 0};
    double* partials = nullptr;
    double* result = nullptr;
    double* staging = nullptr;  // double [max rows][R] for factor transfers
    int* wave_slots = nullptr;
    std::vector<int> wave_off;
    // staged mode
    btc::TileHdr* tiles = nullptr;
    int* slot_tile0 = nullptr;
    int* slot_ntiles = nullptr;
    int4* tent = nullptr;
    unsigned short* tcsr = nullptr;
    unsigned* tsegs = nullptr;
    int* trows = nullptr;
    double* tval64 = nullptr;
    int* counter = nullptr;
    int* unit_off = nullptr;       // device, nunits + 1
    int nunits = 0;
    // BF16 storage: FP32 masters of the hottest rows
    float* master[3] = {nullptr, nullptr, nullptr};
    int* hot_rows[3] = {nullptr, nullptr, nullptr};
    int nhot[3] = {0, 0, 0};
    unsigned epoch = 0;
    int* status = nullptr;
    int st_cap = 0, st_wave = 0, st_grid = 0, st_block = 256, st_G = 0, st_NV = 0, st_repeat = 0;
    size_t st_smem = 0;
    std::vector<float> tile_feat;  // BTC_TILE_FEATURES per tile
    std::vector<int> h_tile0, h_ntiles;  // host copy of each slot's tiles
    // per scheduled block (first use order): cost-model features and tiles
    std::vector<int32_t> blk_ids, blk_tile0, blk_ntiles;
    std::vector<float> blk_feat;
    unsigned* tile_ns = nullptr;   // device, allocated on the first profiled epoch
    bool profile_next = false;
    long long st_rows = 0, st_tiles = 0;
    int64_t updates = 0;
    int nslots = 0;
    bool failed = false;
    std::vector<double> coe_host;  // the schedule's coe weights, 3 per slot (without lr)
};

namespace {

thread_local std::string g_last_error;

btc_status cuda_fail(cudaError_t e, const char* what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return BTC_ERR_CUDA;
}

#define CK(call)                                  \
    do {                                          \
        cudaError_t e_ = (call);                  \
        if (e_ != cudaSuccess)                    \
            return cuda_fail(e_, #call);          \
    } while (0)

int default_threads(const btc_config& c)
{
    return c.host_threads > 0 ? c.host_threads : (int)std::max(1u, std::thread::hardware_concurrency());
}

int resident_blocks(const btc_config& c)
{
    if (c.resident_blocks != 0)
        return c.resident_blocks < 0 ? 0 : c.resident_blocks;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 0;
    }
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, c.device < n ? c.device : 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int per = p.maxBlocksPerMultiProcessor > 0 ? p.maxBlocksPerMultiProcessor : 32;
    return p.multiProcessorCount * per;
}

// Whether every (x, y, z) of n entries lies in [0,I) x [0,J) x [0,K); large
// inputs are checked on host threads.
bool coords_in_range(const int32_t* xyz, int64_t n, int32_t I, int32_t J, int32_t K, int threads)
{
    if (n <= 0)
        return true;
    const int T = n >= (1LL << 22) ? std::max(1, std::min(threads, 32)) : 1;
    std::vector<char> ok((size_t)T, 1);
    auto work = [&](int t) {
        const int64_t lo = n * t / T, hi = n * (t + 1) / T;
        for (int64_t i = lo; i < hi; i++) {
            const int32_t* c = xyz + 3 * i;
            if ((uint32_t)c[0] >= (uint32_t)I || (uint32_t)c[1] >= (uint32_t)J || (uint32_t)c[2] >= (uint32_t)K) {
                ok[(size_t)t] = 0;
                return;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++)
        pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool)
        th.join();
    return std::all_of(ok.begin(), ok.end(), [](char v) { return v != 0; });
}

// fn(lo, hi) over [0, n) split into contiguous shares on up to `threads`
// host threads (one share below `serial_below` items)
void parallel_for(int64_t n, int threads, const std::function<void(int64_t, int64_t)>& fn,
                  int64_t serial_below = 1 << 16)
{
    const int T = n < serial_below ? 1 : std::max(1, std::min(threads, 64));
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++)
        pool.emplace_back(fn, n * t / T, n * (t + 1) / T);
    fn(0, n / T);
    for (auto& th : pool)
        th.join();
}

template <typename T>
void free_dev(T*& p)
{
    if (p)
        cudaFree((void*)p);
    p = nullptr;
}

}  // namespace

extern "C" {

const char* btc_status_string(btc_status s)
{
    switch (s) {
    case BTC_OK: return "ok";
    case BTC_ERR_ARG: return "invalid argument";
    case BTC_ERR_CUDA: return g_last_error.empty() ? "CUDA error" : g_last_error.c_str();
    case BTC_ERR_ALLOC: return "allocation failed";
    case BTC_ERR_STATE: return "invalid state";
    case BTC_ERR_IO: return "I/O error";
    case BTC_ERR_TIMEOUT: return "device wait timed out";
    case BTC_ERR_UNSUPPORTED: return "unsupported";
    case BTC_ERR_RANGE: return "value out of range";
    case BTC_ERR_NO_DEVICE: return "no CUDA device";
    case BTC_ERR_DEVICE: return "kernel reported an error";
    }
    return "unknown status";
}

int32_t btc_abi_version(void) { return BTC_ABI_VERSION; }

btc_status btc_config_default(btc_config* c)
{
    if (!c)
        return BTC_ERR_ARG;
    std::memset(c, 0, sizeof(*c));
    c->I = 144;
    c->J = 288;
    c->K = 168;
    c->epochs = 1000;
    c->rank = 16;
    c->lr = 0.005;
    c->reg = 0.0005;
    c->block_s = 2048;
    c->thread_size = 512;
    c->parallel_sequence_size = 8;
    c->requested_gpu_count = 4;
    c->dtype = BTC_DTYPE_F32;
    c->mode = BTC_MODE_HOGWILD;
    return BTC_OK;
}

btc_status btc_config_validate(const btc_config* c)
{
    if (!c)
        return BTC_ERR_ARG;
    if (c->I <= 0 || c->J <= 0 || c->K <= 0 || c->epochs <= 0)
        return BTC_ERR_ARG;
    if (c->rank <= 0 || c->rank > btc::kMaxRank)
        return BTC_ERR_ARG;
    if (!(c->lr > 0) || !(c->reg >= 0) || c->block_s <= 0)
        return BTC_ERR_ARG;
    if (c->thread_size <= 0 || c->thread_size > 1024 || c->parallel_sequence_size < 0 ||
        c->requested_gpu_count < 0)
        return BTC_ERR_ARG;
    if (c->dtype < 0 || c->dtype > 2 || c->mode < 0 || c->mode > 3 || c->chunk < 0)
        return BTC_ERR_ARG;
    return BTC_OK;
}

/* ---- schedule ---- */

btc_status btc_schedule_build(const btc_config* cfg, const int32_t* xyz, int64_t n, btc_schedule** out)
{
    if (!cfg || !out || (n > 0 && !xyz))
        return BTC_ERR_ARG;
    *out = nullptr;
    btc_schedule* s = new (std::nothrow) btc_schedule();
    if (!s)
        return BTC_ERR_ALLOC;
    btc_status rc;
    try {
        rc = btc::build_schedule(*cfg, xyz, n, resident_blocks(*cfg), default_threads(*cfg), s->s);
    } catch (const std::bad_alloc&) {
        rc = BTC_ERR_ALLOC;
    }
    if (rc != BTC_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return BTC_OK;
}

btc_status btc_schedule_build_learned(const btc_config* cfg, const int32_t* xyz, int64_t n, btc_mlp* model,
                                      btc_schedule** out)
{
    if (!cfg || !out || (n > 0 && !xyz))
        return BTC_ERR_ARG;
    *out = nullptr;
    if (model) {
        int64_t np = 0;
        if (btc_mlp_param_count(model, &np) != BTC_OK || btc_mlp_inputs(model) != BTC_BLOCK_FEATURES)
            return BTC_ERR_ARG;
    }
    btc_schedule* s = new (std::nothrow) btc_schedule();
    if (!s)
        return BTC_ERR_ALLOC;
    std::function<bool(const float*, int64_t, float*)> predict;
    if (model)
        predict = [model](const float* x, int64_t m, float* y) { return btc_mlp_predict(model, x, m, y) == BTC_OK; };
    btc_status rc;
    try {
        rc = btc::build_learned(*cfg, xyz, n, default_threads(*cfg), predict, s->s);
    } catch (const std::bad_alloc&) {
        rc = BTC_ERR_ALLOC;
    }
    if (rc != BTC_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return BTC_OK;
}

btc_status btc_schedule_block_boxes(const btc_schedule* sp, int32_t* boxes)
{
    if (!sp || !boxes)
        return BTC_ERR_ARG;
    if (!sp->s.learned)
        return BTC_ERR_STATE;
    const auto& B = sp->s.blocks;
    for (size_t i = 0; i < B.size(); i++)
        for (int a = 0; a < 3; a++) {
            boxes[6 * i + 2 * a] = B[i].lo[a];
            boxes[6 * i + 2 * a + 1] = B[i].hi[a];
        }
    return BTC_OK;
}

btc_status btc_schedule_summarize(const btc_schedule* sp, btc_schedule_summary* o)
{
    if (!sp || !o)
        return BTC_ERR_ARG;
    const btc::Schedule& s = sp->s;
    std::memset(o, 0, sizeof(*o));
    o->num_blocks = (int32_t)s.blocks.size();
    for (const auto& b : s.blocks)
        o->nonempty_blocks += b.ent.empty() ? 0 : 1;
    o->num_strata = (int32_t)s.strata_off.size() - 1;
    o->max_parallel_cf = s.max_parallel_cf;
    o->target_gpu_blocks = s.target;
    o->num_groups = (int32_t)s.group_off.size() - 1;
    o->num_slots = (int32_t)s.slot_block.size();
    o->max_parallel = s.max_parallel;
    o->scheduled_updates = s.scheduled_updates;
    o->train_nnz = s.train_nnz;
    for (int a = 0; a < 3; a++) {
        o->global_levels[a] = s.global_levels[a];
        o->build_seconds[a] = s.seconds[a];
    }
    return BTC_OK;
}

btc_status btc_schedule_blocks(const btc_schedule* sp, int32_t* meta, uint64_t* codes)
{
    if (!sp || !meta || !codes)
        return BTC_ERR_ARG;
    const auto& B = sp->s.blocks;
    for (size_t i = 0; i < B.size(); i++) {
        meta[4 * i] = (int32_t)B[i].ent.size();
        for (int a = 0; a < 3; a++) {
            meta[4 * i + 1 + a] = B[i].level[a];
            codes[3 * i + a] = B[i].code[a];
        }
    }
    return BTC_OK;
}

btc_status btc_schedule_block_entries(const btc_schedule* sp, int32_t b, int32_t* out, int32_t* n)
{
    if (!sp || !n || b < 0 || b >= (int32_t)sp->s.blocks.size())
        return BTC_ERR_ARG;
    const auto& e = sp->s.blocks[b].ent;
    if (*n < (int32_t)e.size() || (!out && !e.empty())) {
        *n = (int32_t)e.size();
        return BTC_ERR_ARG;
    }
    if (!e.empty())
        std::memcpy(out, e.data(), e.size() * sizeof(int32_t));
    *n = (int32_t)e.size();
    return BTC_OK;
}

btc_status btc_schedule_strata(const btc_schedule* sp, int32_t* off, int32_t* ids)
{
    if (!sp || !off || !ids)
        return BTC_ERR_ARG;
    std::copy(sp->s.strata_off.begin(), sp->s.strata_off.end(), off);
    std::copy(sp->s.strata_ids.begin(), sp->s.strata_ids.end(), ids);
    return BTC_OK;
}

btc_status btc_schedule_groups(const btc_schedule* sp, int32_t* off, int32_t* slot_block, double* coe)
{
    if (!sp || !off || !slot_block || !coe)
        return BTC_ERR_ARG;
    std::copy(sp->s.group_off.begin(), sp->s.group_off.end(), off);
    std::copy(sp->s.slot_block.begin(), sp->s.slot_block.end(), slot_block);
    std::copy(sp->s.slot_coe.begin(), sp->s.slot_coe.end(), coe);
    return BTC_OK;
}

btc_status btc_schedule_write_report(const btc_schedule* sp, const btc_config*, const char* path)
{
    if (!sp || !path)
        return BTC_ERR_ARG;
    std::ofstream f(path, std::ios::out | std::ios::trunc | std::ios::binary);
    if (!f.is_open())
        return BTC_ERR_IO;
    f << btc::report_text(sp->s);
    return f.good() ? BTC_OK : BTC_ERR_IO;
}

void btc_schedule_free(btc_schedule* s) { delete s; }

/* ---- device context ---- */

btc_status btc_ctx_destroy(btc_ctx* c)
{
    if (!c)
        return BTC_OK;
    int dev = c->cfg.device;
    cudaSetDevice(dev);
    if (c->stream)
        cudaStreamSynchronize(c->stream);
    free_dev(c->coo);
    free_dev(c->val64);
    free_dev(c->slot_off);
    free_dev(c->slot_nnz);
    free_dev(c->slot_coe);
    free_dev(c->items);
    for (int a = 0; a < 3; a++)
        free_dev(c->F[a]);
    for (int k = 0; k < 2; k++) {
        free_dev(c->eval_coo[k]);
        free_dev(c->eval_val[k]);
    }
    free_dev(c->partials);
    free_dev(c->result);
    free_dev(c->staging);
    free_dev(c->wave_slots);
    free_dev(c->tiles);
    free_dev(c->slot_tile0);
    free_dev(c->slot_ntiles);
    free_dev(c->tent);
    free_dev(c->tcsr);
    free_dev(c->tsegs);
    free_dev(c->trows);
    free_dev(c->tval64);
    free_dev(c->counter);
    free_dev(c->unit_off);
    free_dev(c->status);
    free_dev(c->tile_ns);
    for (int a = 0; a < 3; a++) {
        free_dev(c->master[a]);
        free_dev(c->hot_rows[a]);
    }
    if (c->ev0)
        cudaEventDestroy(c->ev0);
    if (c->ev1)
        cudaEventDestroy(c->ev1);
    if (c->stream)
        cudaStreamDestroy(c->stream);
    delete c;
    return BTC_OK;
}

static btc_status upload(void** dst, const void* src, size_t bytes, cudaStream_t st)
{
    CK(cudaMalloc(dst, bytes > 0 ? bytes : 16));
    if (bytes > 0)
        CK(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, st));
    return BTC_OK;
}

static btc_status ctx_build(btc_ctx* c, const btc::Schedule& s, const int32_t* txyz, const double* tval,
                            int64_t ntr, const int32_t* sxyz, const double* sval, int64_t nte)
{
    // the slots the context runs: the balanced groups' slots, or for the
    // lock-free mode every non-empty block once in strata order with coe 1
    // (ToMatrix_LF, block.cu:1192-1217)
    std::vector<int32_t> lf_slots;
    std::vector<double> lf_coe;
    if (c->cfg.mode == BTC_MODE_LOCKFREE) {
        for (int32_t b : s.strata_ids)
            if (!s.blocks[(size_t)b].ent.empty())
                lf_slots.push_back(b);
        lf_coe.assign(3 * lf_slots.size(), 1.0);
    }
    const bool lf = c->cfg.mode == BTC_MODE_LOCKFREE;
    const std::vector<int32_t>& slot_block = lf ? lf_slots : s.slot_block;
    const std::vector<double>& slot_coe = lf ? lf_coe : s.slot_coe;
    const btc_config& cfg = c->cfg;
    CK(cudaSetDevice(cfg.device));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, cfg.device));
    c->sms = prop.multiProcessorCount;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    c->dtype = cfg.dtype;
    c->mode = cfg.mode;
    if (c->dtype == BTC_DTYPE_BF16 && c->mode != BTC_MODE_STAGED)
        return BTC_ERR_UNSUPPORTED;  // BF16 storage is served by the staged kernel
    if (c->mode == BTC_MODE_LOCKFREE && s.learned)
        return BTC_ERR_UNSUPPORTED;  // the lock-free rule runs on the reference's strata
    c->esize = c->dtype == BTC_DTYPE_F64 ? 8 : (c->dtype == BTC_DTYPE_BF16 ? 2 : 4);
    c->R = cfg.rank;
    c->Rp = btc::padded_rank(c->dtype, c->R);
    c->chunk = cfg.chunk > 0 ? cfg.chunk : 128;
    c->rows[0] = cfg.I;
    c->rows[1] = cfg.J;
    c->rows[2] = cfg.K;

    // entry stream: each scheduled block once, in order of first use
    const int nslots = (int)slot_block.size();
    c->nslots = nslots;
    std::vector<long long> boff(s.blocks.size(), -1);
    long long total = 0;
    for (int k = 0; k < nslots; k++) {
        int b = slot_block[k];
        if (boff[b] < 0) {
            boff[b] = total;
            total += (long long)s.blocks[b].ent.size();
        }
    }
    std::vector<int4> coo((size_t)total);
    std::vector<double> v64(c->dtype == BTC_DTYPE_F64 ? (size_t)total : 0);
    const int HT = default_threads(cfg);
    parallel_for((int64_t)s.blocks.size(), HT, [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; b++) {
            if (boff[(size_t)b] < 0)
                continue;
            long long o = boff[(size_t)b];
            for (int32_t e : s.blocks[(size_t)b].ent) {
                float fv = (float)tval[e];
                int4 q;
                q.x = txyz[3 * (int64_t)e];
                q.y = txyz[3 * (int64_t)e + 1];
                q.z = txyz[3 * (int64_t)e + 2];
                std::memcpy(&q.w, &fv, 4);
                coo[(size_t)o] = q;
                if (!v64.empty())
                    v64[(size_t)o] = tval[e];
                o++;
            }
        }
    }, 256);
    std::vector<long long> soff(nslots);
    std::vector<int> snnz(nslots);
    std::vector<double> coe64(3 * (size_t)nslots);
    std::vector<float> coe32(3 * (size_t)nslots);
    std::vector<int2> items;
    c->updates = 0;
    for (int k = 0; k < nslots; k++) {
        int b = slot_block[k];
        soff[k] = boff[b];
        snnz[k] = (int)s.blocks[b].ent.size();
        c->updates += snnz[k];
        for (int a = 0; a < 3; a++) {
            coe64[3 * k + a] = slot_coe[3 * k + a] * cfg.lr;  // (coe*lr) as the reference groups it
            coe32[3 * k + a] = (float)coe64[3 * k + a];
        }
        for (int st = 0; st < snnz[k]; st += c->chunk)
            items.push_back(make_int2(k, st));
    }
    c->nitems = (long long)items.size();
    c->coe_host.assign(slot_coe.begin(), slot_coe.end());
    btc_status rc;
    if ((rc = upload((void**)&c->coo, coo.data(), coo.size() * sizeof(int4), c->stream)))
        return rc;
    if (!v64.empty() && (rc = upload((void**)&c->val64, v64.data(), v64.size() * 8, c->stream)))
        return rc;
    if ((rc = upload((void**)&c->slot_off, soff.data(), soff.size() * 8, c->stream)))
        return rc;
    if ((rc = upload((void**)&c->slot_nnz, snnz.data(), snnz.size() * 4, c->stream)))
        return rc;
    if (c->dtype == BTC_DTYPE_F64)
        rc = upload(&c->slot_coe, coe64.data(), coe64.size() * 8, c->stream);
    else
        rc = upload(&c->slot_coe, coe32.data(), coe32.size() * 4, c->stream);
    if (rc)
        return rc;
    if ((rc = upload((void**)&c->items, items.data(), items.size() * sizeof(int2), c->stream)))
        return rc;

    // evaluation entries
    const int32_t* exyz[2] = {txyz, sxyz};
    const double* eval[2] = {tval, sval};
    int64_t en[2] = {ntr, nte};
    for (int k = 0; k < 2; k++) {
        std::vector<int4> q((size_t)en[k]);
        parallel_for(en[k], HT, [&](int64_t lo, int64_t hi) {
            for (int64_t i = lo; i < hi; i++)
                q[(size_t)i] = make_int4(exyz[k][3 * i], exyz[k][3 * i + 1], exyz[k][3 * i + 2], 0);
        });
        if ((rc = upload((void**)&c->eval_coo[k], q.data(), q.size() * sizeof(int4), c->stream)))
            return rc;
        if ((rc = upload((void**)&c->eval_val[k], eval[k], (size_t)en[k] * 8, c->stream)))
            return rc;
        c->eval_n[k] = en[k];
    }
    c->metric_grid = c->sms * 4;
    CK(cudaMalloc((void**)&c->partials, (size_t)c->metric_grid * 3 * sizeof(double)));
    CK(cudaMalloc((void**)&c->result, 4 * sizeof(double)));

    int64_t maxrows = std::max(c->rows[0], std::max(c->rows[1], c->rows[2]));
    for (int a = 0; a < 3; a++) {
        size_t bytes = (size_t)c->rows[a] * c->Rp * c->esize;
        CK(cudaMalloc(&c->F[a], bytes));
        CK(cudaMemsetAsync(c->F[a], 0, bytes, c->stream));
    }
    CK(cudaMalloc((void**)&c->staging, (size_t)maxrows * c->R * sizeof(double)));
    CK(cudaMalloc((void**)&c->status, sizeof(int)));
    CK(cudaMemsetAsync(c->status, 0, sizeof(int), c->stream));


    int occ = btc::hogwild_blocks_per_sm(c->dtype, c->R, c->hw_block);
    c->hw_grid = c->sms * std::max(1, occ);

    if (c->mode == BTC_MODE_STAGED) {
        c->st_wave = std::max(1, std::min(cfg.thread_size, 4096));
        int ctas = cfg.ctas_per_sm > 0 ? cfg.ctas_per_sm : 4;
        c->st_cap = btc::staged_cap_for(c->dtype, c->Rp, c->st_wave, ctas, prop.sharedMemPerMultiprocessor,
                                        prop.sharedMemPerBlockOptin);
        if (c->st_cap < 3)
            return BTC_ERR_UNSUPPORTED;  // one entry needs three staged rows
        btc::TileSet ts;
        // Most entries of one row per tile.  A tile's entries all read the
        // rows as they were when it started, so a row met c times takes a
        // Jacobi step of gain ~ lr * c * |other rows|^2; measured on a
        // skewed 50M-entry tensor (R 32), c = 64 held at lr 0.005 and 0.01
        // and diverged at 0.02, c = 16 held at 0.02, uncapped tiles (c in the
        // hundreds) diverged at 0.01 and at 0.005 once the factors had grown.
        // On a 1B-entry tensor with Zipf(1.3) modes (I = J = 1M, K = 100k,
        // R 32, lr 0.005, lambda 0.02, BF16) c = 64 diverged after 17 epochs
        // and c = 48 after 21, while c = 40 held 30 epochs and c = 32 held 25.
        // The default is the power of two at or below 0.16 / lr, in [16, 512].
        int repeat = cfg.row_repeat;
        if (repeat <= 0) {
            repeat = 16;
            while (repeat < 512 && (double)(repeat * 2) * cfg.lr <= 0.16 + 1e-12)
                repeat *= 2;
        }
        c->st_repeat = repeat;
        btc::build_tiles(s, txyz, tval, cfg.I, cfg.J, cfg.K, c->st_cap, c->st_wave, 16, repeat,
                         c->dtype == BTC_DTYPE_F64, ts, default_threads(cfg));
        std::vector<int> t0(nslots), tn(nslots);
        for (int k = 0; k < nslots; k++) {
            t0[k] = ts.block_tile0[(size_t)slot_block[k]];
            tn[k] = ts.block_ntiles[(size_t)slot_block[k]];
        }
        c->st_tiles = (long long)ts.tiles.size();
        c->st_rows = (long long)ts.rows.size();
        c->h_tile0 = t0;
        c->h_ntiles = tn;
        btc::scheduled_block_features(s, txyz, default_threads(cfg), c->blk_ids, c->blk_feat);
        c->blk_tile0.resize(c->blk_ids.size());
        c->blk_ntiles.resize(c->blk_ids.size());
        for (size_t i = 0; i < c->blk_ids.size(); i++) {
            c->blk_tile0[i] = ts.block_tile0[(size_t)c->blk_ids[i]];
            c->blk_ntiles[i] = ts.block_ntiles[(size_t)c->blk_ids[i]];
        }
        c->tile_feat.assign(ts.tiles.size() * BTC_TILE_FEATURES, 0.f);
        parallel_for((int64_t)ts.tiles.size(), HT, [&](int64_t t0_, int64_t t1_) {
            for (int64_t t = t0_; t < t1_; t++) {
                const btc::TileHdr& h = ts.tiles[(size_t)t];
                int maxseg = 0;
                for (int q = 0; q < h.nseg; q++)
                    maxseg = std::max(maxseg, ts.segs[(size_t)(h.soff + q)].w);
                float* f = &c->tile_feat[(size_t)t * BTC_TILE_FEATURES];
                const float nr = (float)std::max(1, h.nrows);
                f[0] = (float)h.n / (float)c->st_wave;
                f[1] = (float)h.nrows / (float)c->st_cap;
                f[2] = (float)h.nx / nr;
                f[3] = (float)h.ny / nr;
                f[4] = (float)h.nseg / (float)std::max(1, h.n);
                f[5] = (float)maxseg / 16.f;
                f[6] = std::log2(1.f + (float)h.n) / 10.f;
                f[7] = std::log2(1.f + (float)h.nrows) / 10.f;
                f[8] = (float)h.n / nr / 8.f;
                f[9] = 0.f;
            }
        }, 4096);
        for (size_t b = 0; b < ts.block_tile0.size(); b++)
            if (ts.block_tile0[b] >= 0)
                c->tile_feat[(size_t)ts.block_tile0[b] * BTC_TILE_FEATURES + 9] = 1.f;
        if ((rc = upload((void**)&c->tiles, ts.tiles.data(), ts.tiles.size() * sizeof(btc::TileHdr), c->stream)))
            return rc;
        if ((rc = upload((void**)&c->slot_tile0, t0.data(), t0.size() * 4, c->stream)))
            return rc;
        if ((rc = upload((void**)&c->slot_ntiles, tn.data(), tn.size() * 4, c->stream)))
            return rc;
        if ((rc = upload((void**)&c->tent, ts.ent.data(), ts.ent.size() * sizeof(int4), c->stream)))
            return rc;
        if ((rc = upload((void**)&c->tcsr, ts.csr.data(), ts.csr.size() * 2, c->stream)))
            return rc;
        {
            // owner segments packed into one word each, as the kernel reads
            // them: local row (14 bits; cap <= 16383), mode (2), count - 1
            // (4; segments hold <= 16 entries), start in the mode's CSR list
            // (12; a tile holds <= 4096 entries)
            std::vector<uint32_t> seg32(ts.segs.size());
            std::atomic<bool> bad_seg(false);
            parallel_for((int64_t)ts.segs.size(), HT, [&](int64_t lo, int64_t hi) {
                for (int64_t q = lo; q < hi; q++) {
                    const int4& g = ts.segs[(size_t)q];
                    if (g.x < 0 || g.x >= (1 << 14) || g.y < 0 || g.y > 2 || g.w < 1 || g.w > 16 || g.z < 0 ||
                        g.z >= (1 << 12)) {
                        bad_seg = true;
                        return;
                    }
                    seg32[(size_t)q] = (uint32_t)g.x | ((uint32_t)g.y << 14) | ((uint32_t)(g.w - 1) << 16) |
                                       ((uint32_t)g.z << 20);
                }
            });
            if (bad_seg)
                return BTC_ERR_UNSUPPORTED;
            // Within a tile the segments are independent (each adds to its
            // own row), and a warp reduces EPW of them side by side for as
            // many steps as the longest has entries: a stable counting sort
            // by count, longest first, gives each warp segments of about
            // equal length.
            parallel_for((int64_t)ts.tiles.size(), HT, [&](int64_t lo, int64_t hi) {
                std::vector<uint32_t> tmp;
                for (int64_t t = lo; t < hi; t++) {
                    const btc::TileHdr& h = ts.tiles[(size_t)t];
                    uint32_t* sg = seg32.data() + h.soff;
                    tmp.assign(sg, sg + h.nseg);
                    // key 15 - (count - 1): 0 for 16 entries; pos[key + 1]
                    // counts, then the prefix sum makes pos[key] the start
                    int pos[17] = {0};
                    for (uint32_t w : tmp)
                        pos[16 - (int)((w >> 16) & 15)]++;
                    for (int k = 1; k <= 16; k++)
                        pos[k] += pos[k - 1];
                    for (uint32_t w : tmp)
                        sg[pos[15 - (int)((w >> 16) & 15)]++] = w;
                }
            }, 1024);
            if ((rc = upload((void**)&c->tsegs, seg32.data(), seg32.size() * 4, c->stream)))
                return rc;
        }
        if (!ts.val64.empty() && (rc = upload((void**)&c->tval64, ts.val64.data(), ts.val64.size() * 8, c->stream)))
            return rc;
        // Per row and mode, over one epoch's executed updates: how many there
        // are and how much regularisation decay they apply (sum of
        // coe * lr * reg, in e-folds).  A row is FAST when that decay times a
        // tile's share of the epoch (at most 8 CTAs per SM over the tiles)
        // reaches 0.1: its staged updates then decay from the row's value at
        // write time instead of the tile-start snapshot, which concurrent
        // tiles would turn into unstable delayed feedback.  On skewed tensors
        // only the heads of the index distributions qualify.
        std::vector<int64_t> cnts[3];
        std::vector<char> fast[3];
        {
            // counted in a fixed number of slot ranges (partial sums added in
            // range order), so the result does not depend on the thread count
            std::vector<double> decay[3];
            for (int a = 0; a < 3; a++) {
                cnts[a].assign((size_t)c->rows[a], 0);
                decay[a].assign((size_t)c->rows[a], 0.0);
            }
            const int P = c->updates >= (1LL << 24) ? 16 : 1;
            std::vector<std::vector<int64_t>> pc((size_t)P - 1);
            std::vector<std::vector<double>> pd((size_t)P - 1);
            auto count_range = [&](int part) {
                int64_t* cn[3];
                double* dc[3];
                const size_t off[3] = {0, (size_t)c->rows[0], (size_t)(c->rows[0] + c->rows[1])};
                if (part == 0) {
                    for (int a = 0; a < 3; a++) {
                        cn[a] = cnts[a].data();
                        dc[a] = decay[a].data();
                    }
                } else {
                    const size_t all = (size_t)(c->rows[0] + c->rows[1] + c->rows[2]);
                    pc[(size_t)part - 1].assign(all, 0);
                    pd[(size_t)part - 1].assign(all, 0.0);
                    for (int a = 0; a < 3; a++) {
                        cn[a] = pc[(size_t)part - 1].data() + off[a];
                        dc[a] = pd[(size_t)part - 1].data() + off[a];
                    }
                }
                for (int k = (int)((int64_t)nslots * part / P); k < (int)((int64_t)nslots * (part + 1) / P); k++) {
                    double d[3];
                    for (int a = 0; a < 3; a++)
                        d[a] = slot_coe[3 * (size_t)k + a] * cfg.lr * cfg.reg;
                    for (int32_t e : s.blocks[(size_t)slot_block[k]].ent)
                        for (int a = 0; a < 3; a++) {
                            const size_t r = (size_t)txyz[3 * (int64_t)e + a];
                            cn[a][r]++;
                            dc[a][r] += d[a];
                        }
                }
            };
            {
                std::atomic<int> nextp(0);
                const int nt = std::max(1, std::min(HT, P));
                std::vector<std::thread> pool;
                auto worker = [&]() {
                    for (int q; (q = nextp.fetch_add(1)) < P;)
                        count_range(q);
                };
                for (int t = 1; t < nt; t++)
                    pool.emplace_back(worker);
                worker();
                for (auto& th : pool)
                    th.join();
            }
            for (int a = 0; a < 3; a++) {
                const size_t off = a == 0 ? 0 : (a == 1 ? (size_t)c->rows[0] : (size_t)(c->rows[0] + c->rows[1]));
                parallel_for(c->rows[a], HT, [&](int64_t lo, int64_t hi) {
                    for (int q = 0; q + 1 < P; q++)
                        for (int64_t r = lo; r < hi; r++) {
                            cnts[a][(size_t)r] += pc[(size_t)q][off + (size_t)r];
                            decay[a][(size_t)r] += pd[(size_t)q][off + (size_t)r];
                        }
                });
            }
            const double share = (double)c->sms * 8.0 / (double)std::max<size_t>(1, ts.tiles.size());
            for (int a = 0; a < 3; a++) {
                fast[a].assign((size_t)c->rows[a], 0);
                for (size_t r = 0; r < fast[a].size(); r++)
                    fast[a][r] = decay[a][r] * share >= 0.1;
            }
        }
        constexpr int FAST = 1 << 30;  // the kernel's flag bit in a master index
        if (c->dtype == BTC_DTYPE_BF16) {
            std::vector<int> maps[3];
            // FP32 masters for the rows whose BF16 copy would be contended:
            // every row that a tile updates through more than one owner
            // segment (those segments add to it concurrently) and every row
            // updated at least 4x as often as the mean row, and every FAST
            // row; their small updates then accumulate exactly instead of
            // being rounded to BF16 each time.  The other rows take at most
            // one stochastically rounded update per tile visit.
            for (int a = 0; a < 3; a++) {
                const std::vector<int64_t>& cnt = cnts[a];
                int64_t used = 0, total = 0;
                for (int64_t v : cnt)
                    if (v > 0) {
                        used++;
                        total += v;
                    }
                const double thr = used > 0 ? 4.0 * (double)total / (double)used : 0.0;
                std::vector<char> is_hot((size_t)c->rows[a], 0);
                for (int64_t r = 0; r < c->rows[a]; r++)
                    is_hot[(size_t)r] = cnt[(size_t)r] > 0 && (double)cnt[(size_t)r] >= thr;
                {
                    // rows a tile updates through more than one segment; each
                    // thread collects its tiles' rows, then they are marked
                    const int nt = ts.tiles.size() >= 4096 ? std::max(1, std::min(HT, 64)) : 1;
                    std::vector<std::vector<int32_t>> multi((size_t)nt);
                    std::vector<std::thread> pool;
                    auto scan = [&](int t) {
                        const size_t lo = ts.tiles.size() * (size_t)t / (size_t)nt;
                        const size_t hi = ts.tiles.size() * (size_t)(t + 1) / (size_t)nt;
                        for (size_t i = lo; i < hi; i++) {
                            const btc::TileHdr& h = ts.tiles[i];
                            for (int q = 1; q < h.nseg; q++) {
                                const int4& s0 = ts.segs[(size_t)(h.soff + q - 1)];
                                const int4& s1 = ts.segs[(size_t)(h.soff + q)];
                                if (s1.y == a && s0.y == a && s0.x == s1.x)
                                    multi[(size_t)t].push_back(ts.rows[(size_t)(h.roff + s1.x)]);
                            }
                        }
                    };
                    for (int t = 1; t < nt; t++)
                        pool.emplace_back(scan, t);
                    scan(0);
                    for (auto& th : pool)
                        th.join();
                    for (const auto& v : multi)
                        for (int32_t r : v)
                            is_hot[(size_t)r] = 1;
                }
                std::vector<int> hot;
                for (int64_t r = 0; r < c->rows[a]; r++)
                    if (is_hot[(size_t)r] || fast[a][(size_t)r])  // FAST rows decay from their master
                        hot.push_back((int)r);
                if (hot.size() >= (size_t)FAST)
                    return BTC_ERR_UNSUPPORTED;
                std::vector<int> map((size_t)c->rows[a], -1);
                for (size_t h = 0; h < hot.size(); h++)
                    map[(size_t)hot[h]] = (int)h;
                c->nhot[a] = (int)hot.size();
                if ((rc = upload((void**)&c->hot_rows[a], hot.data(), hot.size() * 4, c->stream)))
                    return rc;
                const size_t mb = std::max<size_t>(16, hot.size() * c->Rp * sizeof(float));
                CK(cudaMalloc((void**)&c->master[a], mb));
                CK(cudaMemsetAsync(c->master[a], 0, mb, c->stream));
                maps[a].swap(map);
            }
            // the kernel finds a row's master in its staged row id: ~(master
            // index, FAST bit for a FAST row) instead of the global row, so
            // staging needs no lookup
            parallel_for((int64_t)ts.tiles.size(), HT, [&](int64_t lo, int64_t hi) {
                for (int64_t i = lo; i < hi; i++) {
                    const btc::TileHdr& h = ts.tiles[(size_t)i];
                    for (int r = 0; r < h.nrows; r++) {
                        const int m = r < h.nx ? 0 : (r < h.nx + h.ny ? 1 : 2);
                        int32_t& g = ts.rows[(size_t)(h.roff + r)];
                        const int hm = maps[m][(size_t)g];
                        if (hm >= 0)
                            g = ~(hm | (fast[m][(size_t)g] ? FAST : 0));
                    }
                }
            }, 4096);
        } else {
            // FP32/FP64: a FAST row's staged id is ~row
            parallel_for((int64_t)ts.tiles.size(), HT, [&](int64_t lo, int64_t hi) {
                for (int64_t i = lo; i < hi; i++) {
                    const btc::TileHdr& h = ts.tiles[(size_t)i];
                    for (int r = 0; r < h.nrows; r++) {
                        const int m = r < h.nx ? 0 : (r < h.nx + h.ny ? 1 : 2);
                        int32_t& g = ts.rows[(size_t)(h.roff + r)];
                        if (fast[m][(size_t)g])
                            g = ~g;
                    }
                }
            }, 4096);
        }
        if ((rc = upload((void**)&c->trows, ts.rows.data(), ts.rows.size() * 4, c->stream)))
            return rc;
        CK(cudaMalloc((void**)&c->counter, sizeof(int)));
        {
            std::vector<int> uo((size_t)nslots + 1);
            for (int k = 0; k <= nslots; k++)
                uo[(size_t)k] = k;  // one slot per unit until a packing is chosen
            if ((rc = upload((void**)&c->unit_off, uo.data(), uo.size() * 4, c->stream)))
                return rc;
            c->nunits = nslots;
        }
        size_t smem = btc::staged_smem_bytes(c->dtype, c->Rp, c->st_cap, c->st_wave);
        c->st_smem = smem;
        int occ = btc::staged_blocks_per_sm(c->dtype, c->R, c->st_block, smem);
        if (occ <= 0)
            return BTC_ERR_UNSUPPORTED;
        c->st_grid = c->sms * occ;
        CK(cudaStreamSynchronize(c->stream));  // host tile arrays go out of scope
    }

    if (c->mode == BTC_MODE_DETERMINISTIC || c->mode == BTC_MODE_LOCKFREE) {
        // slots that share any factor row run in schedule order; the others
        // run together (wave = 1 + latest wave of any row the slot touches)
        std::vector<int> last[3];
        for (int a = 0; a < 3; a++)
            last[a].assign((size_t)c->rows[a], 0);
        std::vector<int> wave(nslots);
        int nw = 0;
        for (int k = 0; k < nslots; k++) {
            const auto& ent = s.blocks[slot_block[k]].ent;
            int w = 0;
            for (int32_t e : ent)
                for (int a = 0; a < 3; a++)
                    w = std::max(w, last[a][(size_t)txyz[3 * (int64_t)e + a]]);
            w += 1;
            for (int32_t e : ent)
                for (int a = 0; a < 3; a++)
                    last[a][(size_t)txyz[3 * (int64_t)e + a]] = w;
            wave[k] = w;
            nw = std::max(nw, w);
        }
        c->wave_off.assign((size_t)nw + 2, 0);
        for (int k = 0; k < nslots; k++)
            c->wave_off[(size_t)wave[k] + 1]++;
        for (int w = 1; w <= nw + 1; w++)
            c->wave_off[(size_t)w] += c->wave_off[(size_t)w - 1];
        std::vector<int> ws(nslots);
        std::vector<int> fill(c->wave_off.begin(), c->wave_off.end());
        for (int k = 0; k < nslots; k++)
            ws[(size_t)fill[(size_t)wave[k]]++] = k;
        if ((rc = upload((void**)&c->wave_slots, ws.data(), ws.size() * 4, c->stream)))
            return rc;
    }
    CK(cudaStreamSynchronize(c->stream));
    return BTC_OK;
}

btc_status btc_ctx_create(const btc_config* cfg, const btc_schedule* s, const int32_t* txyz,
                          const double* tval, int64_t ntr, const int32_t* sxyz, const double* sval,
                          int64_t nte, btc_ctx** out)
{
    if (!cfg || !s || !out || (ntr > 0 && (!txyz || !tval)) || (nte > 0 && (!sxyz || !sval)))
        return BTC_ERR_ARG;
    *out = nullptr;
    btc_status rc = btc_config_validate(cfg);
    if (rc)
        return rc;
    if (s->s.train_nnz != ntr || s->s.I != cfg->I || s->s.J != cfg->J || s->s.K != cfg->K)
        return BTC_ERR_ARG;
    // every coordinate the kernels will use as a row index must name a row:
    // an out-of-range train or test entry would read or write past a factor
    if (!coords_in_range(txyz, ntr, cfg->I, cfg->J, cfg->K, default_threads(*cfg)) ||
        !coords_in_range(sxyz, nte, cfg->I, cfg->J, cfg->K, default_threads(*cfg)))
        return BTC_ERR_RANGE;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return BTC_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev)
        return BTC_ERR_ARG;
    btc_ctx* c = new (std::nothrow) btc_ctx();
    if (!c)
        return BTC_ERR_ALLOC;
    c->cfg = *cfg;
    try {
        rc = ctx_build(c, s->s, txyz, tval, ntr, sxyz, sval, nte);
    } catch (const std::bad_alloc&) {
        rc = BTC_ERR_ALLOC;
    }
    if (rc) {
        btc_ctx_destroy(c);
        return rc;
    }
    *out = c;
    return BTC_OK;
}

void* btc_ctx_stream(btc_ctx* c) { return c ? (void*)c->stream : nullptr; }

btc_status btc_ctx_set_rates(btc_ctx* c, double lr, double reg)
{
    if (!c || !(lr > 0) || !(reg >= 0))
        return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    const size_t n = c->coe_host.size();
    if (c->dtype == BTC_DTYPE_F64) {
        std::vector<double> v(n);
        for (size_t i = 0; i < n; i++)
            v[i] = c->coe_host[i] * lr;
        CK(cudaMemcpyAsync(c->slot_coe, v.data(), n * 8, cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    } else {
        std::vector<float> v(n);
        for (size_t i = 0; i < n; i++)
            v[i] = (float)(c->coe_host[i] * lr);
        CK(cudaMemcpyAsync(c->slot_coe, v.data(), n * 4, cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    c->cfg.lr = lr;
    c->cfg.reg = reg;
    return BTC_OK;
}

btc_status btc_ctx_set_factors(btc_ctx* c, int32_t mode, const double* host)
{
    if (!c || mode < 0 || mode > 2 || !host)
        return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    size_t bytes = (size_t)c->rows[mode] * c->R * sizeof(double);
    CK(cudaMemcpyAsync(c->staging, host, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(btc::launch_pack(c->dtype, c->staging, c->F[mode], c->rows[mode], c->R, c->Rp, c->stream));
    if (c->dtype == BTC_DTYPE_BF16)
        CK(btc::launch_master(0, c->staging, nullptr, c->master[mode], nullptr, c->hot_rows[mode], c->nhot[mode],
                              c->R, c->Rp, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return BTC_OK;
}

btc_status btc_ctx_get_factors(btc_ctx* c, int32_t mode, double* host)
{
    if (!c || mode < 0 || mode > 2 || !host)
        return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    size_t bytes = (size_t)c->rows[mode] * c->R * sizeof(double);
    CK(btc::launch_unpack(c->dtype, c->F[mode], c->staging, c->rows[mode], c->R, c->Rp, c->stream));
    if (c->dtype == BTC_DTYPE_BF16)
        CK(btc::launch_master(1, nullptr, c->staging, c->master[mode], nullptr, c->hot_rows[mode], c->nhot[mode],
                              c->R, c->Rp, c->stream));
    CK(cudaMemcpyAsync(host, c->staging, bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return BTC_OK;
}

btc_status btc_ctx_init_factors(btc_ctx* c, uint64_t seed, double lo, double hi)
{
    if (!c || !(hi >= lo))
        return BTC_ERR_ARG;
    for (int m = 0; m < 3; m++) {
        std::vector<double> h((size_t)c->rows[m] * c->R);
        for (int64_t r = 0; r < c->rows[m]; r++)
            for (int q = 0; q < c->R; q++)
                h[(size_t)r * c->R + q] = btc::init_uniform(seed, m, r, q, lo, hi);
        btc_status rc = btc_ctx_set_factors(c, m, h.data());
        if (rc)
            return rc;
    }
    return BTC_OK;
}

static btc::SgdArgs sgd_args(btc_ctx* c)
{
    btc::SgdArgs a{};
    a.coo = c->coo;
    a.val64 = c->val64;
    a.items = c->items;
    a.nitems = c->nitems;
    a.slot_off = c->slot_off;
    a.slot_nnz = c->slot_nnz;
    a.slot_coe = c->slot_coe;
    a.A = c->F[0];
    a.B = c->F[1];
    a.C = c->F[2];
    a.R = c->R;
    a.Rp = c->Rp;
    a.reg = c->cfg.reg;
    a.chunk = c->chunk;
    return a;
}

static btc::StagedArgs staged_args(btc_ctx* c)
{
    btc::StagedArgs s{};
    s.tiles = c->tiles;
    s.slot_tile0 = c->slot_tile0;
    s.slot_ntiles = c->slot_ntiles;
    s.slot_coe = c->slot_coe;
    s.nslots = c->nslots;
    s.unit_off = c->unit_off;
    s.nunits = c->nunits;
    s.ent = c->tent;
    s.csr = c->tcsr;
    s.segs = c->tsegs;
    s.rows = c->trows;
    s.val64 = c->tval64;
    s.A = c->F[0];
    s.B = c->F[1];
    s.C = c->F[2];
    s.R = c->R;
    s.Rp = c->Rp;
    s.reg = c->cfg.reg;
    s.cap = c->st_cap;
    s.wave = c->st_wave;
    s.counter = c->counter;
    s.G = c->st_G;
    s.NV = c->st_NV;
    s.status = c->status;
    for (int a = 0; a < 3; a++)
        s.master[a] = c->master[a];
    return s;
}

static btc_status enqueue_epoch(btc_ctx* c, int* launches)
{
    btc::SgdArgs a = sgd_args(c);
    int n = 0;
    if (c->mode == BTC_MODE_HOGWILD) {
        CK(btc::launch_hogwild(c->dtype, a, c->hw_grid, c->hw_block, c->stream));
        n = c->nitems > 0 ? 1 : 0;
    } else if (c->mode == BTC_MODE_DETERMINISTIC || c->mode == BTC_MODE_LOCKFREE) {
        for (size_t w = 1; w + 1 < c->wave_off.size(); w++) {
            int b = c->wave_off[w], e = c->wave_off[w + 1];
            if (c->mode == BTC_MODE_LOCKFREE)
                CK(btc::launch_lf_wave(c->dtype, c->wave_slots + b, e - b, a, c->stream));
            else
                CK(btc::launch_det_wave(c->dtype, c->wave_slots + b, e - b, a, c->stream));
            n += e > b ? 1 : 0;
        }
    } else if (c->mode == BTC_MODE_STAGED) {
        if (c->nslots > 0) {
            btc::StagedArgs s = staged_args(c);
            s.tile_ns = c->profile_next ? c->tile_ns : nullptr;
            c->epoch++;
            s.seed = (c->epoch * 0x9E3779B9u) ^ 0x5BD1E995u;
            CK(cudaMemsetAsync(c->counter, 0, sizeof(int), c->stream));
            CK(btc::launch_staged(c->dtype, s, c->st_grid, c->st_block, c->stream));
            n = 1;
            if (c->dtype == BTC_DTYPE_BF16)
                for (int a = 0; a < 3; a++) {
                    CK(btc::launch_master(2, nullptr, nullptr, c->master[a], c->F[a], c->hot_rows[a], c->nhot[a],
                                          c->R, c->Rp, c->stream));
                    n += c->nhot[a] > 0 ? 1 : 0;
                }
        }
    } else {
        return BTC_ERR_UNSUPPORTED;
    }
    if (launches)
        *launches = n;
    return BTC_OK;
}

static btc_status check_status(btc_ctx* c, int* word)
{
    int h = 0;
    CK(cudaMemcpy(&h, c->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (word)
        *word = h;
    if (h != 0) {
        CK(cudaMemset(c->status, 0, sizeof(int)));
        return BTC_ERR_DEVICE;
    }
    return BTC_OK;
}

btc_status btc_train_epoch(btc_ctx* c, btc_epoch_stats* st)
{
    if (!c)
        return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    int launches = 0;
    CK(cudaEventRecord(c->ev0, c->stream));
    btc_status rc = enqueue_epoch(c, &launches);
    if (rc)
        return rc;
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    int word = 0;
    btc_status rs = check_status(c, &word);
    if (st) {
        st->kernel_ms = ms;
        st->updates = c->updates;
        st->launches = launches;
        st->device_status = word;
    }
    return rs;
}

btc_status btc_train_epochs(btc_ctx* c, int32_t n, btc_epoch_stats* st)
{
    if (!c || n < 0)
        return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    int launches = 0, total = 0;
    CK(cudaEventRecord(c->ev0, c->stream));
    for (int32_t i = 0; i < n; i++) {
        btc_status rc = enqueue_epoch(c, &launches);
        if (rc)
            return rc;
        total += launches;
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    int word = 0;
    btc_status rs = check_status(c, &word);
    if (st) {
        st->kernel_ms = ms;
        st->updates = c->updates * (int64_t)n;
        st->launches = total;
        st->device_status = word;
    }
    return rs;
}

btc_status btc_ctx_set_work_units(btc_ctx* c, const int32_t* unit_off, int32_t nunits)
{
    if (!c || c->mode != BTC_MODE_STAGED || nunits < 0 || (nunits > 0 && !unit_off))
        return BTC_ERR_ARG;
    if (nunits == 0 || unit_off[0] != 0 || unit_off[nunits] != c->nslots)
        return BTC_ERR_ARG;
    for (int32_t u = 0; u < nunits; u++)
        if (unit_off[u + 1] <= unit_off[u])
            return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    free_dev(c->unit_off);
    btc_status rc = upload((void**)&c->unit_off, unit_off, ((size_t)nunits + 1) * 4, c->stream);
    if (rc)
        return rc;
    CK(cudaStreamSynchronize(c->stream));
    c->nunits = nunits;
    return BTC_OK;
}

btc_status btc_ctx_block_profile(btc_ctx* c, float* features, float* log_us, int64_t* n)
{
    if (!c || !n || c->mode != BTC_MODE_STAGED)
        return BTC_ERR_ARG;
    const int64_t nb = (int64_t)c->blk_ids.size();
    if (*n < nb || (nb > 0 && (!features || !log_us))) {
        *n = nb;
        return BTC_ERR_ARG;
    }
    std::vector<uint32_t> ns((size_t)c->st_tiles);
    btc_epoch_stats es{};
    btc_status rc = btc_train_epoch_profiled(c, ns.data(), &es);
    if (rc)
        return rc;
    int64_t k = 0;
    for (int64_t i = 0; i < nb; i++) {
        double t = 0;
        for (int q = c->blk_tile0[(size_t)i]; q < c->blk_tile0[(size_t)i] + c->blk_ntiles[(size_t)i]; q++)
            t += ns[(size_t)q] * 1e-3;
        if (t <= 0)
            continue;
        std::copy(c->blk_feat.begin() + i * BTC_BLOCK_FEATURES, c->blk_feat.begin() + (i + 1) * BTC_BLOCK_FEATURES,
                  features + k * BTC_BLOCK_FEATURES);
        log_us[k] = (float)std::log(t);
        k++;
    }
    *n = k;
    return BTC_OK;
}

btc_status btc_ctx_slot_tiles(btc_ctx* c, int32_t* tile0, int32_t* ntiles)
{
    if (!c || !tile0 || !ntiles || c->mode != BTC_MODE_STAGED)
        return BTC_ERR_ARG;
    CK(cudaMemcpy(tile0, c->slot_tile0, (size_t)c->nslots * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ntiles, c->slot_ntiles, (size_t)c->nslots * 4, cudaMemcpyDeviceToHost));
    return BTC_OK;
}

// The learned work-unit packing of the staged kernel:
// 1. profile  one training epoch records the time of every tile;
// 2. learn    the MLP (mlp.cu) is trained on the GPU to map a tile's features
//             to log(time in microseconds);
// 3. propose  every tile's time is predicted; a slot's cost is the sum over
//             its tiles plus the measured per-slot overhead (CTA time spent
//             outside tiles: taking work from the global counter, slot
//             set-up); consecutive slots are packed into units of about equal
//             predicted cost, at least 8 per CTA so that no CTA is left with a
//             long last unit;
// 4. trial    epochs with the proposed units and with one slot per unit are
//             timed alternately; the faster packing stays.
btc_status btc_ctx_learn_work_units(btc_ctx* c, btc_mlp* model, int32_t train_steps, int32_t trial_epochs,
                                    btc_learn_report* rep)
{
    if (!c || !model || train_steps < 0 || trial_epochs < 1 || !rep || c->mode != BTC_MODE_STAGED)
        return BTC_ERR_ARG;
    btc_learn_report r{};
    const int64_t ntiles = c->st_tiles;
    if (ntiles == 0 || c->nslots == 0)
        return BTC_ERR_STATE;
    std::vector<int> plain((size_t)c->nslots + 1);
    for (int k = 0; k <= c->nslots; k++)
        plain[(size_t)k] = k;
    btc_status rc = btc_ctx_set_work_units(c, plain.data(), c->nslots);
    if (rc)
        return rc;
    std::vector<uint32_t> ns((size_t)ntiles);
    btc_epoch_stats es{};
    if ((rc = btc_train_epoch_profiled(c, ns.data(), &es)))
        return rc;
    std::vector<float> x, y;
    double tile_us = 0;
    for (int64_t t = 0; t < ntiles; t++) {
        if (ns[(size_t)t] == 0)
            continue;
        x.insert(x.end(), c->tile_feat.begin() + t * BTC_TILE_FEATURES,
                 c->tile_feat.begin() + (t + 1) * BTC_TILE_FEATURES);
        y.push_back(std::log(std::max(1e-3f, (float)ns[(size_t)t] * 1e-3f)));
    }
    // time of each executed tile instance: a block's tiles run once per slot
    for (int k = 0; k < c->nslots; k++)
        for (int t = c->h_tile0[(size_t)k]; t < c->h_tile0[(size_t)k] + c->h_ntiles[(size_t)k]; t++)
            tile_us += ns[(size_t)t] * 1e-3;
    r.samples = (int64_t)y.size();
    if (r.samples < 16)
        return BTC_ERR_STATE;
    if ((rc = btc_mlp_train(model, x.data(), y.data(), r.samples, train_steps, 3e-3f, &r.model_loss)))
        return rc;
    double mean = 0, var = 0;
    for (float v : y)
        mean += v;
    mean /= (double)y.size();
    for (float v : y)
        var += (v - mean) * (v - mean);
    var /= (double)y.size();
    r.model_r2 = var > 0 ? 1.0 - r.model_loss / var : 0.0;
    std::vector<float> pred((size_t)ntiles);
    if ((rc = btc_mlp_predict(model, c->tile_feat.data(), ntiles, pred.data())))
        return rc;
    // per-slot overhead: CTA time of the epoch not spent inside tiles
    const double cta_us = es.kernel_ms * 1e3 * c->st_grid;
    const double overhead = std::max(0.0, (cta_us - tile_us) / c->nslots);
    std::vector<double> cost((size_t)c->nslots);
    double total = 0;
    for (int k = 0; k < c->nslots; k++) {
        double v = overhead;
        for (int t = c->h_tile0[(size_t)k]; t < c->h_tile0[(size_t)k] + c->h_ntiles[(size_t)k]; t++)
            v += std::exp((double)pred[(size_t)t]);
        cost[(size_t)k] = v;
        total += v;
    }
    const double target = total / ((double)c->st_grid * 8.0);
    std::vector<int> units(1, 0);
    double acc = 0;
    for (int k = 0; k < c->nslots; k++) {
        acc += cost[(size_t)k];
        if (acc >= target || k + 1 == c->nslots) {
            units.push_back(k + 1);
            acc = 0;
        }
    }
    r.units = (int32_t)units.size() - 1;
    // trial: alternate the two packings
    double t_plain = 0, t_learn = 0;
    for (int e = 0; e < trial_epochs; e++) {
        btc_epoch_stats a{}, b{};
        if ((rc = btc_ctx_set_work_units(c, plain.data(), c->nslots)) || (rc = btc_train_epoch(c, &a)))
            return rc;
        if ((rc = btc_ctx_set_work_units(c, units.data(), r.units)) || (rc = btc_train_epoch(c, &b)))
            return rc;
        t_plain += a.kernel_ms;
        t_learn += b.kernel_ms;
    }
    r.plain_ms = t_plain / trial_epochs;
    r.learned_ms = t_learn / trial_epochs;
    r.kept = r.learned_ms < r.plain_ms ? 1 : 0;
    if (!r.kept && (rc = btc_ctx_set_work_units(c, plain.data(), c->nslots)))
        return rc;
    *rep = r;
    return BTC_OK;
}

btc_status btc_ctx_autotune(btc_ctx* c, int32_t epochs, btc_autotune_report* rep)
{
    if (!c || epochs < 1 || !rep || c->mode != BTC_MODE_STAGED)
        return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    int G0, NV0;
    btc::staged_default_shape(c->dtype, c->R, &G0, &NV0);
    std::vector<std::pair<int, int>> shapes;
    shapes.push_back({G0, NV0});
    if (G0 >= 2 && btc::staged_shape_exists(c->dtype, c->R, G0 / 2, NV0 * 2))
        shapes.push_back({G0 / 2, NV0 * 2});
    if (NV0 >= 2 && NV0 % 2 == 0 && btc::staged_shape_exists(c->dtype, c->R, G0 * 2, NV0 / 2))
        shapes.push_back({G0 * 2, NV0 / 2});
    const int def_grid = c->st_grid;
    double best = 1e300, def_ms = 0;
    int bG = G0, bNV = NV0, bgrid = def_grid, n = 0;
    for (auto& sh : shapes) {
        int occ = btc::staged_blocks_per_sm_shape(c->dtype, c->R, sh.first, sh.second, c->st_block, c->st_smem);
        for (int k = 2; k <= occ; k++) {
            c->st_G = sh.first;
            c->st_NV = sh.second;
            c->st_grid = c->sms * k;
            btc_epoch_stats st{};
            btc_status rc = btc_train_epochs(c, epochs, &st);
            if (rc)
                return rc;
            const double ms = st.kernel_ms / epochs;
            n++;
            if (sh.first == G0 && sh.second == NV0 && c->st_grid == def_grid)
                def_ms = ms;
            if (ms < best) {
                best = ms;
                bG = sh.first;
                bNV = sh.second;
                bgrid = c->st_grid;
            }
        }
    }
    c->st_G = bG;
    c->st_NV = bNV;
    c->st_grid = bgrid;
    rep->lanes_per_entry = bG;
    rep->vectors_per_lane = bNV;
    rep->ctas_per_sm = bgrid / std::max(1, c->sms);
    rep->candidates = n;
    rep->best_ms = best;
    rep->default_ms = def_ms;
    return BTC_OK;
}

btc_status btc_ctx_tile_count(btc_ctx* c, int64_t* n)
{
    if (!c || !n)
        return BTC_ERR_ARG;
    *n = c->mode == BTC_MODE_STAGED ? (int64_t)c->st_tiles : 0;
    return BTC_OK;
}

btc_status btc_ctx_tile_features(btc_ctx* c, float* f)
{
    if (!c || !f || c->mode != BTC_MODE_STAGED)
        return BTC_ERR_ARG;
    std::copy(c->tile_feat.begin(), c->tile_feat.end(), f);
    return BTC_OK;
}

btc_status btc_train_epoch_profiled(btc_ctx* c, uint32_t* tile_ns, btc_epoch_stats* st)
{
    if (!c || !tile_ns || c->mode != BTC_MODE_STAGED)
        return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    if (!c->tile_ns)
        CK(cudaMalloc((void**)&c->tile_ns, std::max<size_t>(16, (size_t)c->st_tiles * sizeof(unsigned))));
    CK(cudaMemsetAsync(c->tile_ns, 0, std::max<size_t>(16, (size_t)c->st_tiles * sizeof(unsigned)), c->stream));
    c->profile_next = true;
    btc_status rc = btc_train_epoch(c, st);
    c->profile_next = false;
    if (rc)
        return rc;
    CK(cudaMemcpy(tile_ns, c->tile_ns, (size_t)c->st_tiles * sizeof(unsigned), cudaMemcpyDeviceToHost));
    return BTC_OK;
}

btc_status btc_device_count(int32_t* count)
{
    if (!count)
        return BTC_ERR_ARG;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        *count = 0;
        cuda_fail(e, "cudaGetDeviceCount");
        return e == cudaErrorNoDevice ? BTC_ERR_NO_DEVICE : BTC_ERR_CUDA;
    }
    *count = n;
    return BTC_OK;
}

btc_status btc_device_info(int32_t device, char* name, int32_t* sm_count, int64_t* memory_bytes)
{
    cudaDeviceProp p;
    CK(cudaGetDeviceProperties(&p, device));
    if (name) {
        std::strncpy(name, p.name, 255);
        name[255] = 0;
    }
    if (sm_count)
        *sm_count = p.multiProcessorCount;
    if (memory_bytes)
        *memory_bytes = (int64_t)p.totalGlobalMem;
    return BTC_OK;
}

btc_status btc_host_alloc(void** p, int64_t bytes)
{
    if (!p || bytes < 0)
        return BTC_ERR_ARG;
    *p = nullptr;
    CK(cudaHostAlloc(p, (size_t)std::max<int64_t>(bytes, 1), cudaHostAllocDefault));
    return BTC_OK;
}

void btc_host_free(void* p)
{
    if (p)
        cudaFreeHost(p);
}

static void finish_metrics(const double* r, int64_t n, btc_metrics* o)
{
    const double nan = std::numeric_limits<double>::quiet_NaN();
    o->count = n;
    o->sse = r[0];
    o->sae = r[1];
    o->ref2 = r[2];
    if (n == 0) {
        o->rmse = o->mae = o->er = nan;
        return;
    }
    o->rmse = std::sqrt(r[0] / (double)n);
    o->mae = r[1] / (double)n;
    o->er = r[2] > 0 ? r[0] / r[2] : nan;
}

btc_status btc_eval(btc_ctx* c, int32_t split, btc_metrics* out)
{
    if (!c || !out || split < 0 || split > 1)
        return BTC_ERR_ARG;
    CK(cudaSetDevice(c->cfg.device));
    double r[3] = {0, 0, 0};
    int64_t n = c->eval_n[split];
    if (n > 0) {
        CK(btc::launch_metrics(c->dtype, c->eval_coo[split], c->eval_val[split], n, c->F[0], c->F[1],
                               c->F[2], c->R, c->Rp, c->partials, c->metric_grid, c->result, c->stream));
        CK(cudaMemcpyAsync(r, c->result, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    finish_metrics(r, n, out);
    return BTC_OK;
}

btc_status btc_train_epoch_host(btc_ctx* c, double* A, double* B, double* C, btc_epoch_stats* st,
                                btc_metrics* test)
{
    if (!c || !A || !B || !C)
        return BTC_ERR_ARG;
    double* H[3] = {A, B, C};
    btc_status rc;
    for (int m = 0; m < 3; m++)
        if ((rc = btc_ctx_set_factors(c, m, H[m])))
            return rc;
    if ((rc = btc_train_epoch(c, st)))
        return rc;
    if (test && (rc = btc_eval(c, BTC_SPLIT_TEST, test)))
        return rc;
    for (int m = 0; m < 3; m++)
        if ((rc = btc_ctx_get_factors(c, m, H[m])))
            return rc;
    return BTC_OK;
}

struct btc_batch {
    std::vector<btc_ctx*> ctx;
    int dtype = 0, device = 0, nitems = 0, grid = 0;
    size_t smem = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    btc::StagedArgs* args = nullptr;
    int2* items = nullptr;
    int* counter = nullptr;
    unsigned* seed = nullptr;
    btc::RefreshJob* refresh = nullptr;  // BF16: one master refresh job per (context, mode) with hot rows
    int nrefresh = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t updates = 0;
    int launches = 0;
};

btc_status btc_batch_destroy(btc_batch* b)
{
    if (!b)
        return BTC_OK;
    cudaSetDevice(b->device);
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    free_dev(b->args);
    free_dev(b->items);
    free_dev(b->counter);
    free_dev(b->seed);
    free_dev(b->refresh);
    if (b->ev0)
        cudaEventDestroy(b->ev0);
    if (b->ev1)
        cudaEventDestroy(b->ev1);
    if (b->stream)
        cudaStreamDestroy(b->stream);
    delete b;
    return BTC_OK;
}

static btc_status batch_build(btc_batch* b)
{
    CK(cudaSetDevice(b->device));
    CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&b->ev0));
    CK(cudaEventCreate(&b->ev1));
    const int n = (int)b->ctx.size();
    std::vector<btc::StagedArgs> args((size_t)n);
    std::vector<std::pair<double, int2>> order;
    for (int t = 0; t < n; t++) {
        btc_ctx* c = b->ctx[(size_t)t];
        args[(size_t)t] = staged_args(c);
        args[(size_t)t].seed = 0x2545F491u * (unsigned)(t + 1);
        // lanes per entry for the batched kernel: the rank's 16-byte vectors,
        // at most 8 lanes (and at most 4 vectors per lane)
        const int vecs = c->Rp / 4;
        int G = 1;
        while (G < 8 && G < vecs)
            G *= 2;
        if ((vecs + G - 1) / G > 4)
            return BTC_ERR_UNSUPPORTED;
        args[(size_t)t].G = G;
        b->smem = std::max(b->smem, btc::staged_smem_bytes(b->dtype, c->Rp, c->st_cap, c->st_wave));
        b->updates += c->updates;
        // interleave: unit u of tensor t is placed at its progress fraction
        for (int u = 0; u < c->nunits; u++)
            order.push_back({((double)u + 0.5) / (double)c->nunits, make_int2(t, u)});
    }
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<double, int2>& x, const std::pair<double, int2>& y) { return x.first < y.first; });
    std::vector<int2> items;
    items.reserve(order.size());
    for (auto& o : order)
        items.push_back(o.second);
    b->nitems = (int)items.size();
    CK(cudaMalloc((void**)&b->seed, sizeof(unsigned)));
    CK(cudaMemsetAsync(b->seed, 0, sizeof(unsigned), b->stream));
    for (auto& a : args)
        a.seed_ptr = b->seed;
    btc_status rc;
    if ((rc = upload((void**)&b->args, args.data(), args.size() * sizeof(btc::StagedArgs), b->stream)))
        return rc;
    if ((rc = upload((void**)&b->items, items.data(), items.size() * sizeof(int2), b->stream)))
        return rc;
    CK(cudaMalloc((void**)&b->counter, sizeof(int)));
    if (b->dtype == BTC_DTYPE_BF16) {
        std::vector<btc::RefreshJob> jobs;
        for (btc_ctx* c : b->ctx)
            for (int a = 0; a < 3; a++)
                if (c->nhot[a] > 0)
                    jobs.push_back({c->master[a], static_cast<unsigned short*>(c->F[a]), c->hot_rows[a], c->nhot[a],
                                    c->Rp});
        b->nrefresh = (int)jobs.size();
        if ((rc = upload((void**)&b->refresh, jobs.data(), jobs.size() * sizeof(btc::RefreshJob), b->stream)))
            return rc;
    }
    int occ = btc::staged_multi_blocks_per_sm(b->dtype, b->smem);
    if (occ <= 0)
        return BTC_ERR_UNSUPPORTED;
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, b->device));
    b->grid = prop.multiProcessorCount * occ;
    CK(cudaStreamSynchronize(b->stream));
    return BTC_OK;
}

btc_status btc_batch_create(btc_ctx* const* ctxs, int32_t n, btc_batch** out)
{
    if (!ctxs || n <= 0 || !out)
        return BTC_ERR_ARG;
    *out = nullptr;
    const int dtype = ctxs[0]->dtype, device = ctxs[0]->cfg.device;
    for (int i = 0; i < n; i++) {
        const btc_ctx* c = ctxs[i];
        if (!c || c->mode != BTC_MODE_STAGED || c->dtype != dtype || c->cfg.device != device || c->R > 128)
            return BTC_ERR_ARG;
    }
    if (dtype == BTC_DTYPE_F64)
        return BTC_ERR_UNSUPPORTED;
    btc_batch* b = new (std::nothrow) btc_batch();
    if (!b)
        return BTC_ERR_ALLOC;
    b->ctx.assign(ctxs, ctxs + n);
    b->dtype = dtype;
    b->device = device;
    btc_status rc;
    try {
        rc = batch_build(b);
    } catch (const std::bad_alloc&) {
        rc = BTC_ERR_ALLOC;
    }
    if (rc) {
        btc_batch_destroy(b);
        return rc;
    }
    *out = b;
    return BTC_OK;
}

static btc_status batch_enqueue(btc_batch* b, int* launches)
{
    int n = 0;
    CK(cudaMemsetAsync(b->counter, 0, sizeof(int), b->stream));
    CK(btc::launch_staged_multi(b->dtype, b->args, b->items, b->nitems, b->counter, b->smem, b->grid, b->stream));
    n++;
    if (b->nrefresh > 0) {
        // every context's BF16 copies of its hot rows, in one launch
        CK(btc::launch_master_refresh_multi(b->refresh, b->nrefresh, b->stream));
        n++;
    }
    CK(btc::launch_seed_step(b->seed, b->stream));
    n++;
    if (launches)
        *launches = n;
    return BTC_OK;
}

btc_status btc_batch_train_epochs(btc_batch* b, int32_t epochs, int32_t use_graph, btc_epoch_stats* st)
{
    if (!b || epochs < 0)
        return BTC_ERR_ARG;
    CK(cudaSetDevice(b->device));
    int per = 0;
    if (use_graph && !b->exec) {
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        btc_status rc = batch_enqueue(b, &per);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc)
            return rc;
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaStreamEndCapture");
        b->graph = g;
        CK(cudaGraphInstantiate(&b->exec, g, 0));
        b->launches = per;
    }
    CK(cudaEventRecord(b->ev0, b->stream));
    int total = 0;
    for (int e = 0; e < epochs; e++) {
        if (use_graph) {
            CK(cudaGraphLaunch(b->exec, b->stream));
            total += b->launches;
        } else {
            btc_status rc = batch_enqueue(b, &per);
            if (rc)
                return rc;
            total += per;
        }
    }
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaEventSynchronize(b->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    btc_status rs = BTC_OK;
    int word = 0;
    for (btc_ctx* c : b->ctx) {
        int w = 0;
        btc_status r1 = check_status(c, &w);
        if (r1 && !rs)
            rs = r1;
        word |= w;
    }
    if (st) {
        st->kernel_ms = ms;
        st->updates = b->updates * (int64_t)epochs;
        st->launches = total;
        st->device_status = word;
    }
    return rs;
}

}  // extern "C"
