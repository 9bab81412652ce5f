// Launch wrappers of the sm_103a kernels (kernels.cu).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace btc {

// One scheduled slot: a block's entries at [off, off+nnz) of the entry
// stream, with the reference's coe weights already multiplied by lr.
struct SgdArgs {
    const int4* coo;          // (x, y, z, float value bits) per entry, block-ordered
    const double* val64;      // FP64 values (f64 path), else null
    const int2* items;        // Hogwild work items: (slot, first entry in slot)
    long long nitems;
    const long long* slot_off;
    const int* slot_nnz;
    const void* slot_coe;     // 3 per slot, compute type, times lr
    void* A;
    void* B;
    void* C;
    int R;                    // rank
    int Rp;                   // padded row stride (elements)
    double reg;
    int chunk;                // entries per work item
    unsigned long long seed;  // stochastic rounding stream (bf16)
    float* master;            // FP32 master rows for hot rows (bf16), may be null
    const int* hot_map[3];    // row -> master slot, -1 if none (bf16), may be null
};

// Padded row stride for a dtype and rank.
int padded_rank(int dtype, int R);
// Largest rank the kernels support.
constexpr int kMaxRank = 128;

cudaError_t launch_hogwild(int dtype, const SgdArgs& a, int grid, int block, cudaStream_t st);
int hogwild_blocks_per_sm(int dtype, int R, int block);
cudaError_t launch_det_wave(int dtype, const int* wave_slots, int n, const SgdArgs& a,
                            cudaStream_t st);
// One wave of the lock-free rule (slot coe = lr, one block per slot).
cudaError_t launch_lf_wave(int dtype, const int* wave_slots, int n, const SgdArgs& a, cudaStream_t st);
// Metrics: FP64 sums of (ref - dot)^2, |ref - dot| and ref^2 over n entries;
// per-CTA partials then a fixed-order sum into result[0..2].
cudaError_t launch_metrics(int dtype, const int4* coo, const double* val, long long n,
                           const void* A, const void* B, const void* C, int R, int Rp,
                           double* partials, int grid, double* result, cudaStream_t st);
constexpr int kMetricThreads = 256;
// FP32 master rows of a BF16 context: op 0 packs host doubles (src, [rows][R])
// into the masters, op 1 unpacks the masters over dst ([rows][R]), op 2
// refreshes the BF16 copy of every hot row from its master.
cudaError_t launch_master(int op, const double* src, double* dst, float* master, void* bf16, const int* hot_rows,
                          int nhot, int R, int Rp, cudaStream_t st);
// The op-2 refresh of many BF16 contexts in one launch: one job per (context,
// mode) with hot rows.
struct RefreshJob {
    const float* master;
    unsigned short* bf16;
    const int* hot_rows;
    int nhot, Rp;
};
cudaError_t launch_master_refresh_multi(const RefreshJob* jobs, int njobs, cudaStream_t st);
// Advances a device-side rounding seed (one step per replayed epoch).
cudaError_t launch_seed_step(unsigned* p, cudaStream_t st);
// double [rows][R] <-> padded device rows [rows][Rp] of the dtype
cudaError_t launch_pack(int dtype, const double* src, void* dst, long long rows, int R, int Rp,
                        cudaStream_t st);
cudaError_t launch_unpack(int dtype, const void* src, double* dst, long long rows, int R, int Rp,
                          cudaStream_t st);

}  // namespace btc
