// Staged SGD kernel (staged.cu): one CTA per scheduled slot, the slot's rows
// gathered into shared memory, each row written back once per tile.
#pragma once
#include <cuda_runtime.h>

#include "tiles.h"

namespace btc {

struct StagedArgs {
    const TileHdr* tiles;
    const int* slot_tile0;   // first tile of each slot's block
    const int* slot_ntiles;
    const void* slot_coe;    // 3 per slot, compute type, times lr
    int nslots;
    const int* unit_off;     // work units: slots [unit_off[u], unit_off[u+1]) go to one CTA
    int nunits;
    const int4* ent;
    const unsigned short* csr;
    const unsigned* segs;    // owner segments, one packed word each (row 14 bits, mode 2,
                             // count - 1 4, start in the mode's CSR list 12)
    const int* rows;         // global row of every staged row, or ~row for a row
                             // that decays from its value at write time; BF16:
                             // ~(master index, bit 30 = decays at write time) for
                             // a row with an FP32 master
    const double* val64;     // FP64 values (f64), else null
    void* A;
    void* B;
    void* C;
    int R, Rp;
    double reg;
    int cap;                 // rows per tile
    int wave;                // entries per tile
    int* counter;            // next slot to take (zeroed before each launch)
    // BF16 storage only
    float* master[3];        // FP32 master rows of the hottest rows of each mode
    unsigned seed;           // stochastic-rounding stream of this epoch
    int* status;             // device error word read after each epoch (no current
                             // kernel path sets it)
    unsigned* tile_ns;       // when set: nanoseconds each tile took (globaltimer)
    int G, NV;               // lane-group shape; 0 = the default for the rank
    const unsigned* seed_ptr;  // when set, the rounding stream is seed ^ *seed_ptr (graph replays)
};

// Shared-memory layout of one CTA: S rows | entries | errors | row ids (two
// buffers: the current tile's and the next one's, fetched ahead) | two tile
// headers | CSR.  Every region that receives 16-byte copies starts on a
// 16-byte boundary.  es = bytes of one staged row element (8 FP64, 4 FP32,
// 2 BF16); errors are kept in the compute type (8 for FP64, else 4).
struct StagedLayout {
    size_t ent, err, rid, rid2, hdr, csr, total;
    __host__ __device__ StagedLayout(size_t es, int Rp, int cap, int wave)
    {
        auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
        const size_t ee = es == 8 ? 8 : 4;
        ent = al((size_t)cap * Rp * es);
        err = al(ent + (size_t)wave * 16);
        rid = al(err + (size_t)wave * ee);
        rid2 = al(rid + (size_t)cap * 4);
        hdr = al(rid2 + (size_t)cap * 4);
        csr = al(hdr + 2 * sizeof(TileHdr));
        total = al(csr + (3 * (size_t)wave + 8) * 2);
    }
};

// Shared-memory bytes of one CTA for a dtype, rank stride, cap and wave.
size_t staged_smem_bytes(int dtype, int Rp, int cap, int wave);
// Largest cap that fits `ctas_per_sm` CTAs on one SM (at most 16383: a
// segment word holds the local row in 14 bits).
int staged_cap_for(int dtype, int Rp, int wave, int ctas_per_sm, size_t smem_per_sm, size_t smem_per_block);
cudaError_t launch_staged(int dtype, const StagedArgs& a, int grid, int block, cudaStream_t st);
// Many tensors in one launch: `tensors` (device) holds each tensor's
// arguments, `items` (device) the (tensor, unit) work list.
cudaError_t launch_staged_multi(int dtype, const StagedArgs* tensors, const int2* items, int nitems, int* counter,
                                size_t smem, int grid, cudaStream_t st);
int staged_multi_blocks_per_sm(int dtype, size_t smem);
// Lane-group shapes: G lanes per entry, NV 16-byte vectors per lane per row
// (G * NV * vector width must cover the padded rank).
int staged_vector_width(int dtype);
void staged_default_shape(int dtype, int R, int* G, int* NV);
bool staged_shape_exists(int dtype, int R, int G, int NV);
int staged_blocks_per_sm(int dtype, int R, int block, size_t smem);
int staged_blocks_per_sm_shape(int dtype, int R, int G, int NV, int block, size_t smem);

}  // namespace btc
