// Tiles of the staged kernel: a scheduled block cut into runs of entries
// whose distinct factor rows fit in shared memory.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "schedule.h"

namespace btc {

// One tile: entries [eoff, eoff+n) of the tile entry stream, distinct rows
// [roff, roff+nrows) of the row list (x rows, then y rows, then z rows),
// owner segments [soff, soff+nseg).
struct TileHdr {
    long long eoff;
    long long roff;
    long long soff;
    long long coff;  // csr offset (uint16 units, multiple of 8 so 16-byte copies stay aligned)
    int n;
    int nseg;
    int nrows;
    int nx;
    int ny;
    int pad[3];
};

struct TileSet {
    std::vector<TileHdr> tiles;
    std::vector<int4> ent;        // (lx | ly << 16, lz, 0, value bits): local row ids, y/z offset
    std::vector<uint16_t> csr;    // per tile 3 x n (padded to 8): entries of each mode ordered by row
    std::vector<int4> segs;       // (local row, mode, start in that mode's csr, count)
    std::vector<int32_t> rows;    // global row id of every staged row
    std::vector<double> val64;    // FP64 entry values (f64 tiles)
    std::vector<int> block_tile0, block_ntiles;  // per block id, -1 if unscheduled
    int max_rows = 0, max_n = 0;
};

// cap: rows per tile; wave: entries per tile; seg: entries per owner segment;
// repeat: most entries of any one row in a tile; want64: also keep FP64
// entry values; threads: host threads to use (the result does not depend on
// it).
void build_tiles(const Schedule& s, const int32_t* xyz, const double* val, int I, int J, int K, int cap,
                 int wave, int seg, int repeat, bool want64, TileSet& out, int threads = 1);

}  // namespace btc
