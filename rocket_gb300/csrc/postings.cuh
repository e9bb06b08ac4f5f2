// postings.cuh -- key-major (postings) pair engine (declarations).
//
// Products of only the keys two vectors share: for a block of row vectors and a
// block of column vectors, every key window's entries are regrouped by key in
// shared memory (a counting sort into per-key postings), and each key then
// contributes the products of its row entries with its column entries.  The
// products are exact fixed-point integers (2^-46 units) summed with 32-bit
// shared-memory atomics that carry into a high word, so the sums are exact and
// independent of the order in which the atomics land.
#pragma once
#include "allpairs.cuh"
#include "common.cuh"

namespace phylo {

constexpr int PB_SCALE = 46;  // accumulators hold C * 2^46 (int64)

// One unit of work: rows rowids[row0 .. row0 + nrow) x columns colids[col0 ..
// col0 + ncol) over key windows [w0, w1).  diag = 1 when the rows and the
// columns are the same block (each unordered pair and each self product once).
struct PbItem {
    uint32_t row0, nrow;
    uint32_t col0, ncol;
    uint32_t w0, w1;
    uint32_t part;  // index of this item's block x block int64 partial
    uint32_t diag;
};

struct PbArgs {
    ApArena row, col;          // keys are the window-indexed keys (ranks or raw keys)
    uint32_t R;                // windows per vector
    uint32_t wshift;           // window width = 1 << wshift keys
    const uint32_t *rowids, *colids;
    const PbItem *items;
    uint32_t nitems;
    uint32_t *counter;         // work counter (zeroed before launch)
    int64_t *part;             // [parts][block][block]
    uint32_t *status;          // DeviceError bits (may be null)
    int64_t *item_cycles;      // optional per-item clock64 durations (may be null)
};

// Block sizes (vectors per side of a work item): 128 (1024 threads, one CTA per
// SM) or 64 (512 threads, two CTAs per SM).
bool pb_block_ok(int block);
size_t pb_smem_bytes(int block, uint32_t wshift);
uint32_t pb_capacity(int block, uint32_t wshift);  // posting entries per side and chunk
int pb_threads(int block);
cudaError_t pb_prepare(int block, uint32_t wshift, int *ctas_per_sm);
cudaError_t pb_launch(const PbArgs &a, int block, int grid, cudaStream_t st);

// Tile t covers rows rowids[row0..] x columns colids[col0..] with partials
// part[part0 .. part0 + nparts).  C of each pair goes to out[rowid * ldc + colid]
// (and the mirrored entry when `mirror`); in a diag tile the pairs with row
// position < column position, and with `self` also the self products.
struct PbTile {
    uint32_t row0, nrow, col0, ncol;
    uint32_t part0, nparts, diag, pad;
};
struct PbReduceArgs {
    const int64_t *part;
    const PbTile *tiles;
    uint32_t ntiles, block;
    const uint32_t *rowids, *colids;
    double *out;
    uint64_t ldc;
    int self, mirror;
};
cudaError_t pb_reduce_launch(const PbReduceArgs &r, cudaStream_t st);

}  // namespace phylo
