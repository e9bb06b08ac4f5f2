// allpairs.cuh -- batched pair engine (declarations).
#pragma once
#include "common.cuh"

namespace phylo {

constexpr int AP_TI = 16;             // row vectors per item (densified in shared memory)
constexpr int AP_LPC = 4;             // lanes per column vector (2 for 256-column items)

// One unit of work: up to tile_rows row vectors x tile_cols column vectors over
// the key windows [w0, w1).  Vectors are named by positions in rowids / colids.
struct ApItem {
    uint32_t row0, nrow;  // rows: rowids[row0 .. row0 + nrow)
    uint32_t col0, ncol;  // columns: colids[col0 .. col0 + ncol)
    uint32_t w0, w1;      // key windows
    uint32_t part;        // index of this item's tile_rows x tile_cols partial block
    uint32_t tile;        // tile this item contributes to
};

// Rows and columns may live in different arenas (e.g. arriving queries against
// a resident database); for all pairs of one arena both sides are the same.
struct ApArena {
    const uint32_t *keys;
    const float *vals;
    const uint64_t *vec_off;   // [N+1] arena offsets, each a multiple of 4 entries
    const uint32_t *roff;      // [N][R+1] window index
};

struct ApArgs {
    ApArena row, col;
    uint32_t R;                // windows per vector
    uint32_t wshift;           // window width = 1 << wshift keys
    const uint32_t *rowids, *colids;
    const ApItem *items;
    uint32_t nitems;
    uint32_t *counter;         // work counter (zeroed before launch)
    FF *part;                  // [parts][tile rows][tile cols]
    uint32_t fold;             // products per accumulator between compensated folds
    int64_t *item_cycles;      // optional per-item clock64 durations (may be null)
};

// Tile shapes (tile_rows x tile_cols) select the kernel: 16 x 128 (512 threads),
// 16 x 64 (256) and 16 x 32 (128) use 80-byte key records and four lanes per column,
// 16 x 256 (512 threads) the same records and two lanes per column; 32 x 64 uses
// 128-byte swizzled records and eight lanes per column.
bool ap_shape_ok(int tile_rows, int tile_cols);
size_t ap_smem_bytes(uint32_t wshift, int tile_rows, int tile_cols);
int ap_max_wshift(int tile_rows, int tile_cols);
int ap_threads(uint32_t wshift, int tile_rows, int tile_cols);
cudaError_t ap_prepare(uint32_t wshift, int tile_rows, int tile_cols, int *ctas_per_sm);
cudaError_t ap_launch(const ApArgs &a, int tile_rows, int tile_cols, int grid, cudaStream_t st);

// window index: roff[v][r] = number of entries of vector v with key < r << wshift
cudaError_t range_index_launch(const uint32_t *keys, const uint64_t *vec_off, uint32_t N,
                               uint32_t R, uint32_t wshift, uint32_t *roff, cudaStream_t st,
                               uint64_t max_len);

// Tile t (rows rowids[row0..], columns colids[col0..]) has S partial blocks
// part[t * S + s].  Writes out[rowid * ldc + colid] (and the mirrored entry
// when `mirror`), for pairs with row position < column position when `upper` is
// 1, <= when it is 2.
struct ApTile {
    uint32_t row0, nrow, col0, ncol;
};
struct ApReduceArgs {
    const FF *part;            // blocks of ti x tj float pairs
    const ApTile *tiles;
    uint32_t ntiles, S, ti, tj;
    const uint32_t *rowids, *colids;
    double *out;
    uint64_t ldc;
    int upper, mirror;
};
cudaError_t ap_reduce_launch(const ApReduceArgs &r, cudaStream_t st);

// C of each vector with itself (sum of squares, float-float): out[v*ldc+v].
// `part` holds self_dot_part_count(N, max_len) float pairs.
cudaError_t self_dot_launch(const float *vals, const uint64_t *vec_off, uint32_t N, double *out,
                            uint64_t ldc, uint64_t max_len, FF *part, cudaStream_t st);
uint64_t self_dot_part_count(uint32_t N, uint64_t max_len);

}  // namespace phylo
