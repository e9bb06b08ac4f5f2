// compare.cuh -- sparse cosine of one pair (declarations).
#pragma once
#include "common.cuh"

namespace phylo {

// Scratch needed to compare two vectors whose sizes sum to at most max_total.
size_t compare_scratch_bytes(uint64_t max_total);

// Launches the pair kernels on `stream`; writes C (double) to d_out.
// *status_out (device address) receives a DeviceError bit set after completion.
cudaError_t compare_launch(cudaStream_t stream, void *scratch, size_t scratch_size,
                           const uint32_t *lk, const float *lv, uint32_t nl, const uint32_t *rk,
                           const float *rv, uint32_t nr, double *d_out, uint32_t **status_out);

// Same kernels on the library's built-in scratch array (no caller scratch, no
// allocation); at most compare_static_max_entries() entries in the two vectors.
// The first call on a device looks the array's address up (cudaGetSymbolAddress).
cudaError_t compare_launch_static(cudaStream_t stream, const uint32_t *lk, const float *lv,
                                  uint32_t nl, const uint32_t *rk, const float *rv, uint32_t nr,
                                  double *d_out, uint32_t **status_out);
uint64_t compare_static_max_entries();

// Merged elements per tile of the merge-path kernels (the unit of max_tiles).
uint32_t compare_tile_elements();

// Poll limit of every compare CTA's first mbarrier wait (0xffffffff: the default).
// A test hook: 0 makes each CTA give up at once after issuing its copies, which
// exercises the bounded-wait path (status bit, drained copies) without a fault.
void compare_set_first_wait_limit(uint32_t limit);
size_t compare_static_bytes();

// Many pairs per launch: C of pair p = (left vector pa[p], right vector pb[p])
// to out[p].  max_tiles bounds sum over pairs of ceil((nl + nr) / 4096).
size_t compare_many_scratch_bytes(uint32_t P, uint64_t max_tiles);
cudaError_t compare_many_launch(cudaStream_t st, void *scratch, size_t scratch_size,
                                const uint32_t *lkeys, const float *lvals, const uint64_t *loff,
                                const uint32_t *lnnz, const uint32_t *rkeys, const float *rvals,
                                const uint64_t *roff, const uint32_t *rnnz, const uint32_t *pa,
                                const uint32_t *pb, uint32_t P, uint64_t max_tiles, double *out,
                                uint32_t **status_out);

}  // namespace phylo
