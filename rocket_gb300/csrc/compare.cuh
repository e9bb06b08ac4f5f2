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
size_t compare_static_bytes();

}  // namespace phylo
