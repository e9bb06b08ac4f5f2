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

}  // namespace phylo
