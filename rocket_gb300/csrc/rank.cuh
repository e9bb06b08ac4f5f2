// rank.cuh -- dense key ranks over the union of a set of vectors' keys.
#pragma once
#include "common.cuh"

namespace phylo {

// Scratch for key_ranks of N vectors over keys below key_limit (bitmap,
// per-word prefix, 2^16-key range index).
size_t rank_scratch_bytes(uint64_t key_limit, uint32_t N);

// ranks[e] = number of distinct keys of the set below keys[e] (padding keys
// 0xffffffff stay 0xffffffff); *d_union (device) = union size.  Asynchronous.
cudaError_t key_ranks(const uint32_t *keys, const uint64_t *vec_off, uint32_t N, uint64_t max_len,
                      uint64_t key_limit, void *scratch, size_t scratch_size, uint32_t *ranks,
                      uint64_t *d_union, cudaStream_t st);

int key_ranks_launches();

}  // namespace phylo
