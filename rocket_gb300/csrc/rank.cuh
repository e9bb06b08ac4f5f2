// rank.cuh -- dense key ranks over the union of a set of vectors' keys.
#pragma once
#include "common.cuh"

namespace phylo {

// Words of the union bitmap of keys below key_limit (bit k of word k / 32).
size_t rank_bitmap_words(uint64_t key_limit);

// Scratch for key_ranks over keys below key_limit (bitmap + per-word prefix).
size_t rank_scratch_bytes(uint64_t key_limit);

// ranks[e] = number of distinct keys of the set below keys[e] (padding keys
// 0xffffffff stay 0xffffffff; ranks null: only the union prefix is built, for
// key_rank_index); *d_union (device) = union size.  union_bits,
// when not null, is the union bitmap of the set's keys, already marked (the
// batched build can mark it); otherwise it is built here.  Asynchronous.
cudaError_t key_ranks(const uint32_t *keys, const uint64_t *vec_off, uint32_t N, uint64_t max_len,
                      uint64_t key_limit, const uint32_t *union_bits, void *scratch,
                      size_t scratch_size, uint32_t *ranks, uint64_t *d_union, cudaStream_t st);

int key_ranks_launches(bool marked);

// After key_ranks (with ranks null: the union prefix only) on the same scratch,
// key limit and bitmap: the ranks of the set's keys and, in the same pass, the
// window index over them -- roff[v][r] = entries of vector v with rank < r << wshift,
// r = 0..R.  Vectors start on 16-byte boundaries and are padded to multiples of 4
// entries with keys 0xffffffff.  entries = vec_off[N] - vec_off[0] when the
// caller knows it (0 if not): arenas of very uneven vectors are then walked as
// one sequence (two launches) instead of by (slice, vector) CTAs (one launch).
// Asynchronous.
cudaError_t key_rank_index(const uint32_t *keys, const uint64_t *vec_off, uint32_t N,
                           uint64_t max_len, uint64_t entries, uint64_t key_limit,
                           const uint32_t *union_bits,
                           void *scratch, size_t scratch_size, uint32_t wshift, uint32_t R,
                           uint32_t *ranks, uint32_t *roff, cudaStream_t st);

// pw[w] = {set bits of words [0, w) of a bitmap (uint32; the total must stay
// below 2^32), bits[w]}: the prefix stored beside each word, so a rank lookup
// is one 8-byte load; *total = all set bits (device).  partials holds
// bitmap_prefix_partials(nwords) entries.  Three launches.
cudaError_t bitmap_prefix_pairs(const uint32_t *bits, uint64_t nwords, uint64_t *partials,
                                uint2 *pw, uint64_t *total, cudaStream_t st);
uint64_t bitmap_prefix_partials(uint64_t nwords);

}  // namespace phylo
