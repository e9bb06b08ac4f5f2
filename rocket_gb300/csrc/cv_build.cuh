// cv_build.cuh -- device-side composition-vector construction (declarations).
#pragma once
#include "common.cuh"

namespace phylo {

struct BuildGeometry {
    int alpha, k;
    uint32_t A;      // alphabet size (21 protein, 4 DNA)
    uint64_t T1, T2; // A^(K-1), A^(K-2)
    uint64_t NCH;    // chunks of (K-1)-mers per proteome
};

// Everything a build launch needs; plain device pointers, passed by value.
struct BuildArgs {
    int alpha, k, B;
    uint32_t A;
    uint64_t T1, T2, NCH;
    // input: concatenated sequences, seq_off[B+1] (device)
    const uint8_t *seq;
    const uint64_t *seq_off;
    uint64_t *seq_off_store;  // scratch home for seq_off of a single proteome
    uint64_t *tile_base;      // [B+1]
    // dense per-proteome tables
    uint32_t *c1, *coff;      // [B][T1]
    uint32_t *c2, *mask;      // [B][T2]
    uint32_t *tot;            // [B][4]: n0, n1, n2, -
    // per (proteome, chunk)
    uint32_t *chunk_cand;     // candidates per chunk
    uint64_t *chunk_cand_off; // exclusive scan (global over the batch), [nc+1]
    uint32_t *chunk_surv;     // survivors per chunk
    uint64_t *chunk_out_off;  // exclusive scan, [nc+1]
    uint32_t *chunk_m1;       // survivors with alpha^2 == 1
    double *chunk_nhi, *chunk_nlo;
    uint64_t *scan_tmp;
    // per proteome results
    double *norm, *scale;
    uint64_t *nnz, *out_base;
    uint64_t *dst_base, *dst_cap;  // where k_compact writes proteome p
    uint32_t *status;
    // K-mer counts per candidate, replaced by alpha bits
    uint32_t *c0a;
    uint64_t cand_cap;
    // output arena
    uint32_t *out_keys;
    float *out_vals;
};

// Returns 0, -1 (bad alphabet/k) or -2 (keys would not fit uint32).
int build_geometry(int alpha, int k, BuildGeometry *g);
size_t build_scratch_bytes(const BuildGeometry &g, int B, uint64_t cand_cap);
cudaError_t build_carve(const BuildGeometry &g, int B, uint64_t cand_cap, void *scratch,
                        size_t scratch_size, BuildArgs *a);
cudaError_t build_plan(BuildArgs &a, cudaStream_t st);
cudaError_t build_emit(BuildArgs &a, cudaStream_t st);
int build_launches_per_batch();

}  // namespace phylo
