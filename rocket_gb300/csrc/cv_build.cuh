// cv_build.cuh -- device-side composition-vector construction (declarations).
#pragma once
#include "common.cuh"

namespace phylo {

struct BuildGeometry {
    int alpha, k;
    uint32_t A;      // alphabet size (21 protein, 4 DNA)
    uint64_t T1, T2; // A^(K-1), A^(K-2)
    uint64_t T1s;    // per-proteome row length of the (K-1)-mer tables (T1 rounded up to 32)
    uint64_t T2s;    // the same for the (K-2)-mer tables
    uint64_t NCH;    // chunks of the seen bitmap per proteome (CHUNK_THREADS * wpt words)
    uint32_t wpt;    // bitmap words per thread in the candidate passes
};

// Remainder by a run-time constant d (4 <= d < 2^31) for 32-bit numerators:
// with R = ceil(2^32 / d), a = floor(q * R / 2^32) is floor(q / d) or one more
// (q * R / 2^32 exceeds q / d by less than q / 2^32 < 1), so q - a * d is the
// remainder, or the remainder - d, corrected by one conditional add.
struct FastDiv {
    uint32_t R, d;
    __host__ void set(uint32_t divisor) {
        d = divisor;
        R = (uint32_t)((0xffffffffull + divisor) / divisor);  // ceil(2^32 / d)
    }
    __device__ __forceinline__ uint32_t mod(uint32_t q) const {
        const uint32_t r = q - __umulhi(q, R) * d;
        return (int32_t)r < 0 ? r + d : r;
    }
};

// Candidates per k_alpha CTA (proteomes start on multiples of it) and per
// warp segment (survivors are compacted to the start of their segment).
constexpr uint32_t ALPHA_TILE = 2048;
constexpr uint32_t SEG = 256;

// Count -> probability tables are kept for counts below this bound.
constexpr int PROB_TABLE = 4096;

// Alpha / value tables over small count tuples (full, prefix, suffix, middle):
// full in 1..3 (2 bits), prefix and suffix below 8 (3 bits each), middle below
// 128 (7 bits); index = ((full*8 + prefix)*8 + suffix)*128 + middle.
constexpr int TUPLE_FULL = 4, TUPLE_PS = 8, TUPLE_MID = 128;
constexpr int TUPLE_TABLE = TUPLE_FULL * TUPLE_PS * TUPLE_PS * TUPLE_MID;  // 32768
// A candidate whose alpha came from the tuple table keeps TUPLE_TAG | index in
// place of its alpha bits (a negative-NaN pattern no computed alpha produces).
constexpr uint32_t TUPLE_TAG = 0xffff0000u;

// Everything a build launch needs; plain device pointers, passed by value.
struct BuildArgs {
    int alpha, k, B;
    uint32_t A;
    uint64_t T1, T2, T1s, T2s, NCH;
    uint32_t wpt;
    // input: concatenated sequences, seq_off[B+1] (device)
    const uint8_t *seq;
    const uint64_t *seq_off;
    uint64_t *seq_off_store;  // scratch home for seq_off of a single proteome
    uint64_t *tile_base;      // [B+1]
    // (K-1)-mer tables: dense [B][T1s] (coff written for seen (K-1)-mers only), or,
    // when `compact1` (tables beyond 2^20 entries), one entry per seen (K-1)-mer of
    // the batch, at its rank among the seen bits: pw1[word].x + popc(bits below)
    uint32_t *c1, *coff;
    int compact1;
    uint64_t cap1;            // entries of c1 / coff in compact mode
    uint2 *pw1;               // [B * T1s / 32]: {set bits of seen1 before the word, the word}
    uint64_t *p1_partials, *p1_total;
    uint32_t *seen1;          // [B][T1s / 32]: bitmap of the seen (K-1)-mers
    uint32_t *word_cand;      // [B][T1s / 32]: candidates of each bitmap word
    // (K-2)-mer counts: dense [B][T2], or, when `compact2` (beyond 2^20 entries),
    // one entry per seen (K-2)-mer of the batch, at its rank in seen2 (via pw2)
    uint32_t *c2;
    int compact2;
    uint64_t cap2;            // entries of c2 in compact mode
    uint32_t *seen2;          // [B][T2s / 32]: bitmap of the seen (K-2)-mers (compact2)
    uint2 *pw2;               // [B * T2s / 32]: {set bits of seen2 before the word, the word}
    uint64_t *p2_partials, *p2_total;
    uint32_t *tot;            // [B][4]: n0, n1, n2, -
    // per (proteome, chunk of CH (K-1)-mers)
    uint32_t *chunk_cand;     // candidates per chunk
    uint64_t *chunk_cand_off; // exclusive scan (global over the batch), [nc+1]
    // candidate index space: proteome p owns [cbase[p], cbase[p+1]), cbase[p] a
    // multiple of ALPHA_TILE; cbase[B] = *cand_total
    uint64_t *cbase;          // [B+1]
    uint64_t *cand_total;     // [1]
    uint32_t *cq;             // [cand_cap]: the key of each candidate, then of each survivor
    // per segment of SEG candidates (survivors compacted to the segment's start)
    uint32_t *seg_surv;       // [nseg]
    uint64_t *seg_out_off;    // exclusive scan, [nseg+1]
    // per CTA of k_alpha (ALPHA_TILE candidates)
    uint32_t *cta_m1;         // survivors with alpha^2 == 1
    uint64_t *cta_norm;       // [ncta][3]: sum of the other alpha^2 as 192-bit fixed point, 2^-96 units
    uint32_t *cta_bad;        // bit 0 a NaN square, bit 1 an infinite one
    double *prob;             // [B][4][PROB_TABLE]: c/n0, c/n1, c/n2, 1/(c/n2)
    uint32_t *atab;           // [B][TUPLE_TABLE]: alpha bits of each count tuple
    float *vtab;              // [B][TUPLE_TABLE]: float(alpha / sqrt(norm)) of each tuple
    FastDiv fdT2;             // division by A^(K-2)
    uint64_t *scan_tmp;
    // per proteome results
    double *norm, *scale, *rscale;  // sum alpha^2, sqrt of it, RN(1/sqrt)
    uint64_t *nnz, *out_base;
    uint64_t *dst_base, *dst_cap;  // where k_compact writes proteome p
    uint32_t *status;
    // K-mer counts per candidate, replaced by alpha bits
    uint32_t *c0a;
    uint64_t cand_cap;
    // output arena
    uint32_t *out_keys;
    float *out_vals;
    uint32_t *union_bits;     // optional key-rank bitmap: every written key's bit set (and
                              // those of the few candidates whose alpha is 0)
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
