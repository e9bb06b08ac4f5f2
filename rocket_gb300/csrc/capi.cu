// capi.cu -- the C ABI of libphylogenetics.so.
//
// The first three symbols are the drop-in boundary: same names, argument order
// and meaning as the reference's JNA interface
// (src/main/java/nl/esciencecenter/phylogenetics_analysis/Bindings.java:17-45)
// and its C definitions (phylogenetics/src/main/cpp/native.cu:705-780):
//   * the caller owns every device buffer and the stream; the library uses the
//     caller's current context and never allocates, frees or selects a device;
//   * calls are synchronous (the stream is synchronised before returning);
//   * the return value is a cudaError_t code, 0 on success, with a message on
//     stderr for argument errors (cudaErrorUnknown, as the reference).
// compareCompositionVectors returns int (the Java binding's type); the
// reference's C definition says double and returns the code converted to
// double, which a caller binding int reads from the wrong register.
//
// The remaining symbols (phylo*) are new: batched construction into an arena,
// the window index and the pair-engine launches used by the batched and
// serving paths.  They follow the same conventions but are asynchronous unless
// stated.
#include <string.h>

#include <vector>

#include "../../include/phylogenetics.h"
#include "allpairs.cuh"
#include "compare.cuh"
#include "cv_build.cuh"
#include "postings.cuh"
#include "rank.cuh"

using namespace phylo;

namespace {

int parse_alphabet(const char *alphabet) {
    if (!alphabet) return -1;
    if (strcmp(alphabet, "DNA") == 0) return ALPHA_DNA;
    if (strcmp(alphabet, "protein") == 0) return ALPHA_PROTEIN;
    return -1;
}

// Candidate capacity reserved for one proteome of at most max_size entries.
// Candidates = entries + the slots whose alpha is exactly zero; they can never
// exceed the dense slot count A^K.
uint64_t single_cand_cap(const BuildGeometry &g, uint64_t max_size) {
    uint64_t cap = 2 * max_size + (1u << 20);
    const uint64_t dense = (uint64_t)g.T1 * g.A;
    return cap < dense ? cap : dense;
}

__global__ void k_init_single(BuildArgs a, uint64_t len, uint64_t max_size) {
    a.seq_off_store[0] = 0;
    a.seq_off_store[1] = len;
    a.dst_base[0] = 0;
    a.dst_cap[0] = max_size;
}

// arena offsets: vec_off[p] = base + sum of nnz rounded up to 4 entries
__global__ void k_arena_offsets(const uint64_t *nnz, int B, uint64_t base, uint64_t *vec_off,
                                uint64_t *dst_base, uint64_t *dst_cap) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        uint64_t off = base;
        for (int p = 0; p < B; p++) {
            vec_off[p] = off;
            dst_base[p] = off;
            dst_cap[p] = nnz[p];
            off += (nnz[p] + 3) & ~(uint64_t)3;
        }
        vec_off[B] = off;
    }
}

// padding entries after each vector: key 0xffffffff, value 0
__global__ void k_arena_pad(const uint64_t *vec_off, const uint64_t *nnz, int B, uint32_t *keys,
                            float *vals) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= B) return;
    for (uint64_t i = vec_off[p] + nnz[p]; i < vec_off[p + 1]; i++) {
        keys[i] = 0xffffffffu;
        vals[i] = 0.0f;
    }
}

cudaError_t last_status(uint32_t *d_status, cudaStream_t st, uint32_t *out) {
    PHYLO_CHECK(cudaMemcpyAsync(out, d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaStreamSynchronize(st));
    return cudaSuccess;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// drop-in boundary
// ---------------------------------------------------------------------------

long estimateScratchMemory(const char *alphabet, int k, int max_vector_size) {
    // like the reference, any alphabet other than "DNA" is sized as protein
    const int alpha = (alphabet && strcmp(alphabet, "DNA") == 0) ? ALPHA_DNA : ALPHA_PROTEIN;
    const uint64_t max_size = max_vector_size > 0 ? (uint64_t)max_vector_size : 0;
    size_t need = compare_scratch_bytes(2 * max_size);
    BuildGeometry g;
    if (build_geometry(alpha, k, &g) == 0) {
        size_t b = build_scratch_bytes(g, 1, single_cand_cap(g, max_size));
        if (b > need) need = b;
    }
    return (long)need;
}

int buildCompositionVector(uintptr_t stream, uintptr_t d_temp_storage_ptr, long temp_storage_size,
                           const char *alphabet, int k, uintptr_t d_string_ptr, long string_len,
                           uintptr_t d_set_keys_ptr, uintptr_t d_set_values_ptr,
                           uintptr_t set_size_ptr, int max_vector_size) {
    const int alpha = parse_alphabet(alphabet);
    if (alpha < 0) {
        fprintf(stderr, "error: invalid alphabet '%s'\n", alphabet ? alphabet : "(null)");
        return (int)cudaErrorUnknown;
    }
    BuildGeometry g;
    const int gr = build_geometry(alpha, k, &g);
    if (gr == -1) {
        fprintf(stderr, "error: k=%d should be in range 3-10\n", k);
        return (int)cudaErrorUnknown;
    }
    if (gr == -2) {
        fprintf(stderr, "error: k=%d is too large for 32-bit keys with alphabet '%s'\n", k,
                alphabet);
        return (int)cudaErrorUnknown;
    }
    if (string_len < 0 || (uint64_t)string_len > 0xffffffffull || max_vector_size < 0 ||
        temp_storage_size < 0) {
        fprintf(stderr,
                "error: invalid sizes (string_len=%ld, max_vector_size=%d, "
                "temp_storage_size=%ld)\n",
                string_len, max_vector_size, temp_storage_size);
        return (int)cudaErrorInvalidValue;
    }
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t *h_size = (uint32_t *)set_size_ptr;
    const uint64_t max_size = (uint64_t)max_vector_size;
    BuildArgs a;
    memset(&a, 0, sizeof(a));
    cudaError_t err = build_carve(g, 1, single_cand_cap(g, max_size), (void *)d_temp_storage_ptr,
                                  (size_t)temp_storage_size, &a);
    if (err != cudaSuccess) {
        fprintf(stderr, "error: scratch of %ld bytes is smaller than the %zu bytes needed\n",
                temp_storage_size, build_scratch_bytes(g, 1, single_cand_cap(g, max_size)));
        return (int)err;
    }
    a.seq = (const uint8_t *)d_string_ptr;
    a.seq_off = a.seq_off_store;
    a.out_keys = (uint32_t *)d_set_keys_ptr;
    a.out_vals = (float *)d_set_values_ptr;
    k_init_single<<<1, 1, 0, st>>>(a, (uint64_t)string_len, max_size);
    PHYLO_CHECK(cudaGetLastError());
    PHYLO_CHECK(build_plan(a, st));
    uint64_t nnz = 0;
    uint32_t status = 0;
    PHYLO_CHECK(cudaMemcpyAsync(&nnz, a.nnz, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(last_status(a.status, st, &status));
    if (h_size) *h_size = (uint32_t)nnz;
    if (status & DEV_CAPACITY) {
        fprintf(stderr,
                "error: candidate slots exceed the scratch capacity (%llu) for max_vector_size "
                "%d\n",
                (unsigned long long)a.cand_cap, max_vector_size);
        return (int)cudaErrorUnknown;
    }
    if (nnz > max_size) {
        fprintf(stderr,
                "error: size of composition vector (size: %llu) exceeds the given maximum (size: "
                "%d)\n",
                (unsigned long long)nnz, max_vector_size);
        return (int)cudaErrorUnknown;
    }
    PHYLO_CHECK(build_emit(a, st));
    // padding of the unused tail (native.cu:473-474)
    if (max_size > nnz) {
        PHYLO_CHECK(cudaMemsetAsync(a.out_keys + nnz, 0xff, (max_size - nnz) * sizeof(uint32_t), st));
        PHYLO_CHECK(cudaMemsetAsync(a.out_vals + nnz, 0, (max_size - nnz) * sizeof(float), st));
    }
    PHYLO_CHECK(cudaStreamSynchronize(st));
    return (int)cudaGetLastError();
}

int compareCompositionVectors(uintptr_t stream, uintptr_t d_temp_storage_ptr, long temp_storage_size,
                              uintptr_t d_left_keys_ptr, uintptr_t d_left_values_ptr, int left_size,
                              uintptr_t d_right_keys_ptr, uintptr_t d_right_values_ptr,
                              int right_size, uintptr_t d_output_ptr) {
    if (left_size < 0 || right_size < 0 || temp_storage_size < 0) {
        fprintf(stderr, "error: negative size (vectors %d, %d; scratch %ld)\n", left_size,
                right_size, temp_storage_size);
        return (int)cudaErrorInvalidValue;
    }
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t *d_status = nullptr;
    PHYLO_CHECK(compare_launch(st, (void *)d_temp_storage_ptr, (size_t)temp_storage_size,
                               (const uint32_t *)d_left_keys_ptr, (const float *)d_left_values_ptr,
                               (uint32_t)left_size, (const uint32_t *)d_right_keys_ptr,
                               (const float *)d_right_values_ptr, (uint32_t)right_size,
                               (double *)d_output_ptr, &d_status));
    uint32_t status = 0;
    PHYLO_CHECK(last_status(d_status, st, &status));
    if (status) {
        fprintf(stderr, "error: compare kernel reported device status %u\n", status);
        return (int)cudaErrorLaunchTimeout;
    }
    return (int)cudaGetLastError();
}

// For callers that cannot allocate device memory (see include/phylogenetics.h):
// compareCompositionVectors on the library's built-in scratch array.
// Synchronous, like compareCompositionVectors.  No allocation of any kind.
int compareCompositionVectorsStatic(uintptr_t stream, uintptr_t d_left_keys_ptr,
                                    uintptr_t d_left_values_ptr, int left_size,
                                    uintptr_t d_right_keys_ptr, uintptr_t d_right_values_ptr,
                                    int right_size, uintptr_t d_output_ptr) {
    if (left_size < 0 || right_size < 0) {
        fprintf(stderr, "error: negative vector size (%d, %d)\n", left_size, right_size);
        return (int)cudaErrorInvalidValue;
    }
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t *d_status = nullptr;
    cudaError_t e = compare_launch_static(
        st, (const uint32_t *)d_left_keys_ptr, (const float *)d_left_values_ptr,
        (uint32_t)left_size, (const uint32_t *)d_right_keys_ptr,
        (const float *)d_right_values_ptr, (uint32_t)right_size, (double *)d_output_ptr, &d_status);
    if (e != cudaSuccess) return (int)e;
    uint32_t status = 0;
    PHYLO_CHECK(last_status(d_status, st, &status));
    if (status) {
        fprintf(stderr, "error: compare kernel reported device status %u\n", status);
        return (int)cudaErrorLaunchTimeout;
    }
    return (int)cudaGetLastError();
}

int phyloCompareTileElements(void) { return (int)compare_tile_elements(); }

// Test hook of the bounded waits (see include/phylogenetics.h).
void phyloCompareTestWaitLimit(unsigned int limit) { compare_set_first_wait_limit(limit); }

// ---------------------------------------------------------------------------
// batched construction (new)
// ---------------------------------------------------------------------------

// Scratch for building up to max_proteomes proteomes whose candidate slots sum
// to at most max_candidates.
long phyloBuildBatchScratch(const char *alphabet, int k, int max_proteomes, long max_candidates) {
    const int alpha = parse_alphabet(alphabet);
    BuildGeometry g;
    if (alpha < 0 || build_geometry(alpha, k, &g) != 0 || max_proteomes <= 0 || max_candidates < 0)
        return -1;
    return (long)build_scratch_bytes(g, max_proteomes, (uint64_t)max_candidates);
}

// Phase 1: counts, candidate slots, alpha, norms and per-proteome sizes.
// d_seq: concatenated sequence bytes; d_seq_off: uint64[num_proteomes + 1].
// h_nnz (host, num_proteomes entries) receives the vector sizes; h_candidates
// (host, may be null) the total candidate slots.  Synchronous.
int phyloBuildBatchPlan(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                        const char *alphabet, int k, int num_proteomes, uintptr_t d_seq,
                        uintptr_t d_seq_off, long max_candidates, int64_t *h_nnz,
                        int64_t *h_candidates) {
    const int alpha = parse_alphabet(alphabet);
    BuildGeometry g;
    if (alpha < 0 || build_geometry(alpha, k, &g) != 0 || num_proteomes <= 0 ||
        max_candidates < 0 || scratch_size < 0) {
        fprintf(stderr, "error: invalid batch build arguments (alphabet %s, k=%d, n=%d)\n",
                alphabet ? alphabet : "(null)", k, num_proteomes);
        return (int)cudaErrorInvalidValue;
    }
    cudaStream_t st = (cudaStream_t)stream;
    BuildArgs a;
    memset(&a, 0, sizeof(a));
    PHYLO_CHECK(build_carve(g, num_proteomes, (uint64_t)max_candidates, (void *)d_scratch,
                            (size_t)scratch_size, &a));
    a.seq = (const uint8_t *)d_seq;
    a.seq_off = (const uint64_t *)d_seq_off;
    PHYLO_CHECK(build_plan(a, st));
    PHYLO_CHECK(cudaMemcpyAsync(h_nnz, a.nnz, sizeof(uint64_t) * num_proteomes,
                                cudaMemcpyDeviceToHost, st));
    if (h_candidates)
        PHYLO_CHECK(cudaMemcpyAsync(h_candidates, a.cand_total, sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, st));
    uint32_t status = 0;
    PHYLO_CHECK(last_status(a.status, st, &status));
    if (status & DEV_CAPACITY) {
        fprintf(stderr, "error: candidate slots exceed max_candidates=%ld\n", max_candidates);
        return (int)cudaErrorMemoryAllocation;
    }
    return (int)cudaGetLastError();
}

// Phase 1 without waiting: the same kernels, then copies of the results into
// the caller's pinned host buffer h_summary (see the header); the caller
// synchronises the stream (or an event recorded after this call) before
// reading it.
int phyloBuildBatchPlanAsync(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                             const char *alphabet, int k, int num_proteomes, uintptr_t d_seq,
                             uintptr_t d_seq_off, long max_candidates, void *h_summary) {
    const int alpha = parse_alphabet(alphabet);
    BuildGeometry g;
    if (alpha < 0 || build_geometry(alpha, k, &g) != 0 || num_proteomes <= 0 || !h_summary ||
        max_candidates < 0 || scratch_size < 0) {
        fprintf(stderr, "error: invalid batch build arguments (alphabet %s, k=%d, n=%d)\n",
                alphabet ? alphabet : "(null)", k, num_proteomes);
        return (int)cudaErrorInvalidValue;
    }
    cudaStream_t st = (cudaStream_t)stream;
    BuildArgs a;
    memset(&a, 0, sizeof(a));
    PHYLO_CHECK(build_carve(g, num_proteomes, (uint64_t)max_candidates, (void *)d_scratch,
                            (size_t)scratch_size, &a));
    a.seq = (const uint8_t *)d_seq;
    a.seq_off = (const uint64_t *)d_seq_off;
    PHYLO_CHECK(build_plan(a, st));
    // summary layout: int64 nnz[B] | float64 norm[B] | int64 candidates | uint32 status
    char *h = (char *)h_summary;
    const size_t B = (size_t)num_proteomes;
    PHYLO_CHECK(cudaMemcpyAsync(h, a.nnz, 8 * B, cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaMemcpyAsync(h + 8 * B, a.norm, 8 * B, cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaMemcpyAsync(h + 16 * B, a.cand_total, 8, cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaMemcpyAsync(h + 16 * B + 8, a.status, 4, cudaMemcpyDeviceToHost, st));
    return (int)cudaGetLastError();
}

long phyloBuildBatchSummaryBytes(int num_proteomes) {
    return num_proteomes > 0 ? 16L * num_proteomes + 16 : -1;
}

// Phase 2 (after Plan, same scratch): writes vector p at
// d_keys/d_values[vec_off[p] ..], vec_off[p] = arena_base + sum of earlier sizes
// rounded up to 4 entries; d_vec_off (uint64[num_proteomes + 1]) receives the
// offsets.  Padding entries get key 0xffffffff and value 0.  Asynchronous.
int phyloBuildBatchEmit(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                        const char *alphabet, int k, int num_proteomes, long max_candidates,
                        uintptr_t d_keys, uintptr_t d_values, uintptr_t d_vec_off,
                        long arena_base, uintptr_t d_union_bits) {
    const int alpha = parse_alphabet(alphabet);
    BuildGeometry g;
    if (alpha < 0 || build_geometry(alpha, k, &g) != 0 || num_proteomes <= 0 ||
        max_candidates < 0 || scratch_size < 0 || arena_base < 0)
        return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    BuildArgs a;
    memset(&a, 0, sizeof(a));
    PHYLO_CHECK(build_carve(g, num_proteomes, (uint64_t)max_candidates, (void *)d_scratch,
                            (size_t)scratch_size, &a));
    a.out_keys = (uint32_t *)d_keys;
    a.out_vals = (float *)d_values;
    a.union_bits = (uint32_t *)d_union_bits;
    uint64_t *vec_off = (uint64_t *)d_vec_off;
    k_arena_offsets<<<1, 1, 0, st>>>(a.nnz, num_proteomes, (uint64_t)arena_base, vec_off,
                                     a.dst_base, a.dst_cap);
    PHYLO_CHECK(cudaGetLastError());
    PHYLO_CHECK(build_emit(a, st));
    k_arena_pad<<<(num_proteomes + 127) / 128, 128, 0, st>>>(vec_off, a.nnz, num_proteomes,
                                                             a.out_keys, a.out_vals);
    return (int)cudaGetLastError();
}

// Per-proteome norms (sum of alpha^2) of the last Plan, double[num_proteomes].
int phyloBuildBatchNorms(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                         const char *alphabet, int k, int num_proteomes, long max_candidates,
                         double *h_norms) {
    const int alpha = parse_alphabet(alphabet);
    BuildGeometry g;
    if (alpha < 0 || build_geometry(alpha, k, &g) != 0 || num_proteomes <= 0 ||
        max_candidates < 0 || scratch_size < 0 || !h_norms)
        return (int)cudaErrorInvalidValue;
    BuildArgs a;
    memset(&a, 0, sizeof(a));
    PHYLO_CHECK(build_carve(g, num_proteomes, (uint64_t)max_candidates, (void *)d_scratch,
                            (size_t)scratch_size, &a));
    cudaStream_t st = (cudaStream_t)stream;
    PHYLO_CHECK(cudaMemcpyAsync(h_norms, a.norm, sizeof(double) * num_proteomes,
                                cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaStreamSynchronize(st));
    return 0;
}

// Dense (K-1)- and (K-2)-mer count tables and n0/n1/n2 of proteome p of the last
// Plan (for count-parity checks).  Synchronous.
// Compact count table of proteome p (entry pw[w].x + rank of the bit in word w for
// every set bit of the seen bitmap's nw words) expanded into a dense host table of
// `len` entries.
static cudaError_t expand_compact_counts(const uint32_t *d_seen, const uint2 *d_pw,
                                         const uint32_t *d_counts, uint64_t cap, uint64_t nw,
                                         int p, uint64_t len, uint32_t *h_out, cudaStream_t st) {
    std::vector<uint32_t> seen(nw);
    std::vector<uint2> pw(nw);
    PHYLO_CHECK(cudaMemcpyAsync(seen.data(), d_seen + (uint64_t)p * nw, sizeof(uint32_t) * nw,
                                cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaMemcpyAsync(pw.data(), d_pw + (uint64_t)p * nw, sizeof(uint2) * nw,
                                cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaStreamSynchronize(st));
    const uint64_t first = pw[0].x;
    const uint64_t n = pw[nw - 1].x + (uint64_t)__builtin_popcount(seen[nw - 1]) - first;
    if (first + n > cap) return cudaErrorInvalidValue;  // the build ran out of room
    std::vector<uint32_t> cc(n ? n : 1);
    if (n)
        PHYLO_CHECK(cudaMemcpyAsync(cc.data(), d_counts + first, sizeof(uint32_t) * n,
                                    cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaStreamSynchronize(st));
    memset(h_out, 0, sizeof(uint32_t) * len);
    for (uint64_t w = 0; w < nw; w++) {
        uint32_t bits = seen[w], r = pw[w].x - (uint32_t)first;
        while (bits) {
            const int j = __builtin_ctz(bits);
            bits &= bits - 1;
            if (w * 32 + j < len) h_out[w * 32 + j] = cc[r];
            r++;
        }
    }
    return cudaSuccess;
}

int phyloBuildBatchCounts(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                          const char *alphabet, int k, int num_proteomes, long max_candidates,
                          int p, uint32_t *h_c1, uint32_t *h_c2, uint32_t *h_tot) {
    const int alpha = parse_alphabet(alphabet);
    BuildGeometry g;
    if (alpha < 0 || build_geometry(alpha, k, &g) != 0 || p < 0 || p >= num_proteomes ||
        max_candidates < 0 || scratch_size < 0 || !h_c1 || !h_c2 || !h_tot)
        return (int)cudaErrorInvalidValue;
    BuildArgs a;
    memset(&a, 0, sizeof(a));
    PHYLO_CHECK(build_carve(g, num_proteomes, (uint64_t)max_candidates, (void *)d_scratch,
                            (size_t)scratch_size, &a));
    cudaStream_t st = (cudaStream_t)stream;
    if (a.compact1) {
        PHYLO_CHECK(expand_compact_counts(a.seen1, a.pw1, a.c1, a.cap1, g.T1s / 32, p, g.T1, h_c1, st));
    } else {
        PHYLO_CHECK(cudaMemcpyAsync(h_c1, a.c1 + (uint64_t)p * g.T1s, sizeof(uint32_t) * g.T1,
                                    cudaMemcpyDeviceToHost, st));
    }
    if (a.compact2) {
        PHYLO_CHECK(expand_compact_counts(a.seen2, a.pw2, a.c2, a.cap2, g.T2s / 32, p, g.T2, h_c2, st));
    } else {
        PHYLO_CHECK(cudaMemcpyAsync(h_c2, a.c2 + (uint64_t)p * g.T2, sizeof(uint32_t) * g.T2,
                                    cudaMemcpyDeviceToHost, st));
    }
    PHYLO_CHECK(cudaMemcpyAsync(h_tot, a.tot + (uint64_t)p * 4, sizeof(uint32_t) * 3,
                                cudaMemcpyDeviceToHost, st));
    PHYLO_CHECK(cudaStreamSynchronize(st));
    return 0;
}

int phyloBuildLaunchesPerBatch(void) { return build_launches_per_batch(); }

// ---------------------------------------------------------------------------
// pair engine (new)
// ---------------------------------------------------------------------------

// Window index of an arena: roff uint32[num_vectors][R + 1], R = ceil(key_limit / 2^shift).
int phyloWindowIndex(uintptr_t stream, uintptr_t d_keys, uintptr_t d_vec_off, int num_vectors,
                     int window_shift, unsigned int num_windows, long max_vector_len,
                     uintptr_t d_roff) {
    if (num_vectors < 0 || window_shift < 0 || window_shift > 31 || max_vector_len < 0)
        return (int)cudaErrorInvalidValue;
    return (int)range_index_launch((const uint32_t *)d_keys, (const uint64_t *)d_vec_off,
                                   (uint32_t)num_vectors, num_windows, (uint32_t)window_shift,
                                   (uint32_t *)d_roff, (cudaStream_t)stream,
                                   (uint64_t)max_vector_len);
}

// Sets the kernel's shared-memory limit for this window width and reports the
// resident CTAs per SM.
int phyloPairsPrepare(int window_shift, int tile_rows, int tile_cols, int *ctas_per_sm) {
    if (!ap_shape_ok(tile_rows, tile_cols) || window_shift < 4 ||
        window_shift > ap_max_wshift(tile_rows, tile_cols))
        return (int)cudaErrorInvalidValue;
    return (int)ap_prepare((uint32_t)window_shift, tile_rows, tile_cols, ctas_per_sm);
}

int phyloPairsSmemBytes(int window_shift, int tile_rows, int tile_cols) {
    if (!ap_shape_ok(tile_rows, tile_cols)) return -1;
    return (int)ap_smem_bytes((uint32_t)window_shift, tile_rows, tile_cols);
}

int phyloPairsThreads(int window_shift, int tile_rows, int tile_cols) {
    if (!ap_shape_ok(tile_rows, tile_cols)) return -1;
    return ap_threads((uint32_t)window_shift, tile_rows, tile_cols);
}

// Launches the pair kernel over `num_items` items (8 uint32 each, see ApItem);
// row vectors come from the row arena, column vectors from the column arena
// (the same arena for all pairs of one set).  d_counter must be zero.
// d_item_cycles may be 0.
int phyloPairsLaunch(uintptr_t stream, uintptr_t d_row_keys, uintptr_t d_row_values,
                     uintptr_t d_row_vec_off, uintptr_t d_row_roff, uintptr_t d_col_keys,
                     uintptr_t d_col_values, uintptr_t d_col_vec_off, uintptr_t d_col_roff,
                     unsigned int num_windows, int window_shift, uintptr_t d_rowids,
                     uintptr_t d_colids, uintptr_t d_items, int num_items, uintptr_t d_counter,
                     uintptr_t d_part, int fold, uintptr_t d_item_cycles, int tile_rows,
                     int tile_cols, int grid) {
    if (!ap_shape_ok(tile_rows, tile_cols) || window_shift < 4 ||
        window_shift > ap_max_wshift(tile_rows, tile_cols) || num_items < 0 || grid <= 0)
        return (int)cudaErrorInvalidValue;
    ApArgs a;
    a.row.keys = (const uint32_t *)d_row_keys;
    a.row.vals = (const float *)d_row_values;
    a.row.vec_off = (const uint64_t *)d_row_vec_off;
    a.row.roff = (const uint32_t *)d_row_roff;
    a.col.keys = (const uint32_t *)d_col_keys;
    a.col.vals = (const float *)d_col_values;
    a.col.vec_off = (const uint64_t *)d_col_vec_off;
    a.col.roff = (const uint32_t *)d_col_roff;
    a.R = num_windows;
    a.wshift = (uint32_t)window_shift;
    a.rowids = (const uint32_t *)d_rowids;
    a.colids = (const uint32_t *)d_colids;
    a.items = (const ApItem *)d_items;
    a.nitems = (uint32_t)num_items;
    a.counter = (uint32_t *)d_counter;
    a.part = (FF *)d_part;
    // the 16-row kernel adds four products per accumulator between checks
    a.fold = fold >= 4 ? (uint32_t)fold & ~3u : (fold > 0 ? 4u : 28u);
    a.item_cycles = (int64_t *)d_item_cycles;
    return (int)ap_launch(a, tile_rows, tile_cols, grid, (cudaStream_t)stream);
}

// Sums the partial blocks of each tile (4 uint32 per tile: row0, nrow, col0, ncol).
int phyloPairsReduce(uintptr_t stream, uintptr_t d_part, uintptr_t d_tiles, int num_tiles,
                     int segments, int tile_rows, int tile_cols, uintptr_t d_rowids,
                     uintptr_t d_colids, uintptr_t d_out, long ldc, int upper, int mirror) {
    if (!ap_shape_ok(tile_rows, tile_cols) || upper < 0 || upper > 2 || num_tiles < 0 ||
        (num_tiles > 0 && segments <= 0) || ldc <= 0)
        return (int)cudaErrorInvalidValue;
    ApReduceArgs r;
    r.part = (const FF *)d_part;
    r.tiles = (const ApTile *)d_tiles;
    r.ntiles = (uint32_t)num_tiles;
    r.S = (uint32_t)segments;
    r.ti = (uint32_t)tile_rows;
    r.tj = (uint32_t)tile_cols;
    r.rowids = (const uint32_t *)d_rowids;
    r.colids = (const uint32_t *)d_colids;
    r.out = (double *)d_out;
    r.ldc = (uint64_t)ldc;
    r.upper = upper;
    r.mirror = mirror;
    return (int)ap_reduce_launch(r, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// key-major (postings) pair engine (new)
// ---------------------------------------------------------------------------

long phyloPostingsSmemBytes(int block, int window_shift) {
    if (!pb_block_ok(block) || window_shift < 4 || window_shift > 14) return -1;
    const size_t n = pb_smem_bytes(block, (uint32_t)window_shift);
    return n ? (long)n : -1;
}

long phyloPostingsCapacity(int block, int window_shift) {
    if (!pb_block_ok(block) || window_shift < 4 || window_shift > 14) return -1;
    const uint32_t c = pb_capacity(block, (uint32_t)window_shift);
    return c ? (long)c : -1;
}

int phyloPostingsThreads(int block) { return pb_block_ok(block) ? pb_threads(block) : -1; }

int phyloPostingsPrepare(int block, int window_shift, int *ctas_per_sm) {
    if (phyloPostingsCapacity(block, window_shift) < 0) return (int)cudaErrorInvalidValue;
    return (int)pb_prepare(block, (uint32_t)window_shift, ctas_per_sm);
}

int phyloPostingsLaunch(uintptr_t stream, uintptr_t d_row_keys, uintptr_t d_row_values,
                        uintptr_t d_row_vec_off, uintptr_t d_row_roff, uintptr_t d_col_keys,
                        uintptr_t d_col_values, uintptr_t d_col_vec_off, uintptr_t d_col_roff,
                        unsigned int num_windows, int window_shift, uintptr_t d_rowids,
                        uintptr_t d_colids, uintptr_t d_items, int num_items, uintptr_t d_counter,
                        uintptr_t d_part, uintptr_t d_status, uintptr_t d_item_cycles, int block,
                        int grid) {
    if (phyloPostingsCapacity(block, window_shift) < 0 || num_items < 0 || grid <= 0)
        return (int)cudaErrorInvalidValue;
    if (num_items == 0) return 0;
    PbArgs a;
    a.row.keys = (const uint32_t *)d_row_keys;
    a.row.vals = (const float *)d_row_values;
    a.row.vec_off = (const uint64_t *)d_row_vec_off;
    a.row.roff = (const uint32_t *)d_row_roff;
    a.col.keys = (const uint32_t *)d_col_keys;
    a.col.vals = (const float *)d_col_values;
    a.col.vec_off = (const uint64_t *)d_col_vec_off;
    a.col.roff = (const uint32_t *)d_col_roff;
    a.R = num_windows;
    a.wshift = (uint32_t)window_shift;
    a.rowids = (const uint32_t *)d_rowids;
    a.colids = (const uint32_t *)d_colids;
    a.items = (const PbItem *)d_items;
    a.nitems = (uint32_t)num_items;
    a.counter = (uint32_t *)d_counter;
    a.part = (int64_t *)d_part;
    a.status = (uint32_t *)d_status;
    a.item_cycles = (int64_t *)d_item_cycles;
    return (int)pb_launch(a, block, grid, (cudaStream_t)stream);
}

int phyloPostingsReduce(uintptr_t stream, uintptr_t d_part, uintptr_t d_tiles, int num_tiles,
                        int block, uintptr_t d_rowids, uintptr_t d_colids, uintptr_t d_out,
                        long ldc, int self, int mirror) {
    if (!pb_block_ok(block) || num_tiles < 0 || ldc <= 0) return (int)cudaErrorInvalidValue;
    PbReduceArgs r;
    r.part = (const int64_t *)d_part;
    r.tiles = (const PbTile *)d_tiles;
    r.ntiles = (uint32_t)num_tiles;
    r.block = (uint32_t)block;
    r.rowids = (const uint32_t *)d_rowids;
    r.colids = (const uint32_t *)d_colids;
    r.out = (double *)d_out;
    r.ldc = (uint64_t)ldc;
    r.self = self;
    r.mirror = mirror;
    return (int)pb_reduce_launch(r, (cudaStream_t)stream);
}

long phyloKeyRankScratch(long key_limit) {
    if (key_limit <= 0 || key_limit > 0xffffffffl) return -1;
    return (long)rank_scratch_bytes((uint64_t)key_limit);
}

long phyloKeyRankBitmapBytes(long key_limit) {
    if (key_limit <= 0 || key_limit > 0xffffffffl) return -1;
    return (long)(rank_bitmap_words((uint64_t)key_limit) * sizeof(uint32_t));
}

int phyloKeyRanks(uintptr_t stream, uintptr_t d_scratch, long scratch_bytes, long key_limit,
                  uintptr_t d_keys, uintptr_t d_vec_off, int num_vectors, long max_vector_len,
                  uintptr_t d_union_bits, uintptr_t d_rank_keys, uintptr_t d_union_size) {
    if (key_limit <= 0 || key_limit > 0xffffffffl || num_vectors < 0 || max_vector_len < 0 ||
        scratch_bytes < (long)rank_scratch_bytes((uint64_t)key_limit))
        return (int)cudaErrorInvalidValue;
    return (int)key_ranks((const uint32_t *)d_keys, (const uint64_t *)d_vec_off,
                          (uint32_t)num_vectors, (uint64_t)max_vector_len, (uint64_t)key_limit,
                          (const uint32_t *)d_union_bits, (void *)d_scratch, (size_t)scratch_bytes,
                          (uint32_t *)d_rank_keys, (uint64_t *)d_union_size, (cudaStream_t)stream);
}

int phyloKeyRankIndex(uintptr_t stream, uintptr_t d_scratch, long scratch_bytes, long key_limit,
                      uintptr_t d_keys, uintptr_t d_vec_off, int num_vectors, long max_vector_len,
                      long arena_entries, uintptr_t d_union_bits, int window_shift,
                      unsigned int num_windows, uintptr_t d_rank_keys, uintptr_t d_roff) {
    if (key_limit <= 0 || key_limit > 0xffffffffl || num_vectors < 0 || window_shift < 0 ||
        window_shift > 31 || arena_entries < 0 || max_vector_len < 0 ||
        scratch_bytes < (long)rank_scratch_bytes((uint64_t)key_limit))
        return (int)cudaErrorInvalidValue;
    return (int)key_rank_index((const uint32_t *)d_keys, (const uint64_t *)d_vec_off,
                               (uint32_t)num_vectors, (uint64_t)max_vector_len,
                               (uint64_t)arena_entries, (uint64_t)key_limit,
                               (const uint32_t *)d_union_bits, (void *)d_scratch,
                               (size_t)scratch_bytes, (uint32_t)window_shift, num_windows,
                               (uint32_t *)d_rank_keys, (uint32_t *)d_roff, (cudaStream_t)stream);
}

int phyloSelfDot(uintptr_t stream, uintptr_t d_values, uintptr_t d_vec_off, int num_vectors,
                 long max_vector_len, uintptr_t d_part, uintptr_t d_out, long ldc) {
    if (num_vectors < 0 || max_vector_len < 0 || ldc <= 0) return (int)cudaErrorInvalidValue;
    return (int)self_dot_launch((const float *)d_values, (const uint64_t *)d_vec_off,
                                (uint32_t)num_vectors, (double *)d_out, (uint64_t)ldc,
                                (uint64_t)max_vector_len, (FF *)d_part, (cudaStream_t)stream);
}

long phyloSelfDotPartBytes(int num_vectors, long max_vector_len) {
    if (num_vectors < 0 || max_vector_len < 0) return -1;
    return (long)(self_dot_part_count((uint32_t)num_vectors, (uint64_t)max_vector_len) * sizeof(FF));
}

// Scratch bytes of phyloComparePairsMany for P pairs and at most max_tiles
// merge tiles (sum over pairs of ceil((nl + nr) / phyloCompareTileElements())).
long phyloComparePairsManyScratch(int num_pairs, long max_tiles) {
    if (num_pairs < 0 || max_tiles < 0) return -1;
    return (long)compare_many_scratch_bytes((uint32_t)num_pairs, (uint64_t)max_tiles);
}

// C of many pairs in one merge-path launch sequence: pair p compares vector
// pa[p] of the left arena with vector pb[p] of the right arena (arena =
// keys, values, uint64 offsets, uint32 sizes); results to d_out[p] (double).
// Asynchronous.
int phyloComparePairsMany(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                          uintptr_t d_lkeys, uintptr_t d_lvalues, uintptr_t d_loff,
                          uintptr_t d_lnnz, uintptr_t d_rkeys, uintptr_t d_rvalues,
                          uintptr_t d_roff, uintptr_t d_rnnz, uintptr_t d_pa, uintptr_t d_pb,
                          int num_pairs, long max_tiles, uintptr_t d_out) {
    if (num_pairs < 0 || max_tiles < 0 || scratch_size < 0) return (int)cudaErrorInvalidValue;
    return (int)compare_many_launch(
        (cudaStream_t)stream, (void *)d_scratch, (size_t)scratch_size, (const uint32_t *)d_lkeys,
        (const float *)d_lvalues, (const uint64_t *)d_loff, (const uint32_t *)d_lnnz,
        (const uint32_t *)d_rkeys, (const float *)d_rvalues, (const uint64_t *)d_roff,
        (const uint32_t *)d_rnnz, (const uint32_t *)d_pa, (const uint32_t *)d_pb,
        (uint32_t)num_pairs, (uint64_t)max_tiles, (double *)d_out, nullptr);
}

// Pair kernel launch on raw arena pointers for one pair, through the merge
// path, asynchronous (used by the batched engine for vectors whose values
// are not finite).  Scratch from estimateScratchMemory.
int phyloComparePairAsync(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                          uintptr_t d_left_keys, uintptr_t d_left_values, int left_size,
                          uintptr_t d_right_keys, uintptr_t d_right_values, int right_size,
                          uintptr_t d_out) {
    if (left_size < 0 || right_size < 0 || scratch_size < 0) return (int)cudaErrorInvalidValue;
    return (int)compare_launch((cudaStream_t)stream, (void *)d_scratch, (size_t)scratch_size,
                               (const uint32_t *)d_left_keys, (const float *)d_left_values,
                               (uint32_t)left_size, (const uint32_t *)d_right_keys,
                               (const float *)d_right_values, (uint32_t)right_size,
                               (double *)d_out, nullptr);
}

}  // extern "C"
