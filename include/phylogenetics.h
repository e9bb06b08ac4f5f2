/*
 * phylogenetics.h -- C ABI of libphylogenetics.so (GB300 / sm_103a build).
 *
 * Drop-in for the library that Rocket's phylogenetics plug-in loads through
 * JNA (Native.load("phylogenetics"),
 * src/main/java/nl/esciencecenter/phylogenetics_analysis/Bindings.java:15).
 *
 * Conventions of every entry point (as the reference):
 *   - device pointers and the stream are passed as uintptr_t;
 *   - the caller owns every buffer, the stream and the current CUDA context;
 *     the library never allocates, frees or selects a device;
 *   - the return value is a cudaError_t code (0 = cudaSuccess); argument
 *     errors print a message on stderr and return cudaErrorUnknown (999),
 *     except where stated;
 *   - a negative count or byte size (vector lengths, scratch sizes, numbers
 *     of vectors, items, tiles or pairs) returns cudaErrorInvalidValue (1)
 *     before any device work; the size queries (long results) return -1.
 */
#ifndef ROCKET_GB300_PHYLOGENETICS_H
#define ROCKET_GB300_PHYLOGENETICS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------
 * Drop-in boundary
 * ------------------------------------------------------------------------- */

/*
 * Bytes of device scratch a CompositionVectorKernels instance allocates once
 * and passes to every build and compare call.
 * Replaces: native.cu:705-716 (estimateScratchMemory), bound at
 * Bindings.java:17-20, called at CompositionVectorKernels.java:41.
 * Any alphabet other than "DNA" is sized as "protein" (as the reference).
 */
long estimateScratchMemory(const char *alphabet, int k, int max_vector_size);

/*
 * Builds the composition vector of the residue string d_string[0, string_len):
 * sorted keys (uint32, base-21 or base-4 K-mer codes) to d_keys, values
 * (float, alpha / sqrt(sum alpha^2)) to d_values, the size to *set_size_ptr
 * (host int), and pads [size, max_vector_size) with key 0xffffffff and value 0.
 * Fails with cudaErrorUnknown if the size exceeds max_vector_size, if k is
 * outside 3..10, if the keys would not fit 32 bits (protein k >= 8) or if the
 * alphabet is neither "DNA" nor "protein".  Synchronous.
 * Replaces: native.cu:718-752 (buildCompositionVector -> build_composition_vector
 * native.cu:258-477), bound at Bindings.java:22-33, called at
 * CompositionVectorKernels.java:45-66.
 */
int buildCompositionVector(uintptr_t stream, uintptr_t d_temp_storage_ptr, long temp_storage_size,
                           const char *alphabet, int k, uintptr_t d_string_ptr, long string_len,
                           uintptr_t d_set_keys_ptr, uintptr_t d_set_values_ptr,
                           uintptr_t set_size_ptr, int max_vector_size);

/*
 * C = sum over keys present in both vectors of left_value * right_value,
 * written as one double to d_output_ptr (device).  Synchronous.  Returns int:
 * the Java binding's type (Bindings.java:35); the reference's C definition
 * declares double (native.cu:755).
 * Replaces: native.cu:755-780 (compareCompositionVectors ->
 * calculate_cosine_similarity native.cu:645-703), bound at Bindings.java:35-45,
 * called at CompositionVectorKernels.java:68-89.
 */
int compareCompositionVectors(uintptr_t stream, uintptr_t d_temp_storage_ptr, long temp_storage_size,
                              uintptr_t d_left_keys_ptr, uintptr_t d_left_values_ptr, int left_size,
                              uintptr_t d_right_keys_ptr, uintptr_t d_right_values_ptr,
                              int right_size, uintptr_t d_output_ptr);

/*
 * compareCompositionVectors for callers that cannot allocate device memory.
 * No counterpart in the reference.
 *
 * Some callers have no way to call cudaMalloc: a host runtime that divided all
 * device memory into fixed cache slots at start-up (Rocket's device cache works
 * this way) and has no spare buffer for scratch, or a caller whose device
 * memory is owned by another framework's allocator.  This entry point takes no
 * scratch argument and allocates nothing: the compare kernel uses a fixed-size
 * array built into the library (8,448 bytes, present on every GPU that loads the
 * library until the process exits).  The caller still passes the inputs and the
 * output (one double, device memory).
 *
 * Limit: left_size + right_size <= 67,108,864 (2^26); larger inputs are refused
 * with cudaErrorInvalidValue and a message, before any kernel runs.
 * The first call in each CUDA context (one per device, or one per context the
 * caller creates) looks up the array's device address in that context
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the one array: calls whose kernels could overlap on the GPU
 * (other streams, other host threads) must be serialised by the caller.
 * Synchronous; returns a cudaError_t code like compareCompositionVectors.
 */
int compareCompositionVectorsStatic(uintptr_t stream, uintptr_t d_left_keys_ptr,
                                    uintptr_t d_left_values_ptr, int left_size,
                                    uintptr_t d_right_keys_ptr, uintptr_t d_right_values_ptr,
                                    int right_size, uintptr_t d_output_ptr);

/*
 * Test hook of the compare kernels' bounded waits (no counterpart in the
 * reference).  Every mbarrier wait of the compare kernels gives up after a poll
 * limit, records DEV_WAIT_TIMEOUT in the status word, waits (bounded) for its
 * own copies in flight and returns; the synchronous entry points then return
 * cudaErrorLaunchTimeout (702).  This sets the limit of each CTA's first wait
 * (0 = give up at once; 0xffffffff restores the default of 2^22 polls), so that
 * a test can take that path without a fault.  Process-wide; not for production.
 */
void phyloCompareTestWaitLimit(unsigned int limit);

/* ---------------------------------------------------------------------------
 * Batched construction (new; the reference builds one proteome per call,
 * driven per item by DeviceWorker.loadInput, DeviceWorker.java:118-157)
 * ------------------------------------------------------------------------- */

/* Scratch for building up to max_proteomes proteomes with at most
 * max_candidates candidate slots in total; -1 on invalid arguments. */
long phyloBuildBatchScratch(const char *alphabet, int k, int max_proteomes, long max_candidates);

/* Phase 1: counting, candidate slots, Markov alpha, norms, per-proteome sizes.
 * d_seq: concatenated residue bytes; d_seq_off: uint64[num_proteomes + 1].
 * h_nnz (host int64[num_proteomes]) receives the vector sizes, h_candidates
 * (host int64, may be 0) the candidate slots the batch needs (each proteome's
 * rounded up to 2048).  Returns cudaErrorMemoryAllocation (2) when they exceed
 * max_candidates rounded up to 2048 (retry with *h_candidates).  Synchronous. */
int phyloBuildBatchPlan(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                        const char *alphabet, int k, int num_proteomes, uintptr_t d_seq,
                        uintptr_t d_seq_off, long max_candidates, int64_t *h_nnz,
                        int64_t *h_candidates);

/* Phase 1 without waiting for it: the Plan's kernels, then asynchronous
 * copies of the results into h_summary, a pinned host buffer of
 * phyloBuildBatchSummaryBytes bytes laid out as int64 nnz[num_proteomes] |
 * float64 norm[num_proteomes] | int64 candidate slots needed | uint32 status
 * (bit 1: candidate capacity exceeded; retry with a larger max_candidates).
 * Read it only after the stream (or an event recorded after this call) has
 * completed.  Lets a caller overlap the builds of two batches on two streams. */
int phyloBuildBatchPlanAsync(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                             const char *alphabet, int k, int num_proteomes, uintptr_t d_seq,
                             uintptr_t d_seq_off, long max_candidates, void *h_summary);
long phyloBuildBatchSummaryBytes(int num_proteomes);

/* Phase 2 (same scratch and arguments as the Plan): vector p is written at
 * d_keys/d_values[vec_off[p] ..] with vec_off[p] = arena_base + earlier sizes
 * rounded up to 4 entries; d_vec_off (uint64[num_proteomes + 1]) receives the
 * offsets; padding entries get key 0xffffffff, value 0.  d_union_bits, when
 * not 0, is a key bitmap (phyloKeyRankBitmapBytes bytes) in which every
 * written key's bit is set, for phyloKeyRanks; so are the bits of the few
 * candidate keys whose alpha is 0, which are not written (the bitmap is marked
 * per seen (K-1)-mer).  Asynchronous. */
int phyloBuildBatchEmit(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                        const char *alphabet, int k, int num_proteomes, long max_candidates,
                        uintptr_t d_keys, uintptr_t d_values, uintptr_t d_vec_off,
                        long arena_base, uintptr_t d_union_bits);

/* Norms (sum over entries of float(alpha)^2) of the last Plan, host double[]. */
int phyloBuildBatchNorms(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                         const char *alphabet, int k, int num_proteomes, long max_candidates,
                         double *h_norms);

/* Dense (K-1)- and (K-2)-mer count tables and n0/n1/n2 of proteome p of the
 * last Plan (host buffers of A^(K-1), A^(K-2) and 3 uint32).  Where the build
 * keeps counts compact (one entry per seen (K-1)- or (K-2)-mer, tables beyond
 * 2^20 entries: the (K-1)-mer counts from protein K = 6, the (K-2)-mer counts at
 * protein K = 7), they are expanded here on the host. */
int phyloBuildBatchCounts(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                          const char *alphabet, int k, int num_proteomes, long max_candidates,
                          int p, uint32_t *h_c1, uint32_t *h_c2, uint32_t *h_tot);

/* Kernel launches (including memsets) one Plan + Emit issues. */
int phyloBuildLaunchesPerBatch(void);

/* ---------------------------------------------------------------------------
 * Pair engine (new; the reference compares one pair per call,
 * DeviceWorker.submitCorrelation, DeviceWorker.java:237-323)
 * ------------------------------------------------------------------------- */

/* Window index of an arena: d_roff uint32[num_vectors][num_windows + 1],
 * entry [v][r] = number of entries of vector v with key < r << window_shift.
 * max_vector_len bounds the (padded) length of every vector; every vector
 * starts on a 4-entry (16-byte) boundary and is padded to a multiple of 4
 * entries with keys 0xFFFFFFFF (the arena layout of phyloBuildBatchEmit). */
int phyloWindowIndex(uintptr_t stream, uintptr_t d_keys, uintptr_t d_vec_off, int num_vectors,
                     int window_shift, unsigned int num_windows, long max_vector_len,
                     uintptr_t d_roff);

/* The tile shape (tile_rows x tile_cols row x column vectors per work item)
 * selects the pair kernel: 16 x 128, 16 x 64 or 16 x 32 (512, 256 or 128 threads) use
 * 80-byte key records and four lanes per column vector, windows up to 2^11
 * keys; 32 x 64 uses 128-byte swizzled records and eight lanes per column
 * vector, windows up to 2^10 keys.  Partial blocks are tile_rows x tile_cols
 * float pairs. */

/* Sets the pair kernel's shared-memory limit for this window width and
 * reports how many CTAs fit on one SM. */
int phyloPairsPrepare(int window_shift, int tile_rows, int tile_cols, int *ctas_per_sm);

/* Dynamic shared memory of the pair kernel; -1 for an unknown tile shape. */
int phyloPairsSmemBytes(int window_shift, int tile_rows, int tile_cols);

/* Threads per CTA of the pair kernel; -1 for an unknown tile shape. */
int phyloPairsThreads(int window_shift, int tile_rows, int tile_cols);

/* Pair kernel over num_items work items (8 uint32 each: row0, nrow, col0,
 * ncol, w0, w1, part, tile).  Row vectors are read from the row arena and
 * column vectors from the column arena (pass the same arena twice for the
 * pairs of one set; a query batch against a resident database passes two).
 * d_counter (uint32) must be 0; partial blocks of tile_rows x tile_cols float
 * pairs go to d_part; d_item_cycles (int64[num_items]) may be 0.  fold: products per
 * FP32 accumulator between compensated folds, rounded down to a multiple of 4
 * (<= 0: 28); |error of C| <= (fold + 2) * 2^-24 for unit vectors.
 * Asynchronous. */
int phyloPairsLaunch(uintptr_t stream, uintptr_t d_row_keys, uintptr_t d_row_values,
                     uintptr_t d_row_vec_off, uintptr_t d_row_roff, uintptr_t d_col_keys,
                     uintptr_t d_col_values, uintptr_t d_col_vec_off, uintptr_t d_col_roff,
                     unsigned int num_windows, int window_shift, uintptr_t d_rowids,
                     uintptr_t d_colids, uintptr_t d_items, int num_items, uintptr_t d_counter,
                     uintptr_t d_part, int fold, uintptr_t d_item_cycles, int tile_rows,
                     int tile_cols, int grid);

/* Sums the partial blocks of each tile (4 uint32: row0, nrow, col0, ncol) into
 * d_out[rowid * ldc + colid] (double); `upper` 1 keeps pairs whose row position
 * is below the column position, 2 also the diagonal (row position == column
 * position: the self products); `mirror` also writes the transposed entry. */
int phyloPairsReduce(uintptr_t stream, uintptr_t d_part, uintptr_t d_tiles, int num_tiles,
                     int segments, int tile_rows, int tile_cols, uintptr_t d_rowids,
                     uintptr_t d_colids, uintptr_t d_out, long ldc, int upper, int mirror);

/* d_out[v * ldc + v] = sum of squares of vector v (the diagonal the
 * reference's run includes, phylogenetics_analysis/Main.java:196); d_part is
 * device scratch of phyloSelfDotPartBytes bytes. */
int phyloSelfDot(uintptr_t stream, uintptr_t d_values, uintptr_t d_vec_off, int num_vectors,
                 long max_vector_len, uintptr_t d_part, uintptr_t d_out, long ldc);

/* Scratch bytes phyloSelfDot needs. */
long phyloSelfDotPartBytes(int num_vectors, long max_vector_len);

/* Key-major (postings) pair engine.  Replaces, for a whole set of pairs, the
 * per-pair merge path of native.cu:541-703 (one compareCompositionVectors per
 * pair, DeviceWorker.submitCorrelation, DeviceWorker.java:237-323): a work item
 * is a block of row vectors x a block of column vectors (block = 128 or 64) over
 * a run of key windows; each window's entries are regrouped by key in shared
 * memory and only the products of shared keys are formed.  Products are rounded
 * once to a multiple of 2^-46 and summed exactly in 64-bit integers, so C is
 * within (products) * 2^-47 of the exact value and independent of scheduling.
 * Values must satisfy |v| < 2^7 (normalised vectors do); non-finite values count
 * as 0 (recompute those pairs with phyloComparePairsMany).
 *
 * Capacity: posting entries per side that one chunk of a window holds; -1 for
 * an unsupported block / window shift (4..14).  Prepare sets the kernel's
 * shared-memory limit in the current context and reports resident CTAs per SM. */
long phyloPostingsSmemBytes(int block, int window_shift);
long phyloPostingsCapacity(int block, int window_shift);
int phyloPostingsThreads(int block);
int phyloPostingsPrepare(int block, int window_shift, int *ctas_per_sm);

/* Work items: 8 uint32 each (row0, nrow, col0, ncol, w0, w1, part, diag); rows
 * are positions in d_rowids, columns in d_colids; diag = 1 when the rows and the
 * columns are the same block (each unordered pair and self product once).  Each
 * item writes block x block int64 partial sums (units of 2^-46) at d_part + part *
 * block^2 * 8 bytes.  d_counter (uint32) must be 0; d_status (uint32, may be 0)
 * receives DeviceError bits (2: an entry outside its window, 4: a value out of
 * range); d_item_cycles (int64[num_items], may be 0) per-item clock64 durations.
 * The window index (d_roff) and keys are those of phyloWindowIndex /
 * phyloKeyRankIndex.  Asynchronous. */
int phyloPostingsLaunch(uintptr_t stream, uintptr_t d_row_keys, uintptr_t d_row_values,
                        uintptr_t d_row_vec_off, uintptr_t d_row_roff, uintptr_t d_col_keys,
                        uintptr_t d_col_values, uintptr_t d_col_vec_off, uintptr_t d_col_roff,
                        unsigned int num_windows, int window_shift, uintptr_t d_rowids,
                        uintptr_t d_colids, uintptr_t d_items, int num_items, uintptr_t d_counter,
                        uintptr_t d_part, uintptr_t d_status, uintptr_t d_item_cycles, int block,
                        int grid);

/* Sums each tile's partials (tiles: 8 uint32 each: row0, nrow, col0, ncol, part0,
 * nparts, diag, 0) in a fixed order into d_out[rowid * ldc + colid] (double); in a
 * diag tile the pairs of row position < column position, and with `self` the self
 * products too; `mirror` also writes the transposed entry.  Asynchronous. */
int phyloPostingsReduce(uintptr_t stream, uintptr_t d_part, uintptr_t d_tiles, int num_tiles,
                        int block, uintptr_t d_rowids, uintptr_t d_colids, uintptr_t d_out,
                        long ldc, int self, int mirror);

/* Dense key ranks (no counterpart in the reference: an input transform of
 * the batched pair path).  d_rank_keys[e] = number of distinct keys of the
 * num_vectors vectors below d_keys[e] -- a strictly increasing map, so the
 * pair kernel gives the same products on ranks as on keys, over a denser key
 * space; padding keys 0xFFFFFFFF are kept.  key_limit bounds every key (A^K).
 * d_union_bits: a bitmap holding at least the vectors' keys (bit k of uint32
 * word k / 32, phyloKeyRankBitmapBytes bytes), as phyloBuildBatchEmit marks it
 * (ranks then count the marked keys below a key, still strictly increasing over
 * the vectors' keys); 0 to build the exact union here.  d_union_size (uint64, device) receives the union size.
 * d_rank_keys 0: only the union's prefix is built in the scratch, for
 * phyloKeyRankIndex.  Asynchronous. */
long phyloKeyRankScratch(long key_limit);
long phyloKeyRankBitmapBytes(long key_limit);
int phyloKeyRanks(uintptr_t stream, uintptr_t d_scratch, long scratch_bytes, long key_limit,
                  uintptr_t d_keys, uintptr_t d_vec_off, int num_vectors, long max_vector_len,
                  uintptr_t d_union_bits, uintptr_t d_rank_keys, uintptr_t d_union_size);

/* Ranks and window index in one pass: after phyloKeyRanks with d_rank_keys 0
 * on the same scratch, key_limit and d_union_bits, writes the ranks of the
 * vectors' keys to d_rank_keys and the window index over them to d_roff
 * (uint32[num_vectors][num_windows + 1], as phyloWindowIndex on the ranks).
 * num_windows = ceil(union size / 2^window_shift), the union size coming from
 * phyloKeyRanks.  arena_entries = vec_off[num_vectors] - vec_off[0] if known,
 * else 0 (it only chooses the launch shape for arenas of uneven vectors).
 * Arena layout as phyloWindowIndex.  Asynchronous. */
int phyloKeyRankIndex(uintptr_t stream, uintptr_t d_scratch, long scratch_bytes, long key_limit,
                      uintptr_t d_keys, uintptr_t d_vec_off, int num_vectors, long max_vector_len,
                      long arena_entries, uintptr_t d_union_bits, int window_shift,
                      unsigned int num_windows, uintptr_t d_rank_keys, uintptr_t d_roff);

/* Merged elements per tile of the merge-path kernels. */
int phyloCompareTileElements(void);

/* Scratch bytes of phyloComparePairsMany for num_pairs pairs and at most
 * max_tiles merge tiles (sum over pairs of ceil((nl + nr) /
 * phyloCompareTileElements())). */
long phyloComparePairsManyScratch(int num_pairs, long max_tiles);

/* C of many pairs with the merge-path kernels in one launch sequence: pair p
 * compares vector d_pa[p] of the left arena with vector d_pb[p] of the right
 * arena (arena = keys, values, uint64 offsets, uint32 sizes); d_out[p] gets C
 * (double).  Asynchronous. */
int phyloComparePairsMany(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                          uintptr_t d_lkeys, uintptr_t d_lvalues, uintptr_t d_loff,
                          uintptr_t d_lnnz, uintptr_t d_rkeys, uintptr_t d_rvalues,
                          uintptr_t d_roff, uintptr_t d_rnnz, uintptr_t d_pa, uintptr_t d_pb,
                          int num_pairs, long max_tiles, uintptr_t d_out);

/* compareCompositionVectors without the synchronisation (result left on the
 * device); scratch from estimateScratchMemory. */
int phyloComparePairAsync(uintptr_t stream, uintptr_t d_scratch, long scratch_size,
                          uintptr_t d_left_keys, uintptr_t d_left_values, int left_size,
                          uintptr_t d_right_keys, uintptr_t d_right_values, int right_size,
                          uintptr_t d_out);

#ifdef __cplusplus
}
#endif

#endif /* ROCKET_GB300_PHYLOGENETICS_H */
