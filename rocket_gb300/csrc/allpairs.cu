// allpairs.cu -- batched sparse-cosine engine for many pairs of composition vectors.
//
// The reference compares one pair per call (phylogenetics/src/main/cpp/native.cu:
// 645-703, driven pair by pair from DeviceWorker.submitCorrelation).  Here a
// whole block of pairs is computed per launch, reusing every resident vector
// across its row and column of tiles:
//
//   * The key space is cut into windows of W = 2^wshift keys.  A window index
//     roff[v][r] (the multi-way analogue of a merge-path split: the position of
//     key r*W in every sorted list, found once per vector) gives each vector's
//     sub-list in every window.
//   * A work item is 16 row vectors x up to 256 column vectors x a run of
//     windows.  For each window the 16 row sub-lists are scattered into a
//     shared-memory table D[key - r*W][row] (16 floats per key, float4 chunks
//     XOR-swizzled so random gathers spread over the banks; one extra zero row
//     serves masked lanes).  Each thread owns one column vector and streams its
//     sub-list with 16-byte loads; every entry (key, b) adds D[key][i] * b to
//     16 accumulators -- one per row.  Keys absent from a row read 0, so the
//     sum over the column's entries is exactly the intersection sum.
//   * Accumulation: FP32 products summed in FP32 for at most `fold` products,
//     then folded into a float-float (TwoSum) accumulator.  Bound on the error
//     of C: (fold + 2) * 2^-24 * sum|a*b| <= (fold + 2) * 2^-24 for unit
//     vectors (Cauchy-Schwarz).
//   * Items are handed out by an atomic counter to persistent CTAs in the
//     order given (the host sorts them by estimated cost, longest first).
//     Several CTAs share an SM, so one CTA's window barriers overlap another's
//     work.
//   * Each item writes a 16 x 256 float-float partial block; ap_reduce sums the
//     blocks of a tile in a fixed order (double-double), so results do not
//     depend on scheduling.
#include "allpairs.cuh"

namespace phylo {

size_t ap_smem_bytes(uint32_t wshift) { return (((size_t)1 << wshift) + 1) * AP_TI * sizeof(float); }

int ap_max_wshift() { return 11; }

// float index of (key idx, row) in D
__device__ __forceinline__ uint32_t d_slot(uint32_t idx, uint32_t row) {
    return idx * 16u + ((((row >> 2) ^ (idx >> 1)) & 3u) << 2) + (row & 3u);
}

__device__ __forceinline__ void fma_entry(const float *__restrict__ D, uint32_t idx, float b,
                                          float (&acc)[16]) {
    const float4 *rowp = reinterpret_cast<const float4 *>(D + idx * 16u);
    const uint32_t sw = (idx >> 1) & 3u;
    const float4 q0 = rowp[0 ^ sw], q1 = rowp[1 ^ sw], q2 = rowp[2 ^ sw], q3 = rowp[3 ^ sw];
    acc[0] = __fmaf_rn(q0.x, b, acc[0]);
    acc[1] = __fmaf_rn(q0.y, b, acc[1]);
    acc[2] = __fmaf_rn(q0.z, b, acc[2]);
    acc[3] = __fmaf_rn(q0.w, b, acc[3]);
    acc[4] = __fmaf_rn(q1.x, b, acc[4]);
    acc[5] = __fmaf_rn(q1.y, b, acc[5]);
    acc[6] = __fmaf_rn(q1.z, b, acc[6]);
    acc[7] = __fmaf_rn(q1.w, b, acc[7]);
    acc[8] = __fmaf_rn(q2.x, b, acc[8]);
    acc[9] = __fmaf_rn(q2.y, b, acc[9]);
    acc[10] = __fmaf_rn(q2.z, b, acc[10]);
    acc[11] = __fmaf_rn(q2.w, b, acc[11]);
    acc[12] = __fmaf_rn(q3.x, b, acc[12]);
    acc[13] = __fmaf_rn(q3.y, b, acc[13]);
    acc[14] = __fmaf_rn(q3.z, b, acc[14]);
    acc[15] = __fmaf_rn(q3.w, b, acc[15]);
}

__device__ __forceinline__ void fold16(float (&acc)[16], float (&hi)[16], float (&lo)[16]) {
#pragma unroll
    for (int i = 0; i < 16; i++) {
        float s, e;
        two_sum(hi[i], acc[i], s, e);
        hi[i] = s;
        lo[i] = __fadd_rn(lo[i], e);
        acc[i] = 0.0f;
    }
}

__global__ void __launch_bounds__(AP_THREADS, 2) k_allpairs(ApArgs a) {
    extern __shared__ __align__(16) float D[];  // (W + 1) x 16 floats
    __shared__ uint32_t s_item;
    const uint32_t W = 1u << a.wshift, wmask = W - 1u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t Rs = a.R + 1;

    for (uint32_t i = threadIdx.x; i < (W + 1) * 4u; i += AP_THREADS)
        reinterpret_cast<float4 *>(D)[i] = make_float4(0.f, 0.f, 0.f, 0.f);

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= a.nitems) break;
        const ApItem item = a.items[it];
        const int64_t t_start = clock64();

        // this thread's column
        const bool has_col = threadIdx.x < item.ncol;
        const uint32_t cv = has_col ? a.colids[item.col0 + threadIdx.x] : 0u;
        const uint64_t cbase = a.vec_off[cv];
        const uint32_t *cro = a.roff + (uint64_t)cv * Rs;
        // this warp's rows: 2*warp, 2*warp + 1
        uint32_t rv[2];
        uint64_t rbase[2];
        bool has_row[2];
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const uint32_t row = 2 * warp + k;
            has_row[k] = row < item.nrow;
            rv[k] = has_row[k] ? a.rowids[item.row0 + row] : 0u;
            rbase[k] = a.vec_off[rv[k]];
        }

        float acc[16], hi[16], lo[16];
#pragma unroll
        for (int i = 0; i < 16; i++) acc[i] = hi[i] = lo[i] = 0.0f;
        uint32_t nacc = 0;

        // window offsets: rows via lane-held prefetch of 32 windows, column
        // one window ahead
        uint32_t r_lo[2] = {0, 0}, r_hi[2] = {0, 0};
        uint32_t wb = item.w0;
        uint32_t c_lo = has_col ? __ldg(&cro[item.w0]) : 0u;
        uint32_t c_hi_next = has_col ? __ldg(&cro[item.w0 + 1]) : 0u;

        for (uint32_t r = item.w0; r < item.w1; r++) {
            if (r == item.w0 || r - wb >= 32u) {
                wb = r;
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    if (has_row[k]) {
                        const uint32_t *ro = a.roff + (uint64_t)rv[k] * Rs;
                        r_lo[k] = __ldg(&ro[min(r + lane, a.R)]);
                        r_hi[k] = __ldg(&ro[min(r + lane + 1, a.R)]);
                    }
                }
            }
            const int sl = (int)(r - wb);
            const uint32_t c_hi = c_hi_next;
            if (has_col && r + 2 <= a.R) c_hi_next = __ldg(&cro[r + 2]);
            // densify this warp's rows
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const uint32_t lo_k = __shfl_sync(0xffffffffu, r_lo[k], sl);
                const uint32_t hi_k = __shfl_sync(0xffffffffu, r_hi[k], sl);
                if (has_row[k]) {
                    const uint32_t row = 2 * warp + k;
                    for (uint32_t e = lo_k + lane; e < hi_k; e += 32) {
                        const uint32_t key = __ldg(&a.keys[rbase[k] + e]);
                        D[d_slot(key & wmask, row)] = __ldg(&a.vals[rbase[k] + e]);
                    }
                }
            }
            __syncthreads();
            // stream this thread's column entries [c_lo, c_hi)
            if (has_col && c_hi > c_lo) {
                const uint32_t g0 = c_lo & ~3u;
                for (uint32_t g = g0; g < c_hi; g += 4) {
                    const uint4 kk = __ldg(reinterpret_cast<const uint4 *>(a.keys + cbase + g));
                    const float4 vv = __ldg(reinterpret_cast<const float4 *>(a.vals + cbase + g));
                    const uint32_t ks[4] = {kk.x, kk.y, kk.z, kk.w};
                    const float vs[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const uint32_t e = g + u;
                        const bool ok = e >= c_lo && e < c_hi;
                        fma_entry(D, ok ? (ks[u] & wmask) : W, ok ? vs[u] : 0.0f, acc);
                    }
                    nacc += 4;
                    if (nacc >= a.fold) {
                        fold16(acc, hi, lo);
                        nacc = 0;
                    }
                }
            }
            c_lo = c_hi;
            __syncthreads();
            // clear this warp's rows
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const uint32_t lo_k = __shfl_sync(0xffffffffu, r_lo[k], sl);
                const uint32_t hi_k = __shfl_sync(0xffffffffu, r_hi[k], sl);
                if (has_row[k]) {
                    const uint32_t row = 2 * warp + k;
                    for (uint32_t e = lo_k + lane; e < hi_k; e += 32) {
                        const uint32_t key = __ldg(&a.keys[rbase[k] + e]);
                        D[d_slot(key & wmask, row)] = 0.0f;
                    }
                }
            }
        }
        fold16(acc, hi, lo);
        // partial block [16][256]
        FF *dst = a.part + (uint64_t)item.part * (AP_TI * AP_TJ);
#pragma unroll
        for (int i = 0; i < 16; i++) dst[i * AP_TJ + threadIdx.x] = FF{hi[i], lo[i]};
        if (a.item_cycles && threadIdx.x == 0) a.item_cycles[it] = clock64() - t_start;
    }
}

cudaError_t ap_prepare(uint32_t wshift, int *ctas_per_sm) {
    const size_t smem = ap_smem_bytes(wshift);
    PHYLO_CHECK(cudaFuncSetAttribute(k_allpairs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    if (ctas_per_sm) {
        int n = 0;
        PHYLO_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_allpairs, AP_THREADS, smem));
        *ctas_per_sm = n;
    }
    return cudaSuccess;
}

cudaError_t ap_launch(const ApArgs &a, int grid, cudaStream_t st) {
    k_allpairs<<<grid, AP_THREADS, ap_smem_bytes(a.wshift), st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// window index
// ---------------------------------------------------------------------------

// one CTA per vector
__global__ void k_range_index(const uint32_t *__restrict__ keys, const uint64_t *__restrict__ vec_off,
                              uint32_t R, uint32_t wshift, uint32_t *roff) {
    const uint32_t v = blockIdx.x;
    const uint64_t b = vec_off[v];
    const uint32_t n = (uint32_t)(vec_off[v + 1] - b);  // padded length may exceed nnz
    uint32_t *ro = roff + (uint64_t)v * (R + 1);
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
        const uint32_t key = keys[b + e];
        if (key == 0xffffffffu) continue;  // padding
        const uint32_t rt = min(key >> wshift, R);
        const uint32_t prev = e == 0 ? 0u : keys[b + e - 1];
        const int64_t rp = (e == 0) ? -1 : (int64_t)min(prev >> wshift, R);
        for (int64_t r = rp + 1; r <= (int64_t)rt; r++) ro[r] = e;
    }
    // tail: windows after the last real key get the real length
    if (threadIdx.x == 0) {
        uint32_t m = n;
        while (m > 0 && keys[b + m - 1] == 0xffffffffu) m--;
        const int64_t rl = m == 0 ? -1 : (int64_t)min(keys[b + m - 1] >> wshift, R);
        for (int64_t r = rl + 1; r <= (int64_t)R; r++) ro[r] = m;
    }
}

cudaError_t range_index_launch(const uint32_t *keys, const uint64_t *vec_off, uint32_t N,
                               uint32_t R, uint32_t wshift, uint32_t *roff, cudaStream_t st) {
    if (N == 0) return cudaSuccess;
    k_range_index<<<N, 256, 0, st>>>(keys, vec_off, R, wshift, roff);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// reduction of partial blocks
// ---------------------------------------------------------------------------

// grid = ntiles, block = 256 (one column per thread)
__global__ void k_ap_reduce(ApReduceArgs r) {
    const ApTile t = r.tiles[blockIdx.x];
    const uint32_t c = threadIdx.x;
    if (c >= t.ncol) return;
    const uint32_t colid = r.colids[t.col0 + c];
    const FF *base = r.part + (uint64_t)blockIdx.x * r.S * (AP_TI * AP_TJ);
    for (uint32_t i = 0; i < t.nrow; i++) {
        const uint32_t rowpos = t.row0 + i, colpos = t.col0 + c;
        if (r.upper && !(rowpos < colpos)) continue;
        DD acc = {0.0, 0.0};
        for (uint32_t s = 0; s < r.S; s++) {
            const FF p = base[(uint64_t)s * (AP_TI * AP_TJ) + i * AP_TJ + c];
            dd_add(acc, (double)p.hi);
            dd_add(acc, (double)p.lo);
        }
        const double v = __dadd_rn(acc.hi, acc.lo);
        const uint32_t rowid = r.rowids[rowpos];
        r.out[(uint64_t)rowid * r.ldc + colid] = v;
        if (r.mirror) r.out[(uint64_t)colid * r.ldc + rowid] = v;
    }
}

cudaError_t ap_reduce_launch(const ApReduceArgs &r, cudaStream_t st) {
    if (r.ntiles == 0) return cudaSuccess;
    k_ap_reduce<<<r.ntiles, AP_TJ, 0, st>>>(r);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// self products (the diagonal of the reference's run, Main.java:196)
// ---------------------------------------------------------------------------

__global__ void k_self_dot(const float *__restrict__ vals, const uint64_t *__restrict__ vec_off,
                           double *out, uint64_t ldc) {
    const uint32_t v = blockIdx.x;
    const uint64_t b = vec_off[v], n = vec_off[v + 1] - b;
    FF acc = {0.0f, 0.0f};
    for (uint64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const float x = vals[b + e];
        float p, q;
        two_prod(x, x, p, q);
        ff_add(acc, p);
        acc.lo = __fadd_rn(acc.lo, q);
    }
    acc = ff_warp_sum(acc);
    __shared__ FF ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        DD d = {0.0, 0.0};
        for (int w = 0; w < (int)(blockDim.x / 32); w++) {
            dd_add(d, (double)ws[w].hi);
            dd_add(d, (double)ws[w].lo);
        }
        out[(uint64_t)v * ldc + v] = __dadd_rn(d.hi, d.lo);
    }
}

cudaError_t self_dot_launch(const float *vals, const uint64_t *vec_off, uint32_t N, double *out,
                            uint64_t ldc, cudaStream_t st) {
    if (N == 0) return cudaSuccess;
    k_self_dot<<<N, 256, 0, st>>>(vals, vec_off, out, ldc);
    return cudaGetLastError();
}

}  // namespace phylo
