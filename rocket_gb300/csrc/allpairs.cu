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
//     shared-memory table D[key - r*W] of 80-byte records (16 row values +
//     padding: the odd stride spreads random gathers over the banks; one extra
//     zero record serves masked lanes).  The item's columns share the CTA's
//     lanes evenly (two or four lanes per column); a column's lanes stream its
//     sub-list in 16-byte groups through cp.async rings, and every entry (key, b)
//     adds D[key][i] * b to 16 accumulators -- one per row.  Keys absent from a
//     row read 0, so the column's sum is exactly the intersection sum.
//   * Accumulation: FP32 products summed in FP32 for at most `fold` products,
//     then folded into a float-float (TwoSum) accumulator.  Bound on the error
//     of C: (fold + 2) * 2^-24 * sum|a*b| <= (fold + 2) * 2^-24 for unit
//     vectors (Cauchy-Schwarz).
//   * Items are handed out by an atomic counter to persistent CTAs in the
//     order given (the host sorts them by estimated cost, longest first).
//   * Each item writes a 16 x (item width) float-float partial block;
//     ap_reduce sums the blocks of a tile in a fixed order (double-double), so
//     results do not depend on scheduling.
#include "allpairs.cuh"

namespace phylo {

// The row table D holds, for each key of the window, the 16 row values in one
// 80-byte record (64 bytes of values + 16 bytes of padding).  The odd stride
// (5 x 16 bytes) spreads the four 16-byte loads of random keys over all eight
// 16-byte bank groups, and the four loads of a key are one base address plus
// constant offsets.  One extra record (index W) stays zero for masked lanes.
constexpr uint32_t D_STRIDE = 20;  // floats per key record

static size_t ap_ring_bytes(int threads);

// float index of (key idx, row) in D
__device__ __forceinline__ uint32_t d_slot(uint32_t idx, uint32_t row) {
    return idx * D_STRIDE + row;
}

__device__ __forceinline__ void fma_entry(const float *__restrict__ D, uint32_t idx, float b,
                                          float (&acc)[16]) {
    const float4 *rowp = reinterpret_cast<const float4 *>(D + idx * D_STRIDE);
    const float4 q0 = rowp[0], q1 = rowp[1], q2 = rowp[2], q3 = rowp[3];
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

// Per-thread ring of 16-byte column groups (4 keys + 4 values) fetched with
// cp.async (L2 only: a column is read once per item, so caching it in L1 would
// only evict the row side's data), ring_depth(threads) groups ahead of the one
// being used, so a thread's column stream stays in flight across window barriers.
// Four groups for the 512-thread kernels (one CTA per SM; the columns of large
// items stream from DRAM), two for the smaller CTAs, several of which share an SM.
__host__ __device__ constexpr int ring_depth(int threads) { return threads >= 512 ? 4 : 2; }

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(smem)), "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int RING>
__device__ __forceinline__ void cp_async_wait_ring() {
    asm volatile("cp.async.wait_group %0;" ::"n"(RING - 1) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

static size_t ap_ring_bytes(int threads) { return (size_t)ring_depth(threads) * threads * 32; }

// Entries [e0, e1) of a vector's keys and values (widened to whole 16-byte
// groups; vectors start on 16-byte boundaries and are padded to whole groups)
// into L2 with one bulk prefetch each.
__device__ __forceinline__ void prefetch_l2(const uint32_t *keys, const float *vals, uint32_t e0,
                                            uint32_t e1) {
    const uint32_t g0 = e0 & ~3u, g1 = (e1 + 3u) & ~3u;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(keys + g0), "r"(4u * (g1 - g0))
                 : "memory");
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(vals + g0), "r"(4u * (g1 - g0))
                 : "memory");
}

// Lanes of an item's columns: column j takes lanes [s_lane0[j], s_lane0[j + 1]),
// all THREADS lanes split as evenly as possible over the item's columns (at least
// one each), so the lanes of an item with fewer columns than the tile's width
// (at the ragged end of a tile row) are not left idle.  (Weighting the split by
// the columns' entries measured slower on the full uneven1024 workload: the
// largest tiles' items are bound by the column stream, not by lane work.)
template <int THREADS>
__device__ __forceinline__ void assign_lanes(const ApItem &item, uint32_t *s_lane0,
                                             uint16_t *s_col) {
    const uint32_t t = threadIdx.x, nc = item.ncol;
    if (t <= nc && nc > 0) s_lane0[t] = (uint32_t)((uint64_t)t * THREADS / nc);
    __syncthreads();
    if (t < nc)
        for (uint32_t l = s_lane0[t]; l < s_lane0[t + 1]; l++) s_col[l] = (uint16_t)t;
    __syncthreads();
}

// Sums of the lanes of each column, in lane order, into the item's partial block
// (rows x tj float pairs).  The sums pass through `stage` (8 rows x THREADS float
// pairs: the idle cp.async ring), eight rows at a time.
template <int THREADS>
__device__ __forceinline__ void combine_lanes(const float (&hi)[16], const float (&lo)[16],
                                              FF *stage, FF *dst, uint32_t tj, bool has_col,
                                              uint32_t jcol, uint32_t l0, uint32_t q,
                                              uint32_t lpc) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 8; i++) stage[i * THREADS + threadIdx.x] = FF{hi[8 * h + i], lo[8 * h + i]};
        __syncthreads();
        if (has_col) {
            for (uint32_t i = q; i < 8; i += lpc) {
                FF v = stage[i * THREADS + l0];
                for (uint32_t m = 1; m < lpc; m++) v = ff_merge(v, stage[i * THREADS + l0 + m]);
                dst[(8 * h + i) * tj + jcol] = v;
            }
        }
    }
}

// Shape of a 16-row work item for a CTA of THREADS threads: THREADS / LPC
// columns; each warp scatters AP_TI / warps rows, LPR lanes per row, and
// prefetches NPF entries per lane of each row's next window.  (Scattering rows in
// 16-byte groups of four entries was measured slower on every workload.)
template <int THREADS, int LPC>
struct ApShape {
    static constexpr int NW = THREADS / 32;
    static constexpr int TJ = THREADS / LPC;     // column vectors per item
    static constexpr int RPW = AP_TI / NW;       // rows a warp scatters
    static constexpr int LPR = 32 / RPW;         // lanes per scattered row
    static constexpr int NPF = 4;                // prefetched row entries per lane (>= RPW)
    static_assert(RPW <= NPF, "rows per warp");
};

// Column side: the item's columns share the lanes evenly (assign_lanes), lpc
// lanes per column.  Lane q of a column streams the column's 4-entry groups q,
// q + lpc, q + 2 lpc, ... through its cp.async ring, so the lanes of a column fetch
// 16 lpc contiguous bytes per load, and keeps its own 16 accumulators for the
// whole item; the lanes' sums are combined once, at the end of the item.  Row
// side: lane (srow, sj) of a warp scatters entries sj, sj + LPR, ... of row
// warp * RPW + srow; the first NPF * LPR entries of each row's next window are
// prefetched into registers.
template <int THREADS, int MINB, int LPC>
__global__ void __launch_bounds__(THREADS, MINB) k_allpairs(ApArgs a) {
    using S = ApShape<THREADS, LPC>;
    constexpr int TJ = S::TJ, RPW = S::RPW, LPR = S::LPR, NPF = S::NPF;
    constexpr int RING = ring_depth(THREADS);
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t W = 1u << a.wshift, wmask = W - 1u;
    float *D = reinterpret_cast<float *>(smem);                    // (W + 1) x 16
    uint4 *ring_k = reinterpret_cast<uint4 *>(smem + (size_t)(W + 1) * D_STRIDE * 4);
    float4 *ring_v = reinterpret_cast<float4 *>(ring_k + RING * THREADS);
    __shared__ uint32_t s_item;
    __shared__ uint32_t s_lane0[TJ + 1];
    __shared__ uint16_t s_col[THREADS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t srow = lane / LPR, sj = lane % LPR;
    const uint32_t rr = warp * RPW + srow;  // row position this lane scatters
    const int rsrc = (int)(srow * LPR);     // first lane of this row
    const uint32_t Rs = a.R + 1;

    for (uint32_t i = threadIdx.x; i < (W + 1) * (D_STRIDE / 4); i += THREADS)
        reinterpret_cast<float4 *>(D)[i] = make_float4(0.f, 0.f, 0.f, 0.f);

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= a.nitems) break;
        const ApItem item = a.items[it];
        const int64_t t_start = clock64();

        // ---- column side: lpc lanes of column jcol, this one the q-th
        assign_lanes<THREADS>(item, s_lane0, s_col);
        const bool has_col = item.ncol > 0;
        const uint32_t jcol = has_col ? s_col[threadIdx.x] : 0u;
        const uint32_t l0 = has_col ? s_lane0[jcol] : threadIdx.x;
        const uint32_t q = threadIdx.x - l0, lpc = has_col ? s_lane0[jcol + 1] - l0 : 1u;
        const uint32_t cv = has_col ? a.colids[item.col0 + jcol] : 0u;
        const uint64_t cbase = a.col.vec_off[cv];
        const uint32_t *cro = a.col.roff + (uint64_t)cv * Rs;
        uint32_t c_lo = has_col ? __ldg(&cro[item.w0]) : 0u;
        const uint32_t c_end = has_col ? __ldg(&cro[item.w1]) : 0u;
        uint32_t c_hi_next = has_col ? __ldg(&cro[item.w0 + 1]) : 0u;
        // this lane's groups start at entry (c_lo & ~3) + 4q and advance by 16
        uint32_t cur = (c_lo & ~3u) + 4 * q;  // first entry of the oldest unreleased group
        uint32_t fetch = cur;                  // next group to fetch
        uint32_t slot_cur = 0, slot_fetch = 0;
#pragma unroll
        for (int k = 0; k < RING; k++) {
            if (fetch < c_end) {
                cp_async16(&ring_k[slot_fetch * THREADS + threadIdx.x], a.col.keys + cbase + fetch);
                cp_async16(&ring_v[slot_fetch * THREADS + threadIdx.x], a.col.vals + cbase + fetch);
            }
            fetch += 4 * lpc;
            slot_fetch = slot_fetch + 1 == RING ? 0 : slot_fetch + 1;
            cp_async_commit();
        }

        // ---- row side: this lane scatters row rr
        const bool has_row = rr < item.nrow;
        const uint32_t rv = has_row ? a.rowids[item.row0 + rr] : 0u;
        const uint64_t rbase = a.row.vec_off[rv];
        const uint32_t *ro = a.row.roff + (uint64_t)rv * Rs;
        float acc[16], hi[16], lo[16];
#pragma unroll
        for (int i = 0; i < 16; i++) acc[i] = hi[i] = lo[i] = 0.0f;
        uint32_t nacc = 0;

        // window offsets of LPR windows, held by the row's lanes; the first
        // NPF * LPR entries of the row's next window prefetched, NPF per lane
        uint32_t wb = item.w0;
        uint32_t r_lo = 0, r_hi = 0;
        if (has_row) {
            r_lo = __ldg(&ro[min(wb + sj, a.R)]);
            r_hi = __ldg(&ro[min(wb + sj + 1, a.R)]);
        }
        uint32_t pk[NPF];
        float pv[NPF];
        {
            const uint32_t lo0 = __shfl_sync(0xffffffffu, r_lo, rsrc);
            const uint32_t hi0 = __shfl_sync(0xffffffffu, r_hi, rsrc);
#pragma unroll
            for (int t = 0; t < NPF; t++) {
                const uint32_t e = lo0 + sj + t * LPR;
                pk[t] = 0xffffffffu;
                pv[t] = 0.f;
                if (has_row && e < hi0) {
                    pk[t] = __ldg(&a.row.keys[rbase + e]);
                    pv[t] = __ldg(&a.row.vals[rbase + e]);
                }
            }
        }

        for (uint32_t r = item.w0; r < item.w1; r++) {
            const int sl = (int)(r - wb);
            const uint32_t lo_r = __shfl_sync(0xffffffffu, r_lo, rsrc + sl);
            const uint32_t hi_r = __shfl_sync(0xffffffffu, r_hi, rsrc + sl);
            // scatter window r of row rr: first NPF * LPR entries from registers, the rest loaded
            uint32_t ck[NPF];
#pragma unroll
            for (int t = 0; t < NPF; t++) {
                ck[t] = pk[t];
                if (pk[t] != 0xffffffffu) D[d_slot(pk[t] & wmask, rr)] = pv[t];
            }
            if (has_row) {
                for (uint32_t e = lo_r + NPF * LPR + sj; e < hi_r; e += LPR) {
                    const uint32_t key = __ldg(&a.row.keys[rbase + e]);
                    D[d_slot(key & wmask, rr)] = __ldg(&a.row.vals[rbase + e]);
                }
            }
            // prefetch the next window's row offsets and first entries
            if (r + 1 < item.w1) {
                if (r + 1 - wb >= (uint32_t)LPR) {
                    wb = r + 1;
                    if (has_row) {
                        r_lo = __ldg(&ro[min(wb + sj, a.R)]);
                        r_hi = __ldg(&ro[min(wb + sj + 1, a.R)]);
                    }
                }
                const int sn = (int)(r + 1 - wb);
                const uint32_t nlo = __shfl_sync(0xffffffffu, r_lo, rsrc + sn);
                const uint32_t nhi = __shfl_sync(0xffffffffu, r_hi, rsrc + sn);
#pragma unroll
                for (int t = 0; t < NPF; t++) {
                    const uint32_t e = nlo + sj + t * LPR;
                    pk[t] = 0xffffffffu;
                    if (has_row && e < nhi) {
                        pk[t] = __ldg(&a.row.keys[rbase + e]);
                        pv[t] = __ldg(&a.row.vals[rbase + e]);
                    }
                }
                // the rest of the row's next window (the scatter loop's loads) into L2,
                // a whole window's gathers ahead: large rows stream from DRAM
                if (has_row && sj == 0 && nhi > nlo + NPF * LPR)
                    prefetch_l2(a.row.keys + rbase, a.row.vals + rbase, nlo + NPF * LPR, nhi);
            }
            const uint32_t c_hi = c_hi_next;
            if (has_col && r + 2 <= a.R) c_hi_next = __ldg(&cro[r + 2]);
            __syncthreads();
            // this lane's groups of the column that start before c_hi
            if (has_col) {
                while (cur < c_hi) {
                    cp_async_wait_ring<RING>();
                    const uint4 kk = ring_k[slot_cur * THREADS + threadIdx.x];
                    const float4 vv = ring_v[slot_cur * THREADS + threadIdx.x];
                    const uint32_t ks[4] = {kk.x, kk.y, kk.z, kk.w};
                    const float vs[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const uint32_t e = cur + u;
                        const bool ok = e >= c_lo && e < c_hi;
                        fma_entry(D, ok ? (ks[u] & wmask) : W, ok ? vs[u] : 0.0f, acc);
                    }
                    nacc += 4;
                    if (nacc >= a.fold) {
                        fold16(acc, hi, lo);
                        nacc = 0;
                    }
                    if (cur + 4 > c_hi) break;  // reaches into the next window: keep it
                    if (fetch < c_end) {
                        cp_async16(&ring_k[slot_fetch * THREADS + threadIdx.x],
                                   a.col.keys + cbase + fetch);
                        cp_async16(&ring_v[slot_fetch * THREADS + threadIdx.x],
                                   a.col.vals + cbase + fetch);
                    }
                    fetch += 4 * lpc;
                    slot_fetch = slot_fetch + 1 == RING ? 0 : slot_fetch + 1;
                    cp_async_commit();
                    cur += 4 * lpc;
                    slot_cur = slot_cur + 1 == RING ? 0 : slot_cur + 1;
                }
            }
            c_lo = c_hi;
            __syncthreads();
            // clear window r of row rr
#pragma unroll
            for (int t = 0; t < NPF; t++)
                if (ck[t] != 0xffffffffu) D[d_slot(ck[t] & wmask, rr)] = 0.0f;
            if (has_row) {
                for (uint32_t e = lo_r + NPF * LPR + sj; e < hi_r; e += LPR) {
                    const uint32_t key = __ldg(&a.row.keys[rbase + e]);
                    D[d_slot(key & wmask, rr)] = 0.0f;
                }
            }
            __syncwarp();
        }
        cp_async_wait_all();
        fold16(acc, hi, lo);
        combine_lanes<THREADS>(hi, lo, reinterpret_cast<FF *>(ring_k),
                               a.part + (uint64_t)item.part * (AP_TI * TJ), TJ, has_col, jcol, l0,
                               q, lpc);
        if (a.item_cycles && threadIdx.x == 0) a.item_cycles[it] = clock64() - t_start;
    }
}

// ---------------------------------------------------------------------------
// 32-row items
// ---------------------------------------------------------------------------
//
// The same window scheme with 32 row vectors per item and one 128-byte record
// (32 row values) per key.  Eight lanes share a column vector and walk the same
// entries; lane g of the eight holds rows 4g..4g+3, so each entry costs every
// lane one 16-byte shared load and four FMAs.  Record s keeps rows 4c..4c+3 in
// its 16-byte chunk c ^ (s & 7): the eight lanes of a column read the eight
// chunks of one record (one wavefront, never a bank conflict), and the row
// scatter, where lanes hold different keys of the same row, spreads its stores
// over eight bank groups.  Column entries are fetched eight at a time (one per
// lane, three blocks ahead) and passed round the eight lanes by shuffles.  Each
// lane accumulates its own rows, so a column needs no cross-lane combine.

constexpr uint32_t R32_REC = 32;  // floats per key record
constexpr int R32_TJ = 64;        // column vectors per item

__device__ __forceinline__ uint32_t r32_pos(uint32_t slot, uint32_t row) {
    return slot * R32_REC + ((((row >> 2) ^ (slot & 7u)) << 2) | (row & 3u));
}

template <int THREADS>
struct R32Shape {
    static constexpr int NW = THREADS / 32;       // warps
    static constexpr int CPP = NW * 4;            // columns per pass (4 per warp)
    static constexpr int PASSES = R32_TJ / CPP;   // column passes per window
    static constexpr int RPW = 32 / NW;           // rows a warp scatters
    static constexpr int LPR = 32 / RPW;          // lanes per scattered row
    static constexpr int NPF = RPW;               // prefetched entries per lane (NPF * LPR = 32)
    static_assert(PASSES * CPP == R32_TJ, "columns per item");
};

template <int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_allpairs32(ApArgs a) {
    using S = R32Shape<THREADS>;
    constexpr int PASSES = S::PASSES, RPW = S::RPW, LPR = S::LPR, NPF = S::NPF;
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t W = 1u << a.wshift, wmask = W - 1u;
    float *D = reinterpret_cast<float *>(smem);  // (W + 1) records
    __shared__ uint32_t s_item;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t g = lane & 7;               // rows 4g..4g+3 on the column side
    const uint32_t gsrc = lane & ~7u;          // first lane of this column group
    const uint32_t srow = lane / LPR;          // scatter: row of this lane within the warp
    const uint32_t sj = lane % LPR;            // scatter: entry offset within the row
    const uint32_t rr = warp * RPW + srow;     // scatter: row position in the item
    const uint32_t Rs = a.R + 1;

    for (uint32_t i = threadIdx.x; i < (W + 1) * (R32_REC / 4); i += THREADS)
        reinterpret_cast<float4 *>(D)[i] = make_float4(0.f, 0.f, 0.f, 0.f);

    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= a.nitems) break;
        const ApItem item = a.items[it];
        const int64_t t_start = clock64();

        // ---- column side: PASSES column vectors per lane group
        bool has_col[PASSES];
        uint64_t cbase[PASSES];
        const uint32_t *cro[PASSES];
        uint32_t ce[PASSES], c_end[PASSES], blk[PASSES], c_hi_next[PASSES];
        uint32_t bk0[PASSES], bk1[PASSES], bk2[PASSES];
        float bv0[PASSES], bv1[PASSES], bv2[PASSES];
        float acc[PASSES][4], hi[PASSES][4], lo[PASSES][4];
        uint32_t nacc[PASSES];
#pragma unroll
        for (int p = 0; p < PASSES; p++) {
            const uint32_t jc = p * S::CPP + warp * 4 + (lane >> 3);
            has_col[p] = jc < item.ncol;
            const uint32_t cv = has_col[p] ? a.colids[item.col0 + jc] : 0u;
            cbase[p] = a.col.vec_off[cv];
            cro[p] = a.col.roff + (uint64_t)cv * Rs;
            ce[p] = has_col[p] ? __ldg(&cro[p][item.w0]) : 0u;
            c_end[p] = has_col[p] ? __ldg(&cro[p][item.w1]) : 0u;
            c_hi_next[p] = has_col[p] ? __ldg(&cro[p][item.w0 + 1]) : 0u;
            blk[p] = ce[p] & ~7u;
            const uint32_t e0 = blk[p] + g, e1 = e0 + 8, e2 = e0 + 16;
            bk0[p] = e0 < c_end[p] ? __ldg(&a.col.keys[cbase[p] + e0]) : 0u;
            bv0[p] = e0 < c_end[p] ? __ldg(&a.col.vals[cbase[p] + e0]) : 0.f;
            bk1[p] = e1 < c_end[p] ? __ldg(&a.col.keys[cbase[p] + e1]) : 0u;
            bv1[p] = e1 < c_end[p] ? __ldg(&a.col.vals[cbase[p] + e1]) : 0.f;
            bk2[p] = e2 < c_end[p] ? __ldg(&a.col.keys[cbase[p] + e2]) : 0u;
            bv2[p] = e2 < c_end[p] ? __ldg(&a.col.vals[cbase[p] + e2]) : 0.f;
#pragma unroll
            for (int u = 0; u < 4; u++) acc[p][u] = hi[p][u] = lo[p][u] = 0.f;
            nacc[p] = 0;
        }

        // ---- row side: this lane scatters row rr
        const bool has_row = rr < item.nrow;
        const uint32_t rv = has_row ? a.rowids[item.row0 + rr] : 0u;
        const uint64_t rbase = a.row.vec_off[rv];
        const uint32_t *ro = a.row.roff + (uint64_t)rv * Rs;
        // window offsets of LPR windows, held by the row's lanes
        uint32_t wb = item.w0;
        uint32_t r_lo = 0, r_hi = 0;
        if (has_row) {
            r_lo = __ldg(&ro[min(wb + sj, a.R)]);
            r_hi = __ldg(&ro[min(wb + sj + 1, a.R)]);
        }
        const int rsrc = (int)(srow * LPR);
        uint32_t pk[NPF];
        float pv[NPF];
        {
            const uint32_t lo0 = __shfl_sync(0xffffffffu, r_lo, rsrc);
            const uint32_t hi0 = __shfl_sync(0xffffffffu, r_hi, rsrc);
#pragma unroll
            for (int t = 0; t < NPF; t++) {
                const uint32_t e = lo0 + sj + t * LPR;
                pk[t] = 0xffffffffu;
                pv[t] = 0.f;
                if (has_row && e < hi0) {
                    pk[t] = __ldg(&a.row.keys[rbase + e]);
                    pv[t] = __ldg(&a.row.vals[rbase + e]);
                }
            }
        }

        for (uint32_t r = item.w0; r < item.w1; r++) {
            const int sl = (int)(r - wb);
            const uint32_t lo_r = __shfl_sync(0xffffffffu, r_lo, rsrc + sl);
            const uint32_t hi_r = __shfl_sync(0xffffffffu, r_hi, rsrc + sl);
            // scatter window r of row rr
            uint32_t ck[NPF];
#pragma unroll
            for (int t = 0; t < NPF; t++) {
                ck[t] = pk[t];
                if (pk[t] != 0xffffffffu) D[r32_pos(pk[t] & wmask, rr)] = pv[t];
            }
            if (has_row) {
                for (uint32_t e = lo_r + 32 + sj; e < hi_r; e += LPR) {
                    const uint32_t key = __ldg(&a.row.keys[rbase + e]);
                    D[r32_pos(key & wmask, rr)] = __ldg(&a.row.vals[rbase + e]);
                }
            }
            // prefetch the next window's offsets and first entries
            if (r + 1 < item.w1) {
                if (r + 1 - wb >= (uint32_t)LPR) {
                    wb = r + 1;
                    if (has_row) {
                        r_lo = __ldg(&ro[min(wb + sj, a.R)]);
                        r_hi = __ldg(&ro[min(wb + sj + 1, a.R)]);
                    }
                }
                const int sn = (int)(r + 1 - wb);
                const uint32_t nlo = __shfl_sync(0xffffffffu, r_lo, rsrc + sn);
                const uint32_t nhi = __shfl_sync(0xffffffffu, r_hi, rsrc + sn);
#pragma unroll
                for (int t = 0; t < NPF; t++) {
                    const uint32_t e = nlo + sj + t * LPR;
                    pk[t] = 0xffffffffu;
                    if (has_row && e < nhi) {
                        pk[t] = __ldg(&a.row.keys[rbase + e]);
                        pv[t] = __ldg(&a.row.vals[rbase + e]);
                    }
                }
            }
            uint32_t c_hi[PASSES];
#pragma unroll
            for (int p = 0; p < PASSES; p++) {
                c_hi[p] = c_hi_next[p];
                if (has_col[p] && r + 2 <= a.R) c_hi_next[p] = __ldg(&cro[p][r + 2]);
            }
            __syncthreads();
            // column entries of window r
#pragma unroll
            for (int p = 0; p < PASSES; p++) {
                const uint32_t cnt = c_hi[p] - ce[p];  // 0 without a column
                const uint32_t maxc = __reduce_max_sync(0xffffffffu, cnt);
                for (uint32_t t = 0; t < maxc; t++) {
                    const bool act = t < cnt;
                    const uint32_t ee = ce[p] + t;
                    if (act && ee >= blk[p] + 8) {
                        blk[p] += 8;
                        bk0[p] = bk1[p]; bv0[p] = bv1[p];
                        bk1[p] = bk2[p]; bv1[p] = bv2[p];
                        const uint32_t e2 = blk[p] + 16 + g;
                        if (e2 < c_end[p]) {
                            bk2[p] = __ldg(&a.col.keys[cbase[p] + e2]);
                            bv2[p] = __ldg(&a.col.vals[cbase[p] + e2]);
                        }
                    }
                    const int src = (int)(gsrc | (ee & 7u));
                    const uint32_t k = __shfl_sync(0xffffffffu, bk0[p], src);
                    const float v = __shfl_sync(0xffffffffu, bv0[p], src);
                    const uint32_t slot = act ? (k & wmask) : W;
                    const float b = act ? v : 0.f;
                    const float4 q = *reinterpret_cast<const float4 *>(
                        D + slot * R32_REC + ((g ^ (slot & 7u)) << 2));
                    acc[p][0] = __fmaf_rn(q.x, b, acc[p][0]);
                    acc[p][1] = __fmaf_rn(q.y, b, acc[p][1]);
                    acc[p][2] = __fmaf_rn(q.z, b, acc[p][2]);
                    acc[p][3] = __fmaf_rn(q.w, b, acc[p][3]);
                    if (++nacc[p] >= a.fold) {
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            float s2, e2;
                            two_sum(hi[p][u], acc[p][u], s2, e2);
                            hi[p][u] = s2;
                            lo[p][u] = __fadd_rn(lo[p][u], e2);
                            acc[p][u] = 0.f;
                        }
                        nacc[p] = 0;
                    }
                }
                ce[p] += cnt;
            }
            __syncthreads();
            // clear window r of row rr
#pragma unroll
            for (int t = 0; t < NPF; t++)
                if (ck[t] != 0xffffffffu) D[r32_pos(ck[t] & wmask, rr)] = 0.f;
            if (has_row) {
                for (uint32_t e = lo_r + 32 + sj; e < hi_r; e += LPR) {
                    const uint32_t key = __ldg(&a.row.keys[rbase + e]);
                    D[r32_pos(key & wmask, rr)] = 0.f;
                }
            }
            __syncwarp();
        }
        // fold and write: lane g of column jc owns rows 4g..4g+3
        FF *dst = a.part + (uint64_t)item.part * (32 * R32_TJ);
#pragma unroll
        for (int p = 0; p < PASSES; p++) {
            const uint32_t jc = p * S::CPP + warp * 4 + (lane >> 3);
            if (!has_col[p]) continue;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                float s2, e2;
                two_sum(hi[p][u], acc[p][u], s2, e2);
                FF v;
                two_sum(s2, __fadd_rn(lo[p][u], e2), v.hi, v.lo);
                dst[(4 * g + u) * R32_TJ + jc] = v;
            }
        }
        if (a.item_cycles && threadIdx.x == 0) a.item_cycles[it] = clock64() - t_start;
    }
}

// 32-row kernel: 512 threads (one pass over 64 columns) when the table leaves
// room for one CTA per SM, else 256 threads (two passes) and two CTAs per SM.
static size_t r32_smem_bytes(uint32_t wshift) {
    return (((size_t)1 << wshift) + 1) * R32_REC * sizeof(float);
}
static bool r32_wide(uint32_t wshift) { return r32_smem_bytes(wshift) > 100 * 1024; }

bool ap_shape_ok(int tile_rows, int tile_cols) {
    return (tile_rows == 16 &&
            (tile_cols == 256 || tile_cols == 128 || tile_cols == 64 || tile_cols == 32)) ||
           (tile_rows == 32 && tile_cols == 64);
}

// lanes per column vector of the 16-row kernels
static int ap_lpc(int tile_cols) { return tile_cols == 256 ? 2 : AP_LPC; }

size_t ap_smem_bytes(uint32_t wshift, int tile_rows, int tile_cols) {
    if (tile_rows == 32) return r32_smem_bytes(wshift);
    return (((size_t)1 << wshift) + 1) * D_STRIDE * sizeof(float) +
           ap_ring_bytes(tile_cols * ap_lpc(tile_cols));
}

int ap_max_wshift(int tile_rows, int tile_cols) {
    (void)tile_cols;
    return tile_rows == 32 ? 10 : 11;
}

int ap_threads(uint32_t wshift, int tile_rows, int tile_cols) {
    if (tile_rows == 32) return r32_wide(wshift) ? 512 : 256;
    return tile_cols * ap_lpc(tile_cols);
}

static const void *ap_kernel(uint32_t wshift, int tile_rows, int tile_cols) {
    if (tile_rows == 32)
        return r32_wide(wshift) ? (const void *)k_allpairs32<512, 1>
                                : (const void *)k_allpairs32<256, 2>;
    if (tile_cols == 256) return (const void *)k_allpairs<512, 1, 2>;
    if (tile_cols == 128) return (const void *)k_allpairs<512, 1, 4>;
    return tile_cols == 32 ? (const void *)k_allpairs<128, 4, 4> : (const void *)k_allpairs<256, 2, 4>;
}

cudaError_t ap_prepare(uint32_t wshift, int tile_rows, int tile_cols, int *ctas_per_sm) {
    const size_t smem = ap_smem_bytes(wshift, tile_rows, tile_cols);
    const void *fn = ap_kernel(wshift, tile_rows, tile_cols);
    PHYLO_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (ctas_per_sm) {
        int n = 0;
        PHYLO_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &n, fn, ap_threads(wshift, tile_rows, tile_cols), smem));
        *ctas_per_sm = n;
    }
    return cudaSuccess;
}

cudaError_t ap_launch(const ApArgs &a, int tile_rows, int tile_cols, int grid, cudaStream_t st) {
    const size_t smem = ap_smem_bytes(a.wshift, tile_rows, tile_cols);
    if (tile_rows == 32) {
        if (r32_wide(a.wshift))
            k_allpairs32<512, 1><<<grid, 512, smem, st>>>(a);
        else
            k_allpairs32<256, 2><<<grid, 256, smem, st>>>(a);
    } else if (tile_cols == 256) {
        k_allpairs<512, 1, 2><<<grid, 512, smem, st>>>(a);
    } else if (tile_cols == 128) {
        k_allpairs<512, 1, 4><<<grid, 512, smem, st>>>(a);
    } else if (tile_cols == 32) {
        k_allpairs<128, 4, 4><<<grid, 128, smem, st>>>(a);
    } else {
        k_allpairs<256, 2, 4><<<grid, 256, smem, st>>>(a);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// window index
// ---------------------------------------------------------------------------


// grid = (slices, N): CTA (s, v) handles entries [s*RI_SLICE, (s+1)*RI_SLICE) of
// vector v, each thread RI_RUN consecutive entries (16-byte loads; the entry before
// a run comes from the neighbouring lane).  Window r gets the index of the first
// entry whose key is >= r << wshift; the thread holding the last real entry fills
// the windows after it.
constexpr uint32_t RI_RUN = 16;
constexpr uint32_t RI_SLICE = 256 * RI_RUN;  // entries per CTA
__global__ void __launch_bounds__(256) k_range_index(const uint32_t *__restrict__ keys,
                                                     const uint64_t *__restrict__ vec_off,
                                                     uint32_t R, uint32_t wshift, uint32_t *roff) {
    const uint32_t v = blockIdx.y;
    const uint64_t b = vec_off[v];
    const uint32_t n = (uint32_t)(vec_off[v + 1] - b);  // padded length, a multiple of 4
    uint32_t *ro = roff + (uint64_t)v * (R + 1);
    const uint32_t e0 = blockIdx.x * RI_SLICE;
    if (e0 >= n) {
        if (n == 0 && blockIdx.x == 0)
            for (uint32_t r = threadIdx.x; r <= R; r += blockDim.x) ro[r] = 0;
        return;
    }
    const int lane = threadIdx.x & 31;
    const uint32_t s0 = e0 + threadIdx.x * RI_RUN;  // this thread's run
    uint32_t k[RI_RUN];
#pragma unroll
    for (int j = 0; j < (int)RI_RUN; j += 4) {
        uint4 q = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
        if (s0 + j < n) q = *reinterpret_cast<const uint4 *>(keys + b + s0 + j);
        k[j] = q.x; k[j + 1] = q.y; k[j + 2] = q.z; k[j + 3] = q.w;
    }
    // key before the run: the previous lane's last, or a load for lane 0
    uint32_t prev = __shfl_up_sync(0xffffffffu, k[RI_RUN - 1], 1);
    if (lane == 0) prev = s0 == 0 ? 0xffffffffu : (s0 <= n ? keys[b + s0 - 1] : 0xffffffffu);
    // window of the entry before the run (-1 before the first entry)
    int64_t rp = (s0 == 0 || prev == 0xffffffffu) ? -1 : (int64_t)min(prev >> wshift, R);
    if (s0 < n) {
#pragma unroll
        for (int j = 0; j < (int)RI_RUN; j++) {
            const uint32_t e = s0 + j;
            const uint32_t key = k[j];
            if (e >= n || key == 0xffffffffu) break;  // end or padding
            const uint32_t rt = min(key >> wshift, R);
            for (int64_t r = rp + 1; r <= (int64_t)rt; r++) ro[r] = e;
            rp = rt;
            // last real entry: the next key is padding or the end
            const uint32_t nk = j + 1 < (int)RI_RUN ? k[j + 1]
                                : (e + 1 < n ? keys[b + e + 1] : 0xffffffffu);
            if (e + 1 == n || nk == 0xffffffffu)
                for (uint32_t r = rt + 1; r <= R; r++) ro[r] = e + 1;
        }
    }
    // a vector made only of padding
    if (blockIdx.x == 0 && keys[b] == 0xffffffffu)
        for (uint32_t r = threadIdx.x; r <= R; r += blockDim.x) ro[r] = 0;
}

cudaError_t range_index_launch(const uint32_t *keys, const uint64_t *vec_off, uint32_t N,
                               uint32_t R, uint32_t wshift, uint32_t *roff, cudaStream_t st,
                               uint64_t max_len) {
    if (N == 0) return cudaSuccess;
    const uint32_t slices = (uint32_t)div_up(max_len ? max_len : 1, RI_SLICE);
    k_range_index<<<dim3(slices, N), 256, 0, st>>>(keys, vec_off, R, wshift, roff);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// reduction of partial blocks
// ---------------------------------------------------------------------------

// grid = (ntiles, tile rows), block = tile columns: one (row, column) pair per
// thread, its S partials summed in segment order (double-double), so the result
// does not depend on how the items were scheduled.
__global__ void k_ap_reduce(ApReduceArgs r) {
    const ApTile t = r.tiles[blockIdx.x];
    const uint32_t c = threadIdx.x, i = blockIdx.y;
    if (c >= t.ncol || i >= t.nrow) return;
    const uint32_t rowpos = t.row0 + i, colpos = t.col0 + c;
    if (r.upper == 1 && !(rowpos < colpos)) return;
    if (r.upper == 2 && !(rowpos <= colpos)) return;  // with the diagonal
    const uint64_t blk = (uint64_t)r.ti * r.tj;  // float pairs per partial block
    const FF *base = r.part + (uint64_t)blockIdx.x * r.S * blk + i * r.tj + c;
    DD acc = {0.0, 0.0};
    for (uint32_t s = 0; s < r.S; s++) {
        const FF p = base[(uint64_t)s * blk];
        dd_add(acc, (double)p.hi);
        dd_add(acc, (double)p.lo);
    }
    const double v = __dadd_rn(acc.hi, acc.lo);
    const uint32_t rowid = r.rowids[rowpos], colid = r.colids[colpos];
    r.out[(uint64_t)rowid * r.ldc + colid] = v;
    if (r.mirror) r.out[(uint64_t)colid * r.ldc + rowid] = v;
}

cudaError_t ap_reduce_launch(const ApReduceArgs &r, cudaStream_t st) {
    if (r.ntiles == 0) return cudaSuccess;
    k_ap_reduce<<<dim3(r.ntiles, r.ti), r.tj, 0, st>>>(r);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// self products (the diagonal of the reference's run, Main.java:196)
// ---------------------------------------------------------------------------

constexpr uint32_t SD_SLICE = 65536;  // entries per CTA

// grid = (slices, N): float-float sum of squares of one slice -> part[v * slices + s]
__global__ void k_self_dot(const float *__restrict__ vals, const uint64_t *__restrict__ vec_off,
                           uint32_t slices, FF *part) {
    const uint32_t v = blockIdx.y;
    const uint64_t b = vec_off[v], n = vec_off[v + 1] - b;
    const uint64_t e0 = (uint64_t)blockIdx.x * SD_SLICE, e1 = min(n, e0 + SD_SLICE);
    FF acc = {0.0f, 0.0f};
    for (uint64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
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
        FF t = {0.0f, 0.0f};
        for (int w = 0; w < (int)(blockDim.x / 32); w++) t = ff_merge(t, ws[w]);
        part[(uint64_t)v * slices + blockIdx.x] = t;
    }
}

__global__ void k_self_dot_final(const FF *part, uint32_t slices, uint32_t N, double *out,
                                 uint64_t ldc) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= N) return;
    DD d = {0.0, 0.0};
    for (uint32_t s = 0; s < slices; s++) {
        const FF f = part[(uint64_t)v * slices + s];
        dd_add(d, (double)f.hi);
        dd_add(d, (double)f.lo);
    }
    out[(uint64_t)v * ldc + v] = __dadd_rn(d.hi, d.lo);
}

// part must hold N * slices float pairs, slices = ceil(max_len / SD_SLICE)
cudaError_t self_dot_launch(const float *vals, const uint64_t *vec_off, uint32_t N, double *out,
                            uint64_t ldc, uint64_t max_len, FF *part, cudaStream_t st) {
    if (N == 0) return cudaSuccess;
    const uint32_t slices = (uint32_t)div_up(max_len ? max_len : 1, SD_SLICE);
    k_self_dot<<<dim3(slices, N), 256, 0, st>>>(vals, vec_off, slices, part);
    k_self_dot_final<<<(N + 127) / 128, 128, 0, st>>>(part, slices, N, out, ldc);
    return cudaGetLastError();
}

uint64_t self_dot_part_count(uint32_t N, uint64_t max_len) {
    return (uint64_t)N * div_up(max_len ? max_len : 1, SD_SLICE);
}

}  // namespace phylo
