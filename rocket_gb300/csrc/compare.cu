// compare.cu -- sparse cosine of one pair (and of many pairs) of composition vectors.
//
// C = sum over keys present in both lists of a * b, the quantity the reference
// computes with a merge-path partition and one merge step per thread
// (phylogenetics/src/main/cpp/native.cu:513-703).  This version is one launch:
//
//   * k_compare: persistent CTAs take contiguous runs of tiles of 4096 merged
//     elements.  Each CTA first finds the merge-path splits of its own tile
//     boundaries, one warp per boundary by a 32-ary search (about five dependent
//     global loads instead of twenty), ties going to the left list as in
//     native.cu:529.  Then, for each tile, a single thread issues 1-D bulk copies
//     (TMA) of the left and right key/value ranges into shared memory,
//     double-buffered on mbarriers; all threads run a per-thread merge path over
//     16 diagonals in shared memory.  Products are split exactly (TwoProduct) and
//     summed as float-float (TwoSum); warp shuffles and one shared-memory step
//     reduce the CTA, and the last CTA combines the per-CTA partials in a fixed
//     order into the double result.
//   * k_many_intersect does the same over the tiles of many pairs in one index
//     space; each CTA resolves its tiles' pairs, vector offsets and splits up
//     front, so issuing a tile's copies reads only shared memory.
//
// Ranges need not be 16-byte aligned: each copy is widened to 16-byte
// boundaries (never leaving the 16-byte block of a valid element) and the
// consumer indexes from the offset.
#include "compare.cuh"
#include "hostctx.cuh"
#include "scan.cuh"

namespace phylo {

constexpr int CMP_THREADS = 256;
constexpr int CMP_IPT = 16;
constexpr int CMP_TILE = CMP_THREADS * CMP_IPT;  // merged elements per tile
constexpr int CMP_BUF = CMP_TILE + 20;           // entries per stage per type (A + B + look-ahead)
constexpr uint32_t CMP_MAX_RUN = 64;             // tiles per CTA at most
constexpr uint32_t CMP_MIN_CAP = 1024;           // partial slots always carved

// Completion ticket and status first (cleared before every launch), then one
// float-float partial per CTA.
struct CmpState {
    uint32_t ticket;
    uint32_t status;
    uint32_t pad[2];
    FF partial[1];  // [cmp_partials(ntiles)]
};

__host__ __device__ constexpr uint64_t cmp_partials(uint64_t ntiles) {
    return (ntiles + CMP_MAX_RUN - 1) / CMP_MAX_RUN > CMP_MIN_CAP
               ? (ntiles + CMP_MAX_RUN - 1) / CMP_MAX_RUN
               : CMP_MIN_CAP;
}

__host__ __device__ constexpr size_t cmp_state_bytes(uint64_t max_total) {
    return (16 + 8 * cmp_partials((max_total + CMP_TILE - 1) / CMP_TILE) + 255) / 256 * 256;
}

size_t compare_scratch_bytes(uint64_t max_total) { return cmp_state_bytes(max_total); }

// i = number of left elements before merged position d (ties to the left list).
__device__ __forceinline__ uint32_t warp_merge_path(uint64_t d, const uint32_t *__restrict__ A,
                                                    uint32_t na, const uint32_t *__restrict__ B,
                                                    uint32_t nb) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t lo = d > nb ? (uint32_t)(d - nb) : 0u;
    uint32_t hi = d < na ? (uint32_t)d : na;
    while (hi > lo) {
        const uint32_t span = hi - lo;
        const uint32_t step = (span + 31) / 32;
        const uint64_t i = (uint64_t)lo + (uint64_t)(lane + 1) * step;
        bool p = false;
        if (i <= hi) p = __ldg(&A[i - 1]) <= __ldg(&B[d - i]);
        const uint32_t cnt = __popc(__ballot_sync(0xffffffffu, p));
        const uint64_t nlo = (uint64_t)lo + (uint64_t)cnt * step;
        const uint64_t nhi = (uint64_t)lo + (uint64_t)(cnt + 1) * step - 1;
        lo = (uint32_t)nlo;
        hi = nhi < hi ? (uint32_t)nhi : hi;
    }
    return lo;
}

struct Stage {
    uint32_t ka_off, va_off, kb_off, vb_off;  // element offsets of the first wanted entry
    uint32_t na, nb;
    uint32_t nbx;  // nb plus one look-ahead right element when the right list continues
};

// Issues the bulk copies of left [i0, i1) and right [j0, j1x) (j1x = j1 or
// j1 + 1 with the look-ahead element) into one stage buffer; returns the layout.
__device__ __forceinline__ Stage issue_ranges(const uint32_t *Ak, const float *Av, uint32_t i0,
                                              uint32_t i1, const uint32_t *Bk, const float *Bv,
                                              uint32_t j0, uint32_t j1, uint32_t j1x, uint32_t *sk,
                                              float *sv, uint64_t *bar, bool issue) {
    Stage s;
    s.na = i1 - i0;
    s.nb = j1 - j0;
    s.nbx = j1x - j0;
    // widened byte ranges
    const uintptr_t ka0 = (uintptr_t)(Ak + i0), ka1 = (uintptr_t)(Ak + i1);
    const uintptr_t va0 = (uintptr_t)(Av + i0), va1 = (uintptr_t)(Av + i1);
    const uintptr_t kb0 = (uintptr_t)(Bk + j0), kb1 = (uintptr_t)(Bk + j1x);
    const uintptr_t vb0 = (uintptr_t)(Bv + j0), vb1 = (uintptr_t)(Bv + j1x);
    auto lo16 = [](uintptr_t x) { return x & ~(uintptr_t)15; };
    auto hi16 = [](uintptr_t x) { return (x + 15) & ~(uintptr_t)15; };
    const uint32_t bka = s.na ? (uint32_t)(hi16(ka1) - lo16(ka0)) : 0u;
    const uint32_t bva = s.na ? (uint32_t)(hi16(va1) - lo16(va0)) : 0u;
    const uint32_t bkb = s.nbx ? (uint32_t)(hi16(kb1) - lo16(kb0)) : 0u;
    const uint32_t bvb = s.nbx ? (uint32_t)(hi16(vb1) - lo16(vb0)) : 0u;
    // B part starts after the A part (both multiples of 16 bytes)
    s.ka_off = (uint32_t)((ka0 & 15) >> 2);
    s.va_off = (uint32_t)((va0 & 15) >> 2);
    s.kb_off = bka / 4 + (uint32_t)((kb0 & 15) >> 2);
    s.vb_off = bva / 4 + (uint32_t)((vb0 & 15) >> 2);
    if (issue) {
        mbar_arrive_expect_tx(bar, bka + bva + bkb + bvb);
        if (bka) bulk_g2s(sk, (const void *)lo16(ka0), bka, bar);
        if (bva) bulk_g2s(sv, (const void *)lo16(va0), bva, bar);
        if (bkb) bulk_g2s(sk + bka / 4, (const void *)lo16(kb0), bkb, bar);
        if (bvb) bulk_g2s(sv + bva / 4, (const void *)lo16(vb0), bvb, bar);
    }
    return s;
}

// Issues the bulk copies of tile `t` of one pair into a stage buffer; split[]
// holds the left split of tiles t_begin .. t_end (shared memory).
__device__ __forceinline__ Stage issue_tile(uint32_t t, uint32_t t_begin, const uint32_t *split,
                                            uint64_t total, uint32_t nb_total, const uint32_t *Ak,
                                            const float *Av, const uint32_t *Bk, const float *Bv,
                                            uint32_t *sk, float *sv, uint64_t *bar, bool issue) {
    const uint64_t d0 = (uint64_t)t * CMP_TILE;
    const uint64_t d1 = min(d0 + CMP_TILE, total);
    const uint32_t i0 = split[t - t_begin], i1 = split[t - t_begin + 1];
    const uint32_t j0 = (uint32_t)(d0 - i0), j1 = (uint32_t)(d1 - i1);
    // A match whose left element ends this tile can have its equal right element
    // start the next one (ties go left), so one right element past the tile is
    // copied as look-ahead.
    const uint32_t j1x = j1 < nb_total ? j1 + 1 : j1;
    return issue_ranges(Ak, Av, i0, i1, Bk, Bv, j0, j1, j1x, sk, sv, bar, issue);
}

// Per-thread merge path over 16 diagonals of a staged tile; adds the exact
// products of matching keys to acc.
__device__ __forceinline__ void merge_tile(const Stage &s, const uint32_t *skb, const float *svb,
                                           FF &acc) {
    const uint32_t *ka = skb + s.ka_off;
    const float *va = svb + s.va_off;
    const uint32_t *kb = skb + s.kb_off;
    const float *vb = svb + s.vb_off;
    const uint32_t d = threadIdx.x * CMP_IPT;
    const uint32_t n = s.na + s.nb;
    if (d >= n) return;
    uint32_t lo = d > s.nb ? d - s.nb : 0u;
    uint32_t hi = d < s.na ? d : s.na;
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2 + 1;
        if (ka[mid - 1] <= kb[d - mid]) lo = mid; else hi = mid - 1;
    }
    uint32_t i = lo, j = d - lo;
    const uint32_t steps = min((uint32_t)CMP_IPT, n - d);
    for (uint32_t it = 0; it < steps; it++) {
        const bool has_a = i < s.na, has_b = j < s.nb, has_bx = j < s.nbx;
        const uint32_t x = has_a ? ka[i] : 0u, y = has_bx ? kb[j] : 0u;
        const bool take_a = has_a && (!has_b || x <= y);
        if (take_a && has_bx && x == y) {
            float p, e;
            two_prod(va[i], vb[j], p, e);
            ff_add(acc, p);
            acc.lo = __fadd_rn(acc.lo, e);
        }
        i += take_a;
        j += !take_a;
    }
}

__global__ void __launch_bounds__(CMP_THREADS) k_compare(
    const uint32_t *__restrict__ Ak, const float *__restrict__ Av, uint32_t na,
    const uint32_t *__restrict__ Bk, const float *__restrict__ Bv, uint32_t nb, uint32_t ntiles,
    uint32_t per, uint32_t first_wait_limit, CmpState *st, double *out) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    uint32_t *sk[2];
    float *sv[2];
    sk[0] = (uint32_t *)smem_raw;
    sv[0] = (float *)(sk[0] + CMP_BUF);
    sk[1] = (uint32_t *)(sv[0] + CMP_BUF);
    sv[1] = (float *)(sk[1] + CMP_BUF);
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ FF warp_part[CMP_THREADS / 32];
    __shared__ uint32_t s_split[CMP_MAX_RUN + 1];
    __shared__ bool s_last;
    __shared__ bool s_fail;

    const uint64_t total = (uint64_t)na + nb;
    const uint32_t t_begin = blockIdx.x * per;
    const uint32_t t_end = min(ntiles, t_begin + per);

    // merge-path splits of this CTA's tile boundaries t_begin .. t_end, a warp each
    const uint32_t warp = threadIdx.x >> 5;
    for (uint32_t b = warp; t_begin < t_end && b <= t_end - t_begin; b += CMP_THREADS / 32) {
        uint64_t d = (uint64_t)(t_begin + b) * CMP_TILE;
        if (d > total) d = total;
        const uint32_t i = warp_merge_path(d, Ak, na, Bk, nb);
        if ((threadIdx.x & 31) == 0) s_split[b] = i;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        s_fail = false;
    }
    __syncthreads();

    FF acc = {0.0f, 0.0f};
    Stage stg0 = {0, 0, 0, 0, 0, 0, 0}, stg1 = {0, 0, 0, 0, 0, 0, 0};
    // prologue: tiles t_begin, t_begin+1
    if (t_begin < t_end)
        stg0 = issue_tile(t_begin, t_begin, s_split, total, nb, Ak, Av, Bk, Bv, sk[0], sv[0],
                          &bar[0], threadIdx.x == 0);
    if (t_begin + 1 < t_end)
        stg1 = issue_tile(t_begin + 1, t_begin, s_split, total, nb, Ak, Av, Bk, Bv, sk[1], sv[1],
                          &bar[1], threadIdx.x == 0);
    uint32_t fail_at = 0xffffffffu;
    for (uint32_t t = t_begin; t < t_end; t++) {
        const int b = (t - t_begin) & 1;
        const uint32_t phase = ((t - t_begin) >> 1) & 1;
        const uint32_t limit = t == t_begin ? first_wait_limit : (1u << 22);
        if (!mbar_wait_bounded(&bar[b], phase, limit)) s_fail = true;
        __syncthreads();
        if (s_fail) {
            fail_at = t;
            break;
        }
        const Stage s = b ? stg1 : stg0;
        uint32_t *skb = b ? sk[1] : sk[0];
        float *svb = b ? sv[1] : sv[0];
        merge_tile(s, skb, svb, acc);
        __syncthreads();  // everyone done with buffer b
        const uint32_t tn = t + 2;
        if (tn < t_end) {
            if (threadIdx.x == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const Stage ns = issue_tile(tn, t_begin, s_split, total, nb, Ak, Av, Bk, Bv, skb, svb,
                                        &bar[b], threadIdx.x == 0);
            if (b) stg1 = ns; else stg0 = ns;
        }
    }
    if (fail_at != 0xffffffffu) {
        // record the failure, then wait (bounded) for the copies that may still
        // be in flight: the failed tile and the one issued after it
        if (threadIdx.x == 0) atomicOr(&st->status, (uint32_t)DEV_WAIT_TIMEOUT);
        for (uint32_t t = fail_at; t < t_end && t < fail_at + 2; t++) {
            const uint32_t rel = t - t_begin;
            (void)mbar_wait_bounded(&bar[rel & 1], (rel >> 1) & 1, 1u << 16);
        }
        __syncthreads();
    }
    // CTA reduction
    acc = ff_warp_sum(acc);
    if ((threadIdx.x & 31) == 0) warp_part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        FF r = {0.0f, 0.0f};
        for (int w = 0; w < CMP_THREADS / 32; w++) r = ff_merge(r, warp_part[w]);
        st->partial[blockIdx.x] = r;
        __threadfence();
        const uint32_t done = atomicAdd(&st->ticket, 1u);
        s_last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last && threadIdx.x < 32) {
        __threadfence();
        // fixed order: lane l sums partials l, l+32, ... in double-double
        DD dacc = {0.0, 0.0};
        for (uint32_t c = threadIdx.x; c < gridDim.x; c += 32) {
            const volatile float *pp = reinterpret_cast<volatile float *>(&st->partial[c]);
            dd_add(dacc, (double)pp[0]);
            dd_add(dacc, (double)pp[1]);
        }
#pragma unroll
        for (int dd = 16; dd > 0; dd >>= 1) {
            DD o;
            o.hi = __shfl_down_sync(0xffffffffu, dacc.hi, dd);
            o.lo = __shfl_down_sync(0xffffffffu, dacc.lo, dd);
            dacc = dd_merge(dacc, o);
        }
        if (threadIdx.x == 0) *out = __dadd_rn(dacc.hi, dacc.lo);
    }
}

static const size_t kCmpSmem = sizeof(uint32_t) * CMP_BUF * 4;

// Poll limit of each CTA's first wait (a test hook: 0 makes every CTA give up
// at once, after its copies were issued, so the timeout path can be exercised
// without a fault).
static std::atomic<uint32_t> g_first_wait_limit{1u << 22};

void compare_set_first_wait_limit(uint32_t limit) {
    g_first_wait_limit.store(limit == 0xffffffffu ? (1u << 22) : limit);
}

// The kernel's dynamic shared memory limit, set once per context.
static cudaError_t compare_attributes() {
    static PerContext<int> done;
    int v = 0;
    return done.get(&v, [](int *out) -> cudaError_t {
        PHYLO_CHECK(cudaFuncSetAttribute(k_compare, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kCmpSmem));
        *out = 1;
        return cudaSuccess;
    });
}

cudaError_t compare_launch(cudaStream_t stream, void *scratch, size_t scratch_size,
                           const uint32_t *lk, const float *lv, uint32_t nl, const uint32_t *rk,
                           const float *rv, uint32_t nr, double *d_out, uint32_t **status_out) {
    const uint64_t total = (uint64_t)nl + nr;
    const uint32_t ntiles = (uint32_t)div_up(total, CMP_TILE);
    if (scratch_size < cmp_state_bytes(total) || scratch == nullptr) {
        fprintf(stderr,
                "phylogenetics: scratch of %zu bytes too small to compare vectors of sizes %u and "
                "%u\n",
                scratch_size, nl, nr);
        return cudaErrorInvalidValue;
    }
    CmpState *st = (CmpState *)scratch;
    if (status_out) *status_out = &st->status;
    PHYLO_CHECK(cudaMemsetAsync(st, 0, 16, stream));  // ticket and status
    if (ntiles == 0) {
        // empty: C = 0
        PHYLO_CHECK(cudaMemsetAsync(d_out, 0, sizeof(double), stream));
        return cudaSuccess;
    }
    PHYLO_CHECK(compare_attributes());
    // about three CTAs per SM, at most CMP_MAX_RUN tiles each
    const uint32_t sms = (uint32_t)device_sm_count();
    uint32_t grid = min(ntiles, min(3u * sms, CMP_MIN_CAP));
    uint32_t per = (uint32_t)div_up(ntiles, grid);
    if (per > CMP_MAX_RUN) per = CMP_MAX_RUN;
    grid = (uint32_t)div_up(ntiles, per);
    k_compare<<<grid, CMP_THREADS, kCmpSmem, stream>>>(lk, lv, nl, rk, rv, nr, ntiles, per,
                                                       g_first_wait_limit.load(), st, d_out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Compare without caller-provided scratch.
//
// Some callers cannot call cudaMalloc at all: a host runtime that carved all of
// the device memory into fixed cache slots when it started (as Rocket's device
// cache does) and has nothing left to hand out for scratch, or a caller whose
// device memory belongs to another framework's allocator and must not be taken
// behind its back.  For them the pair kernels can also run on a scratch area
// that is part of this library's image: one file-scope device array of fixed
// size, loaded with the module on every GPU that uses the library and kept
// there until the process exits.
//
// Limit: the two vectors may hold at most kStaticCompareMaxEntries entries
// together (2^26 = 67,108,864), which needs kStaticCompareBytes of scratch.
// All calls share the one array and it keeps what the last call left in it;
// the partition kernel clears the completion ticket and the status word at the
// start of every call, and every other byte a call reads it wrote first.  Two
// calls whose kernels overlap on the GPU (different streams, or different host
// threads) would race on the array, so such calls must be serialised.
// ---------------------------------------------------------------------------

constexpr uint64_t kStaticCompareMaxEntries = 1ull << 26;
constexpr size_t kStaticCompareBytes = cmp_state_bytes(kStaticCompareMaxEntries);
static_assert(kStaticCompareBytes >= cmp_state_bytes(kStaticCompareMaxEntries) &&
                  cmp_partials((kStaticCompareMaxEntries + CMP_TILE - 1) / CMP_TILE) >= CMP_MIN_CAP,
              "the built-in scratch holds the state compare_launch carves at its maximum size");

static __device__ __align__(256) unsigned char g_static_compare_scratch[kStaticCompareBytes];

uint64_t compare_static_max_entries() { return kStaticCompareMaxEntries; }
size_t compare_static_bytes() { return kStaticCompareBytes; }

// The host name of the array is only a stand-in; the device address comes from
// cudaGetSymbolAddress, looked up once per context (a device symbol has its own
// address in every context that loads the module) with that context current.
static cudaError_t static_scratch_address(void **ptr) {
    static PerContext<void *> addr;
    return addr.get(ptr, [](void **out) -> cudaError_t {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_compare_scratch);
        if (e != cudaSuccess) {
            fprintf(stderr, "phylogenetics: cudaGetSymbolAddress of the static scratch failed: %s\n",
                    cudaGetErrorString(e));
            return e;
        }
        *out = p;
        return cudaSuccess;
    });
}

cudaError_t compare_launch_static(cudaStream_t stream, const uint32_t *lk, const float *lv,
                                  uint32_t nl, const uint32_t *rk, const float *rv, uint32_t nr,
                                  double *d_out, uint32_t **status_out) {
    if ((uint64_t)nl + nr > kStaticCompareMaxEntries) {
        fprintf(stderr,
                "error: vectors of %u and %u entries exceed the %llu entries the built-in scratch "
                "of compareCompositionVectorsStatic holds; use compareCompositionVectors with "
                "caller scratch\n",
                nl, nr, (unsigned long long)kStaticCompareMaxEntries);
        return cudaErrorInvalidValue;
    }
    void *scratch = nullptr;
    PHYLO_CHECK(static_scratch_address(&scratch));
    return compare_launch(stream, scratch, kStaticCompareBytes, lk, lv, nl, rk, rv, nr, d_out,
                          status_out);
}

// ---------------------------------------------------------------------------
// Many pairs per launch.  Tiles of all pairs form one index space (pair p owns
// tiles [tile_off[p], tile_off[p+1])).  Persistent CTAs take contiguous runs of
// at most CMP_MAX_RUN tiles; each CTA first resolves, a warp per tile boundary,
// the boundary's pair, the pair's vectors and the merge-path split, so the
// double-buffered bulk copies are issued from shared memory alone.  Every tile
// leaves one float-float partial, and k_many_reduce sums each pair's tiles in
// order.
// ---------------------------------------------------------------------------

struct ManyArgs {
    const uint32_t *lkeys; const float *lvals; const uint64_t *loff; const uint32_t *lnnz;
    const uint32_t *rkeys; const float *rvals; const uint64_t *roff; const uint32_t *rnnz;
    const uint32_t *pa, *pb;   // pair p = (left vector pa[p], right vector pb[p])
    uint32_t P;
    uint32_t *ptiles;          // [P] tiles per pair
    uint64_t *tile_off;        // [P+1]
    uint64_t *scan_tmp;
    FF *tile_part;             // [max_tiles]
    uint64_t max_tiles;
    uint32_t per;              // tiles per CTA
    double *out;               // [P]
    uint32_t *status;
};

// Largest p with off[p] <= t (off[0] = 0, off nondecreasing), a warp together:
// each round splits the range into 32 parts with one load per lane.
__device__ __forceinline__ uint32_t warp_owner_of(const uint64_t *off, uint32_t n, uint64_t t) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t lo = 0, hi = n;  // answer in [lo, hi)
    while (hi - lo > 1) {
        const uint32_t span = hi - lo;
        const uint32_t step = (span + 31) / 32;
        const uint32_t i = lo + (lane + 1) * step;  // probe off[i]
        const bool p = i < hi && __ldg(&off[i]) <= t;
        const uint32_t cnt = __popc(__ballot_sync(0xffffffffu, p));
        const uint32_t nlo = lo + cnt * step;
        const uint32_t nhi = lo + (cnt + 1) * step;
        lo = nlo;
        hi = nhi < hi ? nhi : hi;
    }
    return lo;
}

__global__ void k_many_tiles(ManyArgs a) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    const uint64_t tot = (uint64_t)a.lnnz[a.pa[p]] + a.rnnz[a.pb[p]];
    a.ptiles[p] = (uint32_t)div_up(tot, CMP_TILE);
}

// A tile boundary resolved: its pair, that pair's vectors, the merged position
// of the boundary within the pair and the left split there.
struct ManyBound {
    uint64_t lbase, rbase;   // arena offsets of the two vectors
    uint64_t d;              // merged position of the boundary within its pair
    uint32_t p, na, nb, i;   // pair (P: past the last tile), sizes, left split
};

__device__ __forceinline__ Stage many_issue(const ManyArgs &a, const ManyBound *bd, uint32_t rel,
                                            uint32_t *sk, float *sv, uint64_t *bar, bool issue) {
    const ManyBound &b0 = bd[rel];
    const ManyBound &b1 = bd[rel + 1];
    const bool same = b1.p == b0.p;  // the next boundary lies inside this tile's pair
    const uint32_t i0 = b0.i;
    const uint32_t i1 = same ? b1.i : b0.na;
    const uint64_t d1 = same ? b1.d : (uint64_t)b0.na + b0.nb;
    const uint32_t j0 = (uint32_t)(b0.d - i0), j1 = (uint32_t)(d1 - i1);
    const uint32_t j1x = j1 < b0.nb ? j1 + 1 : j1;
    return issue_ranges(a.lkeys + b0.lbase, a.lvals + b0.lbase, i0, i1, a.rkeys + b0.rbase,
                        a.rvals + b0.rbase, j0, j1, j1x, sk, sv, bar, issue);
}

__global__ void __launch_bounds__(CMP_THREADS) k_many_intersect(ManyArgs a) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    uint32_t *sk[2];
    float *sv[2];
    sk[0] = (uint32_t *)smem_raw;
    sv[0] = (float *)(sk[0] + CMP_BUF);
    sk[1] = (uint32_t *)(sv[0] + CMP_BUF);
    sv[1] = (float *)(sk[1] + CMP_BUF);
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ FF warp_part[CMP_THREADS / 32];
    __shared__ ManyBound s_bd[CMP_MAX_RUN + 1];
    __shared__ bool s_fail;
    uint64_t T = a.tile_off[a.P];
    if (blockIdx.x == 0 && threadIdx.x == 0 && T > a.max_tiles)
        atomicOr(a.status, (uint32_t)DEV_CAPACITY);
    if (T > a.max_tiles) T = a.max_tiles;
    const uint64_t t_begin = (uint64_t)blockIdx.x * a.per;
    const uint64_t t_end = min(T, t_begin + a.per);
    if (t_begin >= t_end) return;  // the same for every thread of the CTA
    // resolve the run's boundaries t_begin .. t_end, a warp each
    const uint32_t nbd = (uint32_t)(t_end - t_begin) + 1;
    const uint32_t warp = threadIdx.x >> 5;
    for (uint32_t b = warp; b < nbd; b += CMP_THREADS / 32) {
        const uint64_t t = t_begin + b;
        ManyBound m = {0, 0, 0, a.P, 0, 0, 0};
        if (t < T) {
            m.p = warp_owner_of(a.tile_off, a.P, t);
            const uint32_t va = a.pa[m.p], vb = a.pb[m.p];
            m.na = a.lnnz[va];
            m.nb = a.rnnz[vb];
            m.lbase = a.loff[va];
            m.rbase = a.roff[vb];
            m.d = (t - a.tile_off[m.p]) * CMP_TILE;
            m.i = warp_merge_path(m.d, a.lkeys + m.lbase, m.na, a.rkeys + m.rbase, m.nb);
        }
        if ((threadIdx.x & 31) == 0) s_bd[b] = m;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        s_fail = false;
    }
    __syncthreads();
    Stage stg0 = {0, 0, 0, 0, 0, 0, 0}, stg1 = {0, 0, 0, 0, 0, 0, 0};
    stg0 = many_issue(a, s_bd, 0, sk[0], sv[0], &bar[0], threadIdx.x == 0);
    if (t_begin + 1 < t_end) stg1 = many_issue(a, s_bd, 1, sk[1], sv[1], &bar[1], threadIdx.x == 0);
    uint64_t fail_at = ~0ull;
    for (uint64_t t = t_begin; t < t_end; t++) {
        const uint32_t rel = (uint32_t)(t - t_begin);
        const int b = (int)(rel & 1);
        const uint32_t phase = (rel >> 1) & 1;
        if (!mbar_wait_bounded(&bar[b], phase)) s_fail = true;
        __syncthreads();
        if (s_fail) {
            fail_at = t;
            break;
        }
        FF acc = {0.0f, 0.0f};
        merge_tile(b ? stg1 : stg0, b ? sk[1] : sk[0], b ? sv[1] : sv[0], acc);
        acc = ff_warp_sum(acc);
        if ((threadIdx.x & 31) == 0) warp_part[threadIdx.x >> 5] = acc;
        __syncthreads();  // buffer b consumed, warp partials written
        if (threadIdx.x == 0) {
            FF r = {0.0f, 0.0f};
            for (int w = 0; w < CMP_THREADS / 32; w++) r = ff_merge(r, warp_part[w]);
            a.tile_part[t] = r;
        }
        if (rel + 2 < (uint32_t)(t_end - t_begin)) {
            if (threadIdx.x == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const Stage ns = many_issue(a, s_bd, rel + 2, b ? sk[1] : sk[0], b ? sv[1] : sv[0],
                                        &bar[b], threadIdx.x == 0);
            if (b) stg1 = ns; else stg0 = ns;
        }
        __syncthreads();  // warp_part reused next tile
    }
    if (fail_at != ~0ull) {
        if (threadIdx.x == 0) atomicOr(a.status, (uint32_t)DEV_WAIT_TIMEOUT);
        for (uint64_t t = fail_at; t < t_end && t < fail_at + 2; t++) {
            const uint64_t rel = t - t_begin;
            (void)mbar_wait_bounded(&bar[rel & 1], (uint32_t)((rel >> 1) & 1), 1u << 16);
        }
    }
}

// one warp per pair: its tiles' partials in tile order (each lane a fixed
// strided subset, then a fixed shuffle tree), double-double
__global__ void k_many_reduce(ManyArgs a) {
    const uint32_t p = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (p >= a.P) return;
    const int lane = threadIdx.x & 31;
    const uint64_t t0 = a.tile_off[p], t1 = a.tile_off[p + 1];
    DD acc = {0.0, 0.0};
    for (uint64_t t = t0 + lane; t < t1 && t < a.max_tiles; t += 32) {
        dd_add(acc, (double)a.tile_part[t].hi);
        dd_add(acc, (double)a.tile_part[t].lo);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        DD o;
        o.hi = __shfl_down_sync(0xffffffffu, acc.hi, d);
        o.lo = __shfl_down_sync(0xffffffffu, acc.lo, d);
        acc = dd_merge(acc, o);
    }
    if (lane == 0) a.out[p] = __dadd_rn(acc.hi, acc.lo);
}

size_t compare_many_scratch_bytes(uint32_t P, uint64_t max_tiles) {
    return scratch_bytes<uint32_t>(P) + scratch_bytes<uint64_t>((uint64_t)P + 1) +
           scan_temp_bytes((uint64_t)P + 1) + scratch_bytes<FF>(max_tiles ? max_tiles : 1) +
           scratch_bytes<uint32_t>(4);
}

static cudaError_t many_attributes() {
    static PerContext<int> done;
    int v = 0;
    return done.get(&v, [](int *out) -> cudaError_t {
        PHYLO_CHECK(cudaFuncSetAttribute(k_many_intersect,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kCmpSmem));
        *out = 1;
        return cudaSuccess;
    });
}

cudaError_t compare_many_launch(cudaStream_t st, void *scratch, size_t scratch_size,
                                const uint32_t *lkeys, const float *lvals, const uint64_t *loff,
                                const uint32_t *lnnz, const uint32_t *rkeys, const float *rvals,
                                const uint64_t *roff, const uint32_t *rnnz, const uint32_t *pa,
                                const uint32_t *pb, uint32_t P, uint64_t max_tiles, double *out,
                                uint32_t **status_out) {
    if (P == 0) return cudaSuccess;
    Scratch sc(scratch, scratch_size);
    ManyArgs a;
    a.lkeys = lkeys; a.lvals = lvals; a.loff = loff; a.lnnz = lnnz;
    a.rkeys = rkeys; a.rvals = rvals; a.roff = roff; a.rnnz = rnnz;
    a.pa = pa; a.pb = pb; a.P = P;
    a.ptiles = sc.take<uint32_t>(P);
    a.tile_off = sc.take<uint64_t>((uint64_t)P + 1);
    a.scan_tmp = sc.take<uint64_t>(scan_temp_bytes((uint64_t)P + 1) / 8);
    a.tile_part = sc.take<FF>(max_tiles ? max_tiles : 1);
    a.status = sc.take<uint32_t>(4);
    a.max_tiles = max_tiles;
    a.out = out;
    if (!a.status) return cudaErrorInvalidValue;
    if (status_out) *status_out = a.status;
    PHYLO_CHECK(many_attributes());
    PHYLO_CHECK(cudaMemsetAsync(a.status, 0, sizeof(uint32_t), st));
    k_many_tiles<<<(P + 255) / 256, 256, 0, st>>>(a);
    PHYLO_CHECK(scan_u32_to_u64(a.ptiles, P, a.tile_off, a.scan_tmp, st));
    const uint64_t sms = (uint64_t)device_sm_count();
    uint64_t per = div_up(max_tiles ? max_tiles : 1, 3 * sms);
    if (per > CMP_MAX_RUN) per = CMP_MAX_RUN;
    if (per < 1) per = 1;
    a.per = (uint32_t)per;
    const uint64_t grid = div_up(max_tiles ? max_tiles : 1, per);
    k_many_intersect<<<(unsigned)grid, CMP_THREADS, kCmpSmem, st>>>(a);
    k_many_reduce<<<(P + 7) / 8, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace phylo
