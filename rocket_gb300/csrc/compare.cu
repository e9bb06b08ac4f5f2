// compare.cu -- sparse cosine of one pair (and of many pairs) of composition vectors.
//
// C = sum over keys present in both lists of a * b, the quantity the reference
// computes with a merge-path partition and one merge step per thread
// (phylogenetics/src/main/cpp/native.cu:513-703).  Here the merged sequence of
// a pair is cut into tiles of 4352 elements at merge-path diagonals (ties to the
// left list, native.cu:529), and every CTA runs a warp-specialised pipeline over
// a contiguous run of tiles:
//
//   * one producer warp issues 1-D bulk copies (TMA) of each tile's left and
//     right key/value ranges into a ring of two shared-memory stages, each
//     completed on an mbarrier; the tiles' splits are known before it starts
//     (one pair: the CTA's warps find its few boundaries together; many pairs:
//     a kernel finds every boundary, a thread each);
//   * eight consumer warps merge a staged tile: a per-thread merge path over 17
//     diagonals, products split exactly (TwoProduct) and summed as float-float
//     (TwoSum); each warp releases the stage on the stage's "empty" mbarrier.
//
// Every split is found by a search that starts from the interpolated split
// d * na / (na + nb) and gallops out from it, so its probes read sectors near
// the answer (the ones the tile's copies read) rather than sectors scattered
// over both lists.
//
// k_compare (one pair, one launch) keeps a running sum per thread and combines
// the CTAs' partials in a fixed order in the last CTA; k_many_intersect (many
// pairs, tiles of all pairs in one index space) leaves one partial per tile,
// which k_many_reduce sums per pair in tile order.  Every wait is bounded; a
// timed-out wait records DEV_WAIT_TIMEOUT, the producer stops issuing and waits
// (bounded) for its copies in flight, and the CTA returns.
//
// Ranges need not be 16-byte aligned: each copy is widened to 16-byte
// boundaries (never leaving the 16-byte block of a valid element) and the
// consumer indexes from the offset.
#include "compare.cuh"
#include "hostctx.cuh"
#include "scan.cuh"

namespace phylo {

constexpr int CMP_CONSUMERS = 8;                          // merging warps
constexpr int CMP_CONSUMER_THREADS = CMP_CONSUMERS * 32;  // 256
constexpr int CMP_THREADS = CMP_CONSUMER_THREADS + 32;    // + one producer warp
constexpr int CMP_IPT = 17;  // odd: the lanes' merge runs start on different banks
constexpr int CMP_TILE = CMP_CONSUMER_THREADS * CMP_IPT;  // merged elements per tile
constexpr int CMP_BUF = CMP_TILE + 20;  // entries per stage per type (A + B + look-ahead)
constexpr int CMP_STAGES = 2;  // two stages: three CTAs (24 merging warps) per SM
constexpr uint32_t CMP_MAX_RUN = 64;    // tiles per CTA at most
constexpr uint32_t CMP_MIN_CAP = 1024;  // partial slots always carved
constexpr uint32_t CMP_WAIT = 1u << 22; // default poll limit of a wait
constexpr uint32_t CMP_DRAIN = 1u << 16;

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

// i = number of left elements before merged position d (ties to the left list),
// found by a warp.  The predicate "A[i-1] <= B[d-i]" holds for i up to the split
// and fails above it.  With step > 0 the first round probes 32 positions
// `step` apart around `guess`; when the split lies among them the remaining
// rounds stay inside one step.
__device__ __forceinline__ uint32_t warp_merge_path(uint64_t d, const uint32_t *__restrict__ A,
                                                    uint32_t na, const uint32_t *__restrict__ B,
                                                    uint32_t nb, uint64_t guess, uint32_t step) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t lo = d > nb ? (uint32_t)(d - nb) : 0u;
    uint32_t hi = d < na ? (uint32_t)d : na;
    if (step > 0 && hi - lo > 32u * step) {
        const int64_t first = (int64_t)guess - 16 * (int64_t)step;
        const int64_t i = first + (int64_t)(lane + 1) * step;
        bool p;
        if (i <= (int64_t)lo) p = true;
        else if (i > (int64_t)hi) p = false;
        else p = __ldg(&A[i - 1]) <= __ldg(&B[d - (uint64_t)i]);
        const uint32_t cnt = __popc(__ballot_sync(0xffffffffu, p));
        // split in [first + cnt * step, first + (cnt + 1) * step - 1], clipped to [lo, hi]
        const int64_t nlo = first + (int64_t)cnt * step;
        const int64_t nhi = first + (int64_t)(cnt + 1) * step - 1;
        if (cnt > 0 && nlo > (int64_t)lo) lo = (uint32_t)nlo;
        if (cnt < 32 && nhi < (int64_t)hi) hi = nhi < (int64_t)lo ? lo : (uint32_t)nhi;
    }
    while (hi > lo) {
        const uint32_t span = hi - lo;
        const uint32_t st = (span + 31) / 32;
        const uint64_t i = (uint64_t)lo + (uint64_t)(lane + 1) * st;
        bool p = false;
        if (i <= hi) p = __ldg(&A[i - 1]) <= __ldg(&B[d - i]);
        const uint32_t cnt = __popc(__ballot_sync(0xffffffffu, p));
        const uint64_t nlo = (uint64_t)lo + (uint64_t)cnt * st;
        const uint64_t nhi = (uint64_t)lo + (uint64_t)(cnt + 1) * st - 1;
        lo = (uint32_t)nlo;
        hi = nhi < hi ? (uint32_t)nhi : hi;
    }
    return lo;
}

// Expected left split at merged position d of a pair (keys spread alike).
__device__ __forceinline__ uint64_t split_guess(uint64_t d, uint32_t na, uint32_t nb) {
    const uint64_t n = (uint64_t)na + nb;
    return n ? d * na / n : 0;
}

struct Stage {
    uint32_t ka_off, va_off, kb_off, vb_off;  // element offsets of the first wanted entry
    uint32_t na, nb;
    uint32_t nbx;  // nb plus one look-ahead right element when the right list continues
};

// Layout of left [i0, i1) and right [j0, j1x) (j1x = j1, or j1 + 1 with the
// look-ahead element) in one stage buffer; with `issue`, also arms the stage's
// mbarrier and issues the bulk copies.
__device__ __forceinline__ Stage stage_ranges(const uint32_t *Ak, const float *Av, uint32_t i0,
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

// Per-thread merge path over CMP_IPT diagonals of a staged tile (consumer
// threads 0..255); adds the exact products of matching keys to acc.
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
    // Past either range a key reads as NOKEY, above every key of a list.  The
    // left list then always goes first against the right look-ahead element (the
    // merge path put every remaining left element at or below it), and no step
    // can find both ranges exhausted (each step consumes one of the thread's
    // elements).  The next key of each list is loaded before the comparison, so
    // the loads are off the step-to-step dependency chain.
    constexpr uint32_t NOKEY = 0xffffffffu;
    uint32_t i = lo, j = d - lo;
    const uint32_t steps = min((uint32_t)CMP_IPT, n - d);
    uint32_t x = i < s.na ? ka[i] : NOKEY, y = j < s.nbx ? kb[j] : NOKEY;
    for (uint32_t it = 0; it < steps; it++) {
        const uint32_t xn = i + 1 < s.na ? ka[i + 1] : NOKEY;
        const uint32_t yn = j + 1 < s.nbx ? kb[j + 1] : NOKEY;
        if (x == y && x != NOKEY) {
            float p, e;
            two_prod(va[i], vb[j], p, e);
            ff_add(acc, p);
            acc.lo = __fadd_rn(acc.lo, e);
        }
        if (x <= y) {  // ties go to the left list
            i++;
            x = xn;
        } else {
            j++;
            y = yn;
        }
    }
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// Bounded wait that also gives up when another warp has recorded a failure.
__device__ __forceinline__ bool wait_or_fail(uint64_t *bar, uint32_t phase, uint32_t limit,
                                             volatile uint32_t *fail) {
    for (uint32_t i = 0; i < limit; i++) {
        if (mbar_try_wait(bar, phase)) return true;
        if (*fail) return false;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

// Named barrier of the consumer warps only (the producer warp is not in it).
__device__ __forceinline__ void consumers_sync() {
    asm volatile("bar.sync 1, %0;" ::"n"(CMP_CONSUMER_THREADS) : "memory");
}

// The shared-memory side of the pipeline.
struct Pipe {
    uint64_t full[CMP_STAGES];
    uint64_t empty[CMP_STAGES];
    Stage desc[CMP_STAGES];
    uint64_t tile[CMP_STAGES];
    FF warp_part[CMP_STAGES][CMP_CONSUMERS];
    uint32_t done[CMP_STAGES];
    uint32_t fail;
};

__device__ __forceinline__ uint32_t *stage_keys(uint8_t *raw, int s) {
    return reinterpret_cast<uint32_t *>(raw) + (size_t)s * 2 * CMP_BUF;
}
__device__ __forceinline__ float *stage_vals(uint8_t *raw, int s) {
    return reinterpret_cast<float *>(stage_keys(raw, s) + CMP_BUF);
}

// Left [i0, i1) and right [j0, j1) of one tile of one pair (d0, d1 its merged
// positions): a match whose left element ends the tile can have its equal right
// element start the next one (ties go left), so one right element past the tile
// is staged as look-ahead.
__device__ __forceinline__ Stage tile_ranges(const uint32_t *Ak, const float *Av, uint32_t na,
                                             const uint32_t *Bk, const float *Bv, uint32_t nb,
                                             uint64_t d0, uint32_t i0, uint64_t d1, uint32_t i1,
                                             uint32_t *sk, float *sv, uint64_t *bar, bool issue) {
    const uint32_t j0 = (uint32_t)(d0 - i0), j1 = (uint32_t)(d1 - i1);
    const uint32_t j1x = j1 < nb ? j1 + 1 : j1;
    return stage_ranges(Ak, Av, i0, i1, Bk, Bv, j0, j1, j1x, sk, sv, bar, issue);
}

// Publishes a stage's layout, then arms its barrier and issues the copies (the
// arrive releases the layout to the consumers that acquire the barrier).
template <class F>
__device__ __forceinline__ void issue_stage(Pipe &pp, int s, uint64_t t, F layout) {
    pp.desc[s] = layout(false);
    pp.tile[s] = t;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    (void)layout(true);
}

// After a failure: every copy the producer issued lands before the CTA exits.
__device__ __forceinline__ void producer_drain(Pipe &pp, uint64_t issued, uint32_t *status) {
    if ((threadIdx.x & 31) == 0) {
        atomicOr(status, (uint32_t)DEV_WAIT_TIMEOUT);
        pp.fail = 1;
    }
    const uint64_t from = issued > (uint64_t)CMP_STAGES ? issued - CMP_STAGES : 0;
    for (uint64_t rel = from; rel < issued; rel++)
        (void)mbar_wait_bounded(&pp.full[rel % CMP_STAGES], (uint32_t)(rel / CMP_STAGES) & 1,
                                CMP_DRAIN);
}

// Producer of one pair: the run's splits are in shared memory (split[r] = left
// split of tile t_begin + r).
__device__ __forceinline__ void produce_one(const uint32_t *Ak, const float *Av, uint32_t na,
                                            const uint32_t *Bk, const float *Bv, uint32_t nb,
                                            const uint32_t *split, uint64_t t_begin,
                                            uint64_t t_end, Pipe &pp, uint8_t *raw,
                                            uint32_t *status) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t total = (uint64_t)na + nb;
    uint64_t issued = 0;
    bool failed = false;
    for (uint64_t t = t_begin; t < t_end; t++) {
        const uint64_t rel = t - t_begin;
        const int s = (int)(rel % CMP_STAGES);
        const uint32_t k = (uint32_t)(rel / CMP_STAGES);
        if (k > 0 && !wait_or_fail(&pp.empty[s], (k - 1) & 1, CMP_WAIT, &pp.fail)) {
            failed = true;
            break;
        }
        if (lane == 0) {
            const uint64_t d0 = t * (uint64_t)CMP_TILE, d1 = min(d0 + CMP_TILE, total);
            const uint32_t i0 = split[rel], i1 = split[rel + 1];
            issue_stage(pp, s, t, [&](bool issue) {
                return tile_ranges(Ak, Av, na, Bk, Bv, nb, d0, i0, d1, i1, stage_keys(raw, s),
                                   stage_vals(raw, s), &pp.full[s], issue);
            });
        }
        __syncwarp();
        issued = rel + 1;
    }
    if (failed || pp.fail) producer_drain(pp, issued, status);
}

// A consumer warp's pass over the run.  PER_TILE: each tile's sum goes to
// tile_part[t] (combined by the last warp to finish the tile); otherwise acc
// keeps the running sum.
template <bool PER_TILE>
__device__ __forceinline__ void consume(uint64_t t_begin, uint64_t t_end, Pipe &pp, uint8_t *raw,
                                        uint32_t first_wait_limit, FF *tile_part, FF &acc,
                                        uint32_t *status) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t t = t_begin; t < t_end; t++) {
        const uint64_t rel = t - t_begin;
        const int s = (int)(rel % CMP_STAGES);
        const uint32_t k = (uint32_t)(rel / CMP_STAGES);
        const uint32_t limit = rel == 0 ? first_wait_limit : CMP_WAIT;
        if (!wait_or_fail(&pp.full[s], k & 1, limit, &pp.fail)) {
            if (lane == 0) {
                pp.fail = 1;
                atomicOr(status, (uint32_t)DEV_WAIT_TIMEOUT);
            }
            return;
        }
        const Stage sd = pp.desc[s];
        if (PER_TILE) {
            FF x = {0.0f, 0.0f};
            merge_tile(sd, stage_keys(raw, s), stage_vals(raw, s), x);
            x = ff_warp_sum(x);
            if (lane == 0) {
                pp.warp_part[s][warp] = x;
                __threadfence_block();
                if (atomicAdd(&pp.done[s], 1u) == CMP_CONSUMERS - 1) {
                    __threadfence_block();
                    FF r = {0.0f, 0.0f};
                    for (int w = 0; w < CMP_CONSUMERS; w++) {
                        const volatile float *pw =
                            reinterpret_cast<volatile float *>(&pp.warp_part[s][w]);
                        FF v = {pw[0], pw[1]};
                        r = ff_merge(r, v);
                    }
                    tile_part[pp.tile[s]] = r;
                    pp.done[s] = 0u;
                }
            }
        } else {
            merge_tile(sd, stage_keys(raw, s), stage_vals(raw, s), acc);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&pp.empty[s]);
    }
}

__device__ __forceinline__ void pipe_init(Pipe &pp) {
    if (threadIdx.x == 0) {
        for (int s = 0; s < CMP_STAGES; s++) {
            mbar_init(&pp.full[s], 1);
            mbar_init(&pp.empty[s], CMP_CONSUMERS);
            pp.done[s] = 0u;
        }
        pp.fail = 0u;
        fence_mbar_init();
    }
    __syncthreads();
}

__global__ void __launch_bounds__(CMP_THREADS) k_compare(
    const uint32_t *__restrict__ Ak, const float *__restrict__ Av, uint32_t na,
    const uint32_t *__restrict__ Bk, const float *__restrict__ Bv, uint32_t nb, uint32_t ntiles,
    uint32_t per, uint32_t first_wait_limit, CmpState *st, double *out) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    __shared__ Pipe pp;
    __shared__ uint32_t s_split[CMP_MAX_RUN + 1];
    __shared__ FF s_final[CMP_CONSUMERS];
    __shared__ bool s_last;
    const uint64_t total = (uint64_t)na + nb;
    const uint64_t t_begin = (uint64_t)blockIdx.x * per;
    const uint64_t t_end = min((uint64_t)ntiles, t_begin + per);
    // the splits of this run's boundaries t_begin .. t_end, all warps at once
    const uint32_t warp = threadIdx.x >> 5;
    for (uint64_t b = warp; t_begin < t_end && b <= t_end - t_begin; b += CMP_THREADS / 32) {
        const uint64_t d = min((t_begin + b) * (uint64_t)CMP_TILE, total);
        const uint32_t i = warp_merge_path(d, Ak, na, Bk, nb, split_guess(d, na, nb), 64);
        if ((threadIdx.x & 31) == 0) s_split[b] = i;
    }
    pipe_init(pp);  // (its barrier also publishes the splits)
    if (threadIdx.x >= CMP_CONSUMER_THREADS) {
        if (t_begin < t_end)
            produce_one(Ak, Av, na, Bk, Bv, nb, s_split, t_begin, t_end, pp, smem_raw,
                        &st->status);
        return;
    }
    FF acc = {0.0f, 0.0f};
    consume<false>(t_begin, t_end, pp, smem_raw, first_wait_limit, nullptr, acc, &st->status);
    // CTA reduction (consumer warps), then the last CTA combines in a fixed order
    acc = ff_warp_sum(acc);
    if ((threadIdx.x & 31) == 0) s_final[threadIdx.x >> 5] = acc;
    consumers_sync();
    if (threadIdx.x == 0) {
        FF r = {0.0f, 0.0f};
        for (int w = 0; w < CMP_CONSUMERS; w++) r = ff_merge(r, s_final[w]);
        st->partial[blockIdx.x] = r;
        __threadfence();
        const uint32_t done = atomicAdd(&st->ticket, 1u);
        s_last = (done == gridDim.x - 1);
    }
    consumers_sync();
    if (s_last && threadIdx.x < 32) {
        __threadfence();
        // lane l sums partials l, l+32, ... in double-double, then a fixed tree
        DD dacc = {0.0, 0.0};
        for (uint32_t c = threadIdx.x; c < gridDim.x; c += 32) {
            const volatile float *p = reinterpret_cast<volatile float *>(&st->partial[c]);
            dd_add(dacc, (double)p[0]);
            dd_add(dacc, (double)p[1]);
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

static const size_t kCmpSmem = sizeof(uint32_t) * 2 * CMP_BUF * CMP_STAGES;

// Poll limit of each CTA's first wait (a test hook: 0 makes every CTA give up
// at once, after its copies were issued, so the timeout path can be exercised
// without a fault).
static std::atomic<uint32_t> g_first_wait_limit{CMP_WAIT};

void compare_set_first_wait_limit(uint32_t limit) {
    g_first_wait_limit.store(limit == 0xffffffffu ? CMP_WAIT : limit);
}

uint32_t compare_tile_elements() { return CMP_TILE; }

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
    // two CTAs per SM (three fit): one pair's split searches and the last CTA's
    // combine cost less over fewer, longer runs (synchronous call on 6.6 M entries:
    // 0.045 ms against 0.053 with three); at most CMP_MAX_RUN tiles each
    const uint32_t sms = (uint32_t)device_sm_count();
    uint32_t grid = min(ntiles, min(2u * sms, CMP_MIN_CAP));
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
// tiles [tile_off[p], tile_off[p+1])).  k_many_owner labels every tile with its
// pair, k_many_splits finds every tile boundary's merge-path split (a thread per
// boundary, all at once), and persistent CTAs take contiguous runs of tiles
// through the pipeline, their producer reading the labels and splits of 32
// tiles per coalesced load.  Every tile leaves one float-float partial, and
// k_many_reduce sums each pair's tiles in order.
// ---------------------------------------------------------------------------

struct ManyArgs {
    const uint32_t *lkeys; const float *lvals; const uint64_t *loff; const uint32_t *lnnz;
    const uint32_t *rkeys; const float *rvals; const uint64_t *roff; const uint32_t *rnnz;
    const uint32_t *pa, *pb;   // pair p = (left vector pa[p], right vector pb[p])
    uint32_t P;
    uint32_t *ptiles;          // [P] tiles per pair
    uint64_t *tile_off;        // [P+1]
    uint64_t *scan_tmp;
    uint32_t *owner;           // [max_tiles] pair of each tile
    uint32_t *split;           // [max_tiles] left split at each tile's start
    FF *tile_part;             // [max_tiles]
    uint64_t max_tiles;
    uint32_t per;              // tiles per CTA
    double *out;               // [P]
    uint32_t *status;
};

__global__ void k_many_tiles(ManyArgs a) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    const uint64_t tot = (uint64_t)a.lnnz[a.pa[p]] + a.rnnz[a.pb[p]];
    a.ptiles[p] = (uint32_t)div_up(tot, CMP_TILE);
}

// grid = pairs: CTA p labels tiles [tile_off[p], tile_off[p+1]) with p
__global__ void k_many_owner(ManyArgs a) {
    const uint32_t p = blockIdx.x;
    const uint64_t t0 = a.tile_off[p], t1 = min(a.tile_off[p + 1], a.max_tiles);
    for (uint64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) a.owner[t] = p;
}

// Thread per tile: the left split at the tile's start, by a scalar search that
// gallops out from the interpolated split (its probes stay near the answer).
__global__ void k_many_splits(ManyArgs a) {
    uint64_t T = a.tile_off[a.P];
    if (T > a.max_tiles) T = a.max_tiles;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const uint32_t p = a.owner[t];
    const uint32_t va = a.pa[p], vb = a.pb[p];
    const uint32_t na = a.lnnz[va], nb = a.rnnz[vb];
    const uint32_t *A = a.lkeys + a.loff[va], *B = a.rkeys + a.roff[vb];
    const uint64_t d = (t - a.tile_off[p]) * CMP_TILE;
    // the split is the largest i in [lo, hi] with i == lo or A[i-1] <= B[d-i]
    uint32_t lo = d > nb ? (uint32_t)(d - nb) : 0u;
    uint32_t hi = d < na ? (uint32_t)d : na;
    const uint32_t lo0 = lo;
    auto pred = [&](uint32_t i) { return i <= lo0 || __ldg(&A[i - 1]) <= __ldg(&B[d - i]); };
    const uint64_t g = split_guess(d, na, nb);
    const uint32_t i = (uint32_t)min(max(g, (uint64_t)lo), (uint64_t)hi);
    if (pred(i)) {  // gallop up
        lo = i;
        for (uint32_t step = 1;; step <<= 1) {
            const uint64_t j = (uint64_t)lo + step;
            if (j > hi) break;
            if (!pred((uint32_t)j)) {
                hi = (uint32_t)j - 1;
                break;
            }
            lo = (uint32_t)j;
        }
    } else {  // gallop down (i > lo0 here)
        hi = i - 1;
        for (uint32_t step = 1;; step <<= 1) {
            if (hi < lo + step) break;
            const uint32_t j = hi + 1 - step;  // probe below the current bound
            if (pred(j)) {
                lo = j;
                break;
            }
            hi = j - 1;
        }
    }
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        if (pred(mid)) lo = mid; else hi = mid - 1;
    }
    a.split[t] = lo;
}

// Producer of many pairs: labels and splits of 32 tiles per coalesced load,
// the current pair's vectors cached in registers.
__device__ __forceinline__ void produce_many(const ManyArgs &a, uint64_t T, uint64_t t_begin,
                                             uint64_t t_end, Pipe &pp, uint8_t *raw) {
    const uint32_t lane = threadIdx.x & 31;
    uint64_t issued = 0, base = t_begin;
    bool failed = false;
    uint32_t own = 0, spl = 0, own_x = a.P, spl_x = 0;
    auto load_batch = [&](uint64_t b) {
        const uint64_t t = b + lane;
        own = t < T ? a.owner[t] : a.P;
        spl = t < T ? a.split[t] : 0u;
        own_x = b + 32 < T ? a.owner[b + 32] : a.P;  // the boundary after the batch
        spl_x = b + 32 < T ? a.split[b + 32] : 0u;
    };
    load_batch(base);
    uint32_t cur = a.P, na = 0, nb = 0;
    uint64_t lbase = 0, rbase = 0, toff = 0;
    for (uint64_t t = t_begin; t < t_end; t++) {
        if (t - base == 32) {
            base += 32;
            load_batch(base);
        }
        const uint64_t rel = t - t_begin;
        const int s = (int)(rel % CMP_STAGES);
        const uint32_t k = (uint32_t)(rel / CMP_STAGES);
        if (k > 0 && !wait_or_fail(&pp.empty[s], (k - 1) & 1, CMP_WAIT, &pp.fail)) {
            failed = true;
            break;
        }
        const uint32_t r = (uint32_t)(t - base);
        const uint32_t p = __shfl_sync(0xffffffffu, own, r);
        const uint32_t i0 = __shfl_sync(0xffffffffu, spl, r);
        uint32_t p1 = __shfl_sync(0xffffffffu, own, (r + 1) & 31);
        uint32_t i1n = __shfl_sync(0xffffffffu, spl, (r + 1) & 31);
        if (r == 31) {
            p1 = own_x;
            i1n = spl_x;
        }
        if (p != cur) {
            cur = p;
            const uint32_t va = a.pa[p], vb = a.pb[p];
            na = a.lnnz[va];
            nb = a.rnnz[vb];
            lbase = a.loff[va];
            rbase = a.roff[vb];
            toff = a.tile_off[p];
        }
        if (lane == 0) {
            const uint64_t d0 = (t - toff) * CMP_TILE;
            const bool same = p1 == p;  // the next boundary lies inside this pair
            const uint64_t d1 = same ? d0 + CMP_TILE : (uint64_t)na + nb;
            const uint32_t i1 = same ? i1n : na;
            issue_stage(pp, s, t, [&](bool issue) {
                return tile_ranges(a.lkeys + lbase, a.lvals + lbase, na, a.rkeys + rbase,
                                   a.rvals + rbase, nb, d0, i0, d1, i1, stage_keys(raw, s),
                                   stage_vals(raw, s), &pp.full[s], issue);
            });
        }
        __syncwarp();
        issued = rel + 1;
    }
    if (failed || pp.fail) producer_drain(pp, issued, a.status);
}

__global__ void __launch_bounds__(CMP_THREADS) k_many_intersect(ManyArgs a) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    __shared__ Pipe pp;
    uint64_t T = a.tile_off[a.P];
    if (blockIdx.x == 0 && threadIdx.x == 0 && T > a.max_tiles)
        atomicOr(a.status, (uint32_t)DEV_CAPACITY);
    if (T > a.max_tiles) T = a.max_tiles;
    const uint64_t t_begin = (uint64_t)blockIdx.x * a.per;
    const uint64_t t_end = min(T, t_begin + a.per);
    if (t_begin >= t_end) return;  // the same for every thread of the CTA
    pipe_init(pp);
    if (threadIdx.x >= CMP_CONSUMER_THREADS) {
        produce_many(a, T, t_begin, t_end, pp, smem_raw);
        return;
    }
    FF unused = {0.0f, 0.0f};
    consume<true>(t_begin, t_end, pp, smem_raw, CMP_WAIT, a.tile_part, unused, a.status);
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
    const uint64_t mt = max_tiles ? max_tiles : 1;
    return scratch_bytes<uint32_t>(P) + scratch_bytes<uint64_t>((uint64_t)P + 1) +
           scan_temp_bytes((uint64_t)P + 1) + 2 * scratch_bytes<uint32_t>(mt) +
           scratch_bytes<FF>(mt) + scratch_bytes<uint32_t>(4);
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
    const uint64_t mt = max_tiles ? max_tiles : 1;
    a.ptiles = sc.take<uint32_t>(P);
    a.tile_off = sc.take<uint64_t>((uint64_t)P + 1);
    a.scan_tmp = sc.take<uint64_t>(scan_temp_bytes((uint64_t)P + 1) / 8);
    a.owner = sc.take<uint32_t>(mt);
    a.split = sc.take<uint32_t>(mt);
    a.tile_part = sc.take<FF>(mt);
    a.status = sc.take<uint32_t>(4);
    a.max_tiles = max_tiles;
    a.out = out;
    if (!a.status) return cudaErrorInvalidValue;
    if (status_out) *status_out = a.status;
    PHYLO_CHECK(many_attributes());
    PHYLO_CHECK(cudaMemsetAsync(a.status, 0, sizeof(uint32_t), st));
    k_many_tiles<<<(P + 255) / 256, 256, 0, st>>>(a);
    PHYLO_CHECK(scan_u32_to_u64(a.ptiles, P, a.tile_off, a.scan_tmp, st));
    k_many_owner<<<P, 256, 0, st>>>(a);
    k_many_splits<<<(unsigned)div_up(mt, 256), 256, 0, st>>>(a);
    const uint64_t sms = (uint64_t)device_sm_count();
    uint64_t per = div_up(mt, 3 * sms);
    if (per > CMP_MAX_RUN) per = CMP_MAX_RUN;
    if (per < 1) per = 1;
    a.per = (uint32_t)per;
    const uint64_t grid = div_up(mt, per);
    k_many_intersect<<<(unsigned)grid, CMP_THREADS, kCmpSmem, st>>>(a);
    k_many_reduce<<<(P + 7) / 8, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace phylo
