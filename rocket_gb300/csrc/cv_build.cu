// cv_build.cu -- composition-vector construction on the device.
//
// Same result as the reference pipeline of phylogenetics/src/main/cpp/native.cu
// (count_kmers :220-256, totals :317-345, Markov alpha :350-400, nnz/norm
// :402-428, sorted selection :449-458, normalisation :460-468, padding
// :470-474), computed without the dense A^K table:
//
//   A slot a.m.b (a, b single symbols, m the (K-2)-mer in between) can only be
//   nonzero when its prefix a.m and its suffix m.b were both seen as
//   (K-1)-mers (then the middle m was seen too).  So the candidates are, for
//   every seen (K-1)-mer q = a.m in ascending order, the symbols b of the
//   right-extension set R(m) = { b : m.b seen }, a 21-bit mask per
//   (K-2)-mer.  Enumerated in that order the candidate keys q*A + b are
//   already sorted, and the count of every seen K-mer is scattered straight
//   into its candidate slot (rank of b in R(m)) -- no sort and no A^K table.
//
// Pipeline per batch of proteomes (all kernels take the whole batch):
//   k_prep          tile bases per proteome
//   k_count         (K-2)/(K-1) counts, seen (K-1)-mers (the right-extension
//                   masks are slices of that bitmap), window totals
//   k_cand_count    candidates per chunk of 2048 (K-1)-mers
//   scan, k_cand_bases   candidate offsets; proteome p's candidates start at
//                   cbase[p], a multiple of ALPHA_TILE
//   k_cand_offsets  per-(K-1)-mer candidate offsets; the key of every candidate
//   k_c0_scatter    K-mer counts into candidate slots (zeroed by k_cand_offsets)
//   k_alpha         Markov alpha (reference double order), flat over the
//                   candidates: a seen candidate's count is replaced in place by
//                   its alpha bits (an unseen one keeps count 0: alpha -1);
//                   survivors counted per segment; norm partials
//   scan            -> output offset of every segment
//   k_norm          per-proteome norm, scale, nnz
//   (host reads nnz, checks capacity)
//   k_compact       survivors' keys and normalised values, segment by segment
//   k_union_mark    (with a key bitmap) the candidate keys of every seen (K-1)-mer
#include "cv_build.cuh"
#include "hostctx.cuh"
#include "rank.cuh"
#include "scan.cuh"

namespace phylo {

constexpr int TILE = 512;            // sequence positions per counting tile (few
                                     // proteomes' tables in flight -> L2 hits)
constexpr int COUNT_THREADS = 256;
constexpr int CHUNK_THREADS = 256;

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

// Batch bases (cbase: B + 1 entries) staged in shared memory when they fit, so
// that finding a CTA's proteome is one round of parallel loads instead of a chain
// of dependent ones per thread (k_compact; in the kernels whose tables rely on L1
// the staging measured slower).
constexpr int SMEM_BASES = 256;
__device__ __forceinline__ const uint64_t *stage_bases(const uint64_t *__restrict__ g, int n,
                                                       uint64_t *s) {
    if (n > SMEM_BASES) return g;
    for (int i = threadIdx.x; i <= n; i += blockDim.x) s[i] = g[i];
    __syncthreads();
    return s;
}

__device__ __forceinline__ int find_owner(const uint64_t *__restrict__ base, int n, uint64_t t) {
    // largest p with base[p] <= t, base has n+1 entries, base[0] = 0
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (base[mid] <= t) lo = mid; else hi = mid;
    }
    return lo;
}

// Markov alpha with the reference's operation order (native.cu:387-394):
//   p  = full / n0
//   p0 = ((prefix / n1) * (suffix / n1)) / (middle / n2)
//   alpha = float((p - p0) / p0)
// Every operation is an explicitly rounded IEEE double op, so no FMA
// contraction can change the result.
__device__ __forceinline__ float markov_alpha(uint32_t full, uint32_t prefix, uint32_t suffix,
                                              uint32_t middle, uint32_t n0, uint32_t n1,
                                              uint32_t n2) {
    if (full == 0u && n0 != 0u) return -1.0f;  // (0 - p0) / p0 == -1 exactly (p0 > 0 finite)
    double p = __ddiv_rn((double)full, (double)n0);
    double pp = __ddiv_rn((double)prefix, (double)n1);
    double ps = __ddiv_rn((double)suffix, (double)n1);
    double pm = __ddiv_rn((double)middle, (double)n2);
    double p0 = __ddiv_rn(__dmul_rn(pp, ps), pm);
    return __double2float_rn(__ddiv_rn(__dsub_rn(p, p0), p0));
}

// The same alpha with the FP64 work cut down (GB300 issues FP64 at a small
// fraction of the FP32 rate):
//   * p, prefix/n1, suffix/n1, middle/n2 come from per-proteome tables holding
//     exactly those IEEE quotients for counts below PROB_TABLE;
//   * p0 = RN(a / b) as q0 = RN(a * y), r = a - b*q0 (exact by FMA),
//     RN(q0 + r*y) with y = RN(1/b) from the table -- a correctly rounded
//     quotient (Markstein's reciprocal-correction theorem);
//   * (p - p0) / p0 is only needed rounded to float: a quotient accurate to
//     ~2^-46 from a float reciprocal and one FMA correction gives the same float
//     unless it lies within 256 double ulps of a float rounding midpoint, where
//     the exact IEEE division is used instead.
// Anything outside the tables (large counts, no K-windows) takes markov_alpha.
__device__ __forceinline__ float markov_alpha_fast(uint32_t full, uint32_t prefix,
                                                   uint32_t suffix, uint32_t middle, uint32_t n0,
                                                   uint32_t n1, uint32_t n2,
                                                   const double *__restrict__ prob) {
    if (full == 0u && n0 != 0u) return -1.0f;
    if (n0 == 0u || full >= PROB_TABLE || prefix >= PROB_TABLE || suffix >= PROB_TABLE ||
        middle >= PROB_TABLE)
        return markov_alpha(full, prefix, suffix, middle, n0, n1, n2);
    const double p = __ldg(&prob[full]);
    const double pp = __ldg(&prob[PROB_TABLE + prefix]);
    const double ps = __ldg(&prob[PROB_TABLE + suffix]);
    const double pm = __ldg(&prob[2 * PROB_TABLE + middle]);
    const double ym = __ldg(&prob[3 * PROB_TABLE + middle]);
    const double a = __dmul_rn(pp, ps);
    const double q0 = __dmul_rn(a, ym);
    const double p0 = __fma_rn(__fma_rn(-q0, pm, a), ym, q0);
    const double d = __dsub_rn(p, p0);
    if (d == 0.0) return 0.0f;
    const double y0 = (double)__frcp_rn(__double2float_rn(p0));
    const double g0 = __dmul_rn(d, y0);
    const double g1 = __fma_rn(__fma_rn(-g0, p0, d), y0, g0);
    const long long low = (long long)(__double_as_longlong(g1) & ((1ll << 29) - 1)) - (1ll << 28);
    if (low <= 256 && low >= -256) return __double2float_rn(__ddiv_rn(d, p0));
    return __double2float_rn(g1);
}

// Sum of non-negative floats as an exact 192-bit fixed-point number in units of
// 2^-96 (terms below 2^-73 lose their lowest bits; such squares need
// |alpha| < 2^-36).  Integer addition makes the result independent of order.
struct U192 {
    uint64_t w0, w1, w2;
};

__device__ __forceinline__ void u192_add(U192 &a, uint64_t p0, uint64_t p1, uint64_t p2) {
    asm("add.cc.u64 %0, %0, %3;\n\taddc.cc.u64 %1, %1, %4;\n\taddc.u64 %2, %2, %5;"
        : "+l"(a.w0), "+l"(a.w1), "+l"(a.w2)
        : "l"(p0), "l"(p1), "l"(p2));
}

// Adds a finite square; returns false for a square too large to hold (>= 2^72).
__device__ __forceinline__ bool u192_add_float(U192 &a, float v) {
    const uint32_t bits = __float_as_uint(v);
    const uint32_t e = bits >> 23;
    uint64_t m = e ? ((bits & 0x7fffffu) | 0x800000u) : (bits & 0x7fffffu);
    if (m == 0) return true;
    int sh = (e ? (int)e : 1) - 150 + 96;  // bit position of m's lowest bit
    if (sh < 0) {
        if (sh <= -24) return true;
        m >>= -sh;
        sh = 0;
    }
    uint64_t p0 = 0, p1 = 0, p2 = 0;
    if (sh < 64) {
        p0 = m << sh;
        p1 = sh ? (m >> (64 - sh)) : 0;
    } else if (sh < 128) {
        const int t = sh - 64;
        p1 = m << t;
        p2 = t ? (m >> (64 - t)) : 0;
    } else if (sh <= 192 - 24) {
        p2 = m << (sh - 128);
    } else {
        return false;
    }
    u192_add(a, p0, p1, p2);
    return true;
}

__device__ __forceinline__ U192 u192_shfl_down(const U192 &a, int d) {
    U192 r;
    r.w0 = __shfl_down_sync(0xffffffffu, a.w0, d);
    r.w1 = __shfl_down_sync(0xffffffffu, a.w1, d);
    r.w2 = __shfl_down_sync(0xffffffffu, a.w2, d);
    return r;
}

// value * 2^-96 rounded to nearest-even double
__device__ double u192_to_double(const U192 &a) {
    uint64_t top, next, rest;
    int base;
    if (a.w2) { top = a.w2; next = a.w1; rest = a.w0; base = 128; }
    else if (a.w1) { top = a.w1; next = a.w0; rest = 0; base = 64; }
    else if (a.w0) { top = a.w0; next = 0; rest = 0; base = 0; }
    else return 0.0;
    const int lz = __clzll(top);
    int pos = base + 63 - lz;  // index of the most significant bit
    const uint64_t hi64 = lz ? ((top << lz) | (next >> (64 - lz))) : top;
    const uint64_t below = lz ? (next << lz) : next;
    uint64_t mant = hi64 >> 11;
    const bool round_bit = (hi64 >> 10) & 1;
    const bool sticky = (hi64 & 0x3ffull) || below || rest;
    if (round_bit && (sticky || (mant & 1))) {
        mant++;
        if (mant == (1ull << 53)) {
            mant >>= 1;
            pos++;
        }
    }
    return ldexp((double)mant, pos - 52 - 96);
}

// Index of (K-1)-mer q of proteome p in the c1 / coff tables: q itself (dense
// rows of T1s entries), or its rank among the batch's seen (K-1)-mers (compact).
__device__ __forceinline__ uint64_t c1_index(const BuildArgs &a, int p, uint32_t q) {
    if (!a.compact1) return (uint64_t)p * a.T1s + q;
    const uint2 t = __ldg(&a.pw1[(uint64_t)p * (a.T1s / 32) + (q >> 5)]);  // {prefix, seen word}
    return (uint64_t)t.x + (uint32_t)__popc(t.y & ((1u << (q & 31u)) - 1u));
}

// Index of (K-2)-mer m of proteome p in c2: dense row entry, or its rank among
// the batch's seen (K-2)-mers (compact).
__device__ __forceinline__ uint64_t c2_index(const BuildArgs &a, int p, uint32_t m) {
    if (!a.compact2) return (uint64_t)p * a.T2 + m;
    const uint2 t = __ldg(&a.pw2[(uint64_t)p * (a.T2s / 32) + (m >> 5)]);
    return (uint64_t)t.x + (uint32_t)__popc(t.y & ((1u << (m & 31u)) - 1u));
}

// Right-extension mask of (K-2)-mer m in proteome p: bit b set when the
// (K-1)-mer m.b was seen.  Those are the A bits of the seen bitmap starting at
// bit m * A (the code of m.b is m * A + b), so no separate table is kept.
__device__ __forceinline__ uint32_t ext_mask(const BuildArgs &a, int p, uint32_t m) {
    const uint32_t *sw = a.seen1 + (uint64_t)p * (a.T1s / 32);
    const uint64_t bit = (uint64_t)m * a.A;
    const uint64_t w = bit >> 5;
    const uint32_t off = (uint32_t)bit & 31u;
    uint32_t v = __ldg(&sw[w]) >> off;
    if (off + a.A > 32u) v |= __ldg(&sw[w + 1]) << (32u - off);
    return v & ((1u << a.A) - 1u);
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// prob[p][0][c] = c/n0, [1][c] = c/n1, [2][c] = c/n2, [3][c] = 1/(c/n2): the
// exact IEEE quotients the reference forms for count c.  grid = (PROB_TABLE/256, B)
__global__ void k_tables(BuildArgs a) {
    const int p = blockIdx.y;
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= PROB_TABLE) return;
    const double n0 = (double)a.tot[p * 4 + 0], n1 = (double)a.tot[p * 4 + 1],
                 n2 = (double)a.tot[p * 4 + 2];
    double *t = a.prob + (uint64_t)p * 4 * PROB_TABLE;
    const double pm = __ddiv_rn((double)c, n2);
    t[c] = __ddiv_rn((double)c, n0);
    t[PROB_TABLE + c] = __ddiv_rn((double)c, n1);
    t[2 * PROB_TABLE + c] = pm;
    t[3 * PROB_TABLE + c] = __ddiv_rn(1.0, pm);
}

// tile_base[p] = number of TILE-sized tiles of proteomes < p; tile_base[B] = total.
__global__ void k_prep(int B, const uint64_t *__restrict__ seq_off, uint64_t *tile_base) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        uint64_t acc = 0;
        for (int p = 0; p < B; p++) {
            tile_base[p] = acc;
            acc += div_up(seq_off[p + 1] - seq_off[p], TILE);
        }
        tile_base[B] = acc;
    }
}

// Alpha of every small count tuple, once per proteome (the same arithmetic as
// markov_alpha_fast, so a table hit gives the bits the direct path would).
// grid = (TUPLE_TABLE / 256, B)
__global__ void k_tuple_alpha(BuildArgs a) {
    const int p = blockIdx.y;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint32_t)TUPLE_TABLE) return;
    const uint32_t mid = t % TUPLE_MID, suf = (t / TUPLE_MID) % TUPLE_PS,
                   pre = (t / (TUPLE_MID * TUPLE_PS)) % TUPLE_PS,
                   full = t / (TUPLE_MID * TUPLE_PS * TUPLE_PS);
    const uint32_t n0 = a.tot[p * 4 + 0], n1 = a.tot[p * 4 + 1], n2 = a.tot[p * 4 + 2];
    uint32_t bits = 0;
    if (full >= 1 && pre >= 1 && suf >= 1 && mid >= 1 && n0 != 0)
        bits = __float_as_uint(markov_alpha_fast(full, pre, suf, mid, n0, n1, n2,
                                                 a.prob + (uint64_t)p * 4 * PROB_TABLE));
    a.atab[(uint64_t)p * TUPLE_TABLE + t] = bits;
}

__device__ __forceinline__ float div_by_scale(float f, double scale, double rs) {
    const double x = (double)f;
    const double q = __dmul_rn(x, rs);
    return __double2float_rn(__fma_rn(__fma_rn(-q, scale, x), rs, q));
}

// Normalised value of every tuple, after the norm is known.  grid = (TUPLE_TABLE / 256, B)
__global__ void k_tuple_value(BuildArgs a) {
    const int p = blockIdx.y;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint32_t)TUPLE_TABLE) return;
    const double scale = a.scale[p], rs = a.rscale[p];
    const float f = __uint_as_float(a.atab[(uint64_t)p * TUPLE_TABLE + t]);
    float v;
    if (!(isfinite(scale) && scale > 0.0) || !isfinite(f))
        v = __double2float_rn(__ddiv_rn((double)f, scale));
    else
        v = div_by_scale(f, scale, rs);
    a.vtab[(uint64_t)p * TUPLE_TABLE + t] = v;
}

// Counts (K-2)- and (K-1)-windows, marks right extensions, totals n0/n1/n2.
// A window starting at i counts for length L when its L symbols are all in the
// alphabet and inside the proteome (native.cu:236-252).
template <bool COMPACT>
__global__ void __launch_bounds__(COUNT_THREADS) k_count(BuildArgs a) {
    __shared__ uint8_t dig[TILE + 16];
    __shared__ uint32_t ntot[3];
    const int K = a.k;
    const uint32_t A = a.A;
    const uint64_t total_tiles = a.tile_base[a.B];
    for (uint64_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
        const int p = find_owner(a.tile_base, a.B, t);
        const uint64_t s0 = a.seq_off[p], len = a.seq_off[p + 1] - s0;
        const uint64_t start = (t - a.tile_base[p]) * TILE;
        if (threadIdx.x < 3) ntot[threadIdx.x] = 0;
        for (int j = threadIdx.x; j < TILE + K; j += COUNT_THREADS) {
            uint64_t pos = start + j;
            dig[j] = pos < len ? (uint8_t)char_to_digit(a.alpha, a.seq[s0 + pos]) : (uint8_t)0xff;
        }
        __syncthreads();
        uint32_t *c1 = COMPACT ? nullptr : a.c1 + (uint64_t)p * a.T1s;
        uint32_t *seen = a.seen1 + (uint64_t)p * (a.T1s / 32);
        uint32_t *c2 = a.c2 + (uint64_t)p * a.T2;
        uint32_t *seen2 = a.seen2 + (uint64_t)p * (a.T2s / 32);
        uint32_t cnt0 = 0, cnt1 = 0, cnt2 = 0;
        for (int u = 0; u < TILE / COUNT_THREADS; u++) {
            const int li = u * COUNT_THREADS + threadIdx.x;
            const bool inb = start + li < len;
            uint32_t w = 0, w2 = 0, w1 = 0, last = 0;
            int run = 0;
            if (inb) {
                for (int j = 0; j < K; j++) {
                    uint32_t d = dig[li + j];
                    if (d == 0xffu) break;
                    w = w * A + d;
                    run = j + 1;
                    if (j == K - 3) w2 = w;
                    if (j == K - 2) { w1 = w; last = d; }
                }
            }
            const bool v2 = run >= K - 2, v1 = run >= K - 1, v0 = run >= K;
            cnt2 += v2; cnt1 += v1; cnt0 += v0;
            // counts: reduction atomics (equal keys within a warp are rare, so no
            // aggregation); the first sighting of a (K-1)-mer sets its seen bit,
            // which is also bit `last` of the right-extension mask of its first
            // K-2 symbols (compact tables: only the seen bit here; k_c0_scatter
            // counts once the ranks of the seen (K-1)-mers are known)
            if (v2) {  // compact (K-2)-mer tables: the seen bit; k_c0_scatter counts
                if (a.compact2) atomicOr(&seen2[w2 >> 5], 1u << (w2 & 31u));
                else atomicAdd(&c2[w2], 1u);
            }
            if (v1) {
                if (COMPACT) {
                    atomicOr(&seen[w1 >> 5], 1u << (w1 & 31u));
                } else if (atomicAdd(&c1[w1], 1u) == 0u) {
                    atomicOr(&seen[w1 >> 5], 1u << (w1 & 31u));
                }
            }
        }
        // totals
        cnt0 = __reduce_add_sync(0xffffffffu, cnt0);
        cnt1 = __reduce_add_sync(0xffffffffu, cnt1);
        cnt2 = __reduce_add_sync(0xffffffffu, cnt2);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&ntot[0], cnt0);
            atomicAdd(&ntot[1], cnt1);
            atomicAdd(&ntot[2], cnt2);
        }
        __syncthreads();
        if (threadIdx.x < 3 && ntot[threadIdx.x]) atomicAdd(&a.tot[p * 4 + threadIdx.x], ntot[threadIdx.x]);
        __syncthreads();
    }
}

// Candidates of the seen (K-1)-mers of one word of the seen bitmap (32
// consecutive (K-1)-mers): |R(m)| = popc(ext_mask(m)) for each seen q = a.m.
__device__ __forceinline__ uint32_t word_candidates(const BuildArgs &a, int p, uint32_t q0,
                                                    uint32_t bits) {
    uint32_t s = 0;
    while (bits) {
        const uint32_t j = __ffs(bits) - 1;
        bits &= bits - 1;
        s += __popc(ext_mask(a, p, a.fdT2.mod(q0 + j)));
    }
    return s;
}

// Candidates per chunk of CHUNK_THREADS * wpt bitmap words (wpt consecutive
// words per thread: 4 for the sparse bitmaps of compact (K-1)-mer tables, else 1).
// grid = (NCH, B)
__global__ void __launch_bounds__(CHUNK_THREADS) k_cand_count(BuildArgs a) {
    const int p = blockIdx.y, c = blockIdx.x;
    const uint64_t nw = a.T1s / 32;
    const uint64_t wd0 = ((uint64_t)c * CHUNK_THREADS + threadIdx.x) * a.wpt;
    uint32_t s = 0;
    for (uint32_t i = 0; i < a.wpt; i++) {
        const uint64_t wd = wd0 + i;
        if (wd >= nw) break;
        const uint32_t bits = a.seen1[(uint64_t)p * nw + wd];
        const uint32_t sw = bits ? word_candidates(a, p, (uint32_t)(wd * 32), bits) : 0u;
        a.word_cand[(uint64_t)p * nw + wd] = sw;
        s += sw;
    }
    s = __reduce_add_sync(0xffffffffu, s);
    __shared__ uint32_t ws[CHUNK_THREADS / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < CHUNK_THREADS / 32; w++) t += ws[w];
        a.chunk_cand[(uint64_t)p * a.NCH + c] = t;
    }
}

constexpr int MAX_WPT = 8;  // bitmap words per thread of the chunk kernels, at most

__device__ __forceinline__ uint32_t warp_incl_scan_u32(uint32_t v) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= (uint32_t)d) v += o;
    }
    return v;
}

// The lowest lane k whose (non-decreasing) inclusive scan value incl exceeds i;
// 31 when none does.
__device__ __forceinline__ uint32_t warp_owner(uint32_t incl, uint32_t i) {
    uint32_t k = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        const uint32_t v = __shfl_sync(0xffffffffu, incl, (int)(k + step - 1));
        if (v <= i) k += step;
    }
    return k;
}

// coff[p][q] = candidate offset of seen (K-1)-mer q within proteome p (entries
// of unseen q are not written); cq = the key q * A + b of every candidate (b over
// the right-extension mask of q's suffix, ascending), c0a zeroed.  Thread t of
// the block owns bitmap words [(c * CHUNK_THREADS + t) * wpt, + wpt) and its
// candidates start at the exclusive scan of the word_cand sums; a warp's 32
// threads own a contiguous run of words and candidates, which the warp
// processes together: its seen (K-1)-mers, 32 at a time in order (each lane
// finds its own by a search over the scan of the words' populations), load
// their masks together; a warp scan of the mask populations places their
// candidates, each lane writes its candidates into the warp's shared-memory stage
// at that offset, and the warp stores the stage coalesced.  (One lane per word,
// each writing its word's
// 0..32 A candidates, left most lanes idle; a warp per word wasted its scans on
// the sparse words of K = 7; finding each key's (K-1)-mer by a search over the
// scan cost about three times the instructions of the stage.)
// grid = (NCH, B)
__global__ void __launch_bounds__(CHUNK_THREADS) k_cand_offsets(BuildArgs a) {
    __shared__ uint64_t sw[CHUNK_THREADS / 32 + 1];
    __shared__ uint32_t s_stage[CHUNK_THREADS / 32][32 * 21];  // keys of 32 seen (K-1)-mers (A <= 21)
    uint32_t *stage = s_stage[threadIdx.x >> 5];
    const int p = blockIdx.y, c = blockIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t pc = (uint64_t)p * a.NCH + c;
    const uint64_t nw = a.T1s / 32;
    const uint32_t *seen = a.seen1 + (uint64_t)p * nw;
    const uint64_t wd0 = ((uint64_t)c * CHUNK_THREADS + threadIdx.x) * a.wpt;
    uint32_t s = 0;
    for (uint32_t i = 0; i < a.wpt && wd0 + i < nw; i++) s += a.word_cand[(uint64_t)p * nw + wd0 + i];
    uint64_t tot;
    const uint64_t ex = block_excl_scan_u64<CHUNK_THREADS>(s, sw, &tot);
    const uint32_t run0 =
        (uint32_t)(a.chunk_cand_off[pc] - a.chunk_cand_off[(uint64_t)p * a.NCH] + ex);
    const uint64_t gb = a.cbase[p];
    uint32_t run = __shfl_sync(0xffffffffu, run0, 0);
    const uint32_t r1 = __shfl_sync(0xffffffffu, run0 + s, 31);
    // zero this warp's K-mer count slots (coalesced)
    for (uint64_t i = gb + run + lane; i < gb + r1 && i < a.cand_cap; i += 32) a.c0a[i] = 0u;
    // the warp's words [wbeg, wend), loaded up front (coalesced), lane l holding word
    // wbeg + 32 t + l of group t; the seen (K-1)-mers of a group are taken 32 at a time
    const uint64_t wbeg = __shfl_sync(0xffffffffu, wd0, 0);
    const uint64_t wend = min(wbeg + (uint64_t)32 * a.wpt, nw);
    const uint32_t A = a.A;
    uint32_t wreg[MAX_WPT];
#pragma unroll
    for (int t = 0; t < MAX_WPT; t++) {
        const uint64_t w = wbeg + 32 * t + lane;
        wreg[t] = ((uint32_t)t < a.wpt && w < wend) ? seen[w] : 0u;
    }
#pragma unroll
    for (int t = 0; t < MAX_WPT; t++) {
        if ((uint32_t)t >= a.wpt) break;
        const uint32_t wbits = wreg[t];
        const uint32_t wincl = warp_incl_scan_u32(__popc(wbits));
        const uint32_t nseen = __shfl_sync(0xffffffffu, wincl, 31);
        if (nseen == 0u) continue;
        const uint64_t wfirst = wbeg + 32 * t;
        // compact tables: the rank of the group's first seen (K-1)-mer; the i-th seen
        // (K-1)-mer of the group is then entry P + i
        const uint64_t P = a.compact1 ? (uint64_t)a.pw1[(uint64_t)p * nw + wfirst].x : 0;
        for (uint32_t sb = 0; sb < nseen; sb += 32) {
            const uint32_t i = sb + lane;
            const uint32_t k = warp_owner(wincl, i);
            const uint32_t wk = __shfl_sync(0xffffffffu, wbits, (int)k);
            const uint32_t ik = __shfl_sync(0xffffffffu, wincl, (int)k);
            const bool ok = i < nseen;
            uint32_t q = 0, mask = 0;
            if (ok) {
                q = (uint32_t)((wfirst + k) * 32) + nth_set_bit(wk, i - (ik - (uint32_t)__popc(wk)));
                mask = ext_mask(a, p, a.fdT2.mod(q));
            }
            const uint32_t n = __popc(mask);
            const uint32_t cincl = warp_incl_scan_u32(n);
            const uint32_t ctot = __shfl_sync(0xffffffffu, cincl, 31);
            // every seen (K-1)-mer, also one without candidates: its offset (the next
            // candidate's) and, with compact tables, its count slot (counted by
            // k_c0_scatter)
            if (ok) {
                const uint64_t qi = a.compact1 ? P + i : c1_index(a, p, q);
                if (!a.compact1 || qi < a.cap1) {
                    a.coff[qi] = run + cincl - n;
                    if (a.compact1) a.c1[qi] = 0u;
                }
            }
            // their candidate keys: each lane writes its own (at most A) into the warp's
            // stage at its scanned offset, then the warp stores them coalesced
            {
                uint32_t e = mask, o = cincl - n;
                while (e) {
                    stage[o++] = q * A + (uint32_t)(__ffs(e) - 1);
                    e &= e - 1;
                }
            }
            __syncwarp();
            for (uint32_t ci = lane; ci < ctot; ci += 32) {
                const uint64_t dst = gb + run + ci;
                if (dst < a.cand_cap) a.cq[dst] = stage[ci];
            }
            __syncwarp();
            run += ctot;
        }
    }
}

// cbase[p] = start of proteome p's candidates, rounded up to ALPHA_TILE, so that
// no k_alpha CTA straddles two proteomes.  One thread.
__global__ void k_cand_bases(BuildArgs a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint64_t run = 0;
    for (int p = 0; p < a.B; p++) {
        a.cbase[p] = run;
        const uint64_t n =
            a.chunk_cand_off[(uint64_t)(p + 1) * a.NCH] - a.chunk_cand_off[(uint64_t)p * a.NCH];
        run += div_up(n, (uint64_t)ALPHA_TILE) * ALPHA_TILE;
    }
    a.cbase[a.B] = run;
    *a.cand_total = run;
    if (run > a.cand_cap) atomicOr(a.status, (uint32_t)DEV_CAPACITY);
    if (a.compact1 && *a.p1_total > a.cap1) atomicOr(a.status, (uint32_t)DEV_CAPACITY);
    if (a.compact2 && *a.p2_total > a.cap2) atomicOr(a.status, (uint32_t)DEV_CAPACITY);
}

// Every K-window adds one to the slot of its candidate (native.cu:244); with
// compact (K-1)-mer tables every (K-1)-window also adds one to its count.  A
// thread's windows go through the dependent steps together (codes, rank loads,
// counts, offsets and masks, slot atomics), so their loads are in flight at once.
// The L2 atomics, not those loads, set the pace: the same kernel with four windows
// per thread instead of two measured no faster.
__global__ void __launch_bounds__(COUNT_THREADS) k_c0_scatter(BuildArgs a) {
    __shared__ uint8_t dig[TILE + 16];
    const int K = a.k;
    const uint32_t A = a.A;
    const uint64_t total_tiles = a.tile_base[a.B];
    for (uint64_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
        const int p = find_owner(a.tile_base, a.B, t);
        const uint64_t s0 = a.seq_off[p], len = a.seq_off[p + 1] - s0;
        const uint64_t start = (t - a.tile_base[p]) * TILE;
        for (int j = threadIdx.x; j < TILE + K; j += COUNT_THREADS) {
            uint64_t pos = start + j;
            dig[j] = pos < len ? (uint8_t)char_to_digit(a.alpha, a.seq[s0 + pos]) : (uint8_t)0xff;
        }
        __syncthreads();
        const uint64_t cbase = a.cbase[p];
        constexpr int NU = TILE / COUNT_THREADS;
        // phase 1: every window's (K-1)- and (K-2)-mer codes from the staged digits
        uint32_t w[NU], w2[NU], bd[NU];
        int jj[NU];
#pragma unroll
        for (int u = 0; u < NU; u++) {
            const int li = u * COUNT_THREADS + threadIdx.x;
            w[u] = 0;
            w2[u] = 0;
            bd[u] = 0xffu;
            jj[u] = -1;
            if (start + li < len) {
                uint32_t x = 0, x2 = 0;
                int j;
                for (j = 0; j < K - 1; j++) {
                    if (j == K - 2) x2 = x;
                    uint32_t d = dig[li + j];
                    if (d == 0xffu) break;
                    x = x * A + d;
                }
                w[u] = x;
                w2[u] = x2;
                jj[u] = j;
                bd[u] = dig[li + K - 1];
            }
        }
        // phase 2: all rank loads in flight together
        uint64_t wi[NU], mi[NU];
#pragma unroll
        for (int u = 0; u < NU; u++) {
            wi[u] = jj[u] == K - 1 ? c1_index(a, p, w[u]) : ~0ull;
            mi[u] = (a.compact2 && jj[u] >= K - 2) ? c2_index(a, p, w2[u]) : ~0ull;
        }
        // phase 3: counts, then the candidate offsets and extension masks together
        uint32_t co[NU], em[NU];
#pragma unroll
        for (int u = 0; u < NU; u++) {
            co[u] = 0;
            em[u] = 0;
            if (mi[u] < a.cap2) atomicAdd(&a.c2[mi[u]], 1u);
            if (wi[u] != ~0ull) {
                const bool in_cap = !a.compact1 || wi[u] < a.cap1;
                if (a.compact1 && in_cap) atomicAdd(&a.c1[wi[u]], 1u);
                if (!in_cap || bd[u] == 0xffu) wi[u] = ~0ull;
            }
        }
#pragma unroll
        for (int u = 0; u < NU; u++) {
            if (wi[u] != ~0ull) {
                co[u] = __ldg(&a.coff[wi[u]]);
                em[u] = ext_mask(a, p, a.fdT2.mod(w[u]));
            }
        }
#pragma unroll
        for (int u = 0; u < NU; u++) {
            if (wi[u] != ~0ull) {
                const uint64_t slot = cbase + co[u] + __popc(em[u] & ((1u << bd[u]) - 1u));
                if (slot < a.cand_cap) atomicAdd(&a.c0a[slot], 1u);
            }
        }
        __syncthreads();
    }
}

// Markov alpha of every candidate (alpha bits replace the count, as
// native.cu:399 does), flat over the batch's candidate index space: CTA c takes
// candidates [c * ALPHA_TILE, (c + 1) * ALPHA_TILE) of one proteome, warp w the
// segment of SEG candidates starting at c * ALPHA_TILE + w * SEG.  In place: a
// seen candidate's c0a slot receives its alpha bits (or TUPLE_TAG | tuple), or
// CAND_DROP when alpha is 0 (not written out); an unseen one keeps count 0 and
// stands for alpha -1.  seg_surv = survivors per segment.  Per-CTA norm
// partials.  grid = cand_cap / ALPHA_TILE
//
// Most candidates are K-mers that were not seen (count 0): their alpha is -1
// (native.cu:392 with p = 0) and needs no table loads.  The others are listed
// per warp in shared memory and computed densely, 32 lanes on 32 of them, so
// the long path does not run with most lanes idle.
constexpr int ALPHA_ILP = 1;  // listed candidates per lane in flight together
// c0a value of a seen candidate whose alpha is 0: not written out.  No tuple tag
// (tuple indices stay below TUPLE_TABLE) and no alpha (arithmetic NaNs are
// 0x7fffffff) has these bits.
constexpr uint32_t CAND_DROP = 0xffffffffu;
__global__ void __launch_bounds__(CHUNK_THREADS, 6) k_alpha(BuildArgs a) {
    __shared__ U192 s_norm[CHUNK_THREADS / 32];
    __shared__ uint32_t s_m1[CHUNK_THREADS / 32], s_bad[CHUNK_THREADS / 32];
    __shared__ uint32_t s_lcnt[CHUNK_THREADS / 32][SEG];   // listed candidates: K-mer count,
    __shared__ uint16_t s_lidx[CHUNK_THREADS / 32][SEG];   // index in the segment
    const uint64_t c = blockIdx.x;
    const uint64_t g0 = c * ALPHA_TILE;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t seg = c * (ALPHA_TILE / SEG) + w;
    const uint64_t total = min(*a.cand_total, a.cand_cap);
    if (g0 >= total) {  // past the last proteome
        if (lane == 0) a.seg_surv[seg] = 0;
        if (threadIdx.x == 0) {
            a.cta_m1[c] = 0;
            a.cta_bad[c] = 0;
            a.cta_norm[3 * c] = a.cta_norm[3 * c + 1] = a.cta_norm[3 * c + 2] = 0;
        }
        return;
    }
    const int p = find_owner(a.cbase, a.B, g0);
    const uint32_t np =
        (uint32_t)(a.chunk_cand_off[(uint64_t)(p + 1) * a.NCH] - a.chunk_cand_off[(uint64_t)p * a.NCH]);
    const double *prob = a.prob + (uint64_t)p * 4 * PROB_TABLE;
    const uint32_t *atab = a.atab + (uint64_t)p * TUPLE_TABLE;
    const uint32_t n0 = a.tot[p * 4 + 0], n1 = a.tot[p * 4 + 1], n2 = a.tot[p * 4 + 2];
    const uint32_t A = a.A;
    const uint64_t sbase = g0 + (uint64_t)w * SEG;           // this warp's segment
    const uint32_t loc0 = (uint32_t)(sbase - a.cbase[p]);    // proteome-local index of its start
    U192 acc = {0, 0, 0};
    uint32_t m1 = 0, bad = 0, ndrop = 0;
    constexpr int NI = SEG / 32;  // candidates per lane
    // phase 1: K-mer counts of the whole segment; candidates that need the long path
    // (a seen K-mer, or a proteome without K-windows) are listed
    uint32_t fl[NI];
#pragma unroll
    for (int i = 0; i < NI; i++) {
        const bool ok = loc0 + 32 * i + lane < np;
        fl[i] = ok ? a.c0a[sbase + 32 * i + lane] : 0u;
    }
    uint32_t nlist = 0, nok = 0;
#pragma unroll
    for (int i = 0; i < NI; i++) {
        const bool ok = loc0 + 32 * i + lane < np;
        const bool need = ok && (fl[i] != 0u || n0 == 0u);
        if (ok && !need) m1++;  // an unseen K-mer: alpha -1, square 1
        nok += ok;
        const unsigned bal = __ballot_sync(0xffffffffu, need);
        if (need) {
            const uint32_t pos = nlist + __popc(bal & ((1u << lane) - 1u));
            s_lcnt[w][pos] = fl[i];
            s_lidx[w][pos] = (uint16_t)(32 * i + lane);
        }
        nlist += __popc(bal);
    }
    __syncwarp();
    // phase 2: the listed candidates, ALPHA_ILP per lane with their loads in flight together
    for (uint32_t t0 = 0; t0 < nlist; t0 += 32 * ALPHA_ILP) {
        uint32_t key[ALPHA_ILP], full[ALPHA_ILP], pre[ALPHA_ILP], mid[ALPHA_ILP], suf[ALPHA_ILP];
#pragma unroll
        for (int j = 0; j < ALPHA_ILP; j++) {
            const uint32_t t = t0 + 32 * j + lane;
            const bool ok = t < nlist;
            key[j] = ok ? a.cq[sbase + s_lidx[w][t]] : 0u;
            full[j] = ok ? s_lcnt[w][t] : 0u;
            const uint32_t q = A == 21u ? key[j] / 21u : key[j] >> 2;  // protein or DNA alphabet
            const uint32_t b = key[j] - q * A;
            const uint32_t m = a.fdT2.mod(q);
            const bool seen = ok && full[j] != 0u;
            pre[j] = seen ? __ldg(&a.c1[c1_index(a, p, q)]) : 0u;
            const uint64_t mi = seen ? c2_index(a, p, m) : 0;
            mid[j] = seen && (!a.compact2 || mi < a.cap2) ? __ldg(&a.c2[mi]) : 0u;
            suf[j] = seen ? __ldg(&a.c1[c1_index(a, p, m * A + b)]) : 0u;
        }
#pragma unroll
        for (int j = 0; j < ALPHA_ILP; j++) {
            const uint32_t t = t0 + 32 * j + lane;
            if (t >= nlist) continue;
            uint32_t stored;
            float f;
            if (full[j] - 1u < 3u && pre[j] < (uint32_t)TUPLE_PS && suf[j] < (uint32_t)TUPLE_PS &&
                mid[j] < (uint32_t)TUPLE_MID && n0 != 0u) {
                const uint32_t ti =
                    ((full[j] * TUPLE_PS + pre[j]) * TUPLE_PS + suf[j]) * TUPLE_MID + mid[j];
                const uint32_t tb = __ldg(&atab[ti]);
                f = __uint_as_float(tb);
                stored = tb ? (TUPLE_TAG | ti) : 0u;
            } else {
                f = markov_alpha_fast(full[j], pre[j], suf[j], mid[j], n0, n1, n2, prob);
                stored = __float_as_uint(f);
            }
            // in place: the alpha bits (or tuple tag), or CAND_DROP for alpha 0
            a.c0a[sbase + s_lidx[w][t]] = stored ? stored : CAND_DROP;
            ndrop += stored == 0u;
            if (__float_as_uint(f) != 0u) {
                const float sq = __fmul_rn(f, f);  // float square, as native.cu:421-423
                if (sq == 1.0f) m1++;
                else if (isnan(sq)) bad |= 1u;
                else if (isinf(sq) || !u192_add_float(acc, sq)) bad |= 2u;
            }
        }
    }
    // phase 3: survivors of the segment (k_compact copies them out in place order)
    const uint32_t nsurv = __reduce_add_sync(0xffffffffu, nok - ndrop);
    if (lane == 0) a.seg_surv[seg] = nsurv;
    // norm partials (integer: exact and order independent)
    m1 = __reduce_add_sync(0xffffffffu, m1);
    bad = __reduce_or_sync(0xffffffffu, bad);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const U192 o = u192_shfl_down(acc, d);
        u192_add(acc, o.w0, o.w1, o.w2);
    }
    if (lane == 0) {
        s_norm[w] = acc; s_m1[w] = m1; s_bad[w] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        U192 t = {0, 0, 0};
        uint32_t tm = 0, tb = 0;
        for (int i = 0; i < CHUNK_THREADS / 32; i++) {
            u192_add(t, s_norm[i].w0, s_norm[i].w1, s_norm[i].w2);
            tm += s_m1[i];
            tb |= s_bad[i];
        }
        a.cta_m1[c] = tm;
        a.cta_bad[c] = tb;
        a.cta_norm[3 * c + 0] = t.w0;
        a.cta_norm[3 * c + 1] = t.w1;
        a.cta_norm[3 * c + 2] = t.w2;
    }
}

// Per proteome: norm = exact sum of the squares rounded once to double
// (native.cu:415-428 sums the same float squares in double, in CUB's order),
// scale = sqrt(norm), its reciprocal, nnz, output base.  grid = B, NORM_THREADS
// threads (the CTA partials of a proteome summed exactly, in any order).
constexpr int NORM_THREADS = 256;
__global__ void __launch_bounds__(NORM_THREADS) k_norm(BuildArgs a) {
    __shared__ U192 s_acc[NORM_THREADS / 32];
    __shared__ uint64_t s_m1[NORM_THREADS / 32];
    __shared__ uint32_t s_bad[NORM_THREADS / 32];
    const int p = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t ncta = a.cand_cap / ALPHA_TILE, nseg = a.cand_cap / SEG;
    const uint64_t c0 = min(a.cbase[p] / ALPHA_TILE, ncta);
    const uint64_t c1 = min(a.cbase[p + 1] / ALPHA_TILE, ncta);
    U192 acc = {0, 0, 0};
    uint64_t m1 = 0;
    uint32_t bad = 0;
    for (uint64_t c = c0 + threadIdx.x; c < c1; c += NORM_THREADS) {
        u192_add(acc, a.cta_norm[3 * c], a.cta_norm[3 * c + 1], a.cta_norm[3 * c + 2]);
        m1 += a.cta_m1[c];
        bad |= a.cta_bad[c];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const U192 o = u192_shfl_down(acc, d);
        u192_add(acc, o.w0, o.w1, o.w2);
        m1 += __shfl_down_sync(0xffffffffu, m1, d);
    }
    bad = __reduce_or_sync(0xffffffffu, bad);
    if (lane == 0) {
        s_acc[warp] = acc;
        s_m1[warp] = m1;
        s_bad[warp] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        acc = s_acc[0];
        m1 = s_m1[0];
        bad = s_bad[0];
        for (int w = 1; w < NORM_THREADS / 32; w++) {
            u192_add(acc, s_acc[w].w0, s_acc[w].w1, s_acc[w].w2);
            m1 += s_m1[w];
            bad |= s_bad[w];
        }
        // each unit square adds 1.0 = 2^96 units: bit 32 of the middle word
        u192_add(acc, 0, m1 << 32, m1 >> 32);
        double norm = u192_to_double(acc);
        if (bad & 1u) norm = __longlong_as_double(0x7ff8000000000000ll);
        else if (bad & 2u) norm = __longlong_as_double(0x7ff0000000000000ll);
        const double scale = __dsqrt_rn(norm);
        a.norm[p] = norm;
        a.scale[p] = scale;
        a.rscale[p] = __ddiv_rn(1.0, scale);
        const uint64_t o0 = a.seg_out_off[min(a.cbase[p] / SEG, nseg)];
        const uint64_t o1 = a.seg_out_off[min(a.cbase[p + 1] / SEG, nseg)];
        a.nnz[p] = o1 - o0;
        a.out_base[p] = o0;
    }
}

// Marks in the key bitmap, for every seen (K-1)-mer q of the batch, the keys
// q * A + b of its candidates (b over the right-extension mask of q's suffix):
// one or two atomics per seen (K-1)-mer instead of one per written key.  The
// marked set is a superset of the written keys (a candidate whose alpha is 0 is
// marked but not written), which is all a key-rank bitmap needs: ranks stay
// strictly increasing over the written keys.  grid = (NCH, B)
__global__ void __launch_bounds__(CHUNK_THREADS) k_union_mark(BuildArgs a) {
    const int p = blockIdx.y, c = blockIdx.x;
    const uint64_t nw = a.T1s / 32;
    const uint64_t wd0 = ((uint64_t)c * CHUNK_THREADS + threadIdx.x) * a.wpt;
    for (uint32_t i = 0; i < a.wpt; i++) {
        const uint64_t wd = wd0 + i;
        if (wd >= nw) break;
        uint32_t bits = a.seen1[(uint64_t)p * nw + wd];
        while (bits) {
            const uint32_t q = (uint32_t)(wd * 32) + (uint32_t)(__ffs(bits) - 1);
            bits &= bits - 1;
            const uint32_t m = ext_mask(a, p, a.fdT2.mod(q));
            if (!m) continue;
            const uint64_t bit = (uint64_t)q * a.A;
            const uint64_t w = bit >> 5;
            const uint32_t off = (uint32_t)bit & 31u;
            atomicOr(&a.union_bits[w], m << off);
            if (off + a.A > 32u && (m >> (32u - off))) atomicOr(&a.union_bits[w + 1], m >> (32u - off));
        }
    }
}

// Copies every segment's survivors to the output, in key order: keys and
// float(alpha / scale) (native.cu:460-468).  A candidate with count 0 is an
// unseen K-mer (alpha -1); one marked CAND_DROP had alpha 0 and is skipped.  The
// division by the per-proteome constant scale uses its correctly rounded
// reciprocal and one FMA correction (Markstein), which yields the correctly
// rounded double quotient.  grid = cand_cap / ALPHA_TILE
__global__ void __launch_bounds__(CHUNK_THREADS) k_compact(BuildArgs a) {
    __shared__ uint64_t s_base[SMEM_BASES + 1];
    const uint64_t c = blockIdx.x, g0 = c * ALPHA_TILE;
    if (g0 >= min(*a.cand_total, a.cand_cap)) return;
    const uint64_t *cb = stage_bases(a.cbase, a.B, s_base);
    const int p = find_owner(cb, a.B, g0);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t seg = c * (ALPHA_TILE / SEG) + w;
    if (a.seg_surv[seg] == 0) return;
    const uint64_t src = seg * SEG;
    const uint32_t np =
        (uint32_t)(a.chunk_cand_off[(uint64_t)(p + 1) * a.NCH] - a.chunk_cand_off[(uint64_t)p * a.NCH]);
    const uint32_t loc0 = (uint32_t)(src - cb[p]);
    const uint32_t nc = loc0 < np ? min((uint32_t)SEG, np - loc0) : 0u;  // its candidates
    const uint64_t dst = a.dst_base[p] + (a.seg_out_off[seg] - a.out_base[p]);
    const uint64_t dst_end = a.dst_base[p] + a.dst_cap[p];
    const double scale = a.scale[p];
    const double rs = a.rscale[p];
    const float *vtab = a.vtab + (uint64_t)p * TUPLE_TABLE;
    const bool finite = isfinite(scale) && scale > 0.0;
    const float vm1 = __double2float_rn(-rs);  // RN(-1/scale) == -RN(1/scale)
    // four candidates per lane in flight: loads first, then the stores
    constexpr int U = 4;
    uint32_t out = 0;  // survivors written so far
    for (uint32_t i0 = 0; i0 < nc; i0 += 32 * U) {
        uint32_t bits[U], key[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint32_t i = i0 + 32 * u + lane;
            bits[u] = i < nc ? a.c0a[src + i] : CAND_DROP;
            key[u] = i < nc ? a.cq[src + i] : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const bool surv = bits[u] != CAND_DROP;
            const unsigned bal = __ballot_sync(0xffffffffu, surv);
            if (surv) {
                float v;
                if (bits[u] == 0u) {
                    v = vm1;  // unseen K-mer: alpha -1
                } else if ((bits[u] & TUPLE_TAG) == TUPLE_TAG) {
                    v = __ldg(&vtab[bits[u] & ~TUPLE_TAG]);
                } else {
                    const float f = __uint_as_float(bits[u]);
                    if (!finite || !isfinite(f)) v = __double2float_rn(__ddiv_rn((double)f, scale));
                    else if (f == -1.0f) v = vm1;
                    else v = div_by_scale(f, scale, rs);
                }
                const uint64_t o = dst + out + __popc(bal & ((1u << lane) - 1u));
                if (o < dst_end) {
                    a.out_keys[o] = key[u];
                    a.out_vals[o] = v;
                }
            }
            out += __popc(bal);
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

int build_geometry(int alpha, int k, BuildGeometry *g) {
    if (alpha != ALPHA_PROTEIN && alpha != ALPHA_DNA) return -1;
    if (k < 3 || k > 10) return -1;
    const uint64_t A = alphabet_size(alpha);
    if (ipow64(A, k) > 0xffffffffull) return -2;  // keys must fit uint32
    g->alpha = alpha;
    g->k = k;
    g->A = (uint32_t)A;
    g->T1 = ipow64(A, k - 1);
    g->T1s = (g->T1 + 31) / 32 * 32;  // whole words of the seen bitmap
    g->T2 = ipow64(A, k - 2);
    g->T2s = (g->T2 + 31) / 32 * 32;
    g->wpt = g->T1s > (1ull << 24) ? MAX_WPT : 1;  // sparse bitmaps: eight words per thread
    g->NCH = div_up(g->T1s / 32, (uint64_t)CHUNK_THREADS * g->wpt);
    return 0;
}

// (K-1)-mer tables beyond 2^20 entries per proteome (protein K >= 6) are kept
// compact: one entry per seen (K-1)-mer instead of a dense row.  A batch's
// dense rows (16 MB per proteome at K = 6) would live in DRAM, so every
// (K-1)-window's count would be a DRAM atomic; the compact entries of a batch
// stay in L2, and the zeroing of the dense rows goes away.
static bool compact1_tables(const BuildGeometry &g) { return g.T1s > (1ull << 20); }
// (K-2)-mer counts likewise beyond 2^20 entries (protein K = 7: 16 MB per proteome).
static bool compact2_tables(const BuildGeometry &g) { return g.T2s > (1ull << 20); }

// Candidate capacity rounded up to whole k_alpha CTAs.
static uint64_t cand_cap_rounded(uint64_t cand_cap) {
    return div_up(cand_cap ? cand_cap : 1, (uint64_t)ALPHA_TILE) * ALPHA_TILE;
}

size_t build_scratch_bytes(const BuildGeometry &g, int B, uint64_t cand_cap) {
    const uint64_t nc = (uint64_t)B * g.NCH;
    const uint64_t cap = cand_cap_rounded(cand_cap);
    const uint64_t ncta = cap / ALPHA_TILE, nseg = cap / SEG;
    size_t s = 0;
    const bool compact = compact1_tables(g);
    const uint64_t n1 = compact ? cap : g.T1s * B;  // entries of c1 / coff
    const uint64_t nw1 = g.T1s / 32 * B;
    s += scratch_bytes<uint32_t>(n1);              // c1
    s += scratch_bytes<uint32_t>(n1);              // coff
    s += scratch_bytes<uint2>(compact ? nw1 : 0);                           // pw1
    s += scratch_bytes<uint64_t>(compact ? bitmap_prefix_partials(nw1) : 0);  // p1_partials
    s += scratch_bytes<uint64_t>(1);               // p1_total
    s += scratch_bytes<uint32_t>(g.T1s / 32 * B);  // seen1
    s += scratch_bytes<uint32_t>(g.T1s / 32 * B);  // word_cand
    const bool compact2 = compact2_tables(g);
    const uint64_t nw2 = g.T2s / 32 * B;
    s += scratch_bytes<uint32_t>(compact2 ? cap : g.T2 * B);                    // c2
    s += scratch_bytes<uint32_t>(compact2 ? nw2 : 0);                           // seen2
    s += scratch_bytes<uint2>(compact2 ? nw2 : 0);                              // pw2
    s += scratch_bytes<uint64_t>(compact2 ? bitmap_prefix_partials(nw2) : 0);  // p2_partials
    s += scratch_bytes<uint64_t>(1);                                            // p2_total
    s += scratch_bytes<uint32_t>(4 * (uint64_t)B); // tot
    s += scratch_bytes<uint64_t>(B + 1);           // seq_off (single-proteome path)
    s += scratch_bytes<uint64_t>(B + 1);           // tile_base
    s += scratch_bytes<uint32_t>(nc);              // chunk_cand
    s += scratch_bytes<uint64_t>(nc + 1);          // chunk_cand_off
    s += scratch_bytes<uint64_t>(B + 1);           // cbase
    s += scratch_bytes<uint64_t>(1);               // cand_total
    s += scratch_bytes<uint32_t>(nseg);            // seg_surv
    s += scratch_bytes<uint64_t>(nseg + 1);        // seg_out_off
    s += scratch_bytes<uint32_t>(ncta);            // cta_m1
    s += scratch_bytes<uint64_t>(3 * ncta);        // cta_norm
    s += scratch_bytes<uint32_t>(ncta);            // cta_bad
    s += scratch_bytes<double>(4 * (uint64_t)PROB_TABLE * B);  // prob tables
    s += scratch_bytes<uint32_t>((uint64_t)TUPLE_TABLE * B);   // atab
    s += scratch_bytes<float>((uint64_t)TUPLE_TABLE * B);      // vtab
    s += scratch_bytes<uint64_t>(scan_temp_bytes(max(nc, nseg) + 1) / 8 + 1);  // scan temp
    s += scratch_bytes<double>(B);                 // norm
    s += scratch_bytes<double>(B);                 // scale
    s += scratch_bytes<double>(B);                 // rscale
    s += scratch_bytes<uint64_t>(B);               // nnz
    s += scratch_bytes<uint64_t>(B);               // out_base
    s += scratch_bytes<uint64_t>(B);               // dst_base
    s += scratch_bytes<uint64_t>(B);               // dst_cap
    s += scratch_bytes<uint32_t>(4);               // status
    s += scratch_bytes<uint32_t>(cap);             // c0a
    s += scratch_bytes<uint32_t>(cap);             // cq
    return s;
}

cudaError_t build_carve(const BuildGeometry &g, int B, uint64_t cand_cap, void *scratch,
                        size_t scratch_size, BuildArgs *a) {
    Scratch sc(scratch, scratch_size);
    const uint64_t nc = (uint64_t)B * g.NCH;
    const uint64_t cap = cand_cap_rounded(cand_cap);
    const uint64_t ncta = cap / ALPHA_TILE, nseg = cap / SEG;
    BuildArgs &r = *a;
    r.alpha = g.alpha; r.k = g.k; r.A = g.A; r.T1 = g.T1; r.T2 = g.T2; r.NCH = g.NCH; r.B = B;
    r.wpt = g.wpt;
    r.T1s = g.T1s;
    const bool compact = compact1_tables(g);
    const uint64_t n1 = compact ? cap : g.T1s * B;
    const uint64_t nw1 = g.T1s / 32 * B;
    r.compact1 = compact ? 1 : 0;
    r.cap1 = n1;
    r.c1 = sc.take<uint32_t>(n1);
    r.coff = sc.take<uint32_t>(n1);
    r.pw1 = sc.take<uint2>(compact ? nw1 : 0);
    r.p1_partials = sc.take<uint64_t>(compact ? bitmap_prefix_partials(nw1) : 0);
    r.p1_total = sc.take<uint64_t>(1);
    r.seen1 = sc.take<uint32_t>(g.T1s / 32 * B);
    r.word_cand = sc.take<uint32_t>(g.T1s / 32 * B);
    const bool compact2 = compact2_tables(g);
    const uint64_t nw2 = g.T2s / 32 * B;
    r.compact2 = compact2 ? 1 : 0;
    r.cap2 = compact2 ? cap : g.T2 * B;
    r.T2s = g.T2s;
    r.c2 = sc.take<uint32_t>(r.cap2);
    r.seen2 = sc.take<uint32_t>(compact2 ? nw2 : 0);
    r.pw2 = sc.take<uint2>(compact2 ? nw2 : 0);
    r.p2_partials = sc.take<uint64_t>(compact2 ? bitmap_prefix_partials(nw2) : 0);
    r.p2_total = sc.take<uint64_t>(1);
    r.tot = sc.take<uint32_t>(4 * (uint64_t)B);
    r.seq_off_store = sc.take<uint64_t>(B + 1);
    r.tile_base = sc.take<uint64_t>(B + 1);
    r.chunk_cand = sc.take<uint32_t>(nc);
    r.chunk_cand_off = sc.take<uint64_t>(nc + 1);
    r.cbase = sc.take<uint64_t>(B + 1);
    r.cand_total = sc.take<uint64_t>(1);
    r.seg_surv = sc.take<uint32_t>(nseg);
    r.seg_out_off = sc.take<uint64_t>(nseg + 1);
    r.cta_m1 = sc.take<uint32_t>(ncta);
    r.cta_norm = sc.take<uint64_t>(3 * ncta);
    r.cta_bad = sc.take<uint32_t>(ncta);
    r.prob = sc.take<double>(4 * (uint64_t)PROB_TABLE * B);
    r.atab = sc.take<uint32_t>((uint64_t)TUPLE_TABLE * B);
    r.vtab = sc.take<float>((uint64_t)TUPLE_TABLE * B);
    r.fdT2.set((uint32_t)g.T2);
    r.scan_tmp = sc.take<uint64_t>(scan_temp_bytes(max(nc, nseg) + 1) / 8 + 1);
    r.norm = sc.take<double>(B);
    r.scale = sc.take<double>(B);
    r.rscale = sc.take<double>(B);
    r.nnz = sc.take<uint64_t>(B);
    r.out_base = sc.take<uint64_t>(B);
    r.dst_base = sc.take<uint64_t>(B);
    r.dst_cap = sc.take<uint64_t>(B);
    r.status = sc.take<uint32_t>(4);
    r.c0a = sc.take<uint32_t>(cap);
    r.cq = sc.take<uint32_t>(cap);
    r.cand_cap = cap;
    if (!r.cq) return cudaErrorInvalidValue;  // scratch too small
    return cudaSuccess;
}

// Phase 1: everything up to per-proteome nnz (no host sync inside).
cudaError_t build_plan(BuildArgs &a, cudaStream_t st) {
    const uint64_t nc = (uint64_t)a.B * a.NCH;
    // dense tables c1 | coff | c2 | tot are contiguous in scratch: zero what needs it
    if (!a.compact1) PHYLO_CHECK(cudaMemsetAsync(a.c1, 0, sizeof(uint32_t) * a.T1s * a.B, st));
    PHYLO_CHECK(cudaMemsetAsync(a.seen1, 0, sizeof(uint32_t) * (a.T1s / 32) * a.B, st));
    if (a.compact2) PHYLO_CHECK(cudaMemsetAsync(a.seen2, 0, sizeof(uint32_t) * (a.T2s / 32) * a.B, st));
    else PHYLO_CHECK(cudaMemsetAsync(a.c2, 0, sizeof(uint32_t) * a.T2 * a.B, st));
    PHYLO_CHECK(cudaMemsetAsync(a.tot, 0, sizeof(uint32_t) * 4 * a.B, st));
    PHYLO_CHECK(cudaMemsetAsync(a.status, 0, sizeof(uint32_t) * 4, st));
    k_prep<<<1, 32, 0, st>>>(a.B, a.seq_off, a.tile_base);
    const int grid_seq = device_sm_count() * 8;
    if (a.compact1) {
        k_count<true><<<grid_seq, COUNT_THREADS, 0, st>>>(a);
        PHYLO_CHECK(bitmap_prefix_pairs(a.seen1, a.T1s / 32 * a.B, a.p1_partials, a.pw1,
                                        a.p1_total, st));
    } else {
        k_count<false><<<grid_seq, COUNT_THREADS, 0, st>>>(a);
        PHYLO_CHECK(cudaMemsetAsync(a.p1_total, 0, sizeof(uint64_t), st));
    }
    if (a.compact2) {  // ranks of the seen (K-2)-mers; their counts (k_c0_scatter) start at 0
        PHYLO_CHECK(bitmap_prefix_pairs(a.seen2, a.T2s / 32 * a.B, a.p2_partials, a.pw2,
                                        a.p2_total, st));
        PHYLO_CHECK(cudaMemsetAsync(a.c2, 0, sizeof(uint32_t) * a.cap2, st));
    } else {
        PHYLO_CHECK(cudaMemsetAsync(a.p2_total, 0, sizeof(uint64_t), st));
    }
    k_tables<<<dim3(PROB_TABLE / 256, a.B), 256, 0, st>>>(a);
    k_tuple_alpha<<<dim3(TUPLE_TABLE / 256, a.B), 256, 0, st>>>(a);
    dim3 gch((unsigned)a.NCH, (unsigned)a.B);
    k_cand_count<<<gch, CHUNK_THREADS, 0, st>>>(a);
    PHYLO_CHECK(scan_u32_to_u64(a.chunk_cand, nc, a.chunk_cand_off, a.scan_tmp, st));
    k_cand_bases<<<1, 32, 0, st>>>(a);
    k_cand_offsets<<<gch, CHUNK_THREADS, 0, st>>>(a);
    k_c0_scatter<<<grid_seq, COUNT_THREADS, 0, st>>>(a);
    const unsigned ncta = (unsigned)(a.cand_cap / ALPHA_TILE);
    k_alpha<<<ncta, CHUNK_THREADS, 0, st>>>(a);
    PHYLO_CHECK(scan_u32_to_u64(a.seg_surv, a.cand_cap / SEG, a.seg_out_off, a.scan_tmp, st));
    k_norm<<<a.B, NORM_THREADS, 0, st>>>(a);
    k_tuple_value<<<dim3(TUPLE_TABLE / 256, a.B), 256, 0, st>>>(a);
    return cudaGetLastError();
}

// Phase 2: write survivors to out_keys/out_vals at dst_base[p] (capacity dst_cap[p]).
cudaError_t build_emit(BuildArgs &a, cudaStream_t st) {
    k_compact<<<(unsigned)(a.cand_cap / ALPHA_TILE), CHUNK_THREADS, 0, st>>>(a);
    if (a.union_bits)
        k_union_mark<<<dim3((unsigned)a.NCH, (unsigned)a.B), CHUNK_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

// Kernel counting per launch of build_plan + build_emit (for launch accounting).
// Kernels one batched Plan + Emit launches: plan k_prep, k_count, k_tables,
// k_tuple_alpha, k_cand_count, scan (3), k_cand_bases, k_cand_offsets,
// k_c0_scatter, k_alpha, scan (3), k_norm, k_tuple_value; emit
// k_arena_offsets, k_compact, k_union_mark (with a key bitmap), k_arena_pad.  (Six
// memsets are not counted.)
int build_launches_per_batch() { return 17 + 4; }

}  // namespace phylo
