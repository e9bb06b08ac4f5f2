// postings.cu -- the key-major pair engine.
//
// The reference computes C of one pair by walking the two sorted key lists
// (merge path, phylogenetics/src/main/cpp/native.cu:541-703): every entry of
// both vectors is visited, and a product is formed only where the keys match.
// Over all pairs of a set, the useful work is the sum over keys of
// m(m-1)/2 products, m being the number of vectors that hold the key.
//
// This kernel does only that work.  A work item is a block of row vectors x a
// block of column vectors over a run of key windows.  For each window:
//
//   1. count:   every entry of the block's vectors in the window increments the
//               shared-memory counter of its key (one counter per key of the
//               window, per side);
//   2. scan:    the counters become offsets: the window's postings, one list of
//               (vector position, value) per key, laid out back to back;
//   3. scatter: every entry is written into its key's posting;
//   4. product: lanes take the keys, a group of 16 lanes per key, and form the
//               products of the key's row postings with its column postings
//               (in a diagonal block, each unordered pair and each self product
//               once).
//
// When a window's postings do not fit the shared-memory capacity, its keys are
// processed in consecutive chunks that do (a key has at most one entry per
// vector, so any single key fits).
//
// Products are exact: each value is kept as its 24-bit significand and exponent,
// the 48-bit product of two significands is formed in integer arithmetic and
// rounded once to a multiple of 2^-46.  The block's accumulators are 64-bit
// integers split in shared memory into a low word, updated with atomicAdd, and
// a high word that receives the carry (or the borrow) that the low word's
// returned old value reveals; so every sum is exact and does not depend on the
// order of the atomics.  With |value| <= 1 every product is rounded by at most
// 2^-47, and |C| < 2^17 cannot overflow.
//
// Items are handed out longest first (by the planner's estimate) to persistent
// CTAs through an atomic counter; each item writes its block x block partial
// sums, which k_pb_reduce adds in a fixed order.
#include "postings.cuh"

namespace phylo {

namespace {

constexpr int PB_GROUP = 16;   // lanes per key in the product phase
constexpr uint32_t PB_SMEM_LIMIT = 232448;   // opt-in shared memory per block (227 KB)
constexpr uint32_t PB_SMEM_PER_SM = 233472;  // per SM; 1 KB of it is reserved per block

template <int B>
struct PbConf;
template <>
struct PbConf<128> {
    static constexpr int T = 1024;
    static constexpr int CTAS = 1;
};
template <>
struct PbConf<64> {
    static constexpr int T = 512;
    static constexpr int CTAS = 2;
};

template <int B>
constexpr uint32_t pb_static_bytes() {
    return 4u * 8u * B + 32u * 4u + 64u;
}

template <int B>
constexpr uint32_t pb_budget() {
    return (PbConf<B>::CTAS == 1 ? PB_SMEM_LIMIT : PB_SMEM_PER_SM / PbConf<B>::CTAS - 1024u) -
           pb_static_bytes<B>() - 256u;
}

template <int B>
__host__ __device__ constexpr uint32_t pb_fixed_bytes(uint32_t wshift) {
    // two accumulator words per pair (row stride B + 1), then per side a counter
    // per key and W + 1 offsets
    const uint32_t W = 1u << wshift;
    const uint32_t acc = 2u * B * (B + 1) * 4u;
    const uint32_t ctr = (2u * W + 2u * (W + 1)) * 4u;
    return (acc + ctr + 15u) & ~15u;
}

template <int B>
uint32_t pb_cap(uint32_t wshift) {
    const uint32_t fixed = pb_fixed_bytes<B>(wshift);
    if (fixed + 16u * B > pb_budget<B>()) return 0;
    return ((pb_budget<B>() - fixed) / 16u) & ~31u;
}

// Posting entry: x = block position (bits 0-7) | biased exponent (bits 8-15) |
// sign (bit 31), y = significand with its implicit bit.  Values that are not
// finite count as 0 (the host recomputes their pairs); finite values of
// magnitude 2^7 or more set `range` (their products could overflow the sums).
__device__ __forceinline__ uint2 pb_entry(uint32_t pos, float v, uint32_t &range) {
    const uint32_t b = __float_as_uint(v);
    uint32_t ex = (b >> 23) & 0xffu;
    uint32_t m = b & 0x7fffffu;
    if (ex == 0u) {
        ex = 1u;  // subnormal
    } else if (ex == 255u) {
        ex = 1u;  // inf / NaN
        m = 0u;
    } else {
        m |= 0x800000u;
        if (ex >= 134u) {
            range = 1u;
            ex = 133u;
        }
    }
    return make_uint2(pos | (ex << 8) | (b & 0x80000000u), m);
}

// Adds round(x * y * 2^46) to the accumulator pair at idx.
__device__ __forceinline__ void pb_add(uint32_t *acc_lo, int32_t *acc_hi, uint32_t idx, uint2 x,
                                       uint2 y) {
    const int sh = 254 - (int)((x.x >> 8) & 0xffu) - (int)((y.x >> 8) & 0xffu);
    const uint64_t m = (uint64_t)x.y * (uint64_t)y.y;  // < 2^48
    uint64_t f;
    if (sh <= 0) {
        f = m << (-sh);  // |x|, |y| < 2^7: at most 12 places
    } else {
        const int s = sh < 63 ? sh : 63;
        f = (m + (1ull << (s - 1))) >> s;  // round half up
    }
    const int64_t fs = ((x.x ^ y.x) & 0x80000000u) ? -(int64_t)f : (int64_t)f;
    const uint32_t lo = (uint32_t)fs;
    const int32_t hi = (int32_t)(fs >> 32);
    const uint32_t old = atomicAdd(&acc_lo[idx], lo);
    const int32_t dh = hi + ((old + lo) < old ? 1 : 0);
    if (dh != 0) atomicAdd(&acc_hi[idx], dh);
}

// Counts the entries of n vectors in window w per key (warp per vector).
template <int T>
__device__ __forceinline__ void pb_count(const ApArena &ar, const uint64_t *s_base,
                                         const uint64_t *s_ro, uint32_t n, uint32_t w,
                                         uint32_t r0, uint32_t W, uint32_t *cnt, uint32_t &bad) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t p = warp; p < n; p += T / 32) {
        const uint32_t *ro = ar.roff + s_ro[p];
        const uint32_t s = ro[w], e = ro[w + 1];
        const uint32_t *k = ar.keys + s_base[p];
        for (uint32_t j = s + lane; j < e; j += 32) {
            const uint32_t d = __ldg(&k[j]) - r0;
            if (d < W)
                atomicAdd(&cnt[d], 1u);
            else
                bad = 1u;
        }
    }
}

// Writes the entries of keys [ka, kb) of the window into their postings.
template <int T>
__device__ __forceinline__ void pb_scatter(const ApArena &ar, const uint64_t *s_base,
                                           const uint64_t *s_ro, uint32_t n, uint32_t w,
                                           uint32_t r0, uint32_t ka, uint32_t kb, uint32_t *fill,
                                           const uint32_t *off, uint2 *post, uint32_t &range) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t base = off[ka];
    for (uint32_t p = warp; p < n; p += T / 32) {
        const uint32_t *ro = ar.roff + s_ro[p];
        const uint32_t s = ro[w], e = ro[w + 1];
        const uint32_t *k = ar.keys + s_base[p];
        const float *v = ar.vals + s_base[p];
        for (uint32_t j = s + lane; j < e; j += 32) {
            const uint32_t d = __ldg(&k[j]) - r0;
            if (d >= ka && d < kb) {
                const uint32_t slot = atomicAdd(&fill[d], 1u);
                post[off[d] - base + slot] = pb_entry(p, __ldg(&v[j]), range);
            }
        }
    }
}

// Exclusive prefix of cnt[0, W) into off[0, W]; cnt is left zeroed (the fill
// cursors of the scatter).
template <int T>
__device__ __forceinline__ void pb_scan(uint32_t *cnt, uint32_t *off, uint32_t W,
                                        uint32_t *wsum) {
    const uint32_t per = (W + T - 1) / T;
    const uint32_t i0 = threadIdx.x * per;
    const uint32_t i1 = min(i0 + per, W);
    uint32_t local = 0;
    for (uint32_t i = i0; i < i1; i++) local += cnt[i];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= (uint32_t)d) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = lane < (uint32_t)(T / 32) ? wsum[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= (uint32_t)d) v += y;
        }
        if (lane < (uint32_t)(T / 32)) wsum[lane] = v;
    }
    __syncthreads();
    uint32_t run = (warp ? wsum[warp - 1] : 0u) + x - local;
    for (uint32_t i = i0; i < i1; i++) {
        const uint32_t c = cnt[i];
        off[i] = run;
        run += c;
        cnt[i] = 0u;
    }
    if (threadIdx.x == T - 1) off[W] = wsum[T / 32 - 1];
    __syncthreads();
}

// Products of keys [ka, kb): a group of PB_GROUP lanes per key.
template <int B, int T>
__device__ __forceinline__ void pb_products(uint32_t ka, uint32_t kb, bool diag,
                                            const uint32_t *off_r, const uint32_t *off_c,
                                            const uint2 *post_r, const uint2 *post_c,
                                            uint32_t *acc_lo, int32_t *acc_hi) {
    constexpr uint32_t LD = B + 1;
    constexpr uint32_t NG = T / PB_GROUP;
    const uint32_t g = threadIdx.x / PB_GROUP, lg = threadIdx.x % PB_GROUP;
    const uint32_t base_r = off_r[ka];
    if (diag) {
        for (uint32_t k = ka + g; k < kb; k += NG) {
            const uint32_t br = off_r[k] - base_r, nr = off_r[k + 1] - off_r[k];
            const uint32_t P = nr * (nr + 1) / 2;  // pairs r <= c of the posting
            if (lg >= P) continue;
            uint32_t r = 0, t = lg;
            while (r < nr && t >= nr - r) {
                t -= nr - r;
                r++;
            }
            uint32_t c = r + t;
            for (uint32_t idx = lg; idx < P; idx += PB_GROUP) {
                const uint2 x = post_r[br + r], y = post_r[br + c];
                pb_add(acc_lo, acc_hi, (x.x & 0xffu) * LD + (y.x & 0xffu), x, y);
                c += PB_GROUP;
                while (c >= nr && r + 1 < nr) {
                    c = c - nr + r + 1;
                    r++;
                }
            }
        }
    } else {
        const uint32_t base_c = off_c[ka];
        for (uint32_t k = ka + g; k < kb; k += NG) {
            const uint32_t nr = off_r[k + 1] - off_r[k], nc = off_c[k + 1] - off_c[k];
            const uint32_t P = nr * nc;
            if (lg >= P) continue;
            const uint32_t br = off_r[k] - base_r, bc = off_c[k] - base_c;
            // lg / nc and PB_GROUP / nc (exact for these small operands)
            const float inv = __frcp_rn((float)nc);
            uint32_t r = (uint32_t)(((float)lg + 0.5f) * inv);
            uint32_t c = lg - r * nc;
            const uint32_t rs = (uint32_t)(((float)PB_GROUP + 0.5f) * inv);
            const uint32_t cs = PB_GROUP - rs * nc;
            for (uint32_t idx = lg; idx < P; idx += PB_GROUP) {
                const uint2 x = post_r[br + r], y = post_c[bc + c];
                pb_add(acc_lo, acc_hi, (x.x & 0xffu) * LD + (y.x & 0xffu), x, y);
                c += cs;
                r += rs;
                if (c >= nc) {
                    c -= nc;
                    r++;
                }
            }
        }
    }
}

template <int B>
__global__ void __launch_bounds__(PbConf<B>::T, PbConf<B>::CTAS) k_postings(PbArgs a, uint32_t cap) {
    constexpr int T = PbConf<B>::T;
    constexpr uint32_t LD = B + 1;
    extern __shared__ __align__(16) uint8_t pb_smem[];
    const uint32_t W = 1u << a.wshift;
    uint32_t *acc_lo = reinterpret_cast<uint32_t *>(pb_smem);
    int32_t *acc_hi = reinterpret_cast<int32_t *>(acc_lo + B * LD);
    uint32_t *cnt_r = reinterpret_cast<uint32_t *>(acc_hi + B * LD);
    uint32_t *cnt_c = cnt_r + W;
    uint32_t *off_r = cnt_c + W;
    uint32_t *off_c = off_r + W + 1;
    uint2 *post_r = reinterpret_cast<uint2 *>(pb_smem + pb_fixed_bytes<B>(a.wshift));
    uint2 *post_c = post_r + cap;

    __shared__ uint64_t s_rbase[B], s_cbase[B], s_rro[B], s_cro[B];
    __shared__ uint32_t s_wsum[32];
    __shared__ uint32_t s_item, s_kb;

    uint32_t bad = 0, range = 0;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= a.nitems) break;
        const long long t_start = clock64();
        PbItem m = a.items[it];
        // an item never exceeds the block or the window index
        m.nrow = min(m.nrow, (uint32_t)B);
        m.ncol = min(m.ncol, (uint32_t)B);
        m.w1 = min(m.w1, a.R);
        const bool diag = m.diag != 0;
        for (uint32_t p = threadIdx.x; p < B; p += T) {
            if (p < m.nrow) {
                const uint32_t v = a.rowids[m.row0 + p];
                s_rbase[p] = a.row.vec_off[v];
                s_rro[p] = (uint64_t)v * (a.R + 1);
            }
            if (!diag && p < m.ncol) {
                const uint32_t v = a.colids[m.col0 + p];
                s_cbase[p] = a.col.vec_off[v];
                s_cro[p] = (uint64_t)v * (a.R + 1);
            }
        }
        for (uint32_t i = threadIdx.x; i < 2u * B * LD; i += T) acc_lo[i] = 0u;  // lo and hi
        __syncthreads();
        for (uint32_t w = m.w0; w < m.w1; w++) {
            const uint32_t r0 = w << a.wshift;
            for (uint32_t i = threadIdx.x; i < 2u * W; i += T) cnt_r[i] = 0u;  // both sides
            __syncthreads();
            pb_count<T>(a.row, s_rbase, s_rro, m.nrow, w, r0, W, cnt_r, bad);
            if (!diag) pb_count<T>(a.col, s_cbase, s_cro, m.ncol, w, r0, W, cnt_c, bad);
            __syncthreads();
            pb_scan<T>(cnt_r, off_r, W, s_wsum);
            if (!diag) pb_scan<T>(cnt_c, off_c, W, s_wsum);
            for (uint32_t ka = 0; ka < W;) {
                if (threadIdx.x == 0) {
                    // the longest run of keys from ka whose postings fit on both sides
                    uint32_t lo = ka + 1, hi = W;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1) / 2;
                        const bool fits = off_r[mid] - off_r[ka] <= cap &&
                                          (diag || off_c[mid] - off_c[ka] <= cap);
                        if (fits)
                            lo = mid;
                        else
                            hi = mid - 1;
                    }
                    s_kb = lo;
                }
                __syncthreads();
                const uint32_t kb = s_kb;
                pb_scatter<T>(a.row, s_rbase, s_rro, m.nrow, w, r0, ka, kb, cnt_r, off_r, post_r,
                              range);
                if (!diag)
                    pb_scatter<T>(a.col, s_cbase, s_cro, m.ncol, w, r0, ka, kb, cnt_c, off_c,
                                  post_c, range);
                __syncthreads();
                pb_products<B, T>(ka, kb, diag, off_r, off_c, post_r, post_c, acc_lo, acc_hi);
                __syncthreads();
                ka = kb;
            }
        }
        // the item's partial sums: int64 = hi * 2^32 + lo
        int64_t *dst = a.part + (uint64_t)m.part * B * B;
        for (uint32_t i = threadIdx.x; i < (uint32_t)(B * B); i += T) {
            const uint32_t r = i / B, c = i % B;
            const uint64_t v = ((uint64_t)(uint32_t)acc_hi[r * LD + c] << 32) | acc_lo[r * LD + c];
            dst[i] = (int64_t)v;
        }
        if (a.item_cycles && threadIdx.x == 0) a.item_cycles[it] = clock64() - t_start;
        __syncthreads();
    }
    if ((bad | range) && a.status)
        atomicOr(a.status, (bad ? (uint32_t)DEV_CAPACITY : 0u) | (range ? (uint32_t)DEV_RANGE : 0u));
}

__global__ void k_pb_reduce(PbReduceArgs r) {
    const PbTile t = r.tiles[blockIdx.x];
    const uint32_t i = blockIdx.y;
    if (i >= t.nrow) return;
    const uint64_t blk = (uint64_t)r.block * r.block;
    for (uint32_t c = threadIdx.x; c < t.ncol; c += blockDim.x) {
        if (t.diag && (c < i || (c == i && !r.self))) continue;
        int64_t s = 0;
        const int64_t *pp = r.part + (uint64_t)t.part0 * blk;
        for (uint32_t p = 0; p < t.nparts; p++, pp += blk) {
            s += pp[(uint64_t)i * r.block + c];
            if (t.diag && c != i) s += pp[(uint64_t)c * r.block + i];
        }
        const double v = ldexp((double)s, -PB_SCALE);
        const uint32_t rowid = r.rowids[t.row0 + i], colid = r.colids[t.col0 + c];
        r.out[(uint64_t)rowid * r.ldc + colid] = v;
        if (r.mirror) r.out[(uint64_t)colid * r.ldc + rowid] = v;
    }
}

template <int B>
const void *pb_kernel() {
    return (const void *)k_postings<B>;
}

}  // namespace

bool pb_block_ok(int block) { return block == 128 || block == 64; }

int pb_threads(int block) { return block == 128 ? PbConf<128>::T : PbConf<64>::T; }

uint32_t pb_capacity(int block, uint32_t wshift) {
    if (wshift < 4 || wshift > 14) return 0;
    return block == 128 ? pb_cap<128>(wshift) : (block == 64 ? pb_cap<64>(wshift) : 0u);
}

size_t pb_smem_bytes(int block, uint32_t wshift) {
    const uint32_t cap = pb_capacity(block, wshift);
    if (cap == 0) return 0;
    const uint32_t fixed = block == 128 ? pb_fixed_bytes<128>(wshift) : pb_fixed_bytes<64>(wshift);
    return (size_t)fixed + 16u * (size_t)cap;
}

cudaError_t pb_prepare(int block, uint32_t wshift, int *ctas_per_sm) {
    if (!pb_block_ok(block) || pb_capacity(block, wshift) == 0) return cudaErrorInvalidValue;
    const size_t smem = pb_smem_bytes(block, wshift);
    const void *fn = block == 128 ? pb_kernel<128>() : pb_kernel<64>();
    cudaFuncAttributes fa;
    PHYLO_CHECK(cudaFuncGetAttributes(&fa, fn));
    const uint32_t stat = block == 128 ? pb_static_bytes<128>() : pb_static_bytes<64>();
    if (fa.sharedSizeBytes > stat) {
        fprintf(stderr, "phylogenetics: postings kernel static shared memory %zu > %u\n",
                fa.sharedSizeBytes, stat);
        return cudaErrorInvalidValue;
    }
    PHYLO_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (ctas_per_sm) {
        int n = 0;
        PHYLO_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, pb_threads(block), smem));
        *ctas_per_sm = n;
    }
    return cudaSuccess;
}

cudaError_t pb_launch(const PbArgs &a, int block, int grid, cudaStream_t st) {
    const uint32_t cap = pb_capacity(block, a.wshift);
    if (cap == 0 || grid <= 0) return cudaErrorInvalidValue;
    const size_t smem = pb_smem_bytes(block, a.wshift);
    // the attribute belongs to the caller's current context: set it on every launch
    PHYLO_CHECK(cudaFuncSetAttribute(block == 128 ? pb_kernel<128>() : pb_kernel<64>(),
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (block == 128)
        k_postings<128><<<grid, PbConf<128>::T, smem, st>>>(a, cap);
    else
        k_postings<64><<<grid, PbConf<64>::T, smem, st>>>(a, cap);
    return cudaGetLastError();
}

cudaError_t pb_reduce_launch(const PbReduceArgs &r, cudaStream_t st) {
    if (r.ntiles == 0) return cudaSuccess;
    k_pb_reduce<<<dim3(r.ntiles, r.block), 128, 0, st>>>(r);
    return cudaGetLastError();
}

}  // namespace phylo
