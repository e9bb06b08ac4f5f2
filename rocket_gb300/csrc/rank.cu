// rank.cu -- dense key ranks: every key of a set of vectors replaced by its
// rank in the union of the set's keys.
//
// The window pair kernel cuts the key space into windows of W keys; its cost
// per window (barriers, the row scatter, ragged column groups) is paid whether
// a window holds many entries or few.  Protein keys use a small part of their
// space (K=6: ~31 M of 21^6 = 86 M keys in the union of 64 proteomes; K=7: a
// far smaller part of 21^7), so the pair kernel runs on ranks instead: a
// strictly increasing map, so each vector stays sorted, equal keys stay equal
// and different keys stay different -- the products and their order are those
// of the raw keys, only the windows are denser.
//
//   k_rank_mark     union bitmap of the keys (reduction atomics), unless the
//                   caller passes one (the batched build marks survivors' keys)
//   k_rank_reduce / k_scan_partials / k_rank_prefix
//                   exclusive prefix of the bitmap's population per 32-bit word,
//                   stored beside the word ({prefix, word} pairs: one 8-byte
//                   gather per key, one sector, where the bitmap exceeds L2)
//   k_rank_apply    rank = prefix[key / 32] + popc(word & bits below key)
//   k_rank_index    the same ranks, and in the same pass the window index of the
//                   pair kernel over them (entries of each vector below every
//                   window start), so the ranks are not read back
#include "rank.cuh"
#include "scan.cuh"

namespace phylo {

constexpr uint32_t RK_SLICE = 16384;  // entries per CTA (mark / apply)
constexpr uint32_t RK_THREADS = 256;

// grid = (slices, N)
__global__ void __launch_bounds__(RK_THREADS) k_rank_mark(const uint32_t *__restrict__ keys,
                                                          const uint64_t *__restrict__ vec_off,
                                                          uint32_t *bits) {
    const uint32_t v = blockIdx.y;
    const uint64_t b = vec_off[v];
    const uint32_t n = (uint32_t)(vec_off[v + 1] - b);
    const uint32_t e0 = blockIdx.x * RK_SLICE;
    if (e0 >= n) return;
    const uint32_t e1 = min(n, e0 + RK_SLICE);
    for (uint32_t e = e0 + threadIdx.x; e < e1; e += RK_THREADS) {
        const uint32_t key = keys[b + e];
        if (key != 0xffffffffu) atomicOr(&bits[key >> 5], 1u << (key & 31u));  // padding skipped
    }
}

// Population of SCAN_TILE words per CTA -> partials[cta].
__global__ void __launch_bounds__(SCAN_THREADS) k_rank_reduce(const uint32_t *__restrict__ bits,
                                                              uint64_t nwords, uint64_t *partials) {
    __shared__ uint64_t sw[SCAN_THREADS / 32 + 1];
    const uint64_t first = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint64_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++)
        if (first + i < nwords) s += __popc(bits[first + i]);
    uint64_t tot;
    block_excl_scan_u64<SCAN_THREADS>(s, sw, &tot);
    if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

// pw[w] = {keys of the union below word w, bits[w]}; *total = union size.
__global__ void __launch_bounds__(SCAN_THREADS) k_rank_prefix(const uint32_t *__restrict__ bits,
                                                              uint64_t nwords,
                                                              const uint64_t *__restrict__ partials,
                                                              uint2 *pw, uint64_t *total) {
    __shared__ uint64_t sw[SCAN_THREADS / 32 + 1];
    const uint64_t first = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t wv[SCAN_ITEMS];
    uint64_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        wv[i] = first + i < nwords ? bits[first + i] : 0u;
        s += __popc(wv[i]);
    }
    uint64_t tot;
    uint64_t ex = block_excl_scan_u64<SCAN_THREADS>(s, sw, &tot) + partials[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        if (first + i < nwords) pw[first + i] = make_uint2((uint32_t)ex, wv[i]);
        ex += __popc(wv[i]);
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total = partials[gridDim.x];
}

__device__ __forceinline__ uint32_t rank_of(uint32_t key, const uint2 *__restrict__ pw) {
    if (key == 0xffffffffu) return key;  // padding stays padding
    const uint2 t = __ldg(&pw[key >> 5]);
    return t.x + (uint32_t)__popc(t.y & ((1u << (key & 31u)) - 1u));
}

// grid = (slices, N); padding keys stay 0xffffffff.
__global__ void __launch_bounds__(RK_THREADS) k_rank_apply(const uint32_t *__restrict__ keys,
                                                           const uint64_t *__restrict__ vec_off,
                                                           const uint2 *__restrict__ pw,
                                                           uint32_t *ranks) {
    const uint32_t v = blockIdx.y;
    const uint64_t b = vec_off[v];
    const uint32_t n = (uint32_t)(vec_off[v + 1] - b);
    const uint32_t e0 = blockIdx.x * RK_SLICE;
    if (e0 >= n) return;
    const uint32_t e1 = min(n, e0 + RK_SLICE);
    for (uint32_t e = e0 + threadIdx.x; e < e1; e += RK_THREADS) ranks[b + e] = rank_of(keys[b + e], pw);
}

constexpr uint32_t RX_RUN = 4;                   // entries per thread
constexpr uint32_t RX_SLICE = RK_THREADS * RX_RUN;  // entries per CTA

// Ranks of RX_RUN consecutive entries per thread (16-byte loads and stores; a
// vector starts on a 16-byte boundary and its padded length is a multiple of
// 4), then roff[v][r] = entries of vector v with rank < r << wshift: an entry
// whose window is above its predecessor's writes its index into the windows in
// between; the last real entry fills the windows after it.  grid = (slices, N)
__global__ void __launch_bounds__(RK_THREADS) k_rank_index(const uint32_t *__restrict__ keys,
                                                           const uint64_t *__restrict__ vec_off,
                                                           const uint2 *__restrict__ pw,
                                                           uint32_t R, uint32_t wshift,
                                                           uint32_t *ranks, uint32_t *roff) {
    const uint32_t v = blockIdx.y;
    const uint64_t b = vec_off[v];
    const uint32_t n = (uint32_t)(vec_off[v + 1] - b);
    uint32_t *ro = roff + (uint64_t)v * (R + 1);
    const uint32_t e0 = blockIdx.x * RX_SLICE;
    if (e0 >= n) {
        if (n == 0 && blockIdx.x == 0)
            for (uint32_t r = threadIdx.x; r <= R; r += blockDim.x) ro[r] = 0;
        return;
    }
    const int lane = threadIdx.x & 31;
    const uint32_t s0 = e0 + threadIdx.x * RX_RUN;  // this thread's run
    uint32_t k[RX_RUN];
#pragma unroll
    for (int j = 0; j < (int)RX_RUN; j += 4) {
        uint4 q = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
        if (s0 + j < n) q = *reinterpret_cast<const uint4 *>(keys + b + s0 + j);
        k[j] = q.x; k[j + 1] = q.y; k[j + 2] = q.z; k[j + 3] = q.w;
    }
#pragma unroll
    for (int j = 0; j < (int)RX_RUN; j++) k[j] = rank_of(k[j], pw);
#pragma unroll
    for (int j = 0; j < (int)RX_RUN; j += 4)
        if (s0 + j < n)
            *reinterpret_cast<uint4 *>(ranks + b + s0 + j) = make_uint4(k[j], k[j + 1], k[j + 2], k[j + 3]);
    // rank before the run: the previous lane's last, or computed for lane 0
    uint32_t prev = __shfl_up_sync(0xffffffffu, k[RX_RUN - 1], 1);
    if (lane == 0)
        prev = s0 == 0 ? 0xffffffffu : (s0 <= n ? rank_of(keys[b + s0 - 1], pw) : 0xffffffffu);
    // window of the entry before the run (-1 before the first entry)
    int64_t rp = (s0 == 0 || prev == 0xffffffffu) ? -1 : (int64_t)min(prev >> wshift, R);
    if (s0 < n) {
#pragma unroll
        for (int j = 0; j < (int)RX_RUN; j++) {
            const uint32_t e = s0 + j;
            const uint32_t rk = k[j];
            if (e >= n || rk == 0xffffffffu) break;  // end or padding
            const uint32_t rt = min(rk >> wshift, R);
            for (int64_t r = rp + 1; r <= (int64_t)rt; r++) ro[r] = e;
            rp = rt;
            // last real entry: the next key is padding or the end
            const uint32_t nk = j + 1 < (int)RX_RUN ? k[j + 1]
                                : (e + 1 < n ? keys[b + e + 1] : 0xffffffffu);
            if (e + 1 == n || nk == 0xffffffffu)
                for (uint32_t r = rt + 1; r <= R; r++) ro[r] = e + 1;
        }
    }
    // a vector made only of padding
    if (blockIdx.x == 0 && keys[b] == 0xffffffffu)
        for (uint32_t r = threadIdx.x; r <= R; r += blockDim.x) ro[r] = 0;
}

// k_rank_index over the whole arena as one sequence: the grid (a few CTAs per
// SM) walks it in chunks of RX_SLICE entries, a thread's run of RX_RUN entries
// lying in one vector (vectors are padded to multiples of 4).  For arenas of
// very uneven vectors, where most (slice, vector) CTAs of k_rank_index would
// have no entries.  Vectors that are empty or only padding are
// k_rank_index_fill's.
__global__ void __launch_bounds__(RK_THREADS) k_rank_index_flat(const uint32_t *__restrict__ keys,
                                                           const uint64_t *__restrict__ vec_off,
                                                           uint32_t N, const uint2 *__restrict__ pw,
                                                           uint32_t R, uint32_t wshift,
                                                           uint32_t *ranks, uint32_t *roff) {
    const uint64_t a0 = vec_off[0], a1 = vec_off[N];
    const uint64_t nchunks = div_up(a1 - a0, (uint64_t)RX_SLICE);
    const int lane = threadIdx.x & 31;
    uint32_t v = 0;  // this thread's vector: found once, then advanced with its runs
    {
        const uint64_t g = a0 + (uint64_t)blockIdx.x * RX_SLICE + threadIdx.x * RX_RUN;
        uint32_t lo = 0, hi = N;  // last v < N with vec_off[v] <= g
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (vec_off[mid] <= g) lo = mid; else hi = mid;
        }
        v = lo;
    }
    for (uint64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const uint64_t g = a0 + ch * RX_SLICE + threadIdx.x * RX_RUN;  // this thread's run
        const bool live = g < a1;
        if (live)
            while (vec_off[v + 1] <= g) v++;
        const uint64_t b = vec_off[v];
        const uint32_t n = (uint32_t)(vec_off[v + 1] - b);
        const uint32_t s0 = (uint32_t)(g - b);  // position in the vector
        uint32_t *ro = roff + (uint64_t)v * (R + 1);
        uint32_t k[RX_RUN];
        {
            uint4 q = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
            if (live) q = *reinterpret_cast<const uint4 *>(keys + g);
            k[0] = q.x; k[1] = q.y; k[2] = q.z; k[3] = q.w;
        }
#pragma unroll
        for (int j = 0; j < (int)RX_RUN; j++) k[j] = rank_of(k[j], pw);
        if (live) *reinterpret_cast<uint4 *>(ranks + g) = make_uint4(k[0], k[1], k[2], k[3]);
        // rank before the run: the previous lane's last (the same vector unless the
        // run starts it), or computed for lane 0
        uint32_t prev = __shfl_up_sync(0xffffffffu, k[RX_RUN - 1], 1);
        if (lane == 0 && live && s0 > 0) prev = rank_of(keys[g - 1], pw);
        // window of the entry before the run (-1 before the first entry)
        const int64_t rp0 = (s0 == 0 || prev == 0xffffffffu) ? -1 : (int64_t)min(prev >> wshift, R);
        if (live) {
            int64_t rp = rp0;
#pragma unroll
            for (int j = 0; j < (int)RX_RUN; j++) {
                const uint32_t e = s0 + j;
                const uint32_t rk = k[j];
                if (rk == 0xffffffffu) break;  // padding
                const uint32_t rt = min(rk >> wshift, R);
                for (int64_t r = rp + 1; r <= (int64_t)rt; r++) ro[r] = e;
                rp = rt;
                // last real entry: the next key is padding or the end
                const uint32_t nk = j + 1 < (int)RX_RUN ? k[j + 1]
                                    : (e + 1 < n ? keys[b + e + 1] : 0xffffffffu);
                if (e + 1 == n || nk == 0xffffffffu)
                    for (uint32_t r = rt + 1; r <= R; r++) ro[r] = e + 1;
            }
        }
    }
}

// roff rows of vectors that are empty or only padding: all zero.  grid = N
__global__ void __launch_bounds__(RK_THREADS) k_rank_index_fill(const uint32_t *__restrict__ keys,
                                                                const uint64_t *__restrict__ vec_off,
                                                                uint32_t R, uint32_t *roff) {
    const uint32_t v = blockIdx.x;
    const uint64_t b = vec_off[v];
    if (vec_off[v + 1] > b && keys[b] != 0xffffffffu) return;
    uint32_t *ro = roff + (uint64_t)v * (R + 1);
    for (uint32_t r = threadIdx.x; r <= R; r += blockDim.x) ro[r] = 0;
}

cudaError_t bitmap_prefix_pairs(const uint32_t *bits, uint64_t nwords, uint64_t *partials,
                                uint2 *pw, uint64_t *total, cudaStream_t st) {
    const uint64_t nb = div_up(nwords ? nwords : 1, SCAN_TILE);
    k_rank_reduce<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(bits, nwords, partials);
    k_scan_partials<<<1, SCAN_THREADS, 0, st>>>(partials, nb);
    k_rank_prefix<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(bits, nwords, partials, pw, total);
    return cudaGetLastError();
}

uint64_t bitmap_prefix_partials(uint64_t nwords) { return div_up(nwords ? nwords : 1, SCAN_TILE) + 1; }

static uint64_t rank_words(uint64_t key_limit) { return div_up(key_limit ? key_limit : 1, 32); }

size_t rank_bitmap_words(uint64_t key_limit) { return rank_words(key_limit); }

size_t rank_scratch_bytes(uint64_t key_limit) {
    const uint64_t nw = rank_words(key_limit);
    const uint64_t nb = div_up(nw, SCAN_TILE);
    return scratch_bytes<uint32_t>(nw) + scratch_bytes<uint2>(nw) +
           scratch_bytes<uint64_t>(nb + 1) + scratch_bytes<uint64_t>(1);
}

cudaError_t key_ranks(const uint32_t *keys, const uint64_t *vec_off, uint32_t N, uint64_t max_len,
                      uint64_t key_limit, const uint32_t *union_bits, void *scratch,
                      size_t scratch_size, uint32_t *ranks, uint64_t *d_union, cudaStream_t st) {
    const uint64_t nw = rank_words(key_limit);
    const uint64_t nb = div_up(nw, SCAN_TILE);
    Scratch sc(scratch, scratch_size);
    uint32_t *own = sc.take<uint32_t>(nw);
    uint2 *pw = sc.take<uint2>(nw);
    uint64_t *partials = sc.take<uint64_t>(nb + 1);
    uint64_t *total = sc.take<uint64_t>(1);
    if (!total) return cudaErrorInvalidValue;
    const uint32_t slices = (uint32_t)div_up(max_len ? max_len : 1, RK_SLICE);
    const uint32_t *bits = union_bits;
    if (!bits) {
        PHYLO_CHECK(cudaMemsetAsync(own, 0, sizeof(uint32_t) * nw, st));
        if (N) k_rank_mark<<<dim3(slices, N), RK_THREADS, 0, st>>>(keys, vec_off, own);
        bits = own;
    }
    k_rank_reduce<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(bits, nw, partials);
    k_scan_partials<<<1, SCAN_THREADS, 0, st>>>(partials, nb);
    k_rank_prefix<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(bits, nw, partials, pw, total);
    if (N && ranks) k_rank_apply<<<dim3(slices, N), RK_THREADS, 0, st>>>(keys, vec_off, pw, ranks);
    if (d_union) PHYLO_CHECK(cudaMemcpyAsync(d_union, total, sizeof(uint64_t),
                                             cudaMemcpyDeviceToDevice, st));
    return cudaGetLastError();
}

// launches with a caller's bitmap: reduce, scan, prefix, apply, copy (+ mark without one)
int key_ranks_launches(bool marked) { return marked ? 5 : 6; }

cudaError_t key_rank_index(const uint32_t *keys, const uint64_t *vec_off, uint32_t N,
                           uint64_t max_len, uint64_t entries, uint64_t key_limit,
                           const uint32_t *union_bits,
                           void *scratch, size_t scratch_size, uint32_t wshift, uint32_t R,
                           uint32_t *ranks, uint32_t *roff, cudaStream_t st) {
    const uint64_t nw = rank_words(key_limit);
    Scratch sc(scratch, scratch_size);
    sc.take<uint32_t>(nw);  // the bitmap key_ranks built, unless the caller marked one
    const uint2 *pw = sc.take<uint2>(nw);
    (void)union_bits;       // its words are in the pairs
    if (!pw || !ranks || !roff || wshift > 31) return cudaErrorInvalidValue;
    if (N == 0) return cudaSuccess;
    const uint64_t slices = div_up(max_len ? max_len : 1, RX_SLICE);
    const uint64_t chunks = div_up(entries ? entries : 1, RX_SLICE);
    if (entries && slices * N > 2 * chunks) {  // uneven lengths: walk the arena instead
        int dev = 0, sms = 0;
        PHYLO_CHECK(cudaGetDevice(&dev));
        PHYLO_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        k_rank_index_flat<<<(unsigned)(sms > 0 ? sms : 152) * 8, RK_THREADS, 0, st>>>(
            keys, vec_off, N, pw, R, wshift, ranks, roff);
        k_rank_index_fill<<<N, RK_THREADS, 0, st>>>(keys, vec_off, R, roff);
    } else {
        k_rank_index<<<dim3((unsigned)slices, N), RK_THREADS, 0, st>>>(keys, vec_off, pw, R, wshift,
                                                                      ranks, roff);
    }
    return cudaGetLastError();
}

}  // namespace phylo
