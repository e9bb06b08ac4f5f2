// scan.cuh -- device-wide exclusive scan (uint32 -> uint64) in three launches,
// used to place variable-length per-chunk outputs (candidates, survivors).
#pragma once
#include "common.cuh"

namespace phylo {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // elements per CTA

__device__ __forceinline__ uint64_t warp_incl_scan_u64(uint64_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint64_t o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total (all threads see it).
template <int THREADS>
__device__ __forceinline__ uint64_t block_excl_scan_u64(uint64_t v, uint64_t *smem_warp,
                                                        uint64_t *total) {
    constexpr int W = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t incl = warp_incl_scan_u64(v);
    if (lane == 31) smem_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint64_t t = lane < W ? smem_warp[lane] : 0;
        uint64_t ti = warp_incl_scan_u64(t);
        if (lane < W) smem_warp[lane] = ti - t;  // exclusive per warp
        if (lane == W - 1) smem_warp[W] = ti;
    }
    __syncthreads();
    uint64_t r = smem_warp[warp] + incl - v;
    *total = smem_warp[W];
    __syncthreads();
    return r;
}

static __global__ void k_scan_reduce(const uint32_t *__restrict__ in, uint64_t n, uint64_t *partials) {
    __shared__ uint64_t sw[SCAN_THREADS / 32 + 1];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint64_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        uint64_t idx = base + (uint64_t)i * SCAN_THREADS + threadIdx.x;
        if (idx < n) s += in[idx];
    }
    uint64_t tot;
    block_excl_scan_u64<SCAN_THREADS>(s, sw, &tot);
    if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

// Single CTA: exclusive scan of the partials in place; total to partials[np].
static __global__ void k_scan_partials(uint64_t *partials, uint64_t np) {
    __shared__ uint64_t sw[SCAN_THREADS / 32 + 1];
    uint64_t carry = 0;
    for (uint64_t base = 0; base < np; base += SCAN_THREADS) {
        uint64_t idx = base + threadIdx.x;
        uint64_t v = idx < np ? partials[idx] : 0;
        uint64_t tot;
        uint64_t ex = block_excl_scan_u64<SCAN_THREADS>(v, sw, &tot);
        if (idx < np) partials[idx] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) partials[np] = carry;
}

// Writes out[i] = exclusive prefix; out[n] = total.
static __global__ void k_scan_apply(const uint32_t *__restrict__ in, uint64_t n,
                             const uint64_t *__restrict__ partials, uint64_t *out) {
    __shared__ uint64_t sw[SCAN_THREADS / 32 + 1];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    // each thread owns SCAN_ITEMS consecutive elements
    uint64_t first = base + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint64_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        v[i] = (first + i < n) ? in[first + i] : 0u;
        s += v[i];
    }
    uint64_t tot;
    uint64_t ex = block_excl_scan_u64<SCAN_THREADS>(s, sw, &tot) + partials[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        if (first + i < n) out[first + i] = ex;
        ex += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = partials[gridDim.x];
}

inline size_t scan_temp_bytes(uint64_t n) { return scratch_bytes<uint64_t>(div_up(n, SCAN_TILE) + 1); }

// out must hold n + 1 entries; temp from scan_temp_bytes(n).
inline cudaError_t scan_u32_to_u64(const uint32_t *in, uint64_t n, uint64_t *out, uint64_t *temp,
                                   cudaStream_t st) {
    uint64_t nb = div_up(n, SCAN_TILE);
    if (nb == 0) nb = 1;
    k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, temp);
    k_scan_partials<<<1, SCAN_THREADS, 0, st>>>(temp, nb);
    k_scan_apply<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, temp, out);
    return cudaGetLastError();
}

}  // namespace phylo
