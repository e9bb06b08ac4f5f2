// common.cuh -- shared device/host helpers for the composition-vector library.
//
// Everything here is sm_103a-only code (no multi-arch paths).  The helpers are:
//   * alphabet digit tables (phylogenetics/src/main/cpp/native.cu:50-141),
//   * a scratch bump allocator with the reference's 256-byte rounding
//     (native.cu:27-48) so callers can size one buffer up front,
//   * float-float (compensated) arithmetic used by the dot-product kernels,
//   * bounded mbarrier / bulk-copy (TMA) wrappers: every wait has an
//     iteration limit after which the kernel records an error and returns.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

namespace phylo {

// ------------------------------------------------------------------------
// error handling
// ------------------------------------------------------------------------

#define PHYLO_CHECK(expr)                                                       \
    do {                                                                        \
        cudaError_t _e = (expr);                                                \
        if (_e != cudaSuccess) {                                                \
            fprintf(stderr, "phylogenetics: %s failed: %s (%s:%d)\n", #expr,   \
                    cudaGetErrorString(_e), __FILE__, __LINE__);                \
            return _e;                                                          \
        }                                                                       \
    } while (0)

// Device-side error codes written to a status word in scratch.
enum DeviceError : uint32_t {
    DEV_OK = 0,
    DEV_WAIT_TIMEOUT = 1,     // an mbarrier wait exceeded its iteration limit
    DEV_CAPACITY = 2,         // an output/staging capacity was exceeded
    DEV_RANGE = 4,            // an input value outside the range a kernel accepts
};

// ------------------------------------------------------------------------
// alphabets
// ------------------------------------------------------------------------

// ASCII 'A'..'Z' -> digit, 0xff = not part of the alphabet (breaks a K-mer).
// Protein uses 21 symbols ACDEFGHIKLMNPQRSTVWY + X (X = 20, Y = 19).
__constant__ static uint8_t kProteinMap[26] = {
    0, 255, 1, 2, 3, 4, 5, 6, 7, 255, 8, 9, 10, 11, 255, 12, 13, 14, 15, 16, 255, 17, 18, 20, 19,
    255};
__constant__ static uint8_t kDnaMap[26] = {0,   255, 1,   255, 255, 255, 2,   255, 255,
                                           255, 255, 255, 255, 255, 255, 255, 255, 255,
                                           255, 3,   255, 255, 255, 255, 255, 255};

enum Alphabet : int { ALPHA_PROTEIN = 0, ALPHA_DNA = 1 };

__host__ __device__ inline uint32_t alphabet_size(int alpha) { return alpha == ALPHA_DNA ? 4u : 21u; }

__device__ __forceinline__ uint32_t char_to_digit(int alpha, uint8_t c) {
    uint32_t idx = (uint32_t)c - 'A';
    if (idx >= 26u) return 0xffu;
    return alpha == ALPHA_DNA ? kDnaMap[idx] : kProteinMap[idx];
}

__host__ __device__ inline uint64_t ipow64(uint64_t a, int b) {
    uint64_t r = 1;
    while (b-- > 0) r *= a;
    return r;
}

// ------------------------------------------------------------------------
// scratch bump allocator (256-byte granules)
// ------------------------------------------------------------------------

__host__ __device__ inline size_t round256(size_t n) { return (n + 255) / 256 * 256; }

struct Scratch {
    char *base;
    size_t size;
    size_t used;
    __host__ Scratch(void *b, size_t s) : base((char *)b), size(s), used(0) {}
    template <typename T>
    __host__ T *take(size_t n) {
        size_t bytes = round256(n * sizeof(T));
        if (used + bytes > size) return nullptr;
        T *p = (T *)(base + used);
        used += bytes;
        return p;
    }
};

template <typename T>
__host__ inline size_t scratch_bytes(size_t n) {
    return round256(n * sizeof(T));
}

// ------------------------------------------------------------------------
// compensated arithmetic
// ------------------------------------------------------------------------

// TwoSum (Knuth): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// float-float accumulator
struct FF {
    float hi, lo;
};

__device__ __forceinline__ void ff_add(FF &acc, float x) {
    float s, e;
    two_sum(acc.hi, x, s, e);
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, e);
}

__device__ __forceinline__ FF ff_merge(FF a, FF b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    FF r;
    two_sum(s, e, r.hi, r.lo);
    return r;
}

// Exact product split: p + e == a * b (FMA-based TwoProduct).
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

__device__ __forceinline__ FF ff_shfl_down(FF v, int delta) {
    FF r;
    r.hi = __shfl_down_sync(0xffffffffu, v.hi, delta);
    r.lo = __shfl_down_sync(0xffffffffu, v.lo, delta);
    return r;
}

__device__ __forceinline__ FF ff_warp_sum(FF v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = ff_merge(v, ff_shfl_down(v, d));
    return v;
}

// double-double accumulator (used only for the per-vector norm)
struct DD {
    double hi, lo;
};

__device__ __forceinline__ void dd_add(DD &acc, double x) {
    double s = __dadd_rn(acc.hi, x);
    double bb = __dsub_rn(s, acc.hi);
    double e = __dadd_rn(__dsub_rn(acc.hi, __dsub_rn(s, bb)), __dsub_rn(x, bb));
    acc.hi = s;
    acc.lo = __dadd_rn(acc.lo, e);
}

__device__ __forceinline__ DD dd_merge(DD a, DD b) {
    DD r = a;
    dd_add(r, b.hi);
    r.lo = __dadd_rn(r.lo, b.lo);
    double s = __dadd_rn(r.hi, r.lo);
    double e = __dsub_rn(r.lo, __dsub_rn(s, r.hi));
    r.hi = s;
    r.lo = e;
    return r;
}

// ------------------------------------------------------------------------
// mbarrier + bulk copy (TMA, non-tensor 1-D form) with bounded waits
// ------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                     smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// Returns true when the phase with parity `phase` has completed.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after `limit` polls (each try_wait itself blocks for a
// hardware-defined interval) and reports failure to the caller.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase,
                                                  uint32_t limit = (1u << 22)) {
    for (uint32_t i = 0; i < limit; i++) {
        if (mbar_try_wait(bar, phase)) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

// 1-D bulk copy global -> shared, completion counted on `bar` (bytes % 16 == 0,
// both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_g2s(void *dst_smem, const void *src_gmem, uint32_t bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// ------------------------------------------------------------------------
// misc
// ------------------------------------------------------------------------

// Index of the n-th (0-based) set bit of m (m has more than n set bits).
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t n) {
    uint32_t pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        uint32_t c = __popc(m & ((1u << w) - 1u));
        if (n >= c) {
            n -= c;
            m >>= w;
            pos += w;
        }
    }
    return pos;
}

__host__ __device__ inline uint64_t div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

}  // namespace phylo
