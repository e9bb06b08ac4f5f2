// hostctx.cuh -- host-side state keyed by the caller's CUDA context.
//
// Rocket creates its own contexts (cuCtxCreate, one per device worker) and
// destroys them again; its tests do so once per test.  Anything this library
// looks up once and reuses -- a device symbol's address, a kernel attribute --
// belongs to one context, so it is cached under the current context's unique
// id (cuCtxGetId, never reused within a process), not under the device number.
// The driver entry points are fetched through the runtime, so the library
// needs no link dependency on libcuda.  Every cache is guarded by a mutex:
// Rocket runs one device worker thread per GPU in one process.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

namespace phylo {

// Unique id of the calling thread's current context; 0 (and cudaSuccess) when
// no context is current yet, so the caller does its lookup uncached.
inline cudaError_t current_context_id(unsigned long long *id) {
    typedef CUresult (*GetCurrent)(CUcontext *);
    typedef CUresult (*GetId)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault,
                                             &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess)
            get_current = (GetCurrent)f1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) ==
                cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess)
            get_id = (GetId)f2;
    });
    *id = 0;
    if (!get_current || !get_id) return cudaSuccess;  // uncached lookups
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return cudaSuccess;
    unsigned long long v = 0;
    if (get_id(ctx, &v) != CUDA_SUCCESS) return cudaSuccess;
    *id = v;
    return cudaSuccess;
}

// A small map from context id to one value, for a fixed number of live
// contexts (older entries are overwritten round-robin).
template <typename T, int N = 64>
class PerContext {
  public:
    // Returns the cached value of the current context, or computes it with
    // make(&value) (a cudaError_t-returning callable) and caches it.
    template <typename F>
    cudaError_t get(T *out, F make) {
        unsigned long long id = 0;
        cudaError_t e = current_context_id(&id);
        if (e != cudaSuccess) return e;
        if (id != 0) {
            std::lock_guard<std::mutex> lock(mu_);
            for (int i = 0; i < N; i++)
                if (ids_[i] == id) {
                    *out = vals_[i];
                    return cudaSuccess;
                }
        }
        T v{};
        e = make(&v);
        if (e != cudaSuccess) return e;
        if (id == 0) current_context_id(&id);  // the lookup may have made one current
        if (id != 0) {
            std::lock_guard<std::mutex> lock(mu_);
            ids_[next_] = id;
            vals_[next_] = v;
            next_ = (next_ + 1) % N;
        }
        *out = v;
        return cudaSuccess;
    }

  private:
    std::mutex mu_;
    unsigned long long ids_[N] = {0};
    T vals_[N] = {};
    int next_ = 0;
};

// Streaming multiprocessors of the current device, cached per device number
// (a property of the hardware, the same in every context).
inline int device_sm_count() {
    static std::atomic<int> sms[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 152;
    if (dev < 64) {
        const int c = sms[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
        n = 152;
    if (dev < 64) sms[dev].store(n, std::memory_order_relaxed);
    return n;
}

}  // namespace phylo
