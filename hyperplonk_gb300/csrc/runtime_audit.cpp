// runtime_audit.cpp -- counters of the CUDA runtime calls this library makes,
// and host-side failure injection.
//
// The library is linked with `--wrap` for the runtime entry points below
// (hyperplonk_gb300/build.py), so every reference to, say,
// cudaMemcpyAsync in the library's objects lands on __wrap_cudaMemcpyAsync
// here, which counts the call and forwards it to the real one.  This is the
// GB300 form of the reference's link-time audit of its runtime calls
// (backend/src/ascend910b3/native/CMakeLists.txt:106-116,
// tests/runtime_audit.h): a test reads the counters around a compute window
// and checks that no table-sized transfer and no device allocation happened
// inside it.  The counters are process wide and cost one relaxed atomic add
// per call.
//
// Failure injection (hp_cuda_v1_debug_inject_failure, or HP_CUDA_FAIL_ALLOC_AT
// in the environment): the n-th pool allocation from now fails with
// cudaErrorMemoryAllocation without allocating, or the n-th stream
// synchronisation from now really synchronises and then reports
// cudaErrorLaunchFailure -- an execution failure as the caller sees it,
// while the device and the context stay healthy.  Nothing here touches the
// GPU beyond the forwarded calls.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdlib>

#include "../../include/hp_cuda.h"

extern "C" {
cudaError_t __real_cudaMalloc(void **p, size_t bytes);
cudaError_t __real_cudaHostAlloc(void **p, size_t bytes, unsigned int flags);
cudaError_t __real_cudaMallocHost(void **p, size_t bytes);
cudaError_t __real_cudaMallocAsync(void **p, size_t bytes, cudaStream_t s);
cudaError_t __real_cudaMallocFromPoolAsync(void **p, size_t bytes, cudaMemPool_t pool, cudaStream_t s);
cudaError_t __real_cudaFree(void *p);
cudaError_t __real_cudaFreeHost(void *p);
cudaError_t __real_cudaFreeAsync(void *p, cudaStream_t s);
cudaError_t __real_cudaMemcpy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind);
cudaError_t __real_cudaMemcpyAsync(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s);
cudaError_t __real_cudaMemset(void *p, int v, size_t bytes);
cudaError_t __real_cudaMemsetAsync(void *p, int v, size_t bytes, cudaStream_t s);
cudaError_t __real_cudaStreamSynchronize(cudaStream_t s);
cudaError_t __real_cudaEventSynchronize(cudaEvent_t e);
cudaError_t __real_cudaDeviceSynchronize(void);
}

namespace {

enum Counter {
    kDeviceAllocs,
    kHostAllocs,
    kPoolAllocs,
    kPoolAllocBytes,
    kFrees,
    kH2dCopies,
    kH2dBytes,
    kD2hCopies,
    kD2hBytes,
    kD2dCopies,
    kD2dBytes,
    kOtherCopies,
    kOtherBytes,
    kMemsets,
    kSyncs,
    kInjected,
    kCounters
};

std::atomic<uint64_t> g_counts[kCounters];

// Countdown to the injected failure: 0 = disarmed, else the failure fires on
// the call that takes it from 1 to 0.
std::atomic<uint64_t> g_fail_alloc{0};
std::atomic<uint64_t> g_fail_sync{0};

inline void bump(Counter c, uint64_t v = 1) { g_counts[c].fetch_add(v, std::memory_order_relaxed); }

// True when this call is the armed one.
bool fires(std::atomic<uint64_t> &countdown) {
    uint64_t cur = countdown.load(std::memory_order_relaxed);
    while (cur != 0) {
        if (countdown.compare_exchange_weak(cur, cur - 1, std::memory_order_relaxed)) return cur == 1;
    }
    return false;
}

struct EnvArm {
    EnvArm() {
        if (const char *v = std::getenv("HP_CUDA_FAIL_ALLOC_AT")) {
            const unsigned long long n = std::strtoull(v, nullptr, 10);
            g_fail_alloc.store(n, std::memory_order_relaxed);
        }
    }
} g_env_arm;

void count_copy(size_t bytes, cudaMemcpyKind kind) {
    switch (kind) {
        case cudaMemcpyHostToDevice: bump(kH2dCopies); bump(kH2dBytes, bytes); break;
        case cudaMemcpyDeviceToHost: bump(kD2hCopies); bump(kD2hBytes, bytes); break;
        case cudaMemcpyDeviceToDevice: bump(kD2dCopies); bump(kD2dBytes, bytes); break;
        default: bump(kOtherCopies); bump(kOtherBytes, bytes); break;
    }
}

cudaError_t after_sync(cudaError_t e) {
    bump(kSyncs);
    if (e == cudaSuccess && fires(g_fail_sync)) {
        bump(kInjected);
        return cudaErrorLaunchFailure;
    }
    return e;
}

}  // namespace

extern "C" {

cudaError_t __wrap_cudaMalloc(void **p, size_t bytes) {
    bump(kDeviceAllocs);
    return __real_cudaMalloc(p, bytes);
}
cudaError_t __wrap_cudaHostAlloc(void **p, size_t bytes, unsigned int flags) {
    bump(kHostAllocs);
    return __real_cudaHostAlloc(p, bytes, flags);
}
cudaError_t __wrap_cudaMallocHost(void **p, size_t bytes) {
    bump(kHostAllocs);
    return __real_cudaMallocHost(p, bytes);
}
cudaError_t __wrap_cudaMallocAsync(void **p, size_t bytes, cudaStream_t s) {
    bump(kPoolAllocs);
    bump(kPoolAllocBytes, bytes);
    if (fires(g_fail_alloc)) {
        bump(kInjected);
        if (p) *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return __real_cudaMallocAsync(p, bytes, s);
}
cudaError_t __wrap_cudaMallocFromPoolAsync(void **p, size_t bytes, cudaMemPool_t pool, cudaStream_t s) {
    bump(kPoolAllocs);
    bump(kPoolAllocBytes, bytes);
    if (fires(g_fail_alloc)) {
        bump(kInjected);
        if (p) *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return __real_cudaMallocFromPoolAsync(p, bytes, pool, s);
}
cudaError_t __wrap_cudaFree(void *p) {
    bump(kFrees);
    return __real_cudaFree(p);
}
cudaError_t __wrap_cudaFreeHost(void *p) {
    bump(kFrees);
    return __real_cudaFreeHost(p);
}
cudaError_t __wrap_cudaFreeAsync(void *p, cudaStream_t s) {
    bump(kFrees);
    return __real_cudaFreeAsync(p, s);
}
cudaError_t __wrap_cudaMemcpy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind) {
    count_copy(bytes, kind);
    return __real_cudaMemcpy(dst, src, bytes, kind);
}
cudaError_t __wrap_cudaMemcpyAsync(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
    count_copy(bytes, kind);
    return __real_cudaMemcpyAsync(dst, src, bytes, kind, s);
}
cudaError_t __wrap_cudaMemset(void *p, int v, size_t bytes) {
    bump(kMemsets);
    return __real_cudaMemset(p, v, bytes);
}
cudaError_t __wrap_cudaMemsetAsync(void *p, int v, size_t bytes, cudaStream_t s) {
    bump(kMemsets);
    return __real_cudaMemsetAsync(p, v, bytes, s);
}
cudaError_t __wrap_cudaStreamSynchronize(cudaStream_t s) { return after_sync(__real_cudaStreamSynchronize(s)); }
cudaError_t __wrap_cudaEventSynchronize(cudaEvent_t e) { return after_sync(__real_cudaEventSynchronize(e)); }
cudaError_t __wrap_cudaDeviceSynchronize(void) { return after_sync(__real_cudaDeviceSynchronize()); }

HpCudaStatus hp_cuda_v1_debug_runtime_counters(HpCudaRuntimeCounters *out) {
    if (!out) return HpCudaStatus{HP_CUDA_STATUS_INVALID_PARAMETERS, 0};
    auto get = [](Counter c) { return g_counts[c].load(std::memory_order_relaxed); };
    out->device_allocs = get(kDeviceAllocs);
    out->host_allocs = get(kHostAllocs);
    out->pool_allocs = get(kPoolAllocs);
    out->pool_alloc_bytes = get(kPoolAllocBytes);
    out->frees = get(kFrees);
    out->h2d_copies = get(kH2dCopies);
    out->h2d_bytes = get(kH2dBytes);
    out->d2h_copies = get(kD2hCopies);
    out->d2h_bytes = get(kD2hBytes);
    out->d2d_copies = get(kD2dCopies);
    out->d2d_bytes = get(kD2dBytes);
    out->other_copies = get(kOtherCopies);
    out->other_bytes = get(kOtherBytes);
    out->memsets = get(kMemsets);
    out->syncs = get(kSyncs);
    out->injected_failures = get(kInjected);
    return HpCudaStatus{HP_CUDA_STATUS_SUCCESS, 0};
}

HpCudaStatus hp_cuda_v1_debug_inject_failure(int32_t what, uint64_t nth) {
    switch (what) {
        case HP_CUDA_INJECT_NONE:
            g_fail_alloc.store(0, std::memory_order_relaxed);
            g_fail_sync.store(0, std::memory_order_relaxed);
            break;
        case HP_CUDA_INJECT_POOL_ALLOCATION: g_fail_alloc.store(nth, std::memory_order_relaxed); break;
        case HP_CUDA_INJECT_SYNCHRONIZE: g_fail_sync.store(nth, std::memory_order_relaxed); break;
        default: return HpCudaStatus{HP_CUDA_STATUS_INVALID_PARAMETERS, 0};
    }
    return HpCudaStatus{HP_CUDA_STATUS_SUCCESS, 0};
}

}  // extern "C"
