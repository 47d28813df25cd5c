// runtime.cuh -- context, buffer registry and ABI guard shared by every
// translation unit of libhp_cuda.so.
//
// GB300 design: one context = one device + one non-blocking CUDA stream + one
// private stream-ordered memory pool.  Every device allocation is a
// cudaMallocFromPoolAsync on the context stream and every release a
// cudaFreeAsync on the same stream, so a buffer returns to the pool only after
// all work queued before its release (the reference's "free only after the
// block's recorded stream event completes", bridge.h:17-19, by construction).
// Public MLE addresses are reference counted: prover states and parameter
// objects take a reference, so a retired handle's storage lives as long as any
// of them needs it (bridge_runtime.h in the reference keeps BufferRef copies
// for the same reason).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/hp_cuda.h"
#include "field.cuh"

namespace hp {

struct Failure {
    int32_t kind;
    int32_t code;
};

[[noreturn]] inline void fail(int32_t kind, int32_t code = 0) { throw Failure{kind, code}; }
inline void require(bool cond) {
    if (!cond) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
}
inline void check_cuda(cudaError_t e) {
    if (e != cudaSuccess) fail(HP_CUDA_STATUS_INVALID_STATE, static_cast<int32_t>(e));
}

template <class Fn>
inline HpCudaStatus guard(Fn &&fn) {
    try {
        fn();
        return HpCudaStatus{HP_CUDA_STATUS_SUCCESS, 0};
    } catch (const Failure &f) {
        return HpCudaStatus{f.kind, f.code};
    } catch (const std::bad_alloc &) {
        return HpCudaStatus{HP_CUDA_STATUS_INVALID_STATE, static_cast<int32_t>(cudaErrorMemoryAllocation)};
    } catch (...) {
        return HpCudaStatus{HP_CUDA_STATUS_INVALID_STATE, -1};
    }
}

// Status word bits written by kernels (device flag, read after a sync).
enum : uint32_t {
    kFlagNonCanonical = 1u,
    kFlagZeroDenominator = 2u,
    kFlagPointOffCurve = 4u,
    kFlagTimeout = 8u,
};

constexpr size_t kFrBytes = 32;
constexpr size_t kG1PacketBytes = 97;
constexpr size_t kAffineBytes = 96;
constexpr size_t kMaxNumVars = 30;  // 2^30 Fr = 32 GiB per table

inline size_t table_len(size_t num_vars) { return size_t(1) << num_vars; }

}  // namespace hp

// One asynchronous upload call (hp_cuda_v1_mle_upload_async): the event its
// copies and conversions end with on the ingress stream, and its slot in the
// context's pinned flag words (non-canonical input seen).
struct HpCudaIngress {
    cudaEvent_t ready = nullptr;
    int slot = -1;
    bool *slot_used = nullptr;  // the context's slot flag, freed with this record
    HpCudaIngress() = default;
    HpCudaIngress(const HpCudaIngress &) = delete;
    HpCudaIngress &operator=(const HpCudaIngress &) = delete;
    ~HpCudaIngress() {
        if (ready) cudaEventDestroy(ready);
        if (slot_used) *slot_used = false;
    }
};

struct HpCudaContext {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    uint32_t *d_flags = nullptr;  // device status word
    uint32_t *h_flags = nullptr;  // pinned host mirror
    int sm_count = 0;
    struct Buffer {
        size_t bytes;
        int refs;
        bool public_handle;  // still owned by the caller (not yet retired)
        std::shared_ptr<HpCudaIngress> ingress;  // set while an asynchronous upload may still write it
        // a table built by hp_cuda_v1_mle_build_eq_x_r: its point r (Montgomery
        // Fr, 4 words per coordinate); tables are immutable, so the table is
        // eq(x, r) for as long as the buffer lives
        std::vector<uint64_t> eq_point;
    };
    std::unordered_map<void *, Buffer> buffers;
    // Asynchronous uploads: their own stream, and pinned host words that each
    // upload's validation flag is copied into, one per upload call whose
    // buffers are still pending (created on first use).
    static constexpr int kIngressSlots = 256;
    cudaStream_t ingress_stream = nullptr;
    uint32_t *ingress_flags_h = nullptr;
    bool ingress_used[kIngressSlots] = {};
    // Make `stream` wait for the asynchronous upload that writes `p`, if any.
    void await_ingress(void *p);
    // Event and flag slot for a new asynchronous upload (both released when
    // the last buffer holding the record lets go of it).
    std::shared_ptr<HpCudaIngress> new_ingress();

    // Worker streams for independent work inside one call (fork from and
    // join back into `stream` with events; created on first use).
    static constexpr int kWorkers = 8;
    cudaStream_t workers[kWorkers] = {};
    cudaEvent_t fork_event = nullptr;
    cudaEvent_t join_events[kWorkers] = {};
    // Make the first k workers wait for everything queued on `stream`.
    void fork(int k);
    // Make `stream` wait for everything queued on the first k workers.
    void join(int k);

    // Stream-ordered allocation registered with one reference.
    void *alloc(size_t bytes);
    // Unregistered scratch (freed with scratch_free, stream ordered on `s`,
    // the context stream by default).
    void *scratch(size_t bytes, cudaStream_t s = nullptr);
    void scratch_free(void *p, cudaStream_t s = nullptr);
    void ref(void *p);
    void unref(void *p);
    // True while `p` is a caller-owned handle (allocated, not yet retired).
    bool owns(void *p) const {
        auto it = buffers.find(p);
        return it != buffers.end() && it->second.public_handle;
    }
    // Caller gives up its handle; storage lives while internal refs remain.
    void retire(void *p);
    size_t bytes_of(void *p) const;
    // Kernel timing (off by default): CUDA events around named launches on
    // the context stream, resolved into per-name totals on read.
    bool profiling = false;
    struct Pending {
        const char *name;
        cudaEvent_t start, stop;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    std::map<std::string, std::pair<double, uint64_t>> totals;  // ms, launches
    cudaEvent_t take_event();
    // Returns an index to pass to prof_end, or -1 when profiling is off.
    // Events go on stream `s` (the context stream by default).
    int prof_begin(const char *name, cudaStream_t s = nullptr);
    void prof_end(int token, cudaStream_t s = nullptr);
    void prof_resolve();
    // Pinned, device-mapped host memory for small per-round results that a
    // kernel writes straight into host memory (no copy launch, no staging);
    // grown on demand.  Calls on one context are not concurrent.
    uint8_t *h_mailbox = nullptr;
    void *d_mailbox = nullptr;
    size_t mailbox_bytes = 0;
    // Host pointer to >= `bytes` of the mailbox; *dev gets its device alias.
    uint8_t *mailbox(size_t bytes, void **dev);
    // A host thread beside the calling one that runs one job at a time
    // (created on first use, joined by context_destroy): the Fiat-Shamir loop
    // of a resident sumcheck launch runs there, so the launch call may return
    // only when the kernel has finished (CUDA_LAUNCH_BLOCKING, profilers that
    // serialise launches) while the kernel waits for the loop's challenges.
    struct Responder;
    std::unique_ptr<Responder> responder;
    void respond_start(std::function<void()> job);
    // Waits for the job and rethrows its exception, if any.
    void respond_wait();
    void respond_shutdown();
    // Host worker threads (created on first use, joined by context_destroy)
    // for independent host work of one call: fn(i) for every i < n, spread
    // over the pool and the calling thread; rethrows the first exception.
    struct HostPool;
    std::unique_ptr<HostPool> host_pool;
    void host_parallel_for(size_t n, const std::function<void(size_t)> &fn);
    void host_pool_shutdown();
    // Clear the device status word (stream ordered).
    void clear_flags();
    // Synchronize and return the status word.
    uint32_t sync_flags();
    void sync();
};

namespace hp {

// RAII scratch: stream-ordered allocation and free on one stream.
struct Scratch {
    HpCudaContext *ctx = nullptr;
    void *ptr = nullptr;
    cudaStream_t stream = nullptr;  // null: the context stream
    Scratch() = default;
    Scratch(HpCudaContext *c, size_t bytes, cudaStream_t s = nullptr) : ctx(c), ptr(c->scratch(bytes, s)), stream(s) {}
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    Scratch(Scratch &&o) noexcept : ctx(o.ctx), ptr(o.ptr), stream(o.stream) { o.ptr = nullptr; }
    Scratch &operator=(Scratch &&o) noexcept {
        if (this != &o) {
            if (ptr) ctx->scratch_free(ptr, stream);
            ctx = o.ctx;
            ptr = o.ptr;
            stream = o.stream;
            o.ptr = nullptr;
        }
        return *this;
    }
    ~Scratch() {
        if (ptr) ctx->scratch_free(ptr, stream);
    }
    template <class T>
    T *as() const { return static_cast<T *>(ptr); }
};

// RAII owned output buffer: released unless handed out with release().
struct OwnedBuffer {
    HpCudaContext *ctx = nullptr;
    void *ptr = nullptr;
    OwnedBuffer() = default;
    OwnedBuffer(HpCudaContext *c, size_t bytes) : ctx(c), ptr(c->alloc(bytes)) {}
    OwnedBuffer(const OwnedBuffer &) = delete;
    OwnedBuffer &operator=(const OwnedBuffer &) = delete;
    OwnedBuffer(OwnedBuffer &&o) noexcept : ctx(o.ctx), ptr(o.ptr) { o.ptr = nullptr; }
    ~OwnedBuffer() {
        if (ptr) {
            try { ctx->unref(ptr); } catch (...) {}
        }
    }
    void *release() {
        void *p = ptr;
        ptr = nullptr;
        return p;
    }
    template <class T>
    T *as() const { return static_cast<T *>(ptr); }
};

inline void require_ctx(HpCudaContext *ctx) {
    if (!ctx) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
    check_cuda(cudaSetDevice(ctx->device));
}

// A registered MLE buffer of exactly 2^num_vars Fr.  When an asynchronous
// upload may still be writing it, the context stream waits for that upload
// (on the device): work queued after this call reads the uploaded values.
inline Fr *mle_ptr(HpCudaContext *ctx, HpCudaDeviceAddress a, size_t num_vars) {
    require(a != nullptr && num_vars <= kMaxNumVars);
    require(ctx->owns(a));
    require(ctx->bytes_of(a) == table_len(num_vars) * kFrBytes);
    ctx->await_ingress(a);
    return static_cast<Fr *>(a);
}

// Grid sizing: a multiple of the SM count, capped by the work.
inline unsigned grid_for(const HpCudaContext *ctx, size_t work_items, unsigned block,
                         unsigned blocks_per_sm = 8) {
    size_t need = (work_items + block - 1) / block;
    size_t cap = size_t(ctx->sm_count > 0 ? ctx->sm_count : 152) * blocks_per_sm;
    if (need > cap) need = cap;
    if (need == 0) need = 1;
    return static_cast<unsigned>(need);
}

// Kernels launched by this library since load (every launch site calls
// check_launch right after the launch).
void count_launch();

// Launch-error check after a kernel launch; also counts the launch.
inline void check_launch() {
    count_launch();
    check_cuda(cudaGetLastError());
}

// Canonical host Fr bytes -> device Montgomery values, in a small scratch.
// Host side only validates canonical range; conversion happens on device.
bool host_fr_is_canonical(const uint8_t *bytes);

}  // namespace hp
