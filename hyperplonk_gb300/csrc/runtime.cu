// runtime.cu -- context lifetime, buffer registry, retirement.
// ABI: hp_cuda_v1_context_create / _destroy / _buffer_retire / _context_stream
// (reference bridge.h:43-45, bridge_runtime.cpp).
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <mutex>
#include <thread>

#include "runtime.cuh"

using hp::check_cuda;
using hp::fail;
using hp::guard;
using hp::require;

void *HpCudaContext::alloc(size_t bytes) {
    void *p = nullptr;
    check_cuda(cudaMallocFromPoolAsync(&p, bytes ? bytes : 16, pool, stream));
    try {
        buffers.emplace(p, Buffer{bytes, 1, true});
    } catch (...) {
        cudaFreeAsync(p, stream);
        throw;
    }
    return p;
}

void *HpCudaContext::scratch(size_t bytes, cudaStream_t s) {
    void *p = nullptr;
    check_cuda(cudaMallocFromPoolAsync(&p, bytes ? bytes : 16, pool, s ? s : stream));
    return p;
}

uint8_t *HpCudaContext::mailbox(size_t bytes, void **dev) {
    if (bytes > mailbox_bytes) {
        if (h_mailbox) {
            check_cuda(cudaStreamSynchronize(stream));
            check_cuda(cudaFreeHost(h_mailbox));
            h_mailbox = nullptr;
            d_mailbox = nullptr;
            mailbox_bytes = 0;
        }
        const size_t n = std::max<size_t>(bytes, 4096);
        void *h = nullptr;
        check_cuda(cudaHostAlloc(&h, n, cudaHostAllocMapped));
        void *d = nullptr;
        cudaError_t e = cudaHostGetDevicePointer(&d, h, 0);
        if (e != cudaSuccess) {
            cudaFreeHost(h);
            check_cuda(e);
        }
        h_mailbox = static_cast<uint8_t *>(h);
        d_mailbox = d;
        mailbox_bytes = n;
    }
    *dev = d_mailbox;
    return h_mailbox;
}

void HpCudaContext::scratch_free(void *p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s ? s : stream);
}

void HpCudaContext::fork(int k) {
    if (k > kWorkers) k = kWorkers;
    if (!fork_event) check_cuda(cudaEventCreateWithFlags(&fork_event, cudaEventDisableTiming));
    check_cuda(cudaEventRecord(fork_event, stream));
    for (int i = 0; i < k; i++) {
        if (!workers[i]) check_cuda(cudaStreamCreateWithFlags(&workers[i], cudaStreamNonBlocking));
        if (!join_events[i]) check_cuda(cudaEventCreateWithFlags(&join_events[i], cudaEventDisableTiming));
        check_cuda(cudaStreamWaitEvent(workers[i], fork_event, 0));
    }
}

void HpCudaContext::join(int k) {
    if (k > kWorkers) k = kWorkers;
    for (int i = 0; i < k; i++) {
        check_cuda(cudaEventRecord(join_events[i], workers[i]));
        check_cuda(cudaStreamWaitEvent(stream, join_events[i], 0));
    }
}

void HpCudaContext::ref(void *p) {
    auto it = buffers.find(p);
    if (it == buffers.end()) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
    it->second.refs++;
}

void HpCudaContext::unref(void *p) {
    auto it = buffers.find(p);
    if (it == buffers.end()) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
    if (--it->second.refs == 0) {
        // a buffer an asynchronous upload may still write is freed after it
        if (it->second.ingress) check_cuda(cudaStreamWaitEvent(stream, it->second.ingress->ready, 0));
        buffers.erase(it);
        check_cuda(cudaFreeAsync(p, stream));
    }
}

void HpCudaContext::await_ingress(void *p) {
    auto it = buffers.find(p);
    if (it != buffers.end() && it->second.ingress)
        check_cuda(cudaStreamWaitEvent(stream, it->second.ingress->ready, 0));
}

std::shared_ptr<HpCudaIngress> HpCudaContext::new_ingress() {
    if (!ingress_stream) check_cuda(cudaStreamCreateWithFlags(&ingress_stream, cudaStreamNonBlocking));
    if (!ingress_flags_h) {
        void *h = nullptr;
        check_cuda(cudaHostAlloc(&h, kIngressSlots * sizeof(uint32_t), cudaHostAllocDefault));
        ingress_flags_h = static_cast<uint32_t *>(h);
    }
    int slot = -1;
    for (int i = 0; i < kIngressSlots; i++)
        if (!ingress_used[i]) {
            slot = i;
            break;
        }
    if (slot < 0) fail(HP_CUDA_STATUS_INVALID_STATE);  // too many uploads not yet waited for
    auto in = std::make_shared<HpCudaIngress>();
    check_cuda(cudaEventCreateWithFlags(&in->ready, cudaEventDisableTiming));
    in->slot = slot;
    in->slot_used = &ingress_used[slot];
    ingress_used[slot] = true;
    ingress_flags_h[slot] = 0;
    return in;
}

void HpCudaContext::retire(void *p) {
    auto it = buffers.find(p);
    if (it == buffers.end() || !it->second.public_handle) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
    it->second.public_handle = false;
    unref(p);
}

size_t HpCudaContext::bytes_of(void *p) const {
    auto it = buffers.find(p);
    return it == buffers.end() ? 0 : it->second.bytes;
}

cudaEvent_t HpCudaContext::take_event() {
    if (!event_pool.empty()) {
        cudaEvent_t e = event_pool.back();
        event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    check_cuda(cudaEventCreate(&e));
    return e;
}

int HpCudaContext::prof_begin(const char *name, cudaStream_t s) {
    if (!profiling) return -1;
    Pending p{name, take_event(), take_event()};
    check_cuda(cudaEventRecord(p.start, s ? s : stream));
    pending.push_back(p);
    return int(pending.size()) - 1;
}

void HpCudaContext::prof_end(int token, cudaStream_t s) {
    if (token < 0) return;
    check_cuda(cudaEventRecord(pending[size_t(token)].stop, s ? s : stream));
}

void HpCudaContext::prof_resolve() {
    if (pending.empty()) return;
    check_cuda(cudaStreamSynchronize(stream));
    for (auto &p : pending) {
        float ms = 0.f;
        check_cuda(cudaEventSynchronize(p.stop));
        check_cuda(cudaEventElapsedTime(&ms, p.start, p.stop));
        auto &t = totals[p.name];
        t.first += double(ms);
        t.second += 1;
        event_pool.push_back(p.start);
        event_pool.push_back(p.stop);
    }
    pending.clear();
}

void HpCudaContext::clear_flags() { check_cuda(cudaMemsetAsync(d_flags, 0, sizeof(uint32_t), stream)); }

uint32_t HpCudaContext::sync_flags() {
    check_cuda(cudaMemcpyAsync(h_flags, d_flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    check_cuda(cudaStreamSynchronize(stream));
    return *h_flags;
}

void HpCudaContext::sync() { check_cuda(cudaStreamSynchronize(stream)); }

bool hp::host_fr_is_canonical(const uint8_t *bytes) {
    static const uint8_t P[32] = {0x01, 0x00, 0x00, 0x00, 0xff, 0xff, 0xff, 0xff, 0xfe, 0x5b, 0xfe,
                                  0xff, 0x02, 0xa4, 0xbd, 0x53, 0x05, 0xd8, 0xa1, 0x09, 0x08, 0xd8,
                                  0x39, 0x33, 0x48, 0x7d, 0x9d, 0x29, 0x53, 0xa7, 0xed, 0x73};
    for (int i = 31; i >= 0; i--) {
        if (bytes[i] != P[i]) return bytes[i] < P[i];
    }
    return false;
}

extern "C" HpCudaStatus hp_cuda_v1_context_create(int32_t device_id, HpCudaContext **out) {
    if (out) *out = nullptr;
    return guard([&] {
        require(out != nullptr && device_id >= 0);
        int count = 0;
        check_cuda(cudaGetDeviceCount(&count));
        require(device_id < count);
        check_cuda(cudaSetDevice(device_id));
        HpCudaContext *ctx = new HpCudaContext();
        ctx->device = device_id;
        try {
            check_cuda(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device_id));
            check_cuda(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
            cudaMemPoolProps props;
            std::memset(&props, 0, sizeof props);
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = device_id;
            check_cuda(cudaMemPoolCreate(&ctx->pool, &props));
            uint64_t threshold = UINT64_MAX;
            check_cuda(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &threshold));
            check_cuda(cudaMalloc(&ctx->d_flags, sizeof(uint32_t)));
            check_cuda(cudaMallocHost(&ctx->h_flags, sizeof(uint32_t)));
            check_cuda(cudaMemset(ctx->d_flags, 0, sizeof(uint32_t)));
        } catch (...) {
            if (ctx->d_flags) cudaFree(ctx->d_flags);
            if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
            if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
            if (ctx->stream) cudaStreamDestroy(ctx->stream);
            delete ctx;
            throw;
        }
        *out = ctx;
    });
}

struct HpCudaContext::Responder {
    std::thread thread;
    std::mutex mu;
    std::condition_variable cv;
    std::function<void()> job;
    bool stop = false;
    std::atomic<int> state{0};  // 0 idle, 1 queued or running, 2 finished
    std::exception_ptr error;
};

void HpCudaContext::respond_start(std::function<void()> job) {
    if (!responder) {
        responder = std::make_unique<Responder>();
        Responder *r = responder.get();
        const int dev = device;
        r->thread = std::thread([r, dev] {
            cudaSetDevice(dev);
            std::unique_lock<std::mutex> lk(r->mu);
            for (;;) {
                r->cv.wait(lk, [r] { return r->stop || bool(r->job); });
                if (r->stop) return;
                std::function<void()> j = std::move(r->job);
                r->job = nullptr;
                lk.unlock();
                try {
                    j();
                } catch (...) {
                    r->error = std::current_exception();
                }
                r->state.store(2, std::memory_order_release);
                lk.lock();
            }
        });
    }
    {
        std::lock_guard<std::mutex> lk(responder->mu);
        responder->error = nullptr;
        responder->state.store(1, std::memory_order_relaxed);
        responder->job = std::move(job);
    }
    responder->cv.notify_one();
}

void HpCudaContext::respond_wait() {
    if (!responder) return;
    while (responder->state.load(std::memory_order_acquire) == 1) std::this_thread::yield();
    responder->state.store(0, std::memory_order_relaxed);
    if (responder->error) {
        std::exception_ptr e = responder->error;
        responder->error = nullptr;
        std::rethrow_exception(e);
    }
}

void HpCudaContext::respond_shutdown() {
    if (!responder) return;
    {
        std::lock_guard<std::mutex> lk(responder->mu);
        responder->stop = true;
    }
    responder->cv.notify_one();
    if (responder->thread.joinable()) responder->thread.join();
    responder.reset();
}

// Jobs are handed over under `mu`: a worker takes a job's function and size
// and marks itself busy while holding the lock, and a new job is installed
// only while the lock is held with no worker busy, so a worker never runs
// items of a job other than the one it took.
struct HpCudaContext::HostPool {
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv;
    const std::function<void(size_t)> *fn = nullptr;
    size_t n = 0;
    uint64_t generation = 0;
    bool stop = false;
    int busy = 0;                 // workers inside a job (guarded by mu)
    std::atomic<size_t> next{0};  // next item to take
    std::atomic<size_t> done{0};  // items finished
    std::exception_ptr error;     // first failure (guarded by error_mu)
    std::mutex error_mu;

    void run_items(const std::function<void(size_t)> *f, size_t count) {
        for (size_t i; (i = next.fetch_add(1)) < count;) {
            try {
                (*f)(i);
            } catch (...) {
                std::lock_guard<std::mutex> lk(error_mu);
                if (!error) error = std::current_exception();
            }
            done.fetch_add(1, std::memory_order_release);
        }
    }
};

void HpCudaContext::host_parallel_for(size_t n, const std::function<void(size_t)> &fn) {
    if (n == 0) return;
    if (n == 1) {
        fn(0);
        return;
    }
    if (!host_pool) {
        host_pool = std::make_unique<HostPool>();
        HostPool *p = host_pool.get();
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const unsigned workers = std::min(7u, hw > 1 ? hw - 1 : 1u);
        for (unsigned w = 0; w < workers; w++) {
            p->threads.emplace_back([p] {
                uint64_t seen = 0;
                std::unique_lock<std::mutex> lk(p->mu);
                for (;;) {
                    p->cv.wait(lk, [&] { return p->stop || p->generation != seen; });
                    if (p->stop) return;
                    seen = p->generation;
                    const std::function<void(size_t)> *f = p->fn;
                    const size_t count = p->n;
                    p->busy++;
                    lk.unlock();
                    p->run_items(f, count);
                    lk.lock();
                    p->busy--;
                }
            });
        }
    }
    HostPool *p = host_pool.get();
    {
        std::unique_lock<std::mutex> lk(p->mu);
        while (p->busy != 0) {  // a worker still leaving the previous job
            lk.unlock();
            std::this_thread::yield();
            lk.lock();
        }
        p->fn = &fn;
        p->n = n;
        p->next.store(0);
        p->done.store(0);
        p->error = nullptr;
        p->generation++;
    }
    p->cv.notify_all();
    p->run_items(&fn, n);
    while (p->done.load(std::memory_order_acquire) < n) std::this_thread::yield();
    std::exception_ptr e;
    {
        std::lock_guard<std::mutex> lk(p->error_mu);
        e = p->error;
    }
    if (e) std::rethrow_exception(e);
}

void HpCudaContext::host_pool_shutdown() {
    if (!host_pool) return;
    {
        std::lock_guard<std::mutex> lk(host_pool->mu);
        host_pool->stop = true;
    }
    host_pool->cv.notify_all();
    for (auto &t : host_pool->threads)
        if (t.joinable()) t.join();
    host_pool.reset();
}

extern "C" HpCudaStatus hp_cuda_v1_context_destroy(HpCudaContext *ctx) {
    return guard([&] {
        require(ctx != nullptr);
        ctx->respond_shutdown();
        ctx->host_pool_shutdown();
        cudaSetDevice(ctx->device);
        if (ctx->ingress_stream) cudaStreamSynchronize(ctx->ingress_stream);
        cudaError_t first = cudaStreamSynchronize(ctx->stream);
        for (auto &kv : ctx->buffers) cudaFreeAsync(kv.first, ctx->stream);
        ctx->buffers.clear();
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (first == cudaSuccess) first = e;
        for (auto &p : ctx->pending) {
            cudaEventDestroy(p.start);
            cudaEventDestroy(p.stop);
        }
        for (auto e : ctx->event_pool) cudaEventDestroy(e);
        for (int i = 0; i < HpCudaContext::kWorkers; i++) {
            if (ctx->workers[i]) cudaStreamDestroy(ctx->workers[i]);
            if (ctx->join_events[i]) cudaEventDestroy(ctx->join_events[i]);
        }
        if (ctx->fork_event) cudaEventDestroy(ctx->fork_event);
        cudaFree(ctx->d_flags);
        cudaFreeHost(ctx->h_flags);
        if (ctx->h_mailbox) cudaFreeHost(ctx->h_mailbox);
        if (ctx->ingress_flags_h) cudaFreeHost(ctx->ingress_flags_h);
        if (ctx->ingress_stream) cudaStreamDestroy(ctx->ingress_stream);
        cudaStreamDestroy(ctx->stream);
        cudaMemPoolDestroy(ctx->pool);
        delete ctx;
        check_cuda(first);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_buffer_retire(HpCudaContext *ctx, HpCudaDeviceAddress address) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(address != nullptr && ctx->owns(address));
        ctx->retire(address);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_context_stream(HpCudaContext *ctx, void **out_stream) {
    if (out_stream) *out_stream = nullptr;
    return guard([&] {
        require(ctx != nullptr && out_stream != nullptr);
        *out_stream = static_cast<void *>(ctx->stream);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_context_profile(HpCudaContext *ctx, int32_t enable) {
    return guard([&] {
        hp::require_ctx(ctx);
        ctx->prof_resolve();
        ctx->profiling = enable != 0;
        ctx->totals.clear();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_context_profile_read(HpCudaContext *ctx, const char *kernel, double *total_ms,
                                                         uint64_t *launches) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(kernel != nullptr && total_ms != nullptr && launches != nullptr);
        ctx->prof_resolve();
        auto it = ctx->totals.find(kernel);
        *total_ms = it == ctx->totals.end() ? 0.0 : it->second.first;
        *launches = it == ctx->totals.end() ? 0 : it->second.second;
    });
}

extern "C" HpCudaStatus hp_cuda_v1_context_memory(HpCudaContext *ctx, int32_t reset_high, uint64_t *out3) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(out3 != nullptr);
        uint64_t used = 0, high = 0, reserved = 0;  // the attributes are 64-bit values
        check_cuda(cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrUsedMemCurrent, &used));
        check_cuda(cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrUsedMemHigh, &high));
        check_cuda(cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrReservedMemCurrent, &reserved));
        out3[0] = used;
        out3[1] = high;
        out3[2] = reserved;
        if (reset_high) {
            uint64_t zero = 0;  // resets the mark to the current use
            check_cuda(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrUsedMemHigh, &zero));
        }
    });
}

static std::atomic<uint64_t> g_kernel_launches{0};

void hp::count_launch() { g_kernel_launches.fetch_add(1, std::memory_order_relaxed); }

extern "C" HpCudaStatus hp_cuda_v1_kernel_launch_count(uint64_t *out) {
    return guard([&] {
        require(out != nullptr);
        *out = g_kernel_launches.load(std::memory_order_relaxed);
    });
}
