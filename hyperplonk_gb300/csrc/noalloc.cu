// noalloc.cu -- MLE evaluation that allocates no device memory.
//
// Who needs it: a host that carves all of the GPU's memory into its own arena
// at start-up (a proving service that budgets HBM per request and must not
// have a library allocate behind its back).  Such callers cannot use
// hp_cuda_v1_mle_evaluate, which takes its fold buffers from the context's
// memory pool.  This variant keeps its intermediate values in one fixed
// file-scope device array instead, so a call issues only kernel launches, one
// device-to-host copy into the caller's buffer and a stream synchronisation.
//
// Limits and sharing rules:
//  - num_vars <= kNoAllocMaxVars (24); larger tables return InvalidParameters;
//  - the scratch array (kNoAllocScratchFr Fr = 16,402 x 32 bytes, ~513 KiB) is
//    held on every GPU that loads this library until the process exits;
//  - every call on a device shares that device's array: calls that overlap on
//    the GPU (different streams, or different host threads without ordering)
//    race on it.  Serialise them, e.g. by issuing them on one stream;
//  - nothing in the array needs to start at zero: each pass writes every entry
//    it later reads, so the contents left by the previous call never matter;
//  - `table` must be device memory of the current device (checked with
//    cudaPointerGetAttributes; anything else is InvalidParameters), because
//    the kernels run on the current device;
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) once; make that first call before any stream
//    capture begins.
#include <cstring>
#include <mutex>

#include "host_field.h"
#include "runtime.cuh"

namespace hp {
namespace {

constexpr int kNoAllocMaxVars = 24;
constexpr int kFoldLevels = 10;  // variables fixed per block pass (1024 entries)
// pass outputs: 2^(24-10) + 2^(24-20) entries, then 1 result and 1 canonical copy
constexpr size_t kNoAllocScratchFr = (size_t(1) << 14) + (size_t(1) << 4) + 2;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) Fr g_noalloc_scratch[kNoAllocScratchFr];

// Device address of g_noalloc_scratch per device (host code may not use the
// symbol itself as a pointer: it is a host-side stand-in).
Fr *g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

struct FoldPoint {
    Fr r[kNoAllocMaxVars];
};

// Block b folds src[b * 2^levels, (b+1) * 2^levels) with r[first .. first+levels)
// and writes the single value to dst[b].  2^(levels-1) threads, 2^levels Fr of
// shared memory (<= 32 KiB).
__global__ void k_noalloc_fold_block(const Fr *src, Fr *dst, int levels, FoldPoint pt, int first) {
    __shared__ Fr sm[1 << kFoldLevels];
    const size_t base = size_t(blockIdx.x) << levels;
    const int t = threadIdx.x;
    const int n = 1 << levels;
    for (int i = t; i < n; i += blockDim.x) sm[i] = load_fr(&src[base + i]);
    __syncthreads();
    for (int l = 0; l < levels; l++) {
        const int half = n >> (l + 1);
        Fr v;
        if (t < half) {
            Fr lo = sm[2 * t], hi = sm[2 * t + 1];
            v = lo + pt.r[first + l] * (hi - lo);
        }
        __syncthreads();
        if (t < half) sm[t] = v;
        __syncthreads();
    }
    if (t == 0) store_fr(&dst[blockIdx.x], sm[0]);
}

__global__ void k_noalloc_to_canonical(const Fr *src, Fr *dst) {
    if (threadIdx.x == 0 && blockIdx.x == 0) store_fr(dst, from_mont(load_fr(src)));
}

// Looks up (once per device) the device address of the scratch array.
Fr *scratch_for_current_device(int *device_out) {
    int dev = 0;
    check_cuda(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) fail(HP_CUDA_STATUS_INVALID_STATE);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_ptr[dev] == nullptr) {
        void *ptr = nullptr;
        check_cuda(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
        g_scratch_ptr[dev] = static_cast<Fr *>(ptr);
    }
    *device_out = dev;
    return g_scratch_ptr[dev];
}

}  // namespace
}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_mle_evaluate_noalloc(const void *table, size_t num_vars, const uint8_t *point,
                                                        uint8_t *out_evaluation, void *stream) {
    return hp::guard([&] {
        using namespace hp;
        require(table != nullptr && out_evaluation != nullptr);
        if (num_vars > size_t(kNoAllocMaxVars)) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        require(num_vars == 0 || point != nullptr);
        FoldPoint pt;
        std::memset(&pt, 0, sizeof pt);
        for (size_t i = 0; i < num_vars; i++) {
            host::Fr64 m;
            require(host::from_canonical(point + 32 * i, m));
            std::memcpy(pt.r[i].v, m.v, 32);
        }
        int dev = 0;
        Fr *scratch = scratch_for_current_device(&dev);
        // the table must live on the device the kernels run on: a peer
        // pointer (or a host pointer) would be read across the link or fault
        cudaPointerAttributes attr;
        std::memset(&attr, 0, sizeof attr);
        if (cudaPointerGetAttributes(&attr, table) != cudaSuccess) {
            (void)cudaGetLastError();
            fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        }
        if ((attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) || attr.device != dev)
            fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        // Regions: A = [0, 2^14) pass-1 output, B = [2^14, 2^14+16) pass-2
        // output, then the result slot and its canonical copy.
        Fr *region[2] = {scratch, scratch + (size_t(1) << 14)};
        Fr *result = scratch + (size_t(1) << 14) + 16;
        Fr *canonical = result + 1;
        const Fr *cur = static_cast<const Fr *>(table);
        size_t remaining = num_vars, first = 0;
        int which = 0;
        if (remaining == 0) {
            k_noalloc_to_canonical<<<1, 32, 0, s>>>(cur, canonical);
            check_launch();
        } else {
            while (remaining > 0) {
                int levels = int(remaining < size_t(kFoldLevels) ? remaining : size_t(kFoldLevels));
                size_t blocks = size_t(1) << (remaining - levels);
                Fr *dst = remaining == size_t(levels) ? result : region[which];
                k_noalloc_fold_block<<<unsigned(blocks), (1u << levels) / 2 > 0 ? (1u << levels) / 2 : 1u, 0, s>>>(
                    cur, dst, levels, pt, int(first));
                check_launch();
                cur = dst;
                which ^= 1;
                first += size_t(levels);
                remaining -= size_t(levels);
            }
            k_noalloc_to_canonical<<<1, 32, 0, s>>>(result, canonical);
            check_launch();
        }
        check_cuda(cudaMemcpyAsync(out_evaluation, canonical, 32, cudaMemcpyDeviceToHost, s));
        check_cuda(cudaStreamSynchronize(s));
    });
}
