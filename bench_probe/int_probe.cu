// int_probe.cu -- measures the integer-pipe ceilings the MSM and field
// kernels are held against: the 32-bit multiply-add (IMAD) issue rate and the
// Fq / Fr Montgomery multiplication rate of field.cuh, on the current GPU.
// Built as bench_probe/_build/libhp_probe.so; used by bench.py only to
// report a roofline denominator (no product path calls it).
#include <cuda_runtime.h>

#include <cstdint>

#include "field.cuh"

namespace {

constexpr int kChains = 16;

// Each thread runs kChains independent multiply-add chains; every iteration is
// kChains IMAD instructions (mad.lo.u32).
__global__ void k_imad(uint32_t *sink, int iters, uint32_t seed) {
    uint32_t a[kChains];
#pragma unroll
    for (int j = 0; j < kChains; j++) a[j] = seed + threadIdx.x * 131u + j;
    const uint32_t m = seed | 1u, c = seed ^ 0x9e3779b9u;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < kChains; j++) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[j]) : "r"(m), "r"(c));
    }
    uint32_t acc = 0;
#pragma unroll
    for (int j = 0; j < kChains; j++) acc ^= a[j];
    if (acc == 0x12345678u) sink[0] = acc;
}

// The same with 32x32->64 multiply-adds (mad.wide.u32, 64-bit accumulators):
// the instruction the field products are built from.
__global__ void k_imad_wide(uint32_t *sink, int iters, uint32_t seed) {
    uint64_t a[kChains];
#pragma unroll
    for (int j = 0; j < kChains; j++) a[j] = seed + threadIdx.x * 131u + j;
    const uint32_t m = seed | 1u, c = seed ^ 0x9e3779b9u;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < kChains; j++)  // multiplicand = the chain's own low word: nothing to hoist
            asm volatile("{\n\t.reg .u32 lo;\n\tcvt.u32.u64 lo, %0;\n\tmad.wide.u32 %0, lo, %1, %0;\n\t}"
                         : "+l"(a[j])
                         : "r"(m));
    }
    (void)c;
    uint64_t acc = 0;
#pragma unroll
    for (int j = 0; j < kChains; j++) acc ^= a[j];
    if (acc == 0x12345678u) sink[0] = uint32_t(acc);
}

template <class F>
__global__ void k_field_mul(uint32_t *sink, int iters, uint32_t seed) {
    F a, b, c;
#pragma unroll
    for (int i = 0; i < F::N; i++) {
        a.v[i] = (seed * 2654435761u + threadIdx.x + i) & 0x0fffffffu;
        b.v[i] = (seed * 40503u + blockIdx.x + 7 * i) & 0x0fffffffu;
        c.v[i] = (seed + 3 * i) & 0x0fffffffu;
    }
    for (int i = 0; i < iters; i++) {  // two independent chains
        a = a * b;
        c = c * b;
    }
    uint32_t acc = 0;
#pragma unroll
    for (int i = 0; i < F::N; i++) acc ^= a.v[i] ^ c.v[i];
    if (acc == 0x12345678u) sink[0] = acc;
}

template <class K>
double time_kernel(K launch, int reps) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    launch();  // warm-up
    cudaEventRecord(a);
    for (int r = 0; r < reps; r++) launch();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return double(ms) / 1e3 / reps;
}

}  // namespace

// Writes IMAD/s, Fq mul/s and Fr mul/s measured on `device`; returns a CUDA
// error code (0 on success).
extern "C" int hp_probe_integer_rates(int device, double *imad_per_s, double *fq_mul_per_s,
                                      double *fr_mul_per_s) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return int(e);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t *sink = nullptr;
    e = cudaMalloc(&sink, 4);
    if (e != cudaSuccess) return int(e);
    const unsigned blocks = unsigned(sms) * 8, threads = 256;
    const int imad_iters = 4096, mul_iters = 64;
    double t = time_kernel([&] { k_imad<<<blocks, threads>>>(sink, imad_iters, 7u); }, 5);
    *imad_per_s = double(blocks) * threads * imad_iters * kChains / t;
    t = time_kernel([&] { k_field_mul<hp::Fq><<<blocks, 128>>>(sink, mul_iters, 5u); }, 5);
    *fq_mul_per_s = double(blocks) * 128 * mul_iters * 2 / t;
    t = time_kernel([&] { k_field_mul<hp::Fr><<<blocks, 128>>>(sink, mul_iters, 3u); }, 5);
    *fr_mul_per_s = double(blocks) * 128 * mul_iters * 2 / t;
    e = cudaDeviceSynchronize();
    cudaFree(sink);
    return int(e);
}

// Writes the 32x32->64 multiply-add (mad.wide.u32) issue rate per second
// measured on `device`; returns a CUDA error code (0 on success).
extern "C" int hp_probe_wide_rate(int device, double *wide_per_s) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return int(e);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t *sink = nullptr;
    e = cudaMalloc(&sink, 4);
    if (e != cudaSuccess) return int(e);
    const unsigned blocks = unsigned(sms) * 8, threads = 256;
    const int iters = 2048;
    const double t = time_kernel([&] { k_imad_wide<<<blocks, threads>>>(sink, iters, 11u); }, 5);
    *wide_per_s = double(blocks) * threads * iters * kChains / t;
    e = cudaDeviceSynchronize();
    cudaFree(sink);
    return int(e);
}
