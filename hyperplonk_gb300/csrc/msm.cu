// msm.cu -- variable-base MSM sum_i s_i * P_i over BLS12-381 G1.
//
// Reference value semantics: ark-ec 0.6.0 VariableBaseMSM::msm_unchecked as
// called by backend/src/cpu/multilinear_kzg.rs:55,131.  The reference's
// device MSM (backend/src/ascend910b3/native/msm*.{cpp,asc}) uses unsigned
// windows, LSD radix grouping and an affine bucket tree; this is a different,
// GB300-first design:
//
//  1. prepare (once per SRS layer): window w of base i is 2^(c*w) * P_i,
//     stored affine in HBM, so all ceil(256/c) windows of the signed-digit
//     expansion share ONE set of 2^(c-1) buckets and there is no window
//     combination;
//  2. digits: signed c-bit digits in [-2^(c-1), 2^(c-1)]; a counting sort
//     (histogram -> exclusive scan -> atomic scatter) groups the
//     (window, point, sign) records by bucket -- bucket order inside a group
//     is irrelevant because field arithmetic is exact;
//  3. accumulate: flat chunks of L bucket-ordered records per thread, XYZZ
//     mixed additions (8M + 2S), buckets cut by chunk edges fixed up after;
//  4. reduce: sum_b (b+1) S_b via segments of `seg` buckets (running sums,
//     two XYZZ additions per bucket), then the segment weights j are split
//     into bits: sum_j j R_j = sum_k 2^k sum_{j : bit k} R_j, whose subset sums
//     are parallel tree reductions;
//  5. the host finishes the short Horner chain over those subset sums and
//     converts to affine (one inversion), see host_ec.h.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "msm.cuh"
#include "runtime.cuh"

namespace hp {

int msm_window_bits(size_t n) {
    // tuning override (read when a layer is prepared): HP_MSM_WINDOW_BITS=c, 4 <= c <= 22
    if (const char *env = std::getenv("HP_MSM_WINDOW_BITS")) {
        int c = std::atoi(env);
        if (c >= 4 && c <= 22) return c;
    }
    const MsmTuning t = msm_tuning_alone(n);
    if (t.c && msm_window_fits(n, t.c)) return t.c;
    return msm_window_bits_model(n);
}

bool msm_window_fits(size_t n, int c) {
    if (c < 4 || c > 22) return false;
    // records are (window * n + point) in 31 bits
    if (size_t(msm_windows(c)) * n >= (size_t(1) << 31)) return false;
    // The top window holds only 255 - c(W-1) bits of a scalar (< 2^255): its
    // n records fall into that many bits' worth of buckets.  Skip widths that
    // would pile more than 2048 records onto one bucket.
    const int top_bits = 255 - c * (msm_windows(c) - 1);
    const double top_buckets = top_bits >= 2 ? double(size_t(1) << (top_bits - 1)) : 1.0;
    return c == 4 || double(n) / top_buckets <= 2048.0;
}

int msm_window_bits_model(size_t n) {
    int best = 4;
    double best_cost = 1e300;
    for (int c = 4; c <= 20; c++) {
        if (!msm_window_fits(n, c)) continue;
        double cost = double(msm_windows(c)) * 10.0 * double(n) + 28.0 * double(size_t(1) << (c - 1));
        if (cost < best_cost) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

uint32_t msm_default_seg(int c) {
    // 16-bucket segments from 2^17 buckets up; shorter below, because a
    // segment is a chain of 2 seg dependent additions and smaller MSMs are
    // latency-bound (measured: 2^15 buckets seg 4 1.29 ms vs seg 8 1.42 ms
    // and seg 16 1.70 ms; 2^11 buckets seg 1 best; 2^19 seg 16 9.20 ms vs
    // seg 8 9.56 ms and seg 32 9.47 ms)
    const size_t buckets = size_t(1) << (c - 1);
    size_t seg = std::min<size_t>(16, std::max<size_t>(1, buckets >> 13));
    // the subset reduction takes at most msm_max_segments() segments
    while (buckets / seg > msm_max_segments()) seg *= 2;
    return uint32_t(seg);
}

static bool seg_fits(size_t seg, size_t buckets) {
    return seg >= 1 && seg <= 64 && (seg & (seg - 1)) == 0 && seg <= buckets && buckets / seg <= msm_max_segments();
}

MsmShape msm_shape(const MsmLayer &layer) {
    MsmShape s;
    s.buckets = size_t(1) << (layer.c - 1);
    s.seg = msm_default_seg(layer.c);
    if (layer.seg && seg_fits(layer.seg, s.buckets)) s.seg = layer.seg;
    // tuning override: HP_MSM_SEG=s (power of two, 1..64)
    if (const char *env = std::getenv("HP_MSM_SEG")) {
        const long v = std::atol(env);
        if (v >= 1 && v <= 64 && (v & (v - 1)) == 0) s.seg = std::min<size_t>(s.buckets, size_t(v));
    }
    s.segments = s.buckets / s.seg;
    s.seg_bits = 0;
    while ((size_t(1) << s.seg_bits) < s.segments) s.seg_bits++;
    s.partials = s.seg_bits + 1;
    return s;
}

// ---------------------------------------------------------------------------
// Prepare: packets -> window 0 -> windows 1..W-1
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool fq_canonical_le(const uint8_t *b, Fq &out) {
    Fq v;
#pragma unroll
    for (int i = 0; i < 12; i++)
        v.v[i] = uint32_t(b[4 * i]) | (uint32_t(b[4 * i + 1]) << 8) | (uint32_t(b[4 * i + 2]) << 16) |
                 (uint32_t(b[4 * i + 3]) << 24);
    out = v;
    return is_canonical(v);
}

__global__ void k_unpack_packets(const uint8_t *packets, size_t n, Affine *out, uint32_t *flags) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x) {
        const uint8_t *p = packets + 97 * i;
        Affine a;
        a.x = Fq::zero();
        a.y = Fq::zero();
        uint8_t tag = p[0];
        if (tag == 1) {
            uint32_t any = 0;
            for (int k = 1; k < 97; k++) any |= p[k];
            if (any) atomicOr(flags, kFlagNonCanonical);
        } else if (tag == 0) {
            Fq x, y;
            bool ok = fq_canonical_le(p + 1, x) & fq_canonical_le(p + 49, y);
            if (!ok) atomicOr(flags, kFlagNonCanonical);
            a.x = to_mont(x);
            a.y = to_mont(y);
            if (affine_is_inf(a)) atomicOr(flags, kFlagNonCanonical);  // (0,0) is not a finite point
        } else {
            atomicOr(flags, kFlagNonCanonical);
        }
        store_affine(&out[i], a);
    }
}

// tmp[i] = 2^c * prev[i] (XYZZ)
__global__ void k_window_double(const Affine *prev, Xyzz *tmp, size_t n, int c) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x) {
        Affine a = load_affine(&prev[i]);
        Xyzz p;
        if (affine_is_inf(a)) {
            p = xyzz_inf();
        } else {
            p = xyzz_double_affine(a.x, a.y);
            for (int k = 1; k < c; k++) p = xyzz_double(p);
        }
        store_xyzz(&tmp[i], p);
    }
}

// XYZZ -> affine with one inversion per block (Montgomery trick over
// kNormBlock * kNormChunk points).  `pre` is scratch of n Fq.
constexpr int kNormBlock = 128;
constexpr int kNormChunk = 4;

__global__ void __launch_bounds__(kNormBlock) k_normalize(const Xyzz *in, Affine *out, Fq *pre, size_t n) {
    __shared__ Fq spre[kNormBlock];
    __shared__ Fq ssuf[kNormBlock];
    __shared__ Fq total_inv;
    const int t = threadIdx.x;
    const size_t base = (size_t(blockIdx.x) * kNormBlock + t) * kNormChunk;
    Fq one = Fq::one();
    Fq p = one;
    for (int k = 0; k < kNormChunk; k++) {
        size_t i = base + k;
        if (i < n) {
            Xyzz q = load_xyzz(&in[i]);
            Fq v = xyzz_is_inf(q) ? one : q.zz * q.zzz;
            store_words(reinterpret_cast<uint32_t *>(&pre[i]), p);
            p = p * v;
        }
    }
    spre[t] = p;
    ssuf[t] = p;
    __syncthreads();
    for (int off = 1; off < kNormBlock; off <<= 1) {
        Fq a = (t >= off) ? spre[t - off] * spre[t] : spre[t];
        Fq b = (t + off < kNormBlock) ? ssuf[t + off] * ssuf[t] : ssuf[t];
        __syncthreads();
        spre[t] = a;
        ssuf[t] = b;
        __syncthreads();
    }
    if (t == 0) total_inv = inverse(spre[kNormBlock - 1]);
    __syncthreads();
    Fq inv = total_inv;
    if (t > 0) inv = inv * spre[t - 1];
    if (t + 1 < kNormBlock) inv = inv * ssuf[t + 1];
    for (int k = kNormChunk - 1; k >= 0; k--) {
        size_t i = base + k;
        if (i < n) {
            Xyzz q = load_xyzz(&in[i]);
            Affine a;
            if (xyzz_is_inf(q)) {
                a.x = Fq::zero();
                a.y = Fq::zero();
            } else {
                Fq prefix;
                load_words(prefix, reinterpret_cast<const uint32_t *>(&pre[i]));
                Fq vinv = inv * prefix;            // (zz * zzz)^-1
                inv = inv * (q.zz * q.zzz);
                a.x = q.x * (vinv * q.zzz);        // X / ZZ
                a.y = q.y * (vinv * q.zz);         // Y / ZZZ
            }
            store_affine(&out[i], a);
        }
    }
}

void xyzz_to_affine(HpCudaContext *ctx, const Xyzz *in, Affine *out, Fq *pre, size_t n) {
    size_t per_block = size_t(kNormBlock) * kNormChunk;
    k_normalize<<<unsigned((n + per_block - 1) / per_block), kNormBlock, 0, ctx->stream>>>(in, out, pre, n);
    check_launch();
}

// d_i: 256 pseudo-random bits per index (SplitMix64 finaliser over (seed, i, k)),
// top two bits cleared so d_i < 2^254 < r.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void k_msm_delta(Fr *out, size_t n, uint64_t seed) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        Fr d;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint64_t w = mix64(seed + 0x9e3779b97f4a7c15ull * (4 * uint64_t(i) + uint64_t(k) + 1));
            d.v[2 * k] = uint32_t(w);
            d.v[2 * k + 1] = uint32_t(w >> 32);
        }
        d.v[7] &= 0x3fffffffu;
        store_fr(&out[i], d);
    }
}

__global__ void k_msm_to_mont(Fr *data, size_t n) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        store_fr(&data[i], to_mont(load_fr(&data[i])));
}

// Windows 1..W-1 from window 0 (already in layer.bases), then the randomiser
// d and D = sum d_i P_i.
static void msm_sum_bases(HpCudaContext *ctx, const MsmLayer &layer, const Fr *scalars, uint32_t want,
                          const Xyzz *total, Xyzz *out, int rows, cudaStream_t st, size_t n = 0,
                          const Xyzz *d_sum = nullptr);
static void msm_finish_layer(HpCudaContext *ctx, MsmLayer &layer) {
    const size_t n = layer.n;
    if (layer.windows > 1) {
        Scratch tmp(ctx, n * sizeof(Xyzz)), pre(ctx, n * sizeof(Fq));
        size_t per_block = size_t(kNormBlock) * kNormChunk;
        for (int w = 1; w < layer.windows; w++) {
            k_window_double<<<grid_for(ctx, n, 128), 128, 0, ctx->stream>>>(
                layer.bases + size_t(w - 1) * n, tmp.as<Xyzz>(), n, layer.c);
            check_launch();
            k_normalize<<<unsigned((n + per_block - 1) / per_block), kNormBlock, 0, ctx->stream>>>(
                tmp.as<Xyzz>(), layer.bases + size_t(w) * n, pre.as<Fq>(), n);
            check_launch();
        }
    }
    layer.delta = static_cast<Fr *>(ctx->scratch(n * sizeof(Fr)));
    k_msm_delta<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(layer.delta, n, uint64_t(n) * 0x9e3779b97f4a7c15ull);
    check_launch();
    Scratch dm(ctx, n * sizeof(Fr));
    check_cuda(cudaMemcpyAsync(dm.ptr, layer.delta, n * sizeof(Fr), cudaMemcpyDeviceToDevice, ctx->stream));
    k_msm_to_mont<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(dm.as<Fr>(), n);
    check_launch();
    MsmLayer plain = layer;
    plain.delta = nullptr;
    const MsmShape sh = msm_shape(plain);
    Scratch parts(ctx, size_t(sh.partials) * sizeof(Xyzz));
    msm_run(ctx, plain, dm.as<Fr>(), parts.as<Xyzz>());
    std::vector<host::Xyzz64> hp_parts(size_t(sh.partials));
    check_cuda(cudaMemcpyAsync(hp_parts.data(), parts.ptr, size_t(sh.partials) * sizeof(Xyzz),
                               cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    host::Xyzz64 d = msm_combine_host(sh, hp_parts.data());
    // D on the device for the binary path (same byte layout as Xyzz), -D for the host finish
    layer.d_sum = static_cast<Xyzz *>(ctx->scratch(sizeof(Xyzz)));
    static_assert(sizeof(host::Xyzz64) == sizeof(Xyzz), "host and device XYZZ share a layout");
    check_cuda(cudaMemcpyAsync(layer.d_sum, &d, sizeof(Xyzz), cudaMemcpyHostToDevice, ctx->stream));
    ctx->sync();
    d.y = host::fq_sub(host::Fq64{{0, 0, 0, 0, 0, 0}}, d.y);
    layer.minus_d = d;
    // the sum of all window-0 bases, for 0/1 tables that are mostly ones
    layer.base_sum = static_cast<Xyzz *>(ctx->scratch(sizeof(Xyzz)));
    msm_sum_bases(ctx, layer, nullptr, 1, nullptr, layer.base_sum, 1, ctx->stream);
}

void msm_apply_tuning(MsmLayer &layer) {
    // a tuned segment and chunk belong to the window width they were measured with
    const MsmTuning t = msm_tuning_alone(layer.n);
    layer.seg = t.c == layer.c ? t.seg : 0;
    layer.chunk = t.c == layer.c ? t.chunk : 0;
}

bool msm_prepare_layer(HpCudaContext *ctx, MsmLayer &layer, const uint8_t *packets, size_t n) {
    layer.n = n;
    layer.c = msm_window_bits(n);
    layer.windows = msm_windows(layer.c);
    msm_apply_tuning(layer);
    layer.bases = static_cast<Affine *>(ctx->scratch(size_t(layer.windows) * n * sizeof(Affine)));
    Scratch raw(ctx, n * 97);
    check_cuda(cudaMemcpyAsync(raw.ptr, packets, n * 97, cudaMemcpyHostToDevice, ctx->stream));
    ctx->clear_flags();
    k_unpack_packets<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(raw.as<uint8_t>(), n, layer.bases,
                                                                     ctx->d_flags);
    check_launch();
    uint32_t flags = ctx->sync_flags();
    if (flags & kFlagNonCanonical) return false;
    msm_finish_layer(ctx, layer);
    return true;
}

void msm_prepare_prefix_c(HpCudaContext *ctx, MsmLayer &prefix, const MsmLayer &source, size_t n, int c) {
    require(n >= 1 && n <= source.n && c >= 4 && c <= 22);
    prefix.n = n;
    prefix.c = c;
    prefix.windows = msm_windows(c);
    // records are (window * n + point) in 31 bits
    require(size_t(prefix.windows) * n < (size_t(1) << 31));
    prefix.seg = 0;
    prefix.chunk = 0;
    prefix.bases = static_cast<Affine *>(ctx->scratch(size_t(prefix.windows) * n * sizeof(Affine)));
    check_cuda(cudaMemcpyAsync(prefix.bases, source.bases, n * sizeof(Affine), cudaMemcpyDeviceToDevice,
                               ctx->stream));
    msm_finish_layer(ctx, prefix);
}

void msm_prepare_prefix(HpCudaContext *ctx, MsmLayer &prefix, const MsmLayer &source, size_t n) {
    msm_prepare_prefix_c(ctx, prefix, source, n, msm_window_bits(n));
    msm_apply_tuning(prefix);
}

void msm_retune_layer(HpCudaContext *ctx, MsmLayer &layer) {
    const int c = msm_window_bits(layer.n);
    if (c != layer.c) {
        MsmLayer fresh;
        try {
            msm_prepare_prefix_c(ctx, fresh, layer, layer.n, c);
        } catch (...) {
            msm_release_layer(ctx, fresh);
            throw;
        }
        msm_release_layer(ctx, layer);
        layer = fresh;
    }
    msm_apply_tuning(layer);
}

void msm_random_scalars(HpCudaContext *ctx, Fr *out, size_t n, uint64_t seed, cudaStream_t stream) {
    k_msm_delta<<<grid_for(ctx, n, 256), 256, 0, stream>>>(out, n, seed);
    check_launch();
    k_msm_to_mont<<<grid_for(ctx, n, 256), 256, 0, stream>>>(out, n);
    check_launch();
}

void msm_release_layer(HpCudaContext *ctx, MsmLayer &layer) {
    if (layer.bases) ctx->scratch_free(layer.bases);
    if (layer.delta) ctx->scratch_free(layer.delta);
    if (layer.d_sum) ctx->scratch_free(layer.d_sum);
    if (layer.base_sum) ctx->scratch_free(layer.base_sum);
    layer.bases = nullptr;
    layer.delta = nullptr;
    layer.d_sum = nullptr;
    layer.base_sum = nullptr;
}

// ---------------------------------------------------------------------------
// Digits and counting sort
// ---------------------------------------------------------------------------

// bits [bit, bit + c) of a canonical 256-bit value (c <= 20)
__device__ __forceinline__ uint32_t window_bits(const Fr &s, int bit, int c) {
    if (bit >= 256) return 0;
    int limb = bit >> 5, off = bit & 31;
    uint32_t v = s.v[limb] >> off;
    if (off + c > 32 && limb + 1 < 8) v |= s.v[limb + 1] << (32 - off);
    return v & ((1u << c) - 1);
}

// Signed-digit recoding: calls f(window, magnitude, negative) for nonzero digits.
template <class F>
__device__ __forceinline__ void for_each_digit(const Fr &canon, int c, int windows, F &&f) {
    const uint32_t half = 1u << (c - 1);
    uint32_t carry = 0;
    for (int w = 0; w < windows; w++) {
        uint32_t raw = window_bits(canon, w * c, c) + carry;
        if (raw > half) {
            carry = 1;
            uint32_t mag = (1u << c) - raw;
            if (mag) f(w, mag, true);
        } else {
            carry = 0;
            if (raw) f(w, raw, false);
        }
    }
}

// canonical scalar i, shifted by the layer's randomiser when present
__device__ __forceinline__ Fr msm_scalar(const Fr *scalars, const Fr *delta, size_t i) {
    Fr s = from_mont(load_fr(&scalars[i]));
    if (delta) s = s + load_fr(&delta[i]);  // both < r: one conditional subtraction
    return s;
}

__global__ void k_msm_histogram(const Fr *scalars, const Fr *delta, size_t n, int c, int windows,
                                uint32_t *counts) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x) {
        Fr s = msm_scalar(scalars, delta, i);
        for_each_digit(s, c, windows, [&](int, uint32_t mag, bool) { atomicAdd(&counts[mag - 1], 1u); });
    }
}

// Exclusive scan of the m bucket counts, in tiles of kScanTile: k_msm_scan_sums
// writes one total per tile, then k_msm_scan gives every tile its prefix
// (the sum of the tile totals before it) and scans it, writing offsets[0..m]
// (offsets[m] = total) and a copy of offsets[0..m) into cursor.  Thread i of
// a tile owns counts [4i, 4i+4); loads and stores are coalesced.
constexpr int kScanThreads = 1024;
constexpr int kScanTile = 4 * kScanThreads;

__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t v, uint32_t *warp_tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += u;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < int(blockDim.x >> 5) ? warp_tot[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += u;
        }
        warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    return v + (warp > 0 ? warp_tot[warp - 1] : 0);
}

__global__ void __launch_bounds__(kScanThreads) k_msm_scan_sums(const uint32_t *counts, size_t m,
                                                                uint32_t *tile_sums) {
    __shared__ uint32_t warp_tot[32];
    const size_t i = size_t(blockIdx.x) * kScanTile + 4 * size_t(threadIdx.x);
    uint32_t s = 0;
    for (int k = 0; k < 4; k++) s += i + k < m ? counts[i + k] : 0;
    s = block_inclusive_scan(s, warp_tot);
    if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kScanThreads) k_msm_scan(const uint32_t *counts, size_t m,
                                                           const uint32_t *tile_sums, uint32_t *offsets,
                                                           uint32_t *cursor) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t tile_base;
    // prefix of this tile: sum of the totals of tiles 0..blockIdx.x-1
    uint32_t p = 0;
    for (uint32_t t = threadIdx.x; t < blockIdx.x; t += kScanThreads) p += tile_sums[t];
    p = block_inclusive_scan(p, warp_tot);
    if (threadIdx.x == kScanThreads - 1) tile_base = p;
    __syncthreads();
    const uint32_t base = tile_base;
    __syncthreads();  // warp_tot is reused below
    const size_t i = size_t(blockIdx.x) * kScanTile + 4 * size_t(threadIdx.x);
    uint32_t v[4], s = 0;
    for (int k = 0; k < 4; k++) {
        v[k] = i + k < m ? counts[i + k] : 0;
        s += v[k];
    }
    uint32_t run = base + block_inclusive_scan(s, warp_tot) - s;
    for (int k = 0; k < 4; k++) {
        if (i + k < m) {
            offsets[i + k] = run;
            cursor[i + k] = run;
        }
        run += v[k];
    }
    if (i < m && m <= i + 4) offsets[m] = run;  // the thread holding the last count writes the total
}

__global__ void k_msm_scatter(const Fr *scalars, const Fr *delta, size_t n, size_t stride, int c, int windows,
                              uint32_t *cursor, uint32_t *records) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x) {
        Fr s = msm_scalar(scalars, delta, i);
        for_each_digit(s, c, windows, [&](int w, uint32_t mag, bool neg) {
            uint32_t pos = atomicAdd(&cursor[mag - 1], 1u);
            records[pos] = uint32_t(size_t(w) * stride + i) | (neg ? 0x80000000u : 0u);
        });
    }
}

// ---------------------------------------------------------------------------
// Bucket accumulation: flat record chunks, XYZZ mixed additions
// ---------------------------------------------------------------------------
//
// The records are grouped by bucket (CSR `offsets`).  Thread t owns records
// [t*L, (t+1)*L) regardless of bucket boundaries, so every thread does the
// same number of mixed additions (bucket sizes are Poisson distributed and a
// top window with few bits can pile many records onto a few buckets).  A
// bucket lying inside one chunk is written directly; a bucket cut by chunk
// boundaries leaves one partial sum per chunk it touches (`pieces`, two slots
// per chunk: [2t] = the chunk's first segment when it began before the chunk,
// [2t+1] = its last segment when it runs past the chunk), which
// k_msm_bucket_fixup adds up.

#ifndef HP_ACC_MINBLOCKS
#define HP_ACC_MINBLOCKS 4  // measured on GB300 at 2^20: 9.04 ms at 4, 9.20 at 3, 9.56 at 2
#endif

// Chunk length L = 32 records per thread, one block per 128 chunks, blocks
// scheduled dynamically (measured at 2^20 points, c = 20: L = 32 9.56 ms per
// MSM, 48 9.70, 64 9.60, 96 10.33; a grid of exactly the resident blocks with
// L near 64 9.81).  A chunk is a chain of L dependent mixed additions and a
// bucket of k records cut into k/L pieces leaves a fix-up chain of k/L
// additions, so an MSM of fewer than 2 M records (latency-bound: not enough
// chunks to fill the GPU many times over) uses L = 8 (measured: 2^12 points
// L = 8 0.54 ms, 4 0.63, 16 0.60, 32 0.82; 2^16 L = 8 1.33 ms, 5 1.38,
// 16 1.35, 32 1.38; 2^18 L = 32 3.07 ms, 16 3.12, 8 3.18).
constexpr uint32_t kChunkRecords = 32;
constexpr uint32_t kSmallChunkRecords = 8;

struct AccumulateGeometry {
    uint32_t chunk;   // records per chunk (L)
    size_t chunks;    // ceil(records / L)
    unsigned grid;    // blocks of 128 threads
};

uint32_t msm_default_chunk(size_t records) {
    return records < (size_t(1) << 21) ? kSmallChunkRecords : kChunkRecords;
}

// `tuned`: a chunk length from the tuning table, 0 for the size rule
AccumulateGeometry accumulate_geometry(size_t records, uint32_t tuned) {
    size_t L = tuned >= 2 && tuned <= 1024 ? tuned : msm_default_chunk(records);
    // tuning override: HP_ACC_CHUNK=L (2 <= L <= 1024)
    if (const char *env = std::getenv("HP_ACC_CHUNK")) {
        const long v = std::atol(env);
        if (v >= 2 && v <= 1024) L = size_t(v);
    }
    AccumulateGeometry g;
    g.chunk = uint32_t(L);
    g.chunks = (records + L - 1) / L;
    g.grid = unsigned(std::max<size_t>(1, (g.chunks + 127) / 128));
    return g;
}

// largest b in [0, buckets) with offsets[b] <= k (k < offsets[buckets])
__device__ __forceinline__ uint32_t bucket_of(const uint32_t *offsets, uint32_t buckets, uint32_t k) {
    uint32_t lo = 0, hi = buckets;  // offsets[lo] <= k < offsets[hi]
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (offsets[mid] <= k) lo = mid; else hi = mid;
    }
    return lo;
}

// Base table of a bucket: one layer (a single MSM) ...
struct OneTable {
    const Affine *bases;
    __device__ __forceinline__ void prepare() const {}
    __device__ __forceinline__ const Affine *of(uint32_t) const { return bases; }
};

// ... or the layer of the instance owning the bucket (many MSMs in one
// launch, instance bucket ranges ascending; the table sits in shared memory).
constexpr int kMaxInstances = 64;
struct ManyTables {
    const uint32_t *bucket_base;  // [count]
    const Affine *const *bases;   // [count]
    int count;
    __device__ __forceinline__ void prepare() const {
        __shared__ uint32_t s_base[kMaxInstances];
        __shared__ const Affine *s_tab[kMaxInstances];
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            s_base[i] = bucket_base[i];
            s_tab[i] = bases[i];
        }
        __syncthreads();
        sb = s_base;
        st = s_tab;
    }
    __device__ __forceinline__ const Affine *of(uint32_t b) const {
        int lo = 0, hi = count;  // sb[lo] <= b < sb[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sb[mid] <= b) lo = mid; else hi = mid;
        }
        return st[lo];
    }
    mutable const uint32_t *sb = nullptr;
    mutable const Affine *const *st = nullptr;
};

template <class Tables>
__global__ void __launch_bounds__(128, HP_ACC_MINBLOCKS) k_msm_accumulate(Tables tables, const uint32_t *offsets,
                                                                          const uint32_t *records, uint32_t buckets,
                                                                          uint32_t chunk, Xyzz *bucket_sums,
                                                                          Xyzz *pieces) {
    tables.prepare();
    const uint32_t total = offsets[buckets];
    const uint32_t chunks = (total + chunk - 1) / chunk;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < chunks; t += gridDim.x * blockDim.x) {
        const uint32_t lo = t * chunk, hi = min(lo + chunk, total);
        uint32_t b = bucket_of(offsets, buckets, lo);
        uint32_t b_end = offsets[b + 1];
        const Affine *bases = tables.of(b);
        Xyzz acc = xyzz_inf();
        for (uint32_t k = lo;; k++) {
            if (k == hi || k == b_end) {
                // flush the segment of bucket b that ends at k
                const bool starts_inside = offsets[b] >= lo;
                const bool ends_inside = b_end <= hi;
                if (starts_inside && ends_inside) store_xyzz(&bucket_sums[b], acc);
                else if (!starts_inside) store_xyzz(&pieces[2 * size_t(t)], acc);
                else store_xyzz(&pieces[2 * size_t(t) + 1], acc);
                if (k == hi) break;
                // next non-empty bucket containing record k
                do { b++; b_end = offsets[b + 1]; } while (b_end <= k);
                bases = tables.of(b);
                acc = xyzz_inf();
            }
            uint32_t rec = records[k];
            Affine a = load_affine(&bases[rec & 0x7fffffffu]);
            if (affine_is_inf(a)) continue;
            if (rec & 0x80000000u) a.y = neg(a.y);
            acc = xyzz_add_affine(acc, a.x, a.y);
        }
    }
}

// Buckets cut by chunk boundaries: add their pieces; empty buckets: infinity.
__global__ void k_msm_bucket_fixup(const uint32_t *offsets, uint32_t buckets, uint32_t chunk, const Xyzz *pieces,
                                   Xyzz *bucket_sums) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < buckets; b += gridDim.x * blockDim.x) {
        const uint32_t begin = offsets[b], end = offsets[b + 1];
        if (begin == end) {
            store_xyzz(&bucket_sums[b], xyzz_inf());
            continue;
        }
        const uint32_t t0 = begin / chunk, t1 = (end - 1) / chunk;
        if (t0 == t1) continue;
        Xyzz acc = load_xyzz(&pieces[2 * size_t(t0) + 1]);
        for (uint32_t t = t0 + 1; t <= t1; t++) acc = xyzz_add(acc, load_xyzz(&pieces[2 * size_t(t)]));
        store_xyzz(&bucket_sums[b], acc);
    }
}

// ---------------------------------------------------------------------------
// Bucket reduction
// ---------------------------------------------------------------------------

// Segment j of `seg` buckets: run_j = sum S, acc_j = sum_l (l+1) S_{j*seg+l}.
__global__ void __launch_bounds__(128) k_msm_segments(const Xyzz *buckets, size_t segments, size_t seg,
                                                      Xyzz *acc_out, Xyzz *run_out) {
    for (size_t j = blockIdx.x * size_t(blockDim.x) + threadIdx.x; j < segments;
         j += size_t(gridDim.x) * blockDim.x) {
        Xyzz run = xyzz_inf(), acc = xyzz_inf();
        for (size_t l = seg; l-- > 0;) {
            run = xyzz_add(run, load_xyzz(&buckets[j * seg + l]));
            acc = xyzz_add(acc, run);
        }
        store_xyzz(&acc_out[j], acc);
        store_xyzz(&run_out[j], run);
    }
}

// Subset sums.  Subset y < bits: { run_j : bit y of j set } (segments/2
// elements); subset y == bits: every acc_j.  Block (chunk, y) sums elements
// [chunk * kSubsetPerBlock, ...) of subset y into partial[y * chunks + chunk].
constexpr int kSubsetThreads = 128;
constexpr int kSubsetPerThread = 8;
constexpr int kSubsetPerBlock = kSubsetThreads * kSubsetPerThread;

// k_msm_rows sums at most 64 subset blocks per row
size_t msm_max_segments() { return size_t(64) * kSubsetPerBlock; }

// Blocks of T threads (a power of two <= kSubsetThreads), `per` elements per
// thread: T * per = kSubsetPerBlock when there are several chunks; a single
// chunk of few elements takes fewer threads and elements per thread (the
// dependent-addition depth is per + log2 T).
__global__ void __launch_bounds__(kSubsetThreads) k_msm_subsets(const Xyzz *run, const Xyzz *acc,
                                                                size_t segments, int bits, int chunks, int per,
                                                                Xyzz *partial) {
    __shared__ Xyzz sm[kSubsetThreads];
    const int y = blockIdx.y, t = threadIdx.x, T = blockDim.x;
    const size_t count = y < bits ? segments / 2 : segments;
    const size_t first = size_t(blockIdx.x) * size_t(T) * per;
    Xyzz s = xyzz_inf();
    for (int k = 0; k < per; k++) {
        size_t e = first + size_t(k) * T + t;
        if (e >= count) break;
        Xyzz v;
        if (y < bits) {
            size_t j = ((e >> y) << (y + 1)) | (size_t(1) << y) | (e & ((size_t(1) << y) - 1));
            v = load_xyzz(&run[j]);
        } else {
            v = load_xyzz(&acc[e]);
        }
        s = xyzz_add(s, v);
    }
    sm[t] = s;
    __syncthreads();
    for (int half = T / 2; half > 0; half >>= 1) {
        if (t < half) sm[t] = xyzz_add(sm[t], sm[t + half]);
        __syncthreads();
    }
    if (t == 0) store_xyzz(&partial[size_t(y) * chunks + blockIdx.x], sm[0]);
}

// Row sums of a [rows][cols] partial matrix (cols <= 64) into out[rows].
__global__ void k_msm_rows(const Xyzz *partial, int cols, Xyzz *out) {
    __shared__ Xyzz sm[64];
    const int y = blockIdx.x, t = threadIdx.x;
    sm[t] = t < cols ? load_xyzz(&partial[size_t(y) * cols + t]) : xyzz_inf();
    __syncthreads();
    for (int half = 32; half > 0; half >>= 1) {
        if (t < half) sm[t] = xyzz_add(sm[t], sm[t + half]);
        __syncthreads();
    }
    if (t == 0) store_xyzz(&out[y], sm[0]);
}

void msm_run(HpCudaContext *ctx, const MsmLayer &layer, const Fr *scalars, Xyzz *out_partials,
             cudaStream_t stream, size_t count) {
    const cudaStream_t st = stream ? stream : ctx->stream;
    const size_t n = count ? count : layer.n;  // a prefix of the layer's bases
    const MsmShape sh = msm_shape(layer);
    const size_t B = sh.buckets;
    const size_t records = size_t(layer.windows) * n;
    Scratch counts(ctx, (B + 1) * 4, st), offsets(ctx, (B + 1) * 4, st), cursor(ctx, B * 4, st);
    Scratch recs(ctx, records * 4, st), buckets(ctx, B * sizeof(Xyzz), st);
    int whole = ctx->prof_begin("msm", st);
    check_cuda(cudaMemsetAsync(counts.ptr, 0, (B + 1) * 4, st));
    k_msm_histogram<<<grid_for(ctx, n, 256), 256, 0, st>>>(scalars, layer.delta, n, layer.c, layer.windows,
                                                          counts.as<uint32_t>());
    check_launch();
    const unsigned tiles = unsigned((B + kScanTile - 1) / kScanTile);
    Scratch tile_sums(ctx, size_t(tiles) * 4, st);
    if (tiles > 1) {
        k_msm_scan_sums<<<tiles, kScanThreads, 0, st>>>(counts.as<uint32_t>(), B, tile_sums.as<uint32_t>());
        check_launch();
    }
    k_msm_scan<<<tiles, kScanThreads, 0, st>>>(counts.as<uint32_t>(), B, tile_sums.as<uint32_t>(),
                                              offsets.as<uint32_t>(), cursor.as<uint32_t>());
    check_launch();
    k_msm_scatter<<<grid_for(ctx, n, 256), 256, 0, st>>>(scalars, layer.delta, n, layer.n, layer.c, layer.windows,
                                                        cursor.as<uint32_t>(), recs.as<uint32_t>());
    check_launch();
    const AccumulateGeometry geo = accumulate_geometry(records, layer.chunk);
    Scratch pieces(ctx, std::max<size_t>(2 * geo.chunks, 1) * sizeof(Xyzz), st);
    int tok = ctx->prof_begin("msm_accumulate", st);
    k_msm_accumulate<<<geo.grid, 128, 0, st>>>(OneTable{layer.bases}, offsets.as<uint32_t>(), recs.as<uint32_t>(),
                                               uint32_t(B), geo.chunk, buckets.as<Xyzz>(), pieces.as<Xyzz>());
    check_launch();
    ctx->prof_end(tok, st);
    k_msm_bucket_fixup<<<grid_for(ctx, B, 128, 8), 128, 0, st>>>(offsets.as<uint32_t>(), uint32_t(B), geo.chunk,
                                                                pieces.as<Xyzz>(), buckets.as<Xyzz>());
    check_launch();
    Scratch acc(ctx, sh.segments * sizeof(Xyzz), st), run(ctx, sh.segments * sizeof(Xyzz), st);
    k_msm_segments<<<grid_for(ctx, sh.segments, 128, 16), 128, 0, st>>>(buckets.as<Xyzz>(), sh.segments, sh.seg,
                                                                       acc.as<Xyzz>(), run.as<Xyzz>());
    check_launch();
    const int chunks = int((sh.segments + kSubsetPerBlock - 1) / kSubsetPerBlock);
    if (chunks == 1) {
        // depth per + log2 T: T = the power of two >= segments, 32..128
        int T = 32;
        while (T < kSubsetThreads && size_t(T) < sh.segments) T *= 2;
        const int per = int((sh.segments + T - 1) / T);
        k_msm_subsets<<<dim3(1, sh.partials), T, 0, st>>>(run.as<Xyzz>(), acc.as<Xyzz>(), sh.segments,
                                                          sh.seg_bits, 1, per, out_partials);
        check_launch();
    } else {
        if (chunks > 64) fail(HP_CUDA_STATUS_NOT_IMPLEMENTED);
        Scratch partial(ctx, size_t(chunks) * sh.partials * sizeof(Xyzz), st);
        k_msm_subsets<<<dim3(chunks, sh.partials), kSubsetThreads, 0, st>>>(run.as<Xyzz>(), acc.as<Xyzz>(),
                                                                            sh.segments, sh.seg_bits, chunks,
                                                                            kSubsetPerThread, partial.as<Xyzz>());
        check_launch();
        k_msm_rows<<<sh.partials, 64, 0, st>>>(partial.as<Xyzz>(), chunks, out_partials);
        check_launch();
    }
    ctx->prof_end(whole, st);
}

// ---------------------------------------------------------------------------
// Many MSMs in one launch sequence
// ---------------------------------------------------------------------------
//
// Instances keep their own layer (window width, window table, randomisation)
// and get disjoint ranges of one global bucket array, record array, segment
// array and subset-block range; every phase above is one launch over all
// instances' items, a thread finding its instance by a binary search over
// the (ascending) range starts.  Results are the same per instance as
// msm_run's: the per-bucket, per-segment and per-subset arithmetic is.

struct MsmInst {
    const Fr *scalars;
    const Fr *delta;
    uint32_t n, stride;        // points; the layer's point count (window stride)
    int c, windows;
    uint32_t point_base;       // first global point
    uint32_t bucket_base;      // first global bucket
    uint32_t seg, segments, seg_base;
    int seg_bits, per, chunks;
    uint32_t block_base;       // first subset block: (seg_bits + 1) * chunks blocks
    uint32_t row_base;         // first staged row: seg_bits + 1 rows
    uint32_t out_row;          // first output row
};

template <class Key>
__device__ __forceinline__ int inst_of(const MsmInst *in, int count, uint32_t key, Key k) {
    int lo = 0, hi = count;  // k(in[lo]) <= key < k(in[hi])
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (k(in[mid]) <= key) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void k_msmm_histogram(const MsmInst *in, int count, uint32_t points, uint32_t *counts) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < points; g += gridDim.x * blockDim.x) {
        const MsmInst &m = in[inst_of(in, count, g, [](const MsmInst &x) { return x.point_base; })];
        const Fr s = msm_scalar(m.scalars, m.delta, g - m.point_base);
        uint32_t *cnt = counts + m.bucket_base;
        for_each_digit(s, m.c, m.windows, [&](int, uint32_t mag, bool) { atomicAdd(&cnt[mag - 1], 1u); });
    }
}

__global__ void k_msmm_scatter(const MsmInst *in, int count, uint32_t points, uint32_t *cursor, uint32_t *records) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < points; g += gridDim.x * blockDim.x) {
        const MsmInst &m = in[inst_of(in, count, g, [](const MsmInst &x) { return x.point_base; })];
        const uint32_t i = g - m.point_base;
        const Fr s = msm_scalar(m.scalars, m.delta, i);
        uint32_t *cur = cursor + m.bucket_base;
        for_each_digit(s, m.c, m.windows, [&](int w, uint32_t mag, bool neg) {
            const uint32_t pos = atomicAdd(&cur[mag - 1], 1u);
            records[pos] = uint32_t(size_t(w) * m.stride + i) | (neg ? 0x80000000u : 0u);
        });
    }
}

__global__ void __launch_bounds__(128) k_msmm_segments(const MsmInst *in, int count, uint32_t segments,
                                                       const Xyzz *buckets, Xyzz *acc_out, Xyzz *run_out) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < segments; g += gridDim.x * blockDim.x) {
        const MsmInst &m = in[inst_of(in, count, g, [](const MsmInst &x) { return x.seg_base; })];
        const Xyzz *bk = buckets + m.bucket_base + size_t(g - m.seg_base) * m.seg;
        Xyzz run = xyzz_inf(), acc = xyzz_inf();
        for (uint32_t l = m.seg; l-- > 0;) {
            run = xyzz_add(run, load_xyzz(&bk[l]));
            acc = xyzz_add(acc, run);
        }
        store_xyzz(&acc_out[g], acc);
        store_xyzz(&run_out[g], run);
    }
}

// Block -> (instance, subset y, chunk); writes stage[(row_base + y) * 64 + chunk].
__global__ void __launch_bounds__(kSubsetThreads) k_msmm_subsets(const MsmInst *in, int count, const Xyzz *run,
                                                                 const Xyzz *acc, Xyzz *stage) {
    __shared__ Xyzz sm[kSubsetThreads];
    const MsmInst &m = in[inst_of(in, count, blockIdx.x, [](const MsmInst &x) { return x.block_base; })];
    const uint32_t local = blockIdx.x - m.block_base;
    const int y = int(local / uint32_t(m.chunks)), chunk = int(local % uint32_t(m.chunks));
    const int t = threadIdx.x, T = blockDim.x;
    const size_t count_y = y < m.seg_bits ? m.segments / 2 : m.segments;
    const size_t first = size_t(chunk) * size_t(T) * m.per;
    const Xyzz *r = run + m.seg_base, *a = acc + m.seg_base;
    Xyzz s = xyzz_inf();
    for (int k = 0; k < m.per; k++) {
        const size_t e = first + size_t(k) * T + t;
        if (e >= count_y) break;
        Xyzz v;
        if (y < m.seg_bits) {
            const size_t j = ((e >> y) << (y + 1)) | (size_t(1) << y) | (e & ((size_t(1) << y) - 1));
            v = load_xyzz(&r[j]);
        } else {
            v = load_xyzz(&a[e]);
        }
        s = xyzz_add(s, v);
    }
    sm[t] = s;
    __syncthreads();
    for (int half = T / 2; half > 0; half >>= 1) {
        if (t < half) sm[t] = xyzz_add(sm[t], sm[t + half]);
        __syncthreads();
    }
    if (t == 0) store_xyzz(&stage[(size_t(m.row_base) + y) * 64 + chunk], sm[0]);
}

// Row r (of all instances' rows) = sum of its instance's chunks of stage.
__global__ void k_msmm_rows(const MsmInst *in, int count, const Xyzz *stage, Xyzz *out) {
    __shared__ Xyzz sm[64];
    const uint32_t r = blockIdx.x;
    const MsmInst &m = in[inst_of(in, count, r, [](const MsmInst &x) { return x.row_base; })];
    const int t = threadIdx.x;
    sm[t] = t < m.chunks ? load_xyzz(&stage[size_t(r) * 64 + t]) : xyzz_inf();
    __syncthreads();
    for (int half = 32; half > 0; half >>= 1) {
        if (t < half) sm[t] = xyzz_add(sm[t], sm[t + half]);
        __syncthreads();
    }
    if (t == 0) store_xyzz(&out[m.out_row + (r - m.row_base)], sm[0]);
}

// One group: at most kMaxInstances instances, all of it resident at once.
static void msm_run_group(HpCudaContext *ctx, const MsmTask *tasks, size_t count, Xyzz *out_rows, cudaStream_t st,
                          uint32_t chunk) {
    std::vector<MsmInst> in(count);
    std::vector<uint32_t> bucket_base(count);
    std::vector<const Affine *> tables(count);
    size_t points = 0, B = 0, segs = 0, blocks = 0, rows = 0, records = 0;
    for (size_t i = 0; i < count; i++) {
        const MsmLayer &L = *tasks[i].layer;
        const MsmShape sh = msm_shape(L);
        MsmInst &m = in[i];
        m.scalars = tasks[i].scalars;
        m.delta = L.delta;
        m.n = uint32_t(tasks[i].n);
        m.stride = uint32_t(L.n);
        m.c = L.c;
        m.windows = L.windows;
        m.point_base = uint32_t(points);
        m.bucket_base = uint32_t(B);
        m.seg = uint32_t(sh.seg);
        m.segments = uint32_t(sh.segments);
        m.seg_base = uint32_t(segs);
        m.seg_bits = sh.seg_bits;
        m.per = kSubsetPerThread;
        m.chunks = int((sh.segments + kSubsetPerBlock - 1) / kSubsetPerBlock);
        if (m.chunks > 64) fail(HP_CUDA_STATUS_NOT_IMPLEMENTED);
        m.block_base = uint32_t(blocks);
        m.row_base = uint32_t(rows);
        m.out_row = uint32_t(tasks[i].out_row);
        bucket_base[i] = m.bucket_base;
        tables[i] = L.bases;
        points += tasks[i].n;
        B += sh.buckets;
        segs += sh.segments;
        blocks += size_t(sh.partials) * m.chunks;
        rows += size_t(sh.partials);
        records += size_t(L.windows) * tasks[i].n;
    }
    require(records < (size_t(1) << 31) && B < (size_t(1) << 31));
    Scratch din(ctx, count * sizeof(MsmInst), st), dbase(ctx, count * 4, st), dtab(ctx, count * sizeof(void *), st);
    check_cuda(cudaMemcpyAsync(din.ptr, in.data(), count * sizeof(MsmInst), cudaMemcpyHostToDevice, st));
    check_cuda(cudaMemcpyAsync(dbase.ptr, bucket_base.data(), count * 4, cudaMemcpyHostToDevice, st));
    check_cuda(cudaMemcpyAsync(dtab.ptr, tables.data(), count * sizeof(void *), cudaMemcpyHostToDevice, st));
    const MsmInst *inst = din.as<MsmInst>();
    const int cnt = int(count);
    Scratch counts(ctx, (B + 1) * 4, st), offsets(ctx, (B + 1) * 4, st), cursor(ctx, B * 4, st);
    Scratch recs(ctx, std::max<size_t>(records, 1) * 4, st), buckets(ctx, B * sizeof(Xyzz), st);
    check_cuda(cudaMemsetAsync(counts.ptr, 0, (B + 1) * 4, st));
    k_msmm_histogram<<<grid_for(ctx, points, 256), 256, 0, st>>>(inst, cnt, uint32_t(points), counts.as<uint32_t>());
    check_launch();
    const unsigned tiles = unsigned((B + kScanTile - 1) / kScanTile);
    Scratch tile_sums(ctx, size_t(tiles) * 4, st);
    if (tiles > 1) {
        k_msm_scan_sums<<<tiles, kScanThreads, 0, st>>>(counts.as<uint32_t>(), B, tile_sums.as<uint32_t>());
        check_launch();
    }
    k_msm_scan<<<tiles, kScanThreads, 0, st>>>(counts.as<uint32_t>(), B, tile_sums.as<uint32_t>(),
                                              offsets.as<uint32_t>(), cursor.as<uint32_t>());
    check_launch();
    k_msmm_scatter<<<grid_for(ctx, points, 256), 256, 0, st>>>(inst, cnt, uint32_t(points), cursor.as<uint32_t>(),
                                                              recs.as<uint32_t>());
    check_launch();
    // a launch of one MSM takes that layer's tuned chunk, a shared one the
    // entry for its record count
    if (!chunk && count == 1) chunk = tasks[0].layer->chunk;
    const AccumulateGeometry geo = accumulate_geometry(records, chunk ? chunk : msm_tuning_many_chunk(records));
    Scratch pieces(ctx, std::max<size_t>(2 * geo.chunks, 1) * sizeof(Xyzz), st);
    k_msm_accumulate<<<geo.grid, 128, 0, st>>>(ManyTables{dbase.as<uint32_t>(), dtab.as<const Affine *>(), cnt},
                                               offsets.as<uint32_t>(), recs.as<uint32_t>(), uint32_t(B), geo.chunk,
                                               buckets.as<Xyzz>(), pieces.as<Xyzz>());
    check_launch();
    k_msm_bucket_fixup<<<grid_for(ctx, B, 128, 8), 128, 0, st>>>(offsets.as<uint32_t>(), uint32_t(B), geo.chunk,
                                                                pieces.as<Xyzz>(), buckets.as<Xyzz>());
    check_launch();
    Scratch acc(ctx, segs * sizeof(Xyzz), st), run(ctx, segs * sizeof(Xyzz), st);
    k_msmm_segments<<<grid_for(ctx, segs, 128, 16), 128, 0, st>>>(inst, cnt, uint32_t(segs), buckets.as<Xyzz>(),
                                                                  acc.as<Xyzz>(), run.as<Xyzz>());
    check_launch();
    Scratch stage(ctx, rows * 64 * sizeof(Xyzz), st);
    k_msmm_subsets<<<unsigned(blocks), kSubsetThreads, 0, st>>>(inst, cnt, run.as<Xyzz>(), acc.as<Xyzz>(),
                                                               stage.as<Xyzz>());
    check_launch();
    k_msmm_rows<<<unsigned(rows), 64, 0, st>>>(inst, cnt, stage.as<Xyzz>(), out_rows);
    check_launch();
}

static_assert(kMsmManyMaxInstances == size_t(kMaxInstances), "one instance table per launch");

uint32_t msm_effective_chunk(size_t records, uint32_t tuned) { return accumulate_geometry(records, tuned).chunk; }

bool msm_runs_alone(size_t records) {
    const char *env = std::getenv("HP_MSM_MANY");
    if (env && env[0] == '0') return true;
    if (env && env[0] == '1') return false;
    return records >= (size_t(1) << 22);
}

void msm_run_many(HpCudaContext *ctx, const MsmTask *tasks, size_t count, Xyzz *out_rows, cudaStream_t stream,
                  uint32_t chunk) {
    const cudaStream_t st = stream ? stream : ctx->stream;
    // groups of <= kMaxInstances instances and <= 2^27 records (bounded scratch)
    size_t i = 0;
    int whole = ctx->prof_begin("msm_many", st);
    while (i < count) {
        size_t j = i, records = 0;
        while (j < count && j - i < kMsmManyMaxInstances) {
            const size_t r = size_t(tasks[j].layer->windows) * tasks[j].n;
            if (j > i && records + r > kMsmManyMaxRecords) break;
            records += r;
            j++;
        }
        msm_run_group(ctx, tasks + i, j - i, out_rows, st, chunk);
        i = j;
    }
    ctx->prof_end(whole, st);
}

// ---------------------------------------------------------------------------
// Binary scalars (every scalar 0 or 1)
// ---------------------------------------------------------------------------

// Up to kClassifyList tables per launch, passed by value (no descriptor copy).
constexpr int kClassifyList = 32;
struct ClassifyList {
    const Fr *scalars[kClassifyList];
    size_t n[kClassifyList];
};

// flags[t] = 1 when table t (blockIdx.y) has a scalar outside {0, 1}
// (canonical value).  flags is host-mapped memory zeroed by the host; blocks
// only ever store 1 there, so no atomics cross the link.  ones[t] (device,
// zeroed by the host) counts the scalars equal to 1.
__global__ void k_msm_classify(ClassifyList list, uint32_t *flags, unsigned long long *ones) {
    const Fr *scalars = list.scalars[blockIdx.y];
    const size_t n = list.n[blockIdx.y];
    uint32_t other = 0, count = 0;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const Fr c = from_mont(load_fr(&scalars[i]));
        uint32_t high = c.v[0] >> 1;
#pragma unroll
        for (int k = 1; k < 8; k++) high |= c.v[k];
        other |= high;
        count += c.v[0] & 1u;
    }
    if (__syncthreads_or(other != 0) && threadIdx.x == 0) flags[blockIdx.y] = 1u;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) count += __shfl_down_sync(0xffffffffu, count, off);
    if ((threadIdx.x & 31) == 0 && count) atomicAdd(&ones[blockIdx.y], (unsigned long long)count);
}

std::vector<char> msm_binary_tasks(HpCudaContext *ctx, const MsmTask *tasks, size_t count,
                                   std::vector<uint64_t> *ones) {
    std::vector<char> binary(count, 0);
    if (ones) ones->assign(count, 0);
    const char *env = std::getenv("HP_MSM_BINARY");
    if (count == 0 || (env && env[0] == '0')) return binary;
    // mailbox: the flags, then (8-byte aligned) the ones counts copied back
    const size_t flag_bytes = (count * sizeof(uint32_t) + 7) & ~size_t(7);
    void *dev = nullptr;
    uint8_t *box = ctx->mailbox(flag_bytes + count * sizeof(uint64_t), &dev);
    volatile uint32_t *host = reinterpret_cast<volatile uint32_t *>(box);
    for (size_t i = 0; i < count; i++) host[i] = 0;
    Scratch counts(ctx, count * sizeof(uint64_t));
    check_cuda(cudaMemsetAsync(counts.ptr, 0, count * sizeof(uint64_t), ctx->stream));
    for (size_t first = 0; first < count; first += kClassifyList) {
        const size_t m = std::min<size_t>(kClassifyList, count - first);
        ClassifyList list{};
        size_t max_n = 1;
        for (size_t i = 0; i < m; i++) {
            list.scalars[i] = tasks[first + i].scalars;
            list.n[i] = tasks[first + i].n;
            max_n = std::max(max_n, tasks[first + i].n);
        }
        // a memory pass over every table: about two waves of 256-thread blocks
        const unsigned x = unsigned(std::max<size_t>(
            1, std::min<size_t>((max_n + 255) / 256, (size_t(2) * ctx->sm_count * 8 + m - 1) / m)));
        k_msm_classify<<<dim3(x, unsigned(m)), 256, 0, ctx->stream>>>(list, static_cast<uint32_t *>(dev) + first,
                                                                      counts.as<unsigned long long>() + first);
        check_launch();
    }
    if (ones)
        check_cuda(cudaMemcpyAsync(box + flag_bytes, counts.ptr, count * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    ctx->sync();
    for (size_t i = 0; i < count; i++) binary[i] = host[i] == 0;
    if (ones) std::memcpy(ones->data(), box + flag_bytes, count * sizeof(uint64_t));
    return binary;
}

// A grid of at most 4 blocks per SM (the accumulation kernel's residency:
// 128 registers a thread) strides over the indices, thread t of block b
// taking b * 128 + t + k * (grid * 128) (coalesced loads): mixed additions of
// the selected bases into XYZZ, then a shared-memory tree over the block.
// Measured at 2^20 points: 196 registers and 8-index ranges per thread
// (2 blocks per SM) took 0.98 ms.
constexpr int kBinaryThreads = 128;
constexpr int kBinaryPerThread = 8;  // indices per thread below the grid cap

__global__ void __launch_bounds__(kBinaryThreads, 4) k_msm_binary_blocks(const Affine *bases, const Fr *scalars,
                                                                          size_t n, uint32_t want,
                                                                          Xyzz *block_sums) {
    __shared__ Xyzz sm[kBinaryThreads];
    Xyzz acc = xyzz_inf();
    for (size_t i = size_t(blockIdx.x) * kBinaryThreads + threadIdx.x; i < n;
         i += size_t(gridDim.x) * kBinaryThreads) {
        // classified 0 or 1: the bases whose scalar is `want` (every base without scalars)
        if (scalars && from_mont(load_fr(&scalars[i])).v[0] != want) continue;
        const Affine a = load_affine(&bases[i]);
        if (affine_is_inf(a)) continue;
        acc = xyzz_add_affine(acc, a.x, a.y);
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int half = kBinaryThreads / 2; half > 0; half >>= 1) {
        if (threadIdx.x < half) sm[threadIdx.x] = xyzz_add(sm[threadIdx.x], sm[threadIdx.x + half]);
        __syncthreads();
    }
    if (threadIdx.x == 0) store_xyzz(&block_sums[blockIdx.x], sm[0]);
}

// One block: the sum of the block sums, subtracted from *total_sum when
// given, plus D when present, into the last of `rows` partial rows;
// infinity into the others.
__global__ void __launch_bounds__(kBinaryThreads) k_msm_binary_final(const Xyzz *block_sums, size_t blocks,
                                                                      const Xyzz *total_sum, const Xyzz *d_sum,
                                                                      int rows, Xyzz *out) {
    __shared__ Xyzz sm[kBinaryThreads];
    Xyzz acc = xyzz_inf();
    for (size_t b = threadIdx.x; b < blocks; b += kBinaryThreads) acc = xyzz_add(acc, load_xyzz(&block_sums[b]));
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int half = kBinaryThreads / 2; half > 0; half >>= 1) {
        if (threadIdx.x < half) sm[threadIdx.x] = xyzz_add(sm[threadIdx.x], sm[threadIdx.x + half]);
        __syncthreads();
    }
    for (int r = threadIdx.x; r < rows - 1; r += kBinaryThreads) store_xyzz(&out[r], xyzz_inf());
    if (threadIdx.x == 0) {
        Xyzz total = sm[0];
        if (total_sum) {
            total.y = neg(total.y);
            total = xyzz_add(load_xyzz(total_sum), total);
        }
        if (d_sum) total = xyzz_add(total, load_xyzz(d_sum));
        store_xyzz(&out[rows - 1], total);
    }
}

// The sum of the first n window-0 bases whose scalar is `want` (scalars
// null: all of them), subtracted from *total when given, plus *d_sum when
// given, into the last of `rows` rows at `out` (infinity in the others).
static void msm_sum_bases(HpCudaContext *ctx, const MsmLayer &layer, const Fr *scalars, uint32_t want,
                          const Xyzz *total, Xyzz *out, int rows, cudaStream_t st, size_t n,
                          const Xyzz *d_sum) {
    if (n == 0) n = layer.n;
    const size_t per_block = size_t(kBinaryThreads) * kBinaryPerThread;
    const size_t blocks = std::min<size_t>((n + per_block - 1) / per_block, size_t(4) * ctx->sm_count);
    Scratch sums(ctx, blocks * sizeof(Xyzz), st);
    k_msm_binary_blocks<<<unsigned(blocks), kBinaryThreads, 0, st>>>(layer.bases, scalars, n, want,
                                                                     sums.as<Xyzz>());
    check_launch();
    k_msm_binary_final<<<1, kBinaryThreads, 0, st>>>(sums.as<Xyzz>(), blocks, total, d_sum, rows, out);
    check_launch();
}

void msm_run_binary(HpCudaContext *ctx, const MsmLayer &layer, const Fr *scalars, size_t n, Xyzz *out_partials,
                    cudaStream_t stream, bool complement) {
    const cudaStream_t st = stream ? stream : ctx->stream;
    require(n >= 1 && n <= layer.n);
    complement = complement && n == layer.n && layer.base_sum != nullptr;
    const MsmShape sh = msm_shape(layer);
    int tok = ctx->prof_begin("msm_binary", st);
    msm_sum_bases(ctx, layer, scalars, complement ? 0u : 1u, complement ? layer.base_sum : nullptr, out_partials,
                  sh.partials, st, n, layer.delta ? layer.d_sum : nullptr);
    ctx->prof_end(tok, st);
}

host::Xyzz64 msm_combine_host(const MsmShape &shape, const host::Xyzz64 *device_partials) {
    // device coordinates are in [0, 2p): canonical first
    std::vector<host::Xyzz64> partials(device_partials, device_partials + shape.partials);
    for (auto &q : partials) {
        q.x = host::fq_canonical(q.x);
        q.y = host::fq_canonical(q.y);
        q.zz = host::fq_canonical(q.zz);
        q.zzz = host::fq_canonical(q.zzz);
    }
    // result = A + seg * sum_k 2^k T_k, A = partials[bits], T_k = partials[k]
    host::Xyzz64 h = host::xyzz_inf();
    for (int k = shape.seg_bits - 1; k >= 0; k--) {
        h = host::xyzz_double(h);
        h = host::xyzz_add(h, partials[size_t(k)]);
    }
    for (size_t s = shape.seg; s > 1; s >>= 1) h = host::xyzz_double(h);
    return host::xyzz_add(partials[size_t(shape.seg_bits)], h);
}

host::Xyzz64 msm_result_host(const MsmLayer &layer, const host::Xyzz64 *partials) {
    host::Xyzz64 r = msm_combine_host(msm_shape(layer), partials);
    if (layer.delta) r = host::xyzz_add(r, layer.minus_d);
    return r;
}

void msm_finalize_host(const MsmLayer &layer, const host::Xyzz64 *partials, uint8_t *out97) {
    host::xyzz_to_packet(msm_result_host(layer, partials), out97);
}

}  // namespace hp
