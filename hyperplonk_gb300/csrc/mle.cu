// mle.cu -- resident MLE table kernels and their ABI entries.
//
// Reference semantics: backend/src/cpu/multilinear_polynomial.rs:32-253 (CPU
// backend) and backend/src/common/eq.rs:38-95; device counterparts in the
// reference are the AscendC kernels of backend/src/ascend910b3/native/
// mle_kernels.asc:272-522.  Tables are low-bit-first: entry x holds f at the
// Boolean point whose variable i is bit i of x.
//
// Every kernel here is HBM bound except eq/frac (one Fr multiply per 32-byte
// element moved, near the IMAD/HBM balance point).  Grids are multiples of
// the SM count with grid-stride loops; AoS 32-byte elements are moved as two
// 16-byte vector accesses.
#include <algorithm>
#include <cstring>
#include <vector>

#include "host_field.h"
#include "mle.cuh"
#include "runtime.cuh"

using hp::check_cuda;
using hp::check_launch;
using hp::fail;
using hp::Fr;
using hp::guard;
using hp::require;

namespace hp {

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// In place: canonical -> Montgomery, flagging non-canonical inputs.
__global__ void k_to_mont_check(Fr *data, size_t n, uint32_t *flags) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x) {
        Fr x = load_fr(&data[i]);
        if (!is_canonical(x)) atomicOr(flags, kFlagNonCanonical);
        store_fr(&data[i], to_mont(x));
    }
}

__global__ void k_from_mont(const Fr *src, Fr *dst, size_t n) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
        store_fr(&dst[i], from_mont(load_fr(&src[i])));
}

// out[i] (+)= sum_j c_j polys_j[i].  From three terms on the products are
// summed unreduced (FrAcc) and reduced once per element.
__global__ void k_linear_combination(Fr *out, FrPtrList polys, FrScalarList coefs, int count,
                                     size_t n, bool accumulate) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x) {
        if (count >= 3) {
            FrAcc X;
            acc_zero(X);
            if (accumulate) acc_add_shifted(X, load_fr(&out[i]));
            // four tables' loads in flight before their products
            int j = 0;
            for (; j + 4 <= count; j += 4) {
                const Fr v0 = load_fr(&polys.p[j][i]), v1 = load_fr(&polys.p[j + 1][i]);
                const Fr v2 = load_fr(&polys.p[j + 2][i]), v3 = load_fr(&polys.p[j + 3][i]);
                acc_mul_add(X, v0, coefs.s[j]);
                acc_mul_add(X, v1, coefs.s[j + 1]);
                acc_mul_add(X, v2, coefs.s[j + 2]);
                acc_mul_add(X, v3, coefs.s[j + 3]);
            }
            for (; j < count; j++) acc_mul_add(X, load_fr(&polys.p[j][i]), coefs.s[j]);
            store_fr(&out[i], acc_reduce(X));
        } else {
            Fr acc = accumulate ? load_fr(&out[i]) : Fr::zero();
            for (int j = 0; j < count; j++) acc = acc + load_fr(&polys.p[j][i]) * coefs.s[j];
            store_fr(&out[i], acc);
        }
    }
}

// One fix_variables step: dst[b] = src[2b] + r * (src[2b+1] - src[2b]).
__global__ void k_fold(const Fr *src, Fr *dst, size_t half, Fr r) {
    for (size_t b = blockIdx.x * size_t(blockDim.x) + threadIdx.x; b < half;
         b += size_t(gridDim.x) * blockDim.x) {
        Fr lo = load_fr(&src[2 * b]);
        Fr hi = load_fr(&src[2 * b + 1]);
        store_fr(&dst[b], lo + r * (hi - lo));
    }
}

// Block b folds `levels` variables (levels <= 10, 32 KiB) of the 2^levels
// entries src[b 2^levels ..] in shared memory and writes the value to dst[b].
__global__ void k_fold_tail(const Fr *src, Fr *dst, int levels, FrScalarList r) {
    extern __shared__ Fr sm[];
    size_t n = size_t(1) << levels;
    src += size_t(blockIdx.x) << levels;
    dst += blockIdx.x;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) sm[i] = load_fr(&src[i]);
    __syncthreads();
    for (int l = 0; l < levels; l++) {
        size_t half = n >> (l + 1);
        Fr rl = r.s[l];
        Fr v[4];
        int cnt = 0;
        for (size_t b = threadIdx.x; b < half; b += blockDim.x) {
            Fr lo = sm[2 * b], hi = sm[2 * b + 1];
            v[cnt & 3] = lo + rl * (hi - lo);
            cnt++;
        }
        __syncthreads();
        cnt = 0;
        for (size_t b = threadIdx.x; b < half; b += blockDim.x) sm[b] = v[cnt++ & 3];
        __syncthreads();
    }
    if (threadIdx.x == 0) store_fr(dst, sm[0]);
}

// eq table by direct products: out[x] = prod_j (bit_j(x) ? r_j : 1 - r_j).
__global__ void k_eq_direct(Fr *out, const Fr *r, int m) {
    size_t n = size_t(1) << m;
    Fr one = Fr::one();
    for (size_t x = blockIdx.x * size_t(blockDim.x) + threadIdx.x; x < n;
         x += size_t(gridDim.x) * blockDim.x) {
        Fr acc = one;
        for (int j = 0; j < m; j++) {
            Fr rj = r[j];
            acc = acc * (((x >> j) & 1) ? rj : one - rj);
        }
        store_fr(&out[x], acc);
    }
}

// Both halves of a split eq table in one launch: blocks [0, lo_blocks) write
// lo = eq(r[0..m_lo)), the others hi = eq(r[m_lo..m_lo + m_hi)).
__global__ void k_eq_direct2(Fr *lo, Fr *hi, const Fr *r, int m_lo, int m_hi, unsigned lo_blocks) {
    const bool is_lo = blockIdx.x < lo_blocks;
    Fr *out = is_lo ? lo : hi;
    const Fr *rr = is_lo ? r : r + m_lo;
    const int m = is_lo ? m_lo : m_hi;
    const unsigned b = is_lo ? blockIdx.x : blockIdx.x - lo_blocks;
    const unsigned nb = is_lo ? lo_blocks : gridDim.x - lo_blocks;
    const size_t n = size_t(1) << m;
    const Fr one = Fr::one();
    for (size_t x = b * size_t(blockDim.x) + threadIdx.x; x < n; x += size_t(nb) * blockDim.x) {
        Fr acc = one;
        for (int j = 0; j < m; j++) {
            const Fr rj = rr[j];
            acc = acc * (((x >> j) & 1) ? rj : one - rj);
        }
        store_fr(&out[x], acc);
    }
}

// out[x] = lo[x & mask] * hi[x >> low_bits]
__global__ void k_eq_outer(Fr *out, const Fr *lo, const Fr *hi, int low_bits, size_t n) {
    size_t mask = (size_t(1) << low_bits) - 1;
    for (size_t x = blockIdx.x * size_t(blockDim.x) + threadIdx.x; x < n;
         x += size_t(gridDim.x) * blockDim.x)
        store_fr(&out[x], load_fr(&lo[x & mask]) * load_fr(&hi[x >> low_bits]));
}

// num[i] = prod f_j[i], den[i] = prod g_j[i]; flags zero denominators.
__global__ void k_frac_products(Fr *num, Fr *den, FrPtrList fs, FrPtrList gs, int count, size_t n,
                                bool accumulate, uint32_t *flags, bool check_zero) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x) {
        Fr a = accumulate ? load_fr(&num[i]) : load_fr(&fs.p[0][i]);
        Fr b = accumulate ? load_fr(&den[i]) : load_fr(&gs.p[0][i]);
        for (int j = accumulate ? 0 : 1; j < count; j++) {
            a = a * load_fr(&fs.p[j][i]);
            b = b * load_fr(&gs.p[j][i]);
        }
        if (check_zero && b.is_zero()) atomicOr(flags, kFlagZeroDenominator);
        store_fr(&num[i], a);
        store_fr(&den[i], b);
    }
}

// Block-level Montgomery-trick inversion: out[i] = num[i] / den[i].
// Thread t of block b owns the kInvChunk entries b * kInvBlock * kInvChunk +
// k * kInvBlock + t (k = 0..kInvChunk-1: a warp's accesses are contiguous);
// thread chunk products are combined by shared-memory prefix/suffix scans so
// one field inversion serves kInvBlock * kInvChunk entries.  Zero
// denominators were rejected before.
constexpr int kInvBlock = 256;
constexpr int kInvChunk = 8;

__global__ void __launch_bounds__(kInvBlock) k_batch_div(const Fr *__restrict__ num, const Fr *__restrict__ den,
                                                         Fr *__restrict__ out, size_t n) {
    __shared__ Fr pre[kInvBlock];
    __shared__ Fr suf[kInvBlock];
    __shared__ Fr total_inv;
    const int t = threadIdx.x;
    const size_t base = size_t(blockIdx.x) * kInvBlock * kInvChunk + t;
    Fr one = Fr::one();
    // 1) local prefix products, stored in out[] as scratch
    Fr p = one;
    for (int k = 0; k < kInvChunk; k++) {
        const size_t i = base + size_t(k) * kInvBlock;
        if (i < n) {
            store_fr(&out[i], p);
            p = p * load_fr(&den[i]);
        }
    }
    // 2) inclusive prefix and suffix products of the thread totals
    pre[t] = p;
    suf[t] = p;
    __syncthreads();
    for (int off = 1; off < kInvBlock; off <<= 1) {
        Fr a = (t >= off) ? pre[t - off] * pre[t] : pre[t];
        Fr b = (t + off < kInvBlock) ? suf[t + off] * suf[t] : suf[t];
        __syncthreads();
        pre[t] = a;
        suf[t] = b;
        __syncthreads();
    }
    if (t == 0) total_inv = inverse(pre[kInvBlock - 1]);
    __syncthreads();
    // 3) inverse of this thread's own product = total^-1 * prefix_excl * suffix_excl
    Fr inv = total_inv;
    if (t > 0) inv = inv * pre[t - 1];
    if (t + 1 < kInvBlock) inv = inv * suf[t + 1];
    // 4) backward pass over the chunk
    for (int k = kInvChunk - 1; k >= 0; k--) {
        const size_t i = base + size_t(k) * kInvBlock;
        if (i < n) {
            const Fr inv_i = inv * load_fr(&out[i]);
            inv = inv * load_fr(&den[i]);
            store_fr(&out[i], load_fr(&num[i]) * inv_i);
        }
    }
}

// Product tree, first levels inside one block of 256 threads.  Block b reads
// frac[b*1024, (b+1)*1024) and writes levels k = 0..9: level k holds
// N/2^(k+1) entries starting at base_k = N - N/2^k, and this block's share of
// it is [base_k + b*(512>>k), base_k + (b+1)*(512>>k)).
constexpr int kSubtreeLeaves = 512;  // level-0 entries per block
constexpr int kSubtreeLevels = 10;   // levels 0..9 done in shared memory

__global__ void __launch_bounds__(256) k_prod_subtree(const Fr *frac, Fr *prod, size_t N) {
    __shared__ Fr sm[kSubtreeLeaves];
    const size_t b = blockIdx.x;
    const int t = threadIdx.x;
    for (int i = t; i < kSubtreeLeaves; i += 256) {
        size_t src = (b * kSubtreeLeaves + i) * 2;
        Fr v = load_fr(&frac[src]) * load_fr(&frac[src + 1]);
        sm[i] = v;
        store_fr(&prod[b * kSubtreeLeaves + i], v);
    }
    __syncthreads();
    for (int k = 1; k < kSubtreeLevels; k++) {
        int len = kSubtreeLeaves >> k;
        size_t base = N - (N >> k);
        Fr v;
        if (t < len) v = sm[2 * t] * sm[2 * t + 1];
        __syncthreads();
        if (t < len) {
            sm[t] = v;
            store_fr(&prod[base + b * size_t(len) + t], v);
        }
        __syncthreads();
    }
}

__global__ void k_prod_from_frac(const Fr *frac, Fr *prod, size_t half) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < half;
         i += size_t(gridDim.x) * blockDim.x)
        store_fr(&prod[i], load_fr(&frac[2 * i]) * load_fr(&frac[2 * i + 1]));
}

// One product-tree level above the subtree: prod[idx] = prod[2idx-N] * prod[2idx-N+1]
// for idx in [begin, end).
__global__ void k_prod_level(Fr *prod, size_t begin, size_t end, size_t N) {
    for (size_t idx = begin + blockIdx.x * size_t(blockDim.x) + threadIdx.x; idx < end;
         idx += size_t(gridDim.x) * blockDim.x)
        store_fr(&prod[idx], load_fr(&prod[2 * idx - N]) * load_fr(&prod[2 * idx - N + 1]));
}

__global__ void k_set_zero_last(Fr *prod, size_t N) {
    if (threadIdx.x == 0 && blockIdx.x == 0) store_fr(&prod[N - 1], Fr::zero());
}

// nums/denoms for one column: num = f + beta*(column*N + i) + gamma,
// den = g + beta*perm + gamma.  The identity term advances by beta*stride.
__global__ void k_nums_denoms(const Fr *f, const Fr *g, const Fr *perm, Fr *num, Fr *den, Fr beta,
                              Fr gamma, uint64_t column_offset, size_t n) {
    size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    size_t stride = size_t(gridDim.x) * blockDim.x;
    if (i >= n) return;
    // identity value (column_offset + i) in Montgomery form via two 32-bit halves
    uint64_t v = column_offset + i;
    Fr lo = from_u32<FrParams>(uint32_t(v));
    Fr hi = from_u32<FrParams>(uint32_t(v >> 32));
    Fr two32 = from_u32<FrParams>(65536u) * from_u32<FrParams>(65536u);
    Fr id = beta * (lo + hi * two32);
    Fr step = beta * (from_u32<FrParams>(uint32_t(stride)) +
                      from_u32<FrParams>(uint32_t(uint64_t(stride) >> 32)) * two32);
    for (; i < n; i += stride) {
        store_fr(&num[i], load_fr(&f[i]) + id + gamma);
        store_fr(&den[i], load_fr(&g[i]) + beta * load_fr(&perm[i]) + gamma);
        id = id + step;
    }
}

// p1 = even entries of (frac || prod), p2 = odd entries.
__global__ void k_product_factors(const Fr *frac, const Fr *prod, Fr *p1, Fr *p2, size_t N) {
    size_t half = N / 2;
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < N;
         i += size_t(gridDim.x) * blockDim.x) {
        const Fr *src = i < half ? frac : prod;
        size_t j = i < half ? i : i - half;
        store_fr(&p1[i], load_fr(&src[2 * j]));
        store_fr(&p2[i], load_fr(&src[2 * j + 1]));
    }
}

// ---------------------------------------------------------------------------
// Host helpers shared with other translation units
// ---------------------------------------------------------------------------

Fr host_scalar(const uint8_t *canonical) {
    host::Fr64 m;
    require(canonical != nullptr && host::from_canonical(canonical, m));
    Fr r;
    std::memcpy(r.v, m.v, 32);
    return r;
}

void host_scalars_to_device(HpCudaContext *ctx, const uint8_t *canonical, size_t count, Fr *dst) {
    std::vector<Fr> tmp(count);
    for (size_t i = 0; i < count; i++) tmp[i] = host_scalar(canonical + 32 * i);
    if (count)
        check_cuda(cudaMemcpyAsync(dst, tmp.data(), count * sizeof(Fr), cudaMemcpyHostToDevice,
                                   ctx->stream));
    // tmp is pageable: the copy has been staged before cudaMemcpyAsync returns
    // only for pageable sources, so synchronize to end the host borrow.
    ctx->sync();
}

void mle_to_mont_checked(HpCudaContext *ctx, Fr *data, size_t n) {
    k_to_mont_check<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(data, n, ctx->d_flags);
    check_launch();
}

void download_canonical(HpCudaContext *ctx, const Fr *src, size_t n, uint8_t *out) {
    Scratch tmp(ctx, n * sizeof(Fr));
    k_from_mont<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(src, tmp.as<Fr>(), n);
    check_launch();
    check_cuda(cudaMemcpyAsync(out, tmp.ptr, n * sizeof(Fr), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
}

void fold_to_scalar(HpCudaContext *ctx, const Fr *table, size_t nv, const Fr *point, Fr *dst) {
    // Ten variables per pass: block b folds entries [b 2^10, (b+1) 2^10) in
    // shared memory (one launch per ten variables instead of one per variable).
    constexpr int kTail = 10;
    // A last coordinate b in {0, 1} fixes the top variable: the value is the
    // MLE of the 2^(nv-1) entries from b 2^(nv-1) on at the other coordinates
    // (folding by 0 or 1 keeps one half exactly), so those coordinates only
    // move the table's start; one variable is left for the fold below.
    static const Fr one = [] {
        uint8_t c[32] = {1};
        return host_scalar(c);
    }();
    while (nv > 1) {
        const Fr &c = point[nv - 1];
        if (std::memcmp(c.v, one.v, sizeof(Fr)) == 0) table += table_len(nv - 1);
        else if (!c.is_zero()) break;
        nv--;
    }
    if (nv == 0) {
        check_cuda(cudaMemcpyAsync(dst, table, sizeof(Fr), cudaMemcpyDeviceToDevice, ctx->stream));
        return;
    }
    Scratch a, b;
    const Fr *cur = table;
    size_t level = 0;
    if (nv > kTail) {
        a = Scratch(ctx, table_len(nv - kTail) * sizeof(Fr));
        b = Scratch(ctx, table_len(nv > 2 * kTail ? nv - 2 * kTail : 0) * sizeof(Fr));
        Fr *bufs[2] = {a.as<Fr>(), b.as<Fr>()};
        int which = 0;
        while (nv - level > size_t(kTail)) {
            const size_t blocks = table_len(nv - level - kTail);
            FrScalarList r;
            for (int l = 0; l < kTail; l++) r.s[l] = point[level + l];
            Fr *dstb = bufs[which];
            k_fold_tail<<<unsigned(blocks), 512, table_len(kTail) * sizeof(Fr), ctx->stream>>>(cur, dstb, kTail, r);
            check_launch();
            cur = dstb;
            which ^= 1;
            level += kTail;
        }
    }
    int rest = int(nv - level);
    FrScalarList r;
    for (int l = 0; l < rest; l++) r.s[l] = point[level + l];
    size_t smem = table_len(rest) * sizeof(Fr);  // <= 32 KiB
    k_fold_tail<<<1, 512, smem, ctx->stream>>>(cur, dst, rest, r);
    check_launch();
}

void build_eq(HpCudaContext *ctx, const Fr *r_dev, size_t nv, Fr *out) {
    constexpr size_t kDirect = 12;
    size_t n = table_len(nv);
    if (nv <= kDirect) {
        k_eq_direct<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(out, r_dev, int(nv));
        check_launch();
        return;
    }
    size_t low = nv / 2, high = nv - low;
    Scratch lo(ctx, table_len(low) * sizeof(Fr)), hi(ctx, table_len(high) * sizeof(Fr));
    const unsigned lo_blocks = grid_for(ctx, table_len(low), 256), hi_blocks = grid_for(ctx, table_len(high), 256);
    k_eq_direct2<<<lo_blocks + hi_blocks, 256, 0, ctx->stream>>>(lo.as<Fr>(), hi.as<Fr>(), r_dev, int(low),
                                                                 int(high), lo_blocks);
    check_launch();
    k_eq_outer<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(out, lo.as<Fr>(), hi.as<Fr>(),
                                                              int(low), n);
    check_launch();
}

void product_tree(HpCudaContext *ctx, const Fr *frac, Fr *prod, size_t nv) {
    size_t N = table_len(nv);
    size_t k0;
    if (N >= 2 * size_t(kSubtreeLeaves)) {
        k_prod_subtree<<<unsigned(N / (2 * kSubtreeLeaves)), 256, 0, ctx->stream>>>(frac, prod, N);
        check_launch();
        k0 = kSubtreeLevels;
    } else {
        k_prod_from_frac<<<grid_for(ctx, N / 2, 256), 256, 0, ctx->stream>>>(frac, prod, N / 2);
        check_launch();
        k0 = 1;
    }
    for (size_t k = k0; k < nv; k++) {
        size_t begin = N - (N >> k), len = N >> (k + 1);
        k_prod_level<<<grid_for(ctx, len, 256), 256, 0, ctx->stream>>>(prod, begin, begin + len, N);
        check_launch();
    }
    k_set_zero_last<<<1, 32, 0, ctx->stream>>>(prod, N);
    check_launch();
}

}  // namespace hp

// ---------------------------------------------------------------------------
// ABI entries (reference bridge_mle.cpp; trait backend/src/multilinear_polynomial.rs)
// ---------------------------------------------------------------------------

using hp::kFrBytes;
using hp::kMaxList;
using hp::OwnedBuffer;
using hp::Scratch;
using hp::table_len;

extern "C" HpCudaStatus hp_cuda_v1_mle_upload(HpCudaContext *ctx, size_t num_vars,
                                              const uint8_t *evaluations, size_t evaluation_count,
                                              HpCudaDeviceAddress *out) {
    if (out) *out = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && evaluations != nullptr && num_vars <= hp::kMaxNumVars);
        size_t n = table_len(num_vars);
        require(evaluation_count == n);
        OwnedBuffer buf(ctx, n * kFrBytes);
        ctx->clear_flags();
        check_cuda(cudaMemcpyAsync(buf.ptr, evaluations, n * kFrBytes, cudaMemcpyHostToDevice,
                                   ctx->stream));
        hp::k_to_mont_check<<<hp::grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(buf.as<Fr>(), n,
                                                                               ctx->d_flags);
        check_launch();
        uint32_t flags = ctx->sync_flags();
        if (flags & hp::kFlagNonCanonical) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        *out = buf.release();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_upload_many(HpCudaContext *ctx, size_t num_vars,
                                                   const uint8_t *const *evaluations, size_t count,
                                                   size_t evaluation_count, HpCudaDeviceAddress *out) {
    if (out)
        for (size_t i = 0; i < count; i++) out[i] = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && (count == 0 || evaluations != nullptr) && num_vars <= hp::kMaxNumVars);
        const size_t n = table_len(num_vars);
        require(evaluation_count == n);
        for (size_t i = 0; i < count; i++) require(evaluations[i] != nullptr);
        if (count == 0) return;
        // table i's copy and conversion on worker stream i (mod the worker
        // count), so copies run side by side and each conversion overlaps the
        // next copies; one validation synchronisation for the batch.  A
        // non-canonical table fails the whole call and every buffer of it is
        // released (after the workers have joined back).
        std::vector<OwnedBuffer> bufs;
        bufs.reserve(count);
        for (size_t i = 0; i < count; i++) bufs.emplace_back(ctx, n * kFrBytes);
        ctx->clear_flags();
        {
            const int k = int(std::min<size_t>(count, HpCudaContext::kWorkers));
            ctx->fork(k);
            struct Join {
                HpCudaContext *c;
                int k;
                ~Join() {
                    try {
                        c->join(k);
                    } catch (...) {
                    }
                }
            } join{ctx, k};
            for (size_t i = 0; i < count; i++) {
                const cudaStream_t st = ctx->workers[i % size_t(k)];
                check_cuda(cudaMemcpyAsync(bufs[i].ptr, evaluations[i], n * kFrBytes, cudaMemcpyHostToDevice, st));
                hp::k_to_mont_check<<<hp::grid_for(ctx, n, 256), 256, 0, st>>>(bufs[i].as<Fr>(), n, ctx->d_flags);
                check_launch();
            }
        }
        const uint32_t flags = ctx->sync_flags();
        if (flags & hp::kFlagNonCanonical) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        for (size_t i = 0; i < count; i++) out[i] = bufs[i].release();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_upload_async(HpCudaContext *ctx, size_t num_vars,
                                                    const uint8_t *const *evaluations, size_t count,
                                                    size_t evaluation_count, HpCudaDeviceAddress *out) {
    if (out)
        for (size_t i = 0; i < count; i++) out[i] = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && (count == 0 || evaluations != nullptr) && num_vars <= hp::kMaxNumVars);
        const size_t n = table_len(num_vars);
        require(evaluation_count == n);
        for (size_t i = 0; i < count; i++) require(evaluations[i] != nullptr);
        if (count == 0) return;
        // Everything of this call runs on the ingress stream, after what the
        // context stream holds now (the new buffers' previous owners are
        // done with them): allocation, copies, conversions, the flag copy
        // into the call's pinned slot, then the event that work on these
        // tables waits for.  The host returns at once.
        std::shared_ptr<HpCudaIngress> in = ctx->new_ingress();
        const cudaStream_t st = ctx->ingress_stream;
        cudaEvent_t after_ctx = nullptr;
        check_cuda(cudaEventCreateWithFlags(&after_ctx, cudaEventDisableTiming));
        struct EventGuard {
            cudaEvent_t e;
            ~EventGuard() { cudaEventDestroy(e); }
        } eg{after_ctx};
        check_cuda(cudaEventRecord(after_ctx, ctx->stream));
        check_cuda(cudaStreamWaitEvent(st, after_ctx, 0));
        std::vector<void *> ptrs;
        try {
            void *dflag = ctx->scratch(16, st);
            ptrs.reserve(count);
            for (size_t i = 0; i < count; i++) ptrs.push_back(ctx->scratch(n * kFrBytes, st));
            check_cuda(cudaMemsetAsync(dflag, 0, sizeof(uint32_t), st));
            for (size_t i = 0; i < count; i++) {
                check_cuda(cudaMemcpyAsync(ptrs[i], evaluations[i], n * kFrBytes, cudaMemcpyHostToDevice, st));
                hp::k_to_mont_check<<<hp::grid_for(ctx, n, 256), 256, 0, st>>>(static_cast<Fr *>(ptrs[i]), n,
                                                                                static_cast<uint32_t *>(dflag));
                check_launch();
            }
            check_cuda(cudaMemcpyAsync(ctx->ingress_flags_h + in->slot, dflag, sizeof(uint32_t),
                                       cudaMemcpyDeviceToHost, st));
            ctx->scratch_free(dflag, st);
            check_cuda(cudaEventRecord(in->ready, st));
            for (void *p : ptrs) ctx->buffers.emplace(p, HpCudaContext::Buffer{n * kFrBytes, 1, true, in});
        } catch (...) {
            for (void *p : ptrs) {
                ctx->buffers.erase(p);
                cudaFreeAsync(p, st);
            }
            throw;
        }
        for (size_t i = 0; i < count; i++) out[i] = ptrs[i];
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_upload_wait(HpCudaContext *ctx, const HpCudaDeviceAddress *tables,
                                                   size_t count) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(count == 0 || tables != nullptr);
        for (size_t i = 0; i < count; i++) require(tables[i] != nullptr && ctx->owns(tables[i]));
        // every distinct upload these tables came from: wait for it and read its flag
        std::vector<std::shared_ptr<HpCudaIngress>> ins;
        for (size_t i = 0; i < count; i++) {
            auto &b = ctx->buffers.at(tables[i]);
            if (b.ingress && std::find(ins.begin(), ins.end(), b.ingress) == ins.end()) ins.push_back(b.ingress);
        }
        std::vector<std::shared_ptr<HpCudaIngress>> bad;
        for (auto &in : ins) {
            check_cuda(cudaEventSynchronize(in->ready));
            if (ctx->ingress_flags_h[in->slot] & hp::kFlagNonCanonical) bad.push_back(in);
        }
        if (!bad.empty()) {
            // a non-canonical element: every table of the failing uploads is released
            std::vector<void *> victims;
            for (auto &kv : ctx->buffers)
                if (kv.second.ingress && kv.second.public_handle &&
                    std::find(bad.begin(), bad.end(), kv.second.ingress) != bad.end())
                    victims.push_back(kv.first);
            for (void *p : victims) ctx->retire(p);
            fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        }
        // validated and written: later work need not wait for these uploads
        for (auto &kv : ctx->buffers)
            if (kv.second.ingress && std::find(ins.begin(), ins.end(), kv.second.ingress) != ins.end())
                kv.second.ingress.reset();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_download(HpCudaContext *ctx, HpCudaDeviceAddress polynomial,
                                                size_t num_vars, uint8_t *out_evaluations,
                                                size_t evaluation_count) {
    return guard([&] {
        hp::require_ctx(ctx);
        Fr *src = hp::mle_ptr(ctx, polynomial, num_vars);
        require(out_evaluations != nullptr && evaluation_count == table_len(num_vars));
        hp::download_canonical(ctx, src, evaluation_count, out_evaluations);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_linear_combination(HpCudaContext *ctx, size_t num_vars,
                                                          const HpCudaDeviceAddress *polynomials,
                                                          const uint8_t *coefficients,
                                                          size_t count, HpCudaDeviceAddress *out) {
    if (out) *out = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && polynomials != nullptr && coefficients != nullptr && count > 0);
        require(num_vars <= hp::kMaxNumVars);
        std::vector<const Fr *> ptrs;
        std::vector<Fr> coefs;
        for (size_t j = 0; j < count; j++) {
            const Fr *p = hp::mle_ptr(ctx, polynomials[j], num_vars);
            Fr c = hp::host_scalar(coefficients + 32 * j);
            if (c.v[0] | c.v[1] | c.v[2] | c.v[3] | c.v[4] | c.v[5] | c.v[6] | c.v[7]) {
                ptrs.push_back(p);
                coefs.push_back(c);
            }
        }
        size_t n = table_len(num_vars);
        OwnedBuffer buf(ctx, n * kFrBytes);
        if (ptrs.empty()) {
            check_cuda(cudaMemsetAsync(buf.ptr, 0, n * kFrBytes, ctx->stream));
        }
        for (size_t start = 0; start < ptrs.size(); start += kMaxList) {
            hp::FrPtrList pl{};
            hp::FrScalarList cl{};
            int m = int(std::min(ptrs.size() - start, size_t(kMaxList)));
            for (int j = 0; j < m; j++) {
                pl.p[j] = ptrs[start + j];
                cl.s[j] = coefs[start + j];
            }
            hp::k_linear_combination<<<hp::grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
                buf.as<Fr>(), pl, cl, m, n, start > 0);
            check_launch();
        }
        *out = buf.release();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_evaluate(HpCudaContext *ctx, HpCudaDeviceAddress polynomial,
                                                size_t num_vars, const uint8_t *point,
                                                uint8_t *out_evaluation) {
    return guard([&] {
        hp::require_ctx(ctx);
        const Fr *table = hp::mle_ptr(ctx, polynomial, num_vars);
        require(out_evaluation != nullptr && (num_vars == 0 || point != nullptr));
        std::vector<Fr> pt(num_vars);
        for (size_t i = 0; i < num_vars; i++) pt[i] = hp::host_scalar(point + 32 * i);
        Scratch res(ctx, sizeof(Fr));
        hp::fold_to_scalar(ctx, table, num_vars, pt.data(), res.as<Fr>());
        hp::download_canonical(ctx, res.as<Fr>(), 1, out_evaluation);
    });
}

namespace hp {

struct DotRows {
    uint32_t index[kMaxList];
};

// sum_i a[i] * b[i]: block partials (thread sums, shuffle and shared-memory
// reduction), then one block sums the partials into out.
__device__ __forceinline__ Fr fr_warp_sum(Fr v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Fr o;
#pragma unroll
        for (int i = 0; i < 8; i++) o.v[i] = __shfl_down_sync(0xffffffffu, v.v[i], off);
        v = v + o;
    }
    return v;
}

__device__ __forceinline__ Fr block_sum(Fr v) {  // blockDim.x = 256; result in thread 0
    __shared__ Fr warp_part[8];
    v = fr_warp_sum(v);
    if ((threadIdx.x & 31) == 0) warp_part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < 8 ? warp_part[threadIdx.x] : Fr::zero();
        v = fr_warp_sum(v);
    }
    return v;
}

// Block partials of sum_i a[i] b[i]: each thread's products summed unreduced
// (FrAcc), one reduction per thread.  Row y of the grid takes table a.p[y]
// against the shared b (the polynomials of one point against its eq table)
// and writes partials[y * gridDim.x + blockIdx.x].
__global__ void __launch_bounds__(256) k_dot_partials(FrPtrList tables, const Fr *b, size_t n, Fr *partials) {
    const Fr *a = tables.p[blockIdx.y];
    partials += size_t(blockIdx.y) * gridDim.x;
    FrAcc X;
    acc_zero(X);
    // two elements per iteration, their loads issued before either product
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    for (; i + stride < n; i += 2 * stride) {
        const Fr a0 = load_fr(&a[i]), b0 = load_fr(&b[i]), a1 = load_fr(&a[i + stride]), b1 = load_fr(&b[i + stride]);
        acc_mul_add(X, a0, b0);
        acc_mul_add(X, a1, b1);
    }
    if (i < n) acc_mul_add(X, load_fr(&a[i]), load_fr(&b[i]));
    Fr acc = block_sum(acc_reduce(X));
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// The same with eq(x, point) = lo[x & mask] hi[x >> low_bits] never built:
// the grid's stride is a multiple of 2^low_bits, so a thread's entries all
// share x & mask = l and it sums f[x] hi[x >> low_bits] (unreduced) and
// multiplies by lo[l] once at the end.
__global__ void __launch_bounds__(256) k_dot_split_partials(FrPtrList tables, const Fr *lo, const Fr *hi,
                                                            int low_bits, size_t n, Fr *partials) {
    const Fr *a = tables.p[blockIdx.y];
    partials += size_t(blockIdx.y) * gridDim.x;
    FrAcc X;
    acc_zero(X);
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    const size_t first = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    size_t i = first;
    for (; i + stride < n; i += 2 * stride) {
        const Fr a0 = load_fr(&a[i]), h0 = load_fr(&hi[i >> low_bits]);
        const Fr a1 = load_fr(&a[i + stride]), h1 = load_fr(&hi[(i + stride) >> low_bits]);
        acc_mul_add(X, a0, h0);
        acc_mul_add(X, a1, h1);
    }
    if (i < n) acc_mul_add(X, load_fr(&a[i]), load_fr(&hi[i >> low_bits]));
    Fr v = acc_reduce(X);
    if (first < n) v = v * load_fr(&lo[first & ((size_t(1) << low_bits) - 1)]);
    Fr acc = block_sum(v);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// Block y sums row y of a [rows][count] partial matrix into out[index[y]].
__global__ void __launch_bounds__(256) k_sum_partials(const Fr *partials, int count, Fr *out, DotRows rows) {
    partials += size_t(blockIdx.x) * count;
    out += rows.index[blockIdx.x];
    Fr acc = Fr::zero();
    for (int i = threadIdx.x; i < count; i += blockDim.x) acc = acc + partials[i];
    acc = block_sum(acc);
    if (threadIdx.x == 0) *out = acc;
}

}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_mle_evaluate_many(HpCudaContext *ctx, size_t count,
                                                     const HpCudaDeviceAddress *polynomials,
                                                     const size_t *num_vars, const uint8_t *points,
                                                     uint8_t *out_evaluations) {
    return guard([&] {
        hp::require_ctx(ctx);
        if (count == 0) return;
        require(polynomials != nullptr && num_vars != nullptr && out_evaluations != nullptr);
        std::vector<const Fr *> tables(count);
        std::vector<std::vector<Fr>> pts(count);
        size_t off = 0;
        for (size_t k = 0; k < count; k++) {
            tables[k] = hp::mle_ptr(ctx, polynomials[k], num_vars[k]);
            require(num_vars[k] == 0 || points != nullptr);
            pts[k].resize(num_vars[k]);
            for (size_t i = 0; i < num_vars[k]; i++) pts[k][i] = hp::host_scalar(points + 32 * (off + i));
            off += num_vars[k];
        }
        Scratch res(ctx, count * sizeof(Fr));
        // Polynomials of >= 2^12 entries sharing a point: f(point) = sum_x f[x]
        // eq(x, point), one eq table per distinct point (a streaming dot
        // product per polynomial instead of a fold chain each); the others fold.
        constexpr size_t kDotMinVars = 12;
        std::vector<bool> done(count, false);
        off = 0;
        std::vector<size_t> first(count);
        for (size_t k = 0; k < count; k++) {
            first[k] = off;
            off += num_vars[k];
        }
        for (size_t k = 0; k < count; k++) {
            if (done[k] || num_vars[k] < kDotMinVars) continue;
            std::vector<size_t> group{k};
            for (size_t j = k + 1; j < count; j++)
                if (!done[j] && num_vars[j] == num_vars[k] &&
                    std::memcmp(points + 32 * first[j], points + 32 * first[k], 32 * num_vars[k]) == 0)
                    group.push_back(j);
            if (group.size() < 2) continue;
            const size_t nv = num_vars[k], n = hp::table_len(nv);
            Scratch rd(ctx, nv * sizeof(Fr));
            check_cuda(cudaMemcpyAsync(rd.ptr, pts[k].data(), nv * sizeof(Fr), cudaMemcpyHostToDevice, ctx->stream));
            // a few blocks per SM: long per-thread runs amortise the reduction;
            // the group's dot products in one launch (up to 32 tables per launch)
            const unsigned grid = hp::grid_for(ctx, n, 256, 2);
            const size_t rows = std::min(group.size(), size_t(hp::kMaxList));
            Scratch part(ctx, rows * grid * sizeof(Fr));
            // eq(x, point) as its two half tables (the split of build_eq) when
            // the grid's stride fixes every thread's low half, else in full
            const size_t low = nv / 2, high = nv - low;
            const bool split = nv > 12 && (size_t(grid) * 256) % hp::table_len(low) == 0;
            Scratch eq(ctx, split ? (hp::table_len(low) + hp::table_len(high)) * sizeof(Fr) : n * sizeof(Fr));
            if (split) {
                const unsigned lo_blocks = hp::grid_for(ctx, hp::table_len(low), 256);
                const unsigned hi_blocks = hp::grid_for(ctx, hp::table_len(high), 256);
                hp::k_eq_direct2<<<lo_blocks + hi_blocks, 256, 0, ctx->stream>>>(
                    eq.as<Fr>(), eq.as<Fr>() + hp::table_len(low), rd.as<Fr>(), int(low), int(high), lo_blocks);
                check_launch();
            } else {
                hp::build_eq(ctx, rd.as<Fr>(), nv, eq.as<Fr>());
            }
            for (size_t g0 = 0; g0 < group.size(); g0 += hp::kMaxList) {
                const unsigned m = unsigned(std::min(group.size() - g0, size_t(hp::kMaxList)));
                hp::FrPtrList tl{};
                hp::DotRows dr{};
                for (unsigned y = 0; y < m; y++) {
                    tl.p[y] = tables[group[g0 + y]];
                    dr.index[y] = uint32_t(group[g0 + y]);
                    done[group[g0 + y]] = true;
                }
                if (split)
                    hp::k_dot_split_partials<<<dim3(grid, m), 256, 0, ctx->stream>>>(
                        tl, eq.as<Fr>(), eq.as<Fr>() + hp::table_len(low), int(low), n, part.as<Fr>());
                else
                    hp::k_dot_partials<<<dim3(grid, m), 256, 0, ctx->stream>>>(tl, eq.as<Fr>(), n, part.as<Fr>());
                check_launch();
                hp::k_sum_partials<<<m, 256, 0, ctx->stream>>>(part.as<Fr>(), int(grid), res.as<Fr>(), dr);
                check_launch();
            }
        }
        for (size_t k = 0; k < count; k++)
            if (!done[k]) hp::fold_to_scalar(ctx, tables[k], num_vars[k], pts[k].data(), res.as<Fr>() + k);
        hp::download_canonical(ctx, res.as<Fr>(), count, out_evaluations);
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_build_eq_x_r(HpCudaContext *ctx, const uint8_t *r,
                                                    size_t num_vars, HpCudaDeviceAddress *out) {
    if (out) *out = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && r != nullptr && num_vars > 0 && num_vars <= hp::kMaxNumVars);
        Scratch rd(ctx, num_vars * sizeof(Fr));
        hp::host_scalars_to_device(ctx, r, num_vars, rd.as<Fr>());
        OwnedBuffer buf(ctx, table_len(num_vars) * kFrBytes);
        hp::build_eq(ctx, rd.as<Fr>(), num_vars, buf.as<Fr>());
        // the point rides with the table: a prover state over a product
        // family sharing this factor takes the eq-factored zero-check round
        std::vector<uint64_t> point(4 * num_vars);
        for (size_t i = 0; i < num_vars; i++) {
            const Fr v = hp::host_scalar(r + 32 * i);
            std::memcpy(&point[4 * i], v.v, 32);
        }
        ctx->buffers.at(buf.ptr).eq_point = std::move(point);
        *out = buf.release();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_compute_frac_poly(HpCudaContext *ctx, size_t num_vars,
                                                         const HpCudaDeviceAddress *numerators,
                                                         const HpCudaDeviceAddress *denominators,
                                                         size_t count, HpCudaDeviceAddress *out) {
    if (out) *out = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && numerators != nullptr && denominators != nullptr && count > 0);
        require(num_vars <= hp::kMaxNumVars);
        std::vector<const Fr *> fs(count), gs(count);
        for (size_t j = 0; j < count; j++) {
            fs[j] = hp::mle_ptr(ctx, numerators[j], num_vars);
            gs[j] = hp::mle_ptr(ctx, denominators[j], num_vars);
        }
        size_t n = table_len(num_vars);
        Scratch num(ctx, n * kFrBytes), den(ctx, n * kFrBytes);
        ctx->clear_flags();
        for (size_t start = 0; start < count; start += kMaxList) {
            hp::FrPtrList fl{}, gl{};
            int m = int(std::min(count - start, size_t(kMaxList)));
            for (int j = 0; j < m; j++) {
                fl.p[j] = fs[start + j];
                gl.p[j] = gs[start + j];
            }
            bool last = start + kMaxList >= count;
            hp::k_frac_products<<<hp::grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
                num.as<Fr>(), den.as<Fr>(), fl, gl, m, n, start > 0, ctx->d_flags, last);
            check_launch();
        }
        uint32_t flags = ctx->sync_flags();
        if (flags & hp::kFlagZeroDenominator) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        OwnedBuffer buf(ctx, n * kFrBytes);
        size_t per_block = size_t(hp::kInvBlock) * hp::kInvChunk;
        hp::k_batch_div<<<unsigned((n + per_block - 1) / per_block), hp::kInvBlock, 0,
                          ctx->stream>>>(num.as<Fr>(), den.as<Fr>(), buf.as<Fr>(), n);
        check_launch();
        *out = buf.release();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_compute_product_poly(HpCudaContext *ctx,
                                                            HpCudaDeviceAddress frac,
                                                            size_t num_vars,
                                                            HpCudaDeviceAddress *out) {
    if (out) *out = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && num_vars > 0);
        const Fr *f = hp::mle_ptr(ctx, frac, num_vars);
        OwnedBuffer buf(ctx, table_len(num_vars) * kFrBytes);
        hp::product_tree(ctx, f, buf.as<Fr>(), num_vars);
        *out = buf.release();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_compute_nums_and_denoms(
    HpCudaContext *ctx, size_t num_vars, const uint8_t *beta, const uint8_t *gamma,
    const HpCudaDeviceAddress *fxs, const HpCudaDeviceAddress *gxs,
    const HpCudaDeviceAddress *permutations, size_t count, HpCudaDeviceAddress *out_numerators,
    HpCudaDeviceAddress *out_denominators) {
    if (out_numerators)
        for (size_t j = 0; j < count; j++) out_numerators[j] = nullptr;
    if (out_denominators)
        for (size_t j = 0; j < count; j++) out_denominators[j] = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out_numerators != nullptr && out_denominators != nullptr && fxs != nullptr &&
                gxs != nullptr && permutations != nullptr && count > 0 && beta != nullptr &&
                gamma != nullptr);
        require(num_vars <= hp::kMaxNumVars);
        Fr b = hp::host_scalar(beta), g = hp::host_scalar(gamma);
        size_t n = table_len(num_vars);
        std::vector<OwnedBuffer> nums, dens;
        nums.reserve(count);
        dens.reserve(count);
        for (size_t j = 0; j < count; j++) {
            const Fr *f = hp::mle_ptr(ctx, fxs[j], num_vars);
            const Fr *gx = hp::mle_ptr(ctx, gxs[j], num_vars);
            const Fr *p = hp::mle_ptr(ctx, permutations[j], num_vars);
            nums.emplace_back(ctx, n * kFrBytes);
            dens.emplace_back(ctx, n * kFrBytes);
            hp::k_nums_denoms<<<hp::grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
                f, gx, p, nums.back().as<Fr>(), dens.back().as<Fr>(), b, g, uint64_t(j) * n, n);
            check_launch();
        }
        for (size_t j = 0; j < count; j++) {
            out_numerators[j] = nums[j].release();
            out_denominators[j] = dens[j].release();
        }
    });
}

extern "C" HpCudaStatus hp_cuda_v1_mle_compute_product_factors(HpCudaContext *ctx,
                                                               HpCudaDeviceAddress frac,
                                                               HpCudaDeviceAddress product,
                                                               size_t num_vars,
                                                               HpCudaDeviceAddress *out_p1,
                                                               HpCudaDeviceAddress *out_p2) {
    if (out_p1) *out_p1 = nullptr;
    if (out_p2) *out_p2 = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out_p1 != nullptr && out_p2 != nullptr && num_vars > 0);
        const Fr *f = hp::mle_ptr(ctx, frac, num_vars);
        const Fr *p = hp::mle_ptr(ctx, product, num_vars);
        size_t n = table_len(num_vars);
        OwnedBuffer a(ctx, n * kFrBytes), b(ctx, n * kFrBytes);
        hp::k_product_factors<<<hp::grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
            f, p, a.as<Fr>(), b.as<Fr>(), n);
        check_launch();
        *out_p1 = a.release();
        *out_p2 = b.release();
    });
}
