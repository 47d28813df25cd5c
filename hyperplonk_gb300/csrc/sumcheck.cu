// sumcheck.cu -- SumCheck prover state and the fused fold + round-message
// kernel.
//
// Reference semantics: backend/src/cpu/sum_check.rs:35-217.  Round k (1-based)
// first fixes the lowest variable of every distinct factor with the previous
// challenge (ark-poly fix_variables: f'[b] = f[2b] + r*(f[2b+1] - f[2b])),
// then for every product of arity m evaluates
//     s(t) = sum_b prod_j (f_j[2b] + t*(f_j[2b+1] - f_j[2b]))   for t = 0..m,
// scales by the product coefficient and extends the degree-m polynomial to
// t = 0..max_degree.  The reference extends with barycentric weights; this
// backend evaluates Newton's forward-difference form over the integer nodes,
// which yields the same field elements (the degree-m interpolant is unique).
//
// GB300 shape: one launch per round fuses the fold of round k-1's challenge
// with the message of round k, so each factor table is read once and its
// folded half written once per round.  Per-thread slot sums stay in shared
// memory and are reduced once per block; the last block of the launch sums
// the block partials, extrapolates, scales and writes canonical bytes.
// Rounds of <= 64 pairs run in one block (fold, products and finalize in one
// launch); products of arity > 8 or more than 48 slots use a shared-memory
// kernel and a separate one-block finalize.
#include <algorithm>
#include <cstring>
#include <vector>

#include "host_field.h"
#include "mle.cuh"
#include "runtime.cuh"
#include "sumcheck.cuh"
#include "transcript.h"

using hp::check_cuda;
using hp::check_launch;
using hp::fail;
using hp::Fr;
using hp::guard;
using hp::require;

namespace hp {

// Shared-memory layout per thread (T threads per block, column-major by slot
// so thread t's entries are sm[slot * T + t]):
//   [0, 2F)           lo_f, d_f  (folded pair value and its step)
//   [2F, 2F + M)      running evaluations of the current product
//   [2F + M, ...+S)   accumulators, one per (product, t) slot
__global__ void k_sumcheck_round(SumcheckDesc desc, FrPtrList src, FrMutPtrList dst, bool fold,
                                 Fr r, size_t pairs, Fr *partials) {
    extern __shared__ Fr sm[];
    const int T = blockDim.x;
    const int t = threadIdx.x;
    const int F = desc.factor_count;
    const int M = desc.max_arity;
    const int S = desc.slot_count;
    Fr *fv = sm;
    Fr *ev = sm + 2 * F * T;
    Fr *acc = ev + M * T;
    for (int s = 0; s < S; s++) acc[s * T + t] = Fr::zero();

    for (size_t b = blockIdx.x * size_t(T) + t; b < pairs; b += size_t(gridDim.x) * T) {
        for (int f = 0; f < F; f++) {
            Fr lo, hi;
            if (fold) {
                const Fr *s = src.p[f] + 4 * b;
                Fr a0 = load_fr(s), a1 = load_fr(s + 1), a2 = load_fr(s + 2), a3 = load_fr(s + 3);
                lo = a0 + r * (a1 - a0);
                hi = a2 + r * (a3 - a2);
                Fr *d = dst.p[f] + 2 * b;
                store_fr(d, lo);
                store_fr(d + 1, hi);
            } else {
                const Fr *s = src.p[f] + 2 * b;
                lo = load_fr(s);
                hi = load_fr(s + 1);
            }
            fv[(2 * f) * T + t] = lo;
            fv[(2 * f + 1) * T + t] = hi - lo;
        }
        for (int p = 0; p < desc.product_count; p++) {
            const int begin = desc.offsets[p], m = desc.offsets[p + 1] - begin;
            const int slot = desc.slot_base[p];
            Fr prod = fv[(2 * desc.indices[begin]) * T + t];
            ev[t] = prod;
            for (int j = 1; j < m; j++) {
                Fr v = fv[(2 * desc.indices[begin + j]) * T + t];
                ev[j * T + t] = v;
                prod = prod * v;
            }
            acc[slot * T + t] = acc[slot * T + t] + prod;
            for (int k = 1; k <= m; k++) {
                Fr e = ev[t] + fv[(2 * desc.indices[begin] + 1) * T + t];
                ev[t] = e;
                prod = e;
                for (int j = 1; j < m; j++) {
                    Fr ej = ev[j * T + t] + fv[(2 * desc.indices[begin + j] + 1) * T + t];
                    ev[j * T + t] = ej;
                    prod = prod * ej;
                }
                acc[(slot + k) * T + t] = acc[(slot + k) * T + t] + prod;
            }
        }
    }
    // block tree reduction of every slot
    for (int s = 0; s < S; s++) {
        __syncthreads();
        for (int half = T / 2; half > 0; half >>= 1) {
            if (t < half) acc[s * T + t] = acc[s * T + t] + acc[s * T + t + half];
            __syncthreads();
        }
        if (t == 0) partials[size_t(s) * gridDim.x + blockIdx.x] = acc[s * T];  // slot-major
    }
}

// Register-resident round for products of arity <= MAXM (every VP of the
// prover: degree <= 5).  One pair per thread per iteration; the fold of all
// factors is written to `dst` first, then each product re-reads its factors'
// folded pair (an L1/L2 hit: this thread just wrote it) and evaluates at
// t = 0..m with running values in registers; each (product, t) value is added
// to the thread's own slot sum in shared memory, and the block reduces the
// slot sums once at the end (a warp shuffle reduction per value and pair
// cost as much as the products themselves).
#ifndef HP_ROUND_THREADS
#define HP_ROUND_THREADS 128
#endif
#ifndef HP_ROUND_BLOCKS_PER_SM
#define HP_ROUND_BLOCKS_PER_SM 4
#endif
constexpr int kRoundThreads = HP_ROUND_THREADS;
constexpr int kMaxSlotsV2 = 48;  // slot sums in shared memory: 48 x 128 x 32 B = 192 KiB

__device__ __forceinline__ Fr warp_sum(Fr v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Fr o;
#pragma unroll
        for (int i = 0; i < 8; i++) o.v[i] = __shfl_down_sync(0xffffffffu, v.v[i], off);
        v = v + o;
    }
    return v;
}

__device__ void finalize_from_sums(const SumcheckDesc &desc, Fr *sums, const Fr *coefs, int degree, Fr *out);

__device__ __forceinline__ Fr load_fr_cg(const Fr *p) {  // L2 load: written by other blocks of this launch
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
    const uint4 a = __ldcg(q), b = __ldcg(q + 1);
    Fr r;
    r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
    r.v[4] = b.x; r.v[5] = b.y; r.v[6] = b.z; r.v[7] = b.w;
    return r;
}

// After the block partials (slot-major) are written: the last block of the
// launch to finish (a counter per prover state, reset by that block) sums
// them and writes the round message -- no separate finalize launch.
__device__ __forceinline__ void finish_round_in_last_block(const SumcheckDesc &desc, const Fr *partials,
                                                           unsigned *counter, const Fr *coefs, int degree,
                                                           Fr *out, Fr *sums) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    const int S = desc.slot_count, blocks = gridDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    for (int s = warp; s < S; s += warps) {
        Fr a = Fr::zero();
        for (int b = lane; b < blocks; b += 32) a = a + load_fr_cg(&partials[size_t(s) * blocks + b]);
        a = warp_sum(a);
        if (lane == 0) sums[s] = a;
    }
    __syncthreads();
    finalize_from_sums(desc, sums, coefs, degree, out);
    if (threadIdx.x == 0) *counter = 0u;
}

template <int MAXM>
__global__ void __launch_bounds__(kRoundThreads) k_sumcheck_round_regs(SumcheckDesc desc, FrPtrList src,
                                                                       FrMutPtrList dst, FrPtrList rd, bool fold,
                                                                       Fr r, size_t pairs, Fr *partials,
                                                                       unsigned *counter, const Fr *coefs,
                                                                       int degree, Fr *out) {
    // acc[s * kRoundThreads + t]: thread t's running sum of slot s over its pairs
    extern __shared__ Fr acc[];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int S = desc.slot_count, F = desc.factor_count;
    for (int s = 0; s < S; s++) acc[s * kRoundThreads + t] = Fr::zero();
    for (size_t b = size_t(blockIdx.x) * kRoundThreads + t; b < pairs; b += size_t(gridDim.x) * kRoundThreads) {
        if (fold) {
            for (int f = 0; f < F; f++) {
                const Fr *s = src.p[f] + 4 * b;
                Fr a0 = load_fr(s), a1 = load_fr(s + 1), a2 = load_fr(s + 2), a3 = load_fr(s + 3);
                Fr *d = dst.p[f] + 2 * b;
                store_fr(d, a0 + r * (a1 - a0));
                store_fr(d + 1, a2 + r * (a3 - a2));
            }
        }
        for (int p = 0; p < desc.product_count; p++) {
            const int begin = desc.offsets[p], m = desc.offsets[p + 1] - begin, slot = desc.slot_base[p];
            Fr e[MAXM], st[MAXM];
#pragma unroll
            for (int j = 0; j < MAXM; j++) {
                if (j < m) {
                    const Fr *q = rd.p[desc.indices[begin + j]] + 2 * b;
                    e[j] = load_fr(q);
                    st[j] = load_fr(q + 1) - e[j];
                }
            }
            for (int k = 0; k <= m; k++) {
                if (k > 0) {
#pragma unroll
                    for (int j = 0; j < MAXM; j++)
                        if (j < m) e[j] = e[j] + st[j];
                }
                Fr v = e[0];
#pragma unroll
                for (int j = 1; j < MAXM; j++)
                    if (j < m) v = v * e[j];
                Fr &a = acc[(slot + k) * kRoundThreads + t];
                a = a + v;
            }
        }
    }
    __syncthreads();
    // warp w reduces slots w, w + 4, ...: 4 column values per lane, then shuffles
    for (int s = warp; s < S; s += kRoundThreads / 32) {
        Fr v = acc[s * kRoundThreads + lane];
#pragma unroll
        for (int i = 1; i < kRoundThreads / 32; i++) v = v + acc[s * kRoundThreads + 32 * i + lane];
        v = warp_sum(v);
        if (lane == 0) partials[size_t(s) * gridDim.x + blockIdx.x] = v;  // slot-major
    }
    __syncthreads();  // acc is reused below as the last block's slot sums
    finish_round_in_last_block(desc, partials, counter, coefs, degree, out, acc);
}

// One block.  Warp w sums the block partials of slots w, w + warps, ... (lane
// strided loads, then shuffles) into shared memory and slot_sums.  Thread p
// then turns product p's m+1 sums v(0..m) into its forward differences
// Delta^j v(0) in place, and thread x evaluates the round polynomial at t = x
// as sum_p coef_p sum_{j <= min(x, m)} C(x, j) Delta^j v_p(0) -- Newton's
// form of the unique polynomial of degree <= m through the sums, so equal to
// the slot sum for x <= m and to the reference's barycentric extrapolation
// (backend/src/cpu/sum_check.rs:183-217) beyond.  Writes the d+1 canonical
// evaluations.
// Given the slot sums in shared memory (all threads of the block): turn each
// product's m+1 sums into forward differences in place, then thread x writes
// the canonical round evaluation at t = x.
__device__ void finalize_from_sums(const SumcheckDesc &desc, Fr *sums, const Fr *coefs, int degree, Fr *out) {
    for (int p = threadIdx.x; p < desc.product_count; p += blockDim.x) {
        Fr *v = sums + desc.slot_base[p];
        const int m = desc.offsets[p + 1] - desc.offsets[p];
        for (int j = 1; j <= m; j++)
            for (int i = m; i >= j; i--) v[i] = v[i] - v[i - 1];  // v[i] = Delta^j v(i - j)
    }
    __syncthreads();
    for (int x = threadIdx.x; x <= degree; x += blockDim.x) {
        Fr acc = Fr::zero();
        for (int p = 0; p < desc.product_count; p++) {
            const Fr *v = sums + desc.slot_base[p];
            const int m = desc.offsets[p + 1] - desc.offsets[p];
            Fr val = v[0];
            uint64_t c = 1;  // C(x, j); C(64, j) < 2^61
            for (int j = 1; j <= m && j <= x; j++) {
                c = uint64_t((unsigned __int128)c * uint64_t(x - j + 1) / uint64_t(j));
                Fr cj = Fr::zero();
                cj.v[0] = uint32_t(c);
                cj.v[1] = uint32_t(c >> 32);
                val = val + to_mont(cj) * v[j];
            }
            acc = acc + coefs[p] * val;
        }
        out[x] = from_mont(acc);
    }
}

__global__ void k_sumcheck_finalize(SumcheckDesc desc, const Fr *partials, int blocks,
                                    const Fr *coefs, int degree, Fr *slot_sums, Fr *out) {
    extern __shared__ Fr sums[];
    const int S = desc.slot_count;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    for (int s = warp; s < S; s += warps) {
        Fr a = Fr::zero();
        for (int b = lane; b < blocks; b += 32) a = a + partials[size_t(s) * blocks + b];
        a = warp_sum(a);
        if (lane == 0) {
            sums[s] = a;
            slot_sums[s] = a;
        }
    }
    __syncthreads();
    finalize_from_sums(desc, sums, coefs, degree, out);
}

// A round of at most kSmallPairs pairs in one block, finalize included (the
// last rounds of every sumcheck: latency-bound, so the work is spread over
// (factor, pair) and (product, pair) items instead of one pair per thread).
constexpr int kSmallPairs = 64;
constexpr int kSmallThreads = 256;

template <int MAXM>
__global__ void __launch_bounds__(kSmallThreads) k_sumcheck_round_small(SumcheckDesc desc, FrPtrList src,
                                                                        FrMutPtrList dst, FrPtrList rd, bool fold,
                                                                        Fr r, int pairs, const Fr *coefs, int degree,
                                                                        Fr *out) {
    extern __shared__ Fr sm[];  // vals[S][kSmallPairs], then sums[S]
    const int S = desc.slot_count, F = desc.factor_count;
    Fr *vals = sm, *sums = sm + size_t(S) * kSmallPairs;
    if (fold) {
        for (int idx = threadIdx.x; idx < F * pairs; idx += blockDim.x) {
            const int f = idx / pairs, b = idx % pairs;
            const Fr *q = src.p[f] + 4 * b;
            Fr a0 = load_fr(q), a1 = load_fr(q + 1), a2 = load_fr(q + 2), a3 = load_fr(q + 3);
            Fr *d = dst.p[f] + 2 * b;
            store_fr(d, a0 + r * (a1 - a0));
            store_fr(d + 1, a2 + r * (a3 - a2));
        }
        __syncthreads();  // the folded tables are read below by other threads
    }
    for (int idx = threadIdx.x; idx < desc.product_count * pairs; idx += blockDim.x) {
        const int p = idx / pairs, b = idx % pairs;
        const int begin = desc.offsets[p], m = desc.offsets[p + 1] - begin, slot = desc.slot_base[p];
        Fr e[MAXM], st[MAXM];
#pragma unroll
        for (int j = 0; j < MAXM; j++) {
            if (j < m) {
                const Fr *q = rd.p[desc.indices[begin + j]] + 2 * b;
                e[j] = load_fr(q);
                st[j] = load_fr(q + 1) - e[j];
            }
        }
        for (int k = 0; k <= m; k++) {
            if (k > 0) {
#pragma unroll
                for (int j = 0; j < MAXM; j++)
                    if (j < m) e[j] = e[j] + st[j];
            }
            Fr v = e[0];
#pragma unroll
            for (int j = 1; j < MAXM; j++)
                if (j < m) v = v * e[j];
            vals[(slot + k) * kSmallPairs + b] = v;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int s = warp; s < S; s += kSmallThreads / 32) {
        Fr v = lane < pairs ? vals[s * kSmallPairs + lane] : Fr::zero();
        if (lane + 32 < pairs) v = v + vals[s * kSmallPairs + lane + 32];
        v = warp_sum(v);
        if (lane == 0) sums[s] = v;
    }
    __syncthreads();
    finalize_from_sums(desc, sums, coefs, degree, out);
}

__global__ void k_sumcheck_final_fold(FrPtrList tables, int count, Fr r, Fr *out) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= count) return;
    Fr lo = load_fr(tables.p[f]), hi = load_fr(tables.p[f] + 1);
    out[f] = from_mont(lo + r * (hi - lo));
}

}  // namespace hp

// ---------------------------------------------------------------------------
// Prover state
// ---------------------------------------------------------------------------

struct HpCudaSumCheckProverState {
    size_t num_vars = 0, max_degree = 0, round = 0;
    bool poisoned = false;
    hp::SumcheckDesc desc{};
    std::vector<void *> inputs;  // referenced input factor buffers
    void *fold_a = nullptr;      // F x 2^(nv-1) Fr
    void *fold_b = nullptr;      // F x 2^(nv-2) Fr
    void *coefs = nullptr;       // P Montgomery coefficients (device)
    int current = 0;             // 0: inputs, 1: fold_a, 2: fold_b
};

namespace hp {

static const Fr *state_table(HpCudaSumCheckProverState *s, int which, int f) {
    size_t a_stride = s->num_vars >= 1 ? table_len(s->num_vars - 1) : 1;
    size_t b_stride = s->num_vars >= 2 ? table_len(s->num_vars - 2) : 1;
    if (which == 0) return static_cast<const Fr *>(s->inputs[f]);
    if (which == 1) return static_cast<const Fr *>(s->fold_a) + f * a_stride;
    return static_cast<const Fr *>(s->fold_b) + f * b_stride;
}

static unsigned *round_counter(HpCudaSumCheckProverState *s) {
    const size_t p = std::max(size_t(s->desc.product_count), size_t(1));
    return reinterpret_cast<unsigned *>(static_cast<Fr *>(s->coefs) + p);
}

static void release_state(HpCudaContext *ctx, HpCudaSumCheckProverState *s) {
    for (void *p : s->inputs) {
        try { ctx->unref(p); } catch (...) {}
    }
    s->inputs.clear();
    if (s->fold_a) ctx->scratch_free(s->fold_a);
    if (s->fold_b) ctx->scratch_free(s->fold_b);
    if (s->coefs) ctx->scratch_free(s->coefs);
    s->fold_a = s->fold_b = s->coefs = nullptr;
}

static int round_block_size(const SumcheckDesc &d, size_t *smem_out) {
    size_t per_thread = size_t(2 * d.factor_count + d.max_arity + d.slot_count) * sizeof(Fr);
    int T = 256;
    while (T > 32 && per_thread * T > 200 * 1024) T /= 2;
    if (per_thread * T > 200 * 1024) fail(HP_CUDA_STATUS_NOT_IMPLEMENTED);
    *smem_out = per_thread * T;
    return T;
}

}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_sumcheck_prover_state_create(
    HpCudaContext *ctx, size_t num_vars, size_t max_degree, const HpCudaDeviceAddress *factors,
    size_t factor_count, const uint8_t *coefficients, const size_t *product_offsets,
    size_t product_count, const size_t *factor_indices, size_t index_count,
    HpCudaSumCheckProverState **out) {
    if (out) *out = nullptr;
    return guard([&] {
        hp::require_ctx(ctx);
        require(out != nullptr && product_offsets != nullptr);
        require(num_vars > 0 && num_vars <= hp::kMaxNumVars && max_degree > 0);
        require(factor_count == 0 || factors != nullptr);
        require(product_count == 0 || coefficients != nullptr);
        require(index_count == 0 || factor_indices != nullptr);
        require(product_offsets[0] == 0 && product_offsets[product_count] == index_count);
        for (size_t p = 0; p < product_count; p++) {
            size_t m = product_offsets[p + 1] - product_offsets[p];
            require(product_offsets[p + 1] >= product_offsets[p] && m >= 1 && m <= max_degree);
        }
        for (size_t i = 0; i < index_count; i++) require(factor_indices[i] < factor_count);
        if (factor_count > size_t(hp::kMaxList) || product_count > size_t(hp::kMaxProducts) ||
            index_count > size_t(hp::kMaxIndices) || max_degree > size_t(hp::kMaxDegree))
            fail(HP_CUDA_STATUS_NOT_IMPLEMENTED);

        auto *s = new HpCudaSumCheckProverState();
        try {
            s->num_vars = num_vars;
            s->max_degree = max_degree;
            hp::SumcheckDesc &d = s->desc;
            d.factor_count = int(factor_count);
            d.product_count = int(product_count);
            int slots = 0, max_arity = 1;
            for (size_t p = 0; p < product_count; p++) {
                int m = int(product_offsets[p + 1] - product_offsets[p]);
                d.offsets[p] = uint16_t(product_offsets[p]);
                d.slot_base[p] = uint16_t(slots);
                slots += m + 1;
                max_arity = std::max(max_arity, m);
            }
            d.offsets[product_count] = uint16_t(index_count);
            for (size_t i = 0; i < index_count; i++) d.indices[i] = uint8_t(factor_indices[i]);
            d.slot_count = std::max(slots, 1);
            d.max_arity = max_arity;
            for (size_t f = 0; f < factor_count; f++) {
                hp::mle_ptr(ctx, factors[f], num_vars);
                ctx->ref(factors[f]);
                s->inputs.push_back(factors[f]);
            }
            // coefficients, then one zeroed Fr slot whose first word is the
            // round kernels' last-block counter
            s->coefs = ctx->scratch((std::max(product_count, size_t(1)) + 1) * sizeof(Fr));
            hp::host_scalars_to_device(ctx, coefficients, product_count, static_cast<Fr *>(s->coefs));
            check_cuda(cudaMemsetAsync(static_cast<Fr *>(s->coefs) + std::max(product_count, size_t(1)), 0,
                                       sizeof(Fr), ctx->stream));
            size_t a_len = hp::table_len(num_vars - 1);
            size_t b_len = num_vars >= 2 ? hp::table_len(num_vars - 2) : 1;
            size_t fcount = std::max(factor_count, size_t(1));
            s->fold_a = ctx->scratch(fcount * a_len * sizeof(Fr));
            s->fold_b = ctx->scratch(fcount * b_len * sizeof(Fr));
            size_t smem;
            hp::round_block_size(d, &smem);
        } catch (...) {
            hp::release_state(ctx, s);
            delete s;
            throw;
        }
        *out = s;
    });
}

namespace hp {

// Checks a round request without touching the state (misuse -> InvalidState,
// bad arguments -> InvalidParameters).
static void check_round(HpCudaSumCheckProverState *s, const uint8_t *challenge_or_null, uint8_t *out,
                        size_t evaluation_count) {
    require(s != nullptr && out != nullptr);
    if (s->poisoned) fail(HP_CUDA_STATUS_INVALID_STATE);
    require(evaluation_count == s->max_degree + 1);
    if (s->round >= s->num_vars) fail(HP_CUDA_STATUS_INVALID_STATE);
    if (s->round == 0 && challenge_or_null != nullptr) fail(HP_CUDA_STATUS_INVALID_STATE);
    if (s->round > 0 && challenge_or_null == nullptr) fail(HP_CUDA_STATUS_INVALID_STATE);
}

// Enqueues one round of state s on stream st: fold with r (rounds > 1) and
// message into out_dev (degree + 1 canonical Fr, device).  Scratch is ordered
// on st.  Does not advance the state.
static void enqueue_round(HpCudaContext *ctx, HpCudaSumCheckProverState *s, const Fr &r, cudaStream_t st,
                          Fr *out_dev) {
    const SumcheckDesc &d = s->desc;
    const bool fold = s->round > 0;
    const int src_which = s->current;
    const int dst_which = fold ? (src_which == 1 ? 2 : 1) : src_which;
    size_t pairs = table_len(s->num_vars - s->round - 1);
    FrPtrList src{}, rd{};
    FrMutPtrList dst{};
    for (int f = 0; f < d.factor_count; f++) {
        src.p[f] = state_table(s, src_which, f);
        dst.p[f] = const_cast<Fr *>(state_table(s, dst_which, f));
        rd.p[f] = fold ? dst.p[f] : src.p[f];
    }
    const bool regs = d.max_arity <= 8 && d.slot_count <= kMaxSlotsV2;
    if (regs && pairs <= size_t(kSmallPairs)) {
        int tok = ctx->prof_begin("sumcheck_round", st);
        const size_t smem = size_t(d.slot_count) * (kSmallPairs + 1) * sizeof(Fr);
        auto launch = [&](auto kernel) {
            if (smem > 32 * 1024)
                check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
            kernel<<<1, kSmallThreads, smem, st>>>(d, src, dst, rd, fold, r, int(pairs),
                                                   static_cast<const Fr *>(s->coefs), int(s->max_degree), out_dev);
        };
        if (d.max_arity <= 2) launch(k_sumcheck_round_small<2>);
        else if (d.max_arity <= 4) launch(k_sumcheck_round_small<4>);
        else if (d.max_arity <= 6) launch(k_sumcheck_round_small<6>);
        else launch(k_sumcheck_round_small<8>);
        check_launch();
        ctx->prof_end(tok, st);
        return;
    }
    unsigned grid;
    Scratch partials, sums(ctx, d.slot_count * sizeof(Fr), st);
    int tok = ctx->prof_begin("sumcheck_round", st);
    if (regs) {
        grid = grid_for(ctx, pairs, kRoundThreads, HP_ROUND_BLOCKS_PER_SM);
        partials = Scratch(ctx, size_t(grid) * d.slot_count * sizeof(Fr), st);
        const size_t smem = size_t(d.slot_count) * kRoundThreads * sizeof(Fr);
        auto launch = [&](auto kernel) {
            // the kernel's own static shared memory counts against the same
            // 48 KiB default, so opt in well before the dynamic size reaches it
            if (smem > 32 * 1024)
                check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
            kernel<<<grid, kRoundThreads, smem, st>>>(d, src, dst, rd, fold, r, pairs, partials.as<Fr>(),
                                                      round_counter(s), static_cast<const Fr *>(s->coefs),
                                                      int(s->max_degree), out_dev);
        };
        if (d.max_arity <= 2) launch(k_sumcheck_round_regs<2>);
        else if (d.max_arity <= 4) launch(k_sumcheck_round_regs<4>);
        else if (d.max_arity <= 6) launch(k_sumcheck_round_regs<6>);
        else launch(k_sumcheck_round_regs<8>);
        check_launch();
        ctx->prof_end(tok, st);
        return;
    } else {
        size_t smem;
        int T = round_block_size(d, &smem);
        if (smem > 48 * 1024)
            check_cuda(cudaFuncSetAttribute(k_sumcheck_round, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            int(smem)));
        grid = grid_for(ctx, pairs, unsigned(T), 2);
        partials = Scratch(ctx, size_t(grid) * d.slot_count * sizeof(Fr), st);
        k_sumcheck_round<<<grid, T, smem, st>>>(d, src, dst, fold, r, pairs, partials.as<Fr>());
        check_launch();
    }
    ctx->prof_end(tok, st);
    k_sumcheck_finalize<<<1, 256, size_t(d.slot_count) * sizeof(Fr), st>>>(d, partials.as<Fr>(), int(grid),
                                                           static_cast<const Fr *>(s->coefs), int(s->max_degree),
                                                           sums.as<Fr>(), out_dev);
    check_launch();
}

static void advance(HpCudaSumCheckProverState *s) {
    if (s->round > 0) s->current = s->current == 1 ? 2 : 1;
    s->round++;
}

}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_sumcheck_prover_state_round(HpCudaContext *ctx,
                                                               HpCudaSumCheckProverState *s,
                                                               const uint8_t *challenge_or_null,
                                                               uint8_t *out_evaluations,
                                                               size_t evaluation_count) {
    return guard([&] {
        hp::require_ctx(ctx);
        hp::check_round(s, challenge_or_null, out_evaluations, evaluation_count);
        Fr r = Fr::zero();
        if (challenge_or_null) r = hp::host_scalar(challenge_or_null);
        try {
            hp::Scratch outd(ctx, evaluation_count * sizeof(Fr));
            hp::enqueue_round(ctx, s, r, ctx->stream, outd.as<Fr>());
            check_cuda(cudaMemcpyAsync(out_evaluations, outd.ptr, evaluation_count * sizeof(Fr),
                                       cudaMemcpyDeviceToHost, ctx->stream));
            ctx->sync();
            hp::advance(s);
        } catch (const hp::Failure &f) {
            if (f.kind == HP_CUDA_STATUS_INVALID_STATE) s->poisoned = true;
            throw;
        }
    });
}

extern "C" HpCudaStatus hp_cuda_v1_batch_sumcheck_round(HpCudaContext *ctx, HpCudaSumCheckProverState *const *states,
                                                        const uint8_t *const *challenges_or_null,
                                                        uint8_t *const *out_evaluations,
                                                        const size_t *evaluation_counts, size_t count) {
    return guard([&] {
        hp::require_ctx(ctx);
        if (count == 0) return;
        require(states != nullptr && challenges_or_null != nullptr && out_evaluations != nullptr &&
                evaluation_counts != nullptr);
        std::vector<Fr> rs(count, Fr::zero());
        size_t total = 0;
        for (size_t i = 0; i < count; i++) {
            hp::check_round(states[i], challenges_or_null[i], out_evaluations[i], evaluation_counts[i]);
            for (size_t j = 0; j < i; j++) require(states[j] != states[i]);
            if (challenges_or_null[i]) rs[i] = hp::host_scalar(challenges_or_null[i]);
            total += evaluation_counts[i];
        }
        try {
            hp::Scratch outd(ctx, total * sizeof(Fr));
            std::vector<Fr> host_out(total);
            const int k = int(std::min<size_t>(count, HpCudaContext::kWorkers));
            ctx->fork(k);
            size_t off = 0;
            for (size_t i = 0; i < count; i++) {
                hp::enqueue_round(ctx, states[i], rs[i], ctx->workers[i % size_t(k)], outd.as<Fr>() + off);
                off += evaluation_counts[i];
            }
            ctx->join(k);
            check_cuda(cudaMemcpyAsync(host_out.data(), outd.ptr, total * sizeof(Fr), cudaMemcpyDeviceToHost,
                                       ctx->stream));
            ctx->sync();
            off = 0;
            for (size_t i = 0; i < count; i++) {
                std::memcpy(out_evaluations[i], host_out.data() + off, evaluation_counts[i] * sizeof(Fr));
                off += evaluation_counts[i];
                hp::advance(states[i]);
            }
        } catch (const hp::Failure &f) {
            if (f.kind == HP_CUDA_STATUS_INVALID_STATE)
                for (size_t i = 0; i < count; i++) states[i]->poisoned = true;
            throw;
        }
    });
}

extern "C" HpCudaStatus hp_cuda_v1_sumcheck_prover_state_final_evaluations(
    HpCudaContext *ctx, HpCudaSumCheckProverState *s, const uint8_t *challenge,
    uint8_t *out_evaluations, size_t factor_count) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(s != nullptr && challenge != nullptr && out_evaluations != nullptr);
        if (s->poisoned || s->round != s->num_vars) fail(HP_CUDA_STATUS_INVALID_STATE);
        require(factor_count == size_t(s->desc.factor_count));
        if (factor_count == 0) return;
        Fr r = hp::host_scalar(challenge);
        hp::FrPtrList tl{};
        for (int f = 0; f < s->desc.factor_count; f++) tl.p[f] = hp::state_table(s, s->current, f);
        hp::Scratch outd(ctx, factor_count * sizeof(Fr));
        hp::k_sumcheck_final_fold<<<1, 32, 0, ctx->stream>>>(tl, int(factor_count), r,
                                                             outd.as<Fr>());
        check_launch();
        check_cuda(cudaMemcpyAsync(out_evaluations, outd.ptr, factor_count * sizeof(Fr),
                                   cudaMemcpyDeviceToHost, ctx->stream));
        ctx->sync();
    });
}

extern "C" HpCudaStatus hp_cuda_v1_sumcheck_prove_rounds(HpCudaContext *ctx, HpCudaSumCheckProverState *s,
                                                         HpMerlinTranscript *transcript, size_t rounds,
                                                         uint8_t *out_messages, uint8_t *out_challenges) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(s != nullptr && transcript != nullptr && out_messages != nullptr && out_challenges != nullptr);
        if (s->poisoned || s->round != 0) fail(HP_CUDA_STATUS_INVALID_STATE);
        require(rounds == s->num_vars);
        const size_t d1 = s->max_degree + 1;
        hp::Scratch outd(ctx, d1 * sizeof(Fr));
        // "prover msg" payload: u64 LE element count, then the canonical elements
        std::vector<uint8_t> msg(8 + 32 * d1, 0);
        for (int b = 0; b < 8; b++) msg[b] = uint8_t(uint64_t(d1) >> (8 * b));
        Fr r = Fr::zero();
        for (size_t k = 0; k < rounds; k++) {
            try {
                hp::enqueue_round(ctx, s, r, ctx->stream, outd.as<Fr>());
                check_cuda(cudaMemcpyAsync(msg.data() + 8, outd.ptr, 32 * d1, cudaMemcpyDeviceToHost, ctx->stream));
                ctx->sync();
                hp::advance(s);
            } catch (const hp::Failure &f) {
                if (f.kind == HP_CUDA_STATUS_INVALID_STATE) s->poisoned = true;
                throw;
            }
            std::memcpy(out_messages + 32 * d1 * k, msg.data() + 8, 32 * d1);
            hp::merlin_append(transcript, "prover msg", msg.data(), msg.size());
            // challenge: 64 transcript bytes reduced mod r, re-appended canonically
            uint8_t wide[64], canon[32];
            hp::merlin_challenge(transcript, "Internal round", wide, 64);
            const hp::host::Fr64 c = hp::host::from_wide64(wide);
            hp::host::to_canonical(c, canon);
            hp::merlin_append(transcript, "Internal round", canon, 32);
            std::memcpy(out_challenges + 32 * k, canon, 32);
            std::memcpy(r.v, c.v, 32);
        }
    });
}

extern "C" HpCudaStatus hp_cuda_v1_sumcheck_prover_state_destroy(HpCudaContext *ctx,
                                                                 HpCudaSumCheckProverState *s) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(s != nullptr);
        hp::release_state(ctx, s);
        delete s;
    });
}
