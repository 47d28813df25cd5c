// sumcheck.cu -- SumCheck prover state and the fused fold + round-message
// kernels.
//
// Reference semantics: backend/src/cpu/sum_check.rs:35-217.  Round k (1-based)
// first fixes the lowest variable of every distinct factor with the previous
// challenge (ark-poly fix_variables: f'[b] = f[2b] + r*(f[2b+1] - f[2b])),
// then for every product of arity m evaluates
//     s(t) = sum_b prod_j (f_j[2b] + t*(f_j[2b+1] - f_j[2b]))   for t = 0..m,
// scales by the product coefficient and extends the degree-m polynomial to
// t = 0..max_degree.  The reference extends with barycentric weights; this
// backend applies a per-state matrix of coefficient-scaled Lagrange weights
// over the integer nodes to the slot sums, which yields the same field
// elements (the degree-m interpolant is unique).
//
// GB300 shape: one launch per round fuses the fold of round k-1's challenge
// with the message of round k, so each factor table is read once and its
// folded half written once per round, and the last block of the launch sums
// the block partials, extrapolates, scales and writes canonical bytes.
// Rounds of more than 64 pairs: one (slot, pair) item per thread, so the
// latency chain per thread is one product, not the whole polynomial (large
// rounds after an elementwise fold of every table; smaller ones with the fold
// fused).  Rounds of <= 64 pairs: one block over (factor, pair) and
// (product, pair) items.  Products of any arity up to the degree bound and
// any slot count go through the (slot, pair) kernel; the per-pair kernel
// with per-thread slot sums in shared memory remains for HP_BIG_SLOTS=0.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
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

__device__ void finalize_from_sums(const SumcheckDesc &desc, const Fr *sums, const Fr *weights, int degree,
                                   Fr *out, const Fr *claim);

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
                                                           int per_slot, unsigned *counter, const Fr *weights,
                                                           int degree, Fr *out, Fr *sums, const Fr *claim) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    const int S = desc.slot_count;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    for (int s = warp; s < S; s += warps) {
        Fr a = Fr::zero();
        for (int b = lane; b < per_slot; b += 32) a = a + load_fr_cg(&partials[size_t(s) * per_slot + b]);
        a = warp_sum(a);
        if (lane == 0) sums[s] = a;
    }
    __syncthreads();
    finalize_from_sums(desc, sums, weights, degree, out, claim);
    if (threadIdx.x == 0) *counter = 0u;
}

template <int MAXM>
__global__ void __launch_bounds__(kRoundThreads) k_sumcheck_round_regs(SumcheckDesc desc, FrPtrList src,
                                                                       FrMutPtrList dst, FrPtrList rd, bool fold,
                                                                       Fr r, size_t pairs, Fr *partials,
                                                                       unsigned *counter, const Fr *weights,
                                                                       int degree, Fr *out, Fr claim,
                                                                       bool use_claim) {
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
            const int n0 = desc.node0[p];
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
                if (k < n0) continue;
                Fr v = e[0];
#pragma unroll
                for (int j = 1; j < MAXM; j++)
                    if (j < m) v = v * e[j];
                Fr &a = acc[(slot + k - n0) * kRoundThreads + t];
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
    finish_round_in_last_block(desc, partials, int(gridDim.x), counter, weights, degree, out, acc,
                               use_claim ? &claim : nullptr);
}

// dst_f[i] = src_f[2i] + r (src_f[2i+1] - src_f[2i]) for the `count` factor
// tables, i < 2^log_half: the fold of a large round, ahead of the (slot, pair)
// kernel below (elementwise, so every pass is coalesced and HBM-bound).
__global__ void __launch_bounds__(256) k_sumcheck_fold(FrPtrList src, FrMutPtrList dst, int count, int log_half,
                                                       Fr r) {
    const size_t half = size_t(1) << log_half, total = size_t(count) << log_half;
    for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
         idx += size_t(gridDim.x) * blockDim.x) {
        const int f = int(idx >> log_half);
        const size_t i = idx & (half - 1);
        const Fr *q = src.p[f] + 2 * i;
        const Fr a0 = load_fr(q), a1 = load_fr(q + 1);
        store_fr(dst.p[f] + i, a0 + r * (a1 - a0));
    }
}

// One thread per (slot, pair) item, slot = (product p, node t), products of
// any arity (MAXM = the largest, unrolled; 0: a runtime loop): the thread
// steps the m factors of p to t at its pair and multiplies them, a chain of
// m - 1 products with the last one accumulated unreduced -- no per-thread
// slot table, so occupancy is set by registers alone.  Block = kWideThreads
// pairs of one slot; blocks interleave slots (block b: slot b % S) so that
// resident blocks share their pairs' factor rows in L2.  Each block covers
// pairs blk*T + t + i*bps*T (bps = blocks per slot); one partial per block,
// slot-major; the last block finishes the round.
//   fold = true (rounds of up to a few thousand pairs): the thread folds its
// factors from `src` with r itself (a factor is re-folded once per slot
// that reads it: cheap at these sizes, and it saves a launch); the item at a
// factor's first occurrence (desc.writer) and t = 0 stores the folded pair,
// so every folded table is written exactly once.
//   fold = false: `src` holds this round's tables (the inputs in round 1,
// else the k_sumcheck_fold output).
constexpr int kWideThreads = 128;
static_assert(kMaxFactors == kMaxList, "one writer entry per factor pointer");

// (HP_WIDE_MINBLOCKS: a minimum-blocks-per-SM bound, a tuning hook; none by
// default, ~80 registers, 6 blocks per SM)
#ifdef HP_WIDE_MINBLOCKS
#define HP_WIDE_BOUNDS __launch_bounds__(kWideThreads, HP_WIDE_MINBLOCKS)
#else
#define HP_WIDE_BOUNDS __launch_bounds__(kWideThreads)
#endif

// e = lo + k (hi - lo) = hi + (k - 1)(hi - lo), then the slot value's
// running product v (factor j of m), the last factor into the accumulator
__device__ __forceinline__ void slot_step(FrAcc &X, Fr &v, const Fr &lo, const Fr &hi, int j, int m, int k) {
    Fr e = k == 0 ? lo : hi;
    if (k >= 2) {
        const Fr step = hi - lo;
        for (int i = 1; i < k; i++) e = e + step;
    }
    if (j == m - 1) {
        if (m == 1) acc_add_shifted(X, e);
        else acc_mul_add(X, v, e);
    } else {
        v = j == 0 ? e : v * e;
    }
}

template <int MAXM>
__global__ void HP_WIDE_BOUNDS k_sumcheck_round_wide(SumcheckDesc desc, FrPtrList src, FrMutPtrList dst, bool fold,
                                                     Fr r, size_t pairs, int blocks_per_slot, Fr *partials,
                                                     unsigned *counter, const Fr *weights, int degree, Fr *out,
                                                     Fr claim, bool use_claim) {
    extern __shared__ Fr sums[];  // S slot sums, used by the last block
    __shared__ Fr wsum[kWideThreads / 32];
    const int S = desc.slot_count;
    const int s = int(blockIdx.x % unsigned(S)), blk = int(blockIdx.x / unsigned(S));
    int p = 0;
    while (p + 1 < desc.product_count && desc.slot_base[p + 1] <= s) p++;
    const int begin = desc.offsets[p], m = desc.offsets[p + 1] - begin, k = s - desc.slot_base[p] + desc.node0[p];
    FrAcc X;
    acc_zero(X);
    const size_t stride = size_t(blocks_per_slot) * kWideThreads;
    for (size_t b = size_t(blk) * kWideThreads + threadIdx.x; b < pairs; b += stride) {
        Fr v;
        auto factor = [&](int j) {
            const int f = desc.indices[begin + j];
            Fr lo, hi;
            if (fold) {
                const Fr *q = src.p[f] + 4 * b;
                const Fr a0 = load_fr(q), a1 = load_fr(q + 1), a2 = load_fr(q + 2), a3 = load_fr(q + 3);
                lo = a0 + r * (a1 - a0);
                hi = a2 + r * (a3 - a2);
                if (k == desc.node0[p] && desc.writer[f] == begin + j) {  // the product's first slot
                    Fr *d = dst.p[f] + 2 * b;
                    store_fr(d, lo);
                    store_fr(d + 1, hi);
                }
            } else {
                const Fr *q = src.p[f] + 2 * b;
                lo = load_fr(q);
                hi = load_fr(q + 1);
            }
            slot_step(X, v, lo, hi, j, m, k);
        };
        if constexpr (MAXM > 0) {
#pragma unroll
            for (int j = 0; j < MAXM; j++)
                if (j < m) factor(j);
        } else {
            for (int j = 0; j < m; j++) factor(j);
        }
    }
    Fr a = acc_reduce(X);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    a = warp_sum(a);
    if (lane == 0) wsum[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        Fr t = wsum[0];
#pragma unroll
        for (int w = 1; w < kWideThreads / 32; w++) t = t + wsum[w];
        partials[size_t(s) * blocks_per_slot + blk] = t;
    }
    finish_round_in_last_block(desc, partials, blocks_per_slot, counter, weights, degree, out, sums,
                               use_claim ? &claim : nullptr);
}

// Zero-check rounds.  A state whose products all contain one factor exactly
// once, that factor an eq table eq(x, r) built by hp_cuda_v1_mle_build_eq_x_r
// (the context records its point; tables are immutable), has round
// polynomials p(t) = eq1(t; r_i) Q(t): with the challenges c_0..c_{i-1}
// folded in, the eq table's pair b is (a_b (1 - r_i), a_b r_i) with
// a_b = prod_{j<i} eq1(c_j; r_j) eq(b; r_{i+1..}), so its pair sum
// w_b = eq[2b] + eq[2b+1] is a_b and
//     Q(t) = sum_b w_b g_b(t),
// g the polynomial with that factor removed from every product (degree
// d - 1).  Q needs d nodes instead of p's d + 1, and every product one
// multiplication fewer per node (the round split of A. Gruen, "Some
// improvements for the PIOP for ZeroCheck", IACR ePrint 2024, here read
// off the folded eq table).  From round 2 on the claim
// p(0) + p(1) = (1 - r_i) Q(0) + r_i Q(1) gives Q(0) = u + v Q(1) (u =
// claim / (1 - r_i), v = -r_i / (1 - r_i), host-computed; not when r_i = 1).
// The message is the same field elements as the generic kernels': p(x) =
// (a + b x) Q(x) at x = 0..d, a = 1 - r_i, b = 2 r_i - 1, Q(x) from its
// nodes by fixed Lagrange weights.  Items are (node, pair) as in the (slot,
// pair) kernel; each evaluates every product at its node and accumulates
// w_b g_b(t) unreduced; the last block finishes the round.
struct EqRoundDesc {
    int product_count;
    int eq_factor;
    uint16_t offsets[kMaxProducts + 1];  // the products without the eq factor, into indices
    uint8_t indices[kMaxIndices];
    uint8_t coef_kind[kMaxProducts];  // 0: c = 1, 1: c = -1, 2: c = coefs[p]
};

// (HP_EQ_MINBLOCKS: a minimum-blocks-per-SM bound, a tuning hook; none by
// default, ~89 registers, 5 blocks per SM)
#ifdef HP_EQ_MINBLOCKS
#define HP_EQ_BOUNDS __launch_bounds__(kWideThreads, HP_EQ_MINBLOCKS)
#else
#define HP_EQ_BOUNDS __launch_bounds__(kWideThreads)
#endif

template <int MAXR>
__global__ void HP_EQ_BOUNDS k_sumcheck_round_eq(EqRoundDesc ed, FrPtrList tables, size_t pairs, int node0,
                                                   int nodes, int blocks_per_node, const Fr *coefs, Fr *partials,
                                                   unsigned *counter, const Fr *lag, int degree, Fr a, Fr b, Fr u,
                                                   Fr v, Fr *out) {
    __shared__ Fr wsum[kWideThreads / 32];
    __shared__ Fr q[kMaxDegree + 1];
    __shared__ bool last;
    const int ni = int(blockIdx.x % unsigned(nodes)), blk = int(blockIdx.x / unsigned(nodes));
    const int k = node0 + ni;
    const Fr one = Fr::one();
    const Fr *eqt = tables.p[ed.eq_factor];
    FrAcc X;
    acc_zero(X);
    const size_t stride = size_t(blocks_per_node) * kWideThreads;
    for (size_t pb = size_t(blk) * kWideThreads + threadIdx.x; pb < pairs; pb += stride) {
        const Fr w = load_fr(eqt + 2 * pb) + load_fr(eqt + 2 * pb + 1);
        Fr g = Fr::zero();
        for (int p = 0; p < ed.product_count; p++) {
            const int begin = ed.offsets[p], m = ed.offsets[p + 1] - begin;
            Fr val = one;
            auto factor = [&](int j) {
                const Fr *t = tables.p[ed.indices[begin + j]] + 2 * pb;
                const Fr lo = load_fr(t), hi = load_fr(t + 1);
                Fr e = k == 0 ? lo : hi;
                if (k >= 2) {
                    const Fr step = hi - lo;
                    for (int i = 1; i < k; i++) e = e + step;
                }
                val = j == 0 ? e : val * e;
            };
            if constexpr (MAXR > 0) {
#pragma unroll
                for (int j = 0; j < MAXR; j++)
                    if (j < m) factor(j);
            } else {
                for (int j = 0; j < m; j++) factor(j);
            }
            const int kind = ed.coef_kind[p];
            if (kind == 0) g = g + val;
            else if (kind == 1) g = g - val;
            else g = g + val * coefs[p];
        }
        acc_mul_add(X, w, g);
    }
    Fr s = acc_reduce(X);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s = warp_sum(s);
    if (lane == 0) wsum[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        Fr t = wsum[0];
#pragma unroll
        for (int w2 = 1; w2 < kWideThreads / 32; w2++) t = t + wsum[w2];
        partials[size_t(ni) * blocks_per_node + blk] = t;
    }
    // the last block to finish sums the partials of every node and writes p
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    for (int n = warp; n < nodes; n += kWideThreads / 32) {
        Fr t = Fr::zero();
        for (int j = lane; j < blocks_per_node; j += 32) t = t + load_fr_cg(&partials[size_t(n) * blocks_per_node + j]);
        t = warp_sum(t);
        if (lane == 0) q[node0 + n] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0 && node0 == 1) q[0] = u + v * q[1];
    __syncthreads();
    for (int x = threadIdx.x; x <= degree; x += blockDim.x) {
        Fr qx = Fr::zero();
        for (int j = 0; j < degree; j++) qx = qx + lag[size_t(x) * degree + j] * q[j];
        Fr ex = a;
        for (int i = 0; i < x; i++) ex = ex + b;
        out[x] = from_mont(ex * qx);
    }
    if (threadIdx.x == 0) *counter = 0u;
}

// One thread per (product, pair) item, for the large rounds (more than
// wide_max_pairs() pairs) of products of arity <= 3: the thread loads its
// product's m factor rows at its pair once and evaluates all m + 1 slot
// values of the product (t = 0..m) from those registers.  Per pair, 2m Fr
// loads feed m + 1 products of m factors, where a (slot, pair) item loads 2m
// Fr for one.  With `fold` the thread folds its factors with r on the way
// (the item at a factor's first occurrence, desc.writer, stores the folded
// pair, so every folded table is written exactly once); that form re-folds a
// factor once per product reading it and stays opt-in (HP_SUMCHECK_PP_FOLD):
// by default the separate fold pass runs first.  Products of arity <= 2 keep
// their slot sums unreduced (17-limb accumulators, one Montgomery reduction
// per thread at the end); arity 3 keeps reduced sums.  Blocks interleave
// products (block b: product b % P) so that products sharing a factor read
// its rows from L2.  One partial per (slot, block), slot-major; the last
// block finishes the round.  Measured on GB300 (degree-2 sumcheck, 6 tables
// of 2^20, round 1): 138 us against 161 us for the (slot, pair) kernel; the
// middle rounds stay with the (slot, pair) kernel, whose shorter per-thread
// chains hide latency better at a few thousand pairs.
constexpr int kPpThreads = 128;
constexpr int kPpBlocksPerSm = HP_ROUND_BLOCKS_PER_SM;

// (HP_PP_MINBLOCKS: a minimum-blocks-per-SM bound, a tuning hook)
#ifdef HP_PP_MINBLOCKS
#define HP_PP_BOUNDS __launch_bounds__(kPpThreads, HP_PP_MINBLOCKS)
#else
#define HP_PP_BOUNDS __launch_bounds__(kPpThreads)
#endif

// kNode0: the first node of every product (SumcheckDesc::node0, the same for
// all products of the launch's layout: 0 in the first round, 1 in later
// rounds when every product's arity is the degree), a compile-time constant
// so that the node loop keeps its fixed shape (a per-product run-time node
// measured 100 us against 82 us for the full 12-slot form at 2^18 pairs).
template <int MAXM, int kNode0>
__global__ void HP_PP_BOUNDS k_sumcheck_round_pp(SumcheckDesc desc, FrPtrList src, FrMutPtrList dst,
                                                                  bool fold, Fr r, size_t pairs,
                                                                  int blocks_per_product, Fr *partials,
                                                                  unsigned *counter, const Fr *weights, int degree,
                                                                  Fr *out, Fr claim, bool use_claim) {
    constexpr bool kUnreduced = MAXM <= 2;
    extern __shared__ Fr sums[];  // S slot sums, used by the last block
    __shared__ Fr wsum[kPpThreads / 32][MAXM + 1];
    const int P = desc.product_count;
    const int p = int(blockIdx.x % unsigned(P)), blk = int(blockIdx.x / unsigned(P));
    const int begin = desc.offsets[p], m = desc.offsets[p + 1] - begin, slot0 = desc.slot_base[p];
    constexpr int n0 = kNode0;  // slot slot0 holds node n0
    FrAcc X[kUnreduced ? MAXM + 1 : 1];
    Fr A[kUnreduced ? 1 : MAXM + 1];
#pragma unroll
    for (int t = 0; t <= MAXM; t++) {
        if constexpr (kUnreduced) acc_zero(X[t]);
        else A[t] = Fr::zero();
    }
    const size_t stride = size_t(blocks_per_product) * kPpThreads;
    for (size_t b = size_t(blk) * kPpThreads + threadIdx.x; b < pairs; b += stride) {
        Fr e[MAXM], st[MAXM];
#pragma unroll
        for (int j = 0; j < MAXM; j++) {
            if (j < m) {
                const int f = desc.indices[begin + j];
                Fr lo, hi;
                if (fold) {
                    const Fr *q = src.p[f] + 4 * b;
                    const Fr a0 = load_fr(q), a1 = load_fr(q + 1), a2 = load_fr(q + 2), a3 = load_fr(q + 3);
                    lo = a0 + r * (a1 - a0);
                    hi = a2 + r * (a3 - a2);
                    if (desc.writer[f] == begin + j) {
                        Fr *d = dst.p[f] + 2 * b;
                        store_fr(d, lo);
                        store_fr(d + 1, hi);
                    }
                } else {
                    const Fr *q = src.p[f] + 2 * b;
                    lo = load_fr(q);
                    hi = load_fr(q + 1);
                }
                e[j] = lo;
                st[j] = hi - lo;
            }
        }
#pragma unroll
        for (int t = 0; t <= MAXM; t++) {
            if (t <= m) {
                if (t > 0) {
#pragma unroll
                    for (int j = 0; j < MAXM; j++)
                        if (j < m) e[j] = e[j] + st[j];  // factor j at node t
                }
                if (t < n0) continue;
                Fr v;
#pragma unroll
                for (int j = 0; j < MAXM; j++) {
                    if (j + 1 < m) {
                        v = j == 0 ? e[0] : v * e[j];
                    } else if (j + 1 == m) {  // the last factor goes into the slot sum
                        if constexpr (kUnreduced) {
                            if (j == 0) acc_add_shifted(X[t], e[0]);
                            else acc_mul_add(X[t], v, e[j]);
                        } else {
                            A[t] = A[t] + (j == 0 ? e[0] : v * e[j]);
                        }
                    }
                }
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t <= MAXM; t++) {
        if (t <= m && t >= n0) {
            Fr a;
            if constexpr (kUnreduced) a = acc_reduce(X[t]);
            else a = A[t];
            a = warp_sum(a);
            if (lane == 0) wsum[warp][t] = a;
        }
    }
    __syncthreads();
    if (int(threadIdx.x) <= m && int(threadIdx.x) >= n0) {
        const int t = threadIdx.x;
        Fr a = wsum[0][t];
#pragma unroll
        for (int w = 1; w < kPpThreads / 32; w++) a = a + wsum[w][t];
        partials[size_t(slot0 + t - n0) * blocks_per_product + blk] = a;
    }
    finish_round_in_last_block(desc, partials, blocks_per_product, counter, weights, degree, out, sums,
                               use_claim ? &claim : nullptr);
}

// Given the slot sums (Montgomery, shared memory) of a round, writes the d+1
// canonical round evaluations out[x] = sum_s W[x][s] * sums[s], one warp per
// x.  W (per prover state, built on the host) holds for slot
// s = slot_base[p] + i the product coefficient times the Lagrange basis
// polynomial l_i of the nodes 0..m (m = arity of p) at x: the slot sums are
// the product's values at t = 0..m, so the row is the unique polynomial of
// degree <= m through them -- equal to the slot sum for x <= m and to the
// reference's barycentric extrapolation (backend/src/cpu/sum_check.rs:183-217)
// beyond -- scaled and summed over products.
__device__ void finalize_from_sums(const SumcheckDesc &desc, const Fr *sums, const Fr *weights, int degree,
                                   Fr *out, const Fr *claim) {
    const int S = desc.slot_count;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    for (int x = warp; x <= degree; x += warps) {
        Fr a = Fr::zero();
        for (int s = lane; s < S; s += 32) a = a + weights[size_t(x) * S + s] * sums[s];
        a = warp_sum(a);
        // with a claim, row 0 of W is minus row 1: p(0) = claim - p(1)
        if (lane == 0) out[x] = from_mont(x == 0 && claim != nullptr ? a + *claim : a);
    }
}

// A round of at most kSmallPairs pairs in one block, finalize included (the
// last rounds of every sumcheck: latency-bound, so the work is spread over
// (factor, pair) and (product, pair) items instead of one pair per thread).
constexpr int kSmallPairs = 64;
constexpr int kSmallThreads = 256;

template <int MAXM>
__global__ void __launch_bounds__(kSmallThreads) k_sumcheck_round_small(SumcheckDesc desc, FrPtrList src,
                                                                        FrMutPtrList dst, FrPtrList rd, bool fold,
                                                                        Fr r, int pairs, const Fr *weights,
                                                                        int degree, Fr *out, Fr claim,
                                                                        bool use_claim) {
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
        const int n0 = desc.node0[p];
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
            if (k < n0) continue;
            Fr v = e[0];
#pragma unroll
            for (int j = 1; j < MAXM; j++)
                if (j < m) v = v * e[j];
            vals[(slot + k - n0) * kSmallPairs + b] = v;
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
    finalize_from_sums(desc, sums, weights, degree, out, use_claim ? &claim : nullptr);
}

// Host handshake of the resident rounds (the one-block tail below and the
// cooperative grid after it), in pinned, device-mapped host memory: hdr[0]
// counts the messages written (device), hdr[1] the challenges written (host),
// hdr[2] is set when a block gave up waiting for a challenge; `challenges`
// holds one Montgomery challenge per resident round but the last (host
// writes), `messages` (degree + 1) canonical evaluations per round (device
// writes), `claims` the claim p_prev(r_prev) of every resident round after
// the first (Montgomery, written with the previous round's challenge), and
// `messages` (degree + 1) canonical evaluations per round (device writes).
// A block waits for challenge j with at most kTailSpinLimit polls.
struct Handshake {
    uint32_t *hdr;
    Fr *challenges;
    Fr *claims;
    Fr *messages;
};
constexpr uint32_t kTailSpinLimit = 1u << 22;  // polls of host memory (~1 us each): gives up after seconds
constexpr uint32_t kRelaySpinLimit = 1u << 24;  // polls of the device relay (>= 256 ns each)

__device__ __forceinline__ uint32_t load_acquire_sys(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.sys.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void store_release_sys(uint32_t *p, uint32_t v) {
    asm volatile("st.release.sys.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t load_acquire_gpu(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void store_release_gpu(uint32_t *p, uint32_t v) {
    asm volatile("st.release.gpu.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 of a block, after a barrier that follows every thread's writes of
// message j: one system-scope fence (cumulative over the writes the barrier
// ordered before it), then the release of the message count.
__device__ __forceinline__ void release_message(const Handshake &hs, int j) {
    __threadfence_system();
    store_release_sys(&hs.hdr[0], uint32_t(j + 1));
}

// Thread 0 of a block: waits (bounded) until the host has written challenge
// j, copies it to *out and the claim of round j + 1 to *claim; false when the
// wait ran out (hdr[2] is then set).
__device__ __forceinline__ bool wait_host_challenge(const Handshake &hs, int j, Fr *out, Fr *claim) {
    uint32_t it = 0;
    while (load_acquire_sys(&hs.hdr[1]) < uint32_t(j + 1) && ++it < kTailSpinLimit) __nanosleep(32);
    if (it >= kTailSpinLimit) {
        store_release_sys(&hs.hdr[2], 1u);
        return false;
    }
    const volatile uint32_t *c = reinterpret_cast<const volatile uint32_t *>(&hs.challenges[j]);
    const volatile uint32_t *q = reinterpret_cast<const volatile uint32_t *>(&hs.claims[j + 1]);
#pragma unroll
    for (int w = 0; w < 8; w++) {
        out->v[w] = c[w];
        claim->v[w] = q[w];
    }
    return true;
}

// The last rounds of a sumcheck (at most tail_pairs() pairs) in one launch
// of one block that stays resident between rounds: the factor tables live in
// shared memory, each round's message goes to the handshake followed by a
// release of its sequence number, and the block waits for the host's
// challenge before folding it in and running the next round.  This removes
// a launch and a stream synchronisation per round from
// hp_cuda_v1_sumcheck_prove_rounds, whose host side polls the mapped
// sequence numbers instead; the messages are the same field elements as the
// one-launch-per-round path's (same node sums, same weight matrix).
constexpr int kTailThreads = 256;
constexpr int kTailMaxPairs = 256;  // at most 9 rounds

template <int MAXM>
__global__ void __launch_bounds__(kTailThreads) k_sumcheck_tail(SumcheckDesc desc, FrPtrList src, FrMutPtrList dst,
                                                                bool fold_first, Fr r0, int pairs0, int rounds,
                                                                const Fr *weights, int degree, Fr claim0,
                                                                Handshake hs) {
    extern __shared__ Fr tsm[];
    __shared__ int abort_round;
    __shared__ Fr challenge, claim;
    const int F = desc.factor_count, S = desc.slot_count, P = desc.product_count;
    const int row = 2 * pairs0;                     // table row stride
    Fr *tab = tsm;                                  // F x 2 pairs0
    Fr *tmp = tab + size_t(F) * row;                // F x pairs0 (fold staging)
    Fr *vals = tmp + size_t(F) * pairs0;            // S x pairs0
    Fr *sums = vals + size_t(S) * pairs0;           // S
    int pairs = pairs0;
    for (int idx = threadIdx.x; idx < F * 2 * pairs; idx += blockDim.x) {
        const int f = idx / (2 * pairs), e = idx - f * 2 * pairs;
        Fr v;
        if (fold_first) {
            const Fr a0 = load_fr(src.p[f] + 2 * e), a1 = load_fr(src.p[f] + 2 * e + 1);
            v = a0 + r0 * (a1 - a0);
        } else {
            v = load_fr(src.p[f] + e);
        }
        tab[f * row + e] = v;
    }
    if (threadIdx.x == 0) claim = claim0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    for (int j = 0; j < rounds; j++) {
        for (int idx = threadIdx.x; idx < P * pairs; idx += blockDim.x) {
            const int p = idx / pairs, b = idx - p * pairs;
            const int begin = desc.offsets[p], m = desc.offsets[p + 1] - begin, slot = desc.slot_base[p];
            const int n0 = desc.node0[p];
            Fr e[MAXM], st[MAXM];
#pragma unroll
            for (int q = 0; q < MAXM; q++) {
                if (q < m) {
                    const Fr *t = tab + desc.indices[begin + q] * row + 2 * b;
                    e[q] = t[0];
                    st[q] = t[1] - e[q];
                }
            }
            for (int k = 0; k <= m; k++) {
                if (k > 0) {
#pragma unroll
                    for (int q = 0; q < MAXM; q++)
                        if (q < m) e[q] = e[q] + st[q];
                }
                if (k < n0) continue;
                Fr v = e[0];
#pragma unroll
                for (int q = 1; q < MAXM; q++)
                    if (q < m) v = v * e[q];
                vals[(slot + k - n0) * pairs0 + b] = v;
            }
        }
        __syncthreads();
        for (int sl = warp; sl < S; sl += warps) {
            Fr a = Fr::zero();
            for (int b = lane; b < pairs; b += 32) a = a + vals[sl * pairs0 + b];
            a = warp_sum(a);
            if (lane == 0) sums[sl] = a;
        }
        __syncthreads();
        finalize_from_sums(desc, sums, weights, degree, hs.messages + size_t(j) * (degree + 1), &claim);
        __syncthreads();
        if (threadIdx.x == 0) release_message(hs, j);
        if (j + 1 == rounds) break;
        if (threadIdx.x == 0) abort_round = !wait_host_challenge(hs, j, &challenge, &claim);
        __syncthreads();
        if (abort_round) return;
        const Fr r = challenge;
        for (int idx = threadIdx.x; idx < F * pairs; idx += blockDim.x) {
            const int f = idx / pairs, b = idx - f * pairs;
            const Fr lo = tab[f * row + 2 * b], hi = tab[f * row + 2 * b + 1];
            tmp[f * pairs0 + b] = lo + r * (hi - lo);
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < F * pairs; idx += blockDim.x) {
            const int f = idx / pairs, b = idx - f * pairs;
            tab[f * row + b] = tmp[f * pairs0 + b];
        }
        __syncthreads();
        pairs >>= 1;
    }
    // the state's tables after the last message (folded by every challenge but
    // the last, which final_evaluations folds in)
    for (int idx = threadIdx.x; idx < F * 2 * pairs; idx += blockDim.x) {
        const int f = idx / (2 * pairs), e = idx - f * 2 * pairs;
        store_fr(dst.p[f] + e, tab[f * row + e]);
    }
}

// The middle and last rounds of a sumcheck (from resident_pairs() pairs
// down) in one cooperative launch whose blocks stay resident between rounds.
// Round j (pairs_j = pairs0 >> j): the first `active` blocks (at least
// kResMinPairs pairs each; a block past that count returns, since ranges only
// shrink) each take a contiguous range of pairs and, tile by tile, fold the
// previous challenge into the factor rows of the range (reading the previous
// round's tables through L2, since other blocks wrote them; writing the
// folded rows to the state's next fold buffer and to shared memory), then
// accumulate their (slot, pair) items from shared memory with one thread
// group per slot (unreduced 17-limb sums).  Each block adds its slot sums
// limb by limb into 64-bit counters of the round (double-buffered by round
// parity, cleared by their reader); the last block to arrive (a counter
// ticket) reads them, writes the message into the handshake and releases its
// sequence number (a round of one active block skips the counters).  Block 0 then waits
// for the host's challenge and relays it through device memory (relay[0]:
// rounds relayed, relay[1]: abort, relay + 8: the challenge, relay + 16: the
// next round's claim) to the other
// blocks, which wait for it with a bounded spin as well.  Every round's
// writes precede its ticket, and the next round starts only after the host
// has answered that round's message, so a block can read rows that any other
// block wrote in the previous round.  The fold buffers follow the per-round
// path's ping-pong (inputs -> fold_a -> fold_b -> fold_a ...), so the state
// after the launch is the one the per-round calls leave.
constexpr int kResThreads = 256;
constexpr size_t kResMinPairs = 32;

// sum_i l[i] 2^(32 i) mod r: block partial sums (Montgomery values < r)
// accumulated limb by limb in 64-bit counters (at most 2^31 terms), carried
// into 256 bits plus a top word w (< 2^32), then reduced: the 256-bit part is
// < 3r (two conditional subtractions), and w 2^256 = to_mont(w) mod r.
__device__ Fr fr_from_limb_sums(const uint64_t *l) {
    Fr r;
    uint64_t c = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint64_t t = l[i] + c;
        r.v[i] = uint32_t(t);
        c = t >> 32;
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
        uint32_t u[8];
        u[0] = sub_cc(r.v[0], FrParams::p(0));
#pragma unroll
        for (int i = 1; i < 8; i++) u[i] = subc_cc(r.v[i], FrParams::p(i));
        const uint32_t borrow = subc(0, 0);
#pragma unroll
        for (int i = 0; i < 8; i++) r.v[i] = borrow ? r.v[i] : u[i];
    }
    Fr w = Fr::zero();
    w.v[0] = uint32_t(c);
    return r + to_mont(w);
}

struct FoldBuffers {
    FrPtrList inputs;
    Fr *a, *b;
    size_t a_stride, b_stride;
    __device__ __forceinline__ Fr *table(int which, int f) const {
        return which == 0 ? const_cast<Fr *>(inputs.p[f]) : which == 1 ? a + f * a_stride : b + f * b_stride;
    }
};

template <int MAXM>
__global__ void __launch_bounds__(kResThreads) k_sumcheck_resident(SumcheckDesc desc, FoldBuffers buf, int which0,
                                                                   bool fold_first, Fr r0, size_t pairs0,
                                                                   int rounds, int tile, const Fr *weights,
                                                                   int degree, Fr claim0, uint64_t *limb_sums,
                                                                   unsigned *counter, uint32_t *relay, Handshake hs) {
    extern __shared__ Fr rsm[];  // tile rows: F x 2 tile; then kResThreads reduced sums
    __shared__ Fr challenge, claim;
    __shared__ Fr sums[kMaxSlotsV2];
    __shared__ int stop;
    __shared__ bool last;
    const int F = desc.factor_count, S = desc.slot_count;
    const int row = 2 * tile;
    Fr *tab = rsm;
    Fr *red = rsm + size_t(F) * row;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = kResThreads / 32;
    // thread group of slot s: tps threads, each over pairs g, g + tps, ...
    const int tps = kResThreads / S;
    const int s = int(threadIdx.x) / tps, g = int(threadIdx.x) - s * tps;
    int begin = 0, m = 1, k = 0;
    if (s < S) {
        int p = 0;
        while (p + 1 < desc.product_count && desc.slot_base[p + 1] <= s) p++;
        begin = desc.offsets[p];
        m = desc.offsets[p + 1] - begin;
        k = s - desc.slot_base[p] + desc.node0[p];
    }
    if (threadIdx.x == 0) claim = claim0;
    int which = which0;
    bool fold = fold_first;
    Fr r = r0;
    for (int j = 0; j < rounds; j++) {
        const size_t pairs = pairs0 >> j;
        const unsigned active = unsigned(min(size_t(gridDim.x), (pairs + kResMinPairs - 1) / kResMinPairs));
        const size_t b0 = pairs * blockIdx.x / active, b1 = pairs * (blockIdx.x + 1) / active;
        const int dst = fold ? (which == 1 ? 2 : 1) : which;
        FrAcc X;
        acc_zero(X);
        for (size_t pb = b0; pb < b1; pb += size_t(tile)) {
            const int np = int(min(size_t(tile), b1 - pb));
            for (int idx = threadIdx.x; idx < F * 2 * np; idx += kResThreads) {
                const int f = idx / (2 * np), e = idx - f * 2 * np;
                const size_t ge = 2 * pb + size_t(e);
                Fr v;
                if (fold) {
                    const Fr *q = buf.table(which, f) + 2 * ge;
                    const Fr a0 = load_fr_cg(q), a1 = load_fr_cg(q + 1);
                    v = a0 + r * (a1 - a0);
                    store_fr(buf.table(dst, f) + ge, v);
                } else {
                    v = load_fr(buf.table(which, f) + ge);
                }
                tab[f * row + e] = v;
            }
            __syncthreads();
            if (s < S) {
                for (int b = g; b < np; b += tps) {
                    Fr v;
                    auto factor = [&](int q) {
                        const Fr *t = tab + desc.indices[begin + q] * row + 2 * b;
                        slot_step(X, v, t[0], t[1], q, m, k);
                    };
#pragma unroll
                    for (int q = 0; q < MAXM; q++)
                        if (q < m) factor(q);
                }
            }
            __syncthreads();
        }
        red[threadIdx.x] = s < S ? acc_reduce(X) : Fr::zero();
        __syncthreads();
        for (int sl = warp; sl < S; sl += warps) {
            Fr a = Fr::zero();
            for (int i = lane; i < tps; i += 32) a = a + red[sl * tps + i];
            a = warp_sum(a);
            if (lane == 0) sums[sl] = a;
        }
        __syncthreads();
        bool finish = active == 1;  // one block: its slot sums are the round's
        if (!finish) {
            // add the block's slot sums limb by limb into this round's 64-bit
            // counters, then the ticket: thread 0 fences once for the block
            // (cumulative over the additions the barrier ordered before it)
            uint64_t *acc = limb_sums + size_t(j & 1) * 8 * kMaxSlotsV2;
            for (int i = threadIdx.x; i < 8 * S; i += kResThreads)
                atomicAdd(reinterpret_cast<unsigned long long *>(&acc[i]),
                          (unsigned long long)sums[i >> 3].v[i & 7]);
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                last = atomicAdd(counter, 1u) == active - 1;
            }
            __syncthreads();
            if (last) {
                // read and clear the counters (their next use is two rounds on)
                uint64_t *lim = reinterpret_cast<uint64_t *>(red);
                for (int i = threadIdx.x; i < 8 * S; i += kResThreads)
                    lim[i] = atomicExch(reinterpret_cast<unsigned long long *>(&acc[i]), 0ull);
                __syncthreads();
                if (threadIdx.x < S) sums[threadIdx.x] = fr_from_limb_sums(lim + 8 * threadIdx.x);
                __syncthreads();
                finish = true;
            }
        }
        if (finish) {
            finalize_from_sums(desc, sums, weights, degree, hs.messages + size_t(j) * (degree + 1), &claim);
            __syncthreads();
            if (threadIdx.x == 0) {
                *counter = 0u;
                release_message(hs, j);
            }
        }
        if (j + 1 == rounds) break;
        const size_t next = pairs >> 1;
        if (blockIdx.x >= unsigned(min(size_t(gridDim.x), (next + kResMinPairs - 1) / kResMinPairs))) return;
        if (threadIdx.x == 0) {
            bool ok;
            if (blockIdx.x == 0) {
                ok = wait_host_challenge(hs, j, &challenge, &claim);
                if (ok) {
                    store_fr(reinterpret_cast<Fr *>(relay + 8), challenge);
                    store_fr(reinterpret_cast<Fr *>(relay + 16), claim);
                    store_release_gpu(&relay[0], uint32_t(j + 1));
                } else {
                    store_release_gpu(&relay[1], 1u);
                }
            } else {
                uint32_t it = 0;
                while (load_acquire_gpu(&relay[0]) < uint32_t(j + 1) && load_acquire_gpu(&relay[1]) == 0u &&
                       ++it < kRelaySpinLimit)
                    __nanosleep(256);
                ok = it < kRelaySpinLimit && load_acquire_gpu(&relay[0]) >= uint32_t(j + 1);
                if (ok) {
                    challenge = load_fr_cg(reinterpret_cast<const Fr *>(relay + 8));
                    claim = load_fr_cg(reinterpret_cast<const Fr *>(relay + 16));
                }
                else store_release_sys(&hs.hdr[2], 1u);
            }
            stop = ok ? 0 : 1;
        }
        __syncthreads();
        if (stop) return;
        r = challenge;
        which = dst;
        fold = true;
    }
}

// One round over shared-memory tiles staged by bulk asynchronous copies.
// Block b takes a contiguous range of pairs, in tiles of `tile` pairs: thread
// 0 issues, per factor, one cp.async.bulk of the tile's source rows (4 Fr per
// pair when the previous challenge is folded in, 2 otherwise) into one of
// kTileStages shared-memory stages, completing on that stage's mbarrier, up
// to kTileStages - 1 tiles ahead of the one being computed.  Each tile: the
// fold writes the folded rows to `dst` and to a shared tile (a factor folded
// once, whatever the number of products reading it), then one thread group
// per slot accumulates its (slot, pair) items from shared memory into an
// unreduced 17-limb sum.  Block slot sums go into the state's 64-bit limb
// counters; the last block (ticket) turns them into field elements, clears
// them and writes the message.  A stage wait that runs out (kTileWaitLimit
// polls) makes the block skip its remaining tiles, wait (bounded) for its
// copies still in flight and flag the launch; the last block then writes a
// message of non-canonical bytes, which the host rejects.
constexpr int kTileThreads = 256;
constexpr int kTileStages = 3;
constexpr uint32_t kTileWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    uint32_t it = 0;
    while (!mbar_try_wait(bar, parity))
        if (++it >= kTileWaitLimit) return false;
    return true;
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Shared memory of the tiled kernel: the barriers, kTileStages stages of raw
// rows, the folded tile, the per-thread reduced sums.
static size_t tiled_smem(int factors, int tile, bool fold) {
    const size_t row = fold ? 4 : 2;
    return 128 + (size_t(kTileStages) * factors * row * tile + size_t(factors) * 2 * tile + kTileThreads) * sizeof(Fr);
}

template <int MAXM>
__global__ void __launch_bounds__(kTileThreads) k_sumcheck_round_tiled(SumcheckDesc desc, FrPtrList src,
                                                                       FrMutPtrList dst, bool fold, Fr r,
                                                                       size_t pairs, int tile, const Fr *weights,
                                                                       int degree, Fr *out, Fr claim, bool use_claim,
                                                                       uint64_t *limb_sums, unsigned *counter,
                                                                       uint32_t *err) {
    extern __shared__ __align__(128) uint8_t tile_smem[];
    __shared__ Fr sums[kMaxSlotsV2];
    __shared__ bool last;
    __shared__ int bad;
    const int F = desc.factor_count, S = desc.slot_count;
    const int rowlen = fold ? 4 : 2;
    uint64_t *bar = reinterpret_cast<uint64_t *>(tile_smem);
    Fr *raw = reinterpret_cast<Fr *>(tile_smem + 128);
    const size_t stage_fr = size_t(F) * rowlen * tile;
    Fr *tab = raw + kTileStages * stage_fr;  // F x 2 tile folded rows
    Fr *red = tab + size_t(F) * 2 * tile;    // kTileThreads
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = kTileThreads / 32;
    const int tps = kTileThreads / S;
    const int s = int(threadIdx.x) / tps, g = int(threadIdx.x) - s * tps;
    int begin = 0, m = 1, k = 0;
    if (s < S) {
        int p = 0;
        while (p + 1 < desc.product_count && desc.slot_base[p + 1] <= s) p++;
        begin = desc.offsets[p];
        m = desc.offsets[p + 1] - begin;
        k = s - desc.slot_base[p] + desc.node0[p];
    }
    const size_t b0 = pairs * blockIdx.x / gridDim.x, b1 = pairs * (blockIdx.x + 1) / gridDim.x;
    const int ntiles = int((b1 - b0 + size_t(tile) - 1) / size_t(tile));
    if (threadIdx.x == 0) {
        for (int i = 0; i < kTileStages; i++) mbar_init(&bar[i]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        bad = 0;
    }
    __syncthreads();
    auto issue = [&](int t) {  // thread 0: the copies of tile t
        const size_t pb = b0 + size_t(t) * tile;
        const int np = int(min(size_t(tile), b1 - pb));
        const int st = t % kTileStages;
        const uint32_t bytes = uint32_t(size_t(rowlen) * np * sizeof(Fr));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bar[st], bytes * uint32_t(F));
        for (int f = 0; f < F; f++)
            bulk_load(raw + st * stage_fr + size_t(f) * rowlen * tile, src.p[f] + size_t(rowlen) * pb, bytes,
                      &bar[st]);
    };
    int issued = 0;
    if (threadIdx.x == 0)
        for (; issued < kTileStages - 1 && issued < ntiles; issued++) issue(issued);
    FrAcc X;
    acc_zero(X);
    int t = 0;
    for (; t < ntiles; t++) {
        const size_t pb = b0 + size_t(t) * tile;
        const int np = int(min(size_t(tile), b1 - pb));
        const int st = t % kTileStages;
        // the stage of tile t + kTileStages - 1 was last read in tile t - 1,
        // which every thread has finished (barrier at the end of the loop)
        if (threadIdx.x == 0 && issued < ntiles) issue(issued++);
        if (!mbar_wait_bounded(&bar[st], uint32_t(t / kTileStages) & 1u)) bad = 1;
        __syncthreads();
        if (bad) break;
        const Fr *rows = raw + st * stage_fr;
        const Fr *tb = rows;  // unfolded: the stage holds this round's rows, 2 tile apart
        if (fold) {
            for (int idx = threadIdx.x; idx < F * 2 * np; idx += kTileThreads) {
                const int f = idx / (2 * np), e = idx - f * 2 * np;
                const Fr a0 = rows[size_t(f) * 4 * tile + 2 * e], a1 = rows[size_t(f) * 4 * tile + 2 * e + 1];
                const Fr v = a0 + r * (a1 - a0);
                tab[f * 2 * tile + e] = v;
                store_fr(dst.p[f] + 2 * pb + size_t(e), v);
            }
            __syncthreads();
            tb = tab;
        }
        if (s < S) {
            for (int b = g; b < np; b += tps) {
                Fr v;
                auto factor = [&](int q) {
                    const Fr *row = tb + desc.indices[begin + q] * 2 * tile + 2 * b;
                    slot_step(X, v, row[0], row[1], q, m, k);
                };
#pragma unroll
                for (int q = 0; q < MAXM; q++)
                    if (q < m) factor(q);
            }
        }
        __syncthreads();
    }
    if (bad && threadIdx.x == 0) {
        // the copies still in flight: the timed-out tile's and those issued after it
        for (int u = t; u < issued; u++) mbar_wait_bounded(&bar[u % kTileStages], uint32_t(u / kTileStages) & 1u);
        atomicOr(err, 1u);
    }
    red[threadIdx.x] = s < S ? acc_reduce(X) : Fr::zero();
    __syncthreads();
    for (int sl = warp; sl < S; sl += warps) {
        Fr a = Fr::zero();
        for (int i = lane; i < tps; i += 32) a = a + red[sl * tps + i];
        a = warp_sum(a);
        if (lane == 0) sums[sl] = a;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * S; i += kTileThreads)
        atomicAdd(reinterpret_cast<unsigned long long *>(&limb_sums[i]), (unsigned long long)sums[i >> 3].v[i & 7]);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    uint64_t *lim = reinterpret_cast<uint64_t *>(red);
    for (int i = threadIdx.x; i < 8 * S; i += kTileThreads)
        lim[i] = atomicExch(reinterpret_cast<unsigned long long *>(&limb_sums[i]), 0ull);
    if (threadIdx.x == 0) bad = atomicExch(err, 0u) != 0u;
    __syncthreads();
    if (threadIdx.x < S) sums[threadIdx.x] = fr_from_limb_sums(lim + 8 * threadIdx.x);
    __syncthreads();
    if (!bad) {
        finalize_from_sums(desc, sums, weights, degree, out, use_claim ? &claim : nullptr);
    } else if (threadIdx.x <= degree) {
        Fr poison;
#pragma unroll
        for (int w = 0; w < 8; w++) poison.v[w] = 0xffffffffu;
        out[threadIdx.x] = poison;  // not canonical: the host reading the message fails
    }
    if (threadIdx.x == 0) *counter = 0u;
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
    // device: three zeroed Fr slots -- the round kernels' last-block counter
    // (first word), the resident grid's relay words and its relayed
    // challenge -- then the (max_degree + 1) x slot_count extrapolation
    // weights (Montgomery) of finalize_from_sums
    void *weights = nullptr;
    void *partials = nullptr;  // block partials of a round, reused every round
    size_t partials_bytes = 0;
    int current = 0;             // 0: inputs, 1: fold_a, 2: fold_b
    // Rounds after the first: products of arity = degree without their t = 0
    // slot (SumcheckDesc::node0), with their own weight matrix after the
    // first one in `weights` (row 0 = minus row 1, the claim added to it).
    hp::SumcheckDesc desc_red{};
    bool red_uniform = false;  // every product of desc_red starts at node 1
    size_t weights_full = 0;   // Fr entries of the first round's matrix
    size_t weights_red = 0;    // Fr entries of the later rounds' matrix
    // 1 / prod_{y != x} (x - y) for x = 0..max_degree: Lagrange weights of a
    // round message over the nodes 0..max_degree
    std::vector<hp::host::Fr64> lag_den;
    // the latest round message (Montgomery) and the round that produced it
    std::vector<hp::host::Fr64> last_msg;
    size_t last_round = SIZE_MAX;
    // Zero-check states (k_sumcheck_round_eq): the factor that is an eq table
    // eq(x, r) occurring once in every product (-1: none), r (Montgomery),
    // the products without it, the largest of their arities, and a device
    // buffer [product coefficients (Montgomery)][(max_degree + 1) x
    // max_degree Lagrange weights of Q over the nodes 0..max_degree-1].
    int eq_factor = -1;
    std::vector<hp::host::Fr64> eq_r;
    std::vector<hp::host::Fr64> eq_inv_a;  // 1 / (1 - r_i), 0 where r_i = 1
    hp::EqRoundDesc eq_desc{};
    int eq_max_rest = 0;
    void *eq_buf = nullptr;
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
    return reinterpret_cast<unsigned *>(s->weights);
}

// The state's relay words (zeroed at prover_init): [0] rounds relayed and [1]
// abort of the resident grid, [2] the tiled kernel's error flag; the
// resident grid's relayed challenge and claim follow at words 8 and 16.
static uint32_t *state_relay(HpCudaSumCheckProverState *s) {
    return reinterpret_cast<uint32_t *>(static_cast<Fr *>(s->weights) + 1);
}
static const Fr *state_weights(HpCudaSumCheckProverState *s) { return static_cast<const Fr *>(s->weights) + 4; }
static const Fr *state_weights_red(HpCudaSumCheckProverState *s) {
    return static_cast<const Fr *>(s->weights) + 4 + s->weights_full;
}
// The tiled kernel's 8 x kMaxSlotsV2 limb counters after both matrices
// (zeroed at prover_init, cleared again by every launch's last block).
static uint64_t *state_tile_limbs(HpCudaSumCheckProverState *s) {
    return reinterpret_cast<uint64_t *>(static_cast<Fr *>(s->weights) + 4 + s->weights_full + s->weights_red);
}
constexpr size_t kTileLimbFr = 8 * kMaxSlotsV2 * sizeof(uint64_t) / sizeof(Fr);

// Stores round `round`'s message (canonical bytes) for the next round's claim.
static void record_message(HpCudaSumCheckProverState *s, size_t round, const uint8_t *bytes) {
    s->last_msg.resize(s->max_degree + 1);
    for (size_t x = 0; x <= s->max_degree; x++)
        if (!host::from_canonical(bytes + 32 * x, s->last_msg[x])) fail(HP_CUDA_STATUS_INVALID_STATE);
    s->last_round = round;
}

// The claim of the state's current round: the previous message's polynomial
// at the previous challenge r, sum_x L_x(r) m[x] with the Lagrange basis of
// the nodes 0..d (prefix and suffix products of r - y); false when the
// previous message was not recorded.
static host::Fr64 message_at(const std::vector<host::Fr64> &msg, const std::vector<host::Fr64> &lag_den,
                             const host::Fr64 &r) {
    const size_t D = lag_den.size() - 1;
    std::vector<host::Fr64> diff(D + 1), pre(D + 1), suf(D + 1);
    for (size_t y = 0; y <= D; y++) diff[y] = host::add(r, host::neg(host::from_u64(uint64_t(y))));
    pre[0] = host::one();
    for (size_t x = 1; x <= D; x++) pre[x] = host::mont_mul(pre[x - 1], diff[x - 1]);
    suf[D] = host::one();
    for (size_t x = D; x-- > 0;) suf[x] = host::mont_mul(suf[x + 1], diff[x + 1]);
    host::Fr64 acc{{0, 0, 0, 0}};
    for (size_t x = 0; x <= D; x++) {
        const host::Fr64 l = host::mont_mul(host::mont_mul(pre[x], suf[x]), lag_den[x]);
        acc = host::add(acc, host::mont_mul(l, msg[x]));
    }
    return acc;
}
static bool round_claim(const HpCudaSumCheckProverState *s, const host::Fr64 &r, host::Fr64 &out) {
    if (s->round == 0 || s->last_round != s->round - 1) return false;
    out = message_at(s->last_msg, s->lag_den, r);
    return true;
}

static size_t big_blocks_per_sm();

// Block partials of any round of the state: the largest grid x slots of the
// round kernels (per-pair grid kernel, (slot, pair) kernel, shared-memory
// kernel).
static size_t partials_capacity(const SumcheckDesc &d, int sm_count) {
    const size_t sms = size_t(sm_count > 0 ? sm_count : 152), S = size_t(d.slot_count);
    size_t n = sms * HP_ROUND_BLOCKS_PER_SM * S;
    n = std::max(n, sms * 2 * S);
    n = std::max(n, size_t(64) * S);
    n = std::max(n, sms * big_blocks_per_sm() + S);
    // the resident grid's limb counters: 2 rounds x 8 limbs x kMaxSlotsV2 slots
    n = std::max(n, size_t(2 * 8 * kMaxSlotsV2) * sizeof(uint64_t) / sizeof(Fr));
    return n * sizeof(Fr);
}

// The state's partials buffer when it holds `bytes`, else `fallback`.
static Fr *round_partials(HpCudaContext *ctx, HpCudaSumCheckProverState *s, size_t bytes, Scratch &fallback,
                          cudaStream_t st) {
    if (bytes <= s->partials_bytes) return static_cast<Fr *>(s->partials);
    fallback = Scratch(ctx, bytes, st);
    return fallback.as<Fr>();
}

// The (degree + 1) x slot_count matrix W of finalize_from_sums, Montgomery
// form: W[x][slot_base[p] + i] = c_p * l_{m,i}(x), where l_{m,i} is the
// Lagrange basis polynomial of the nodes 0..m (m = arity of product p):
// l_{m,i}(x) = [x == i] for x <= m, else
// prod_{k != i} (x - k) / ((-1)^(m-i) i! (m-i)!).
// 1 / prod_{y != x} (x - y) = (-1)^(D - x) / (x! (D - x)!) for x = 0..D
static std::vector<host::Fr64> lagrange_denominators(size_t D) {
    std::vector<host::Fr64> fact(D + 1), inv_fact(D + 1), out(D + 1);
    fact[0] = host::one();
    for (size_t k = 1; k <= D; k++) fact[k] = host::mont_mul(fact[k - 1], host::from_u64(uint64_t(k)));
    inv_fact[D] = host::inverse(fact[D]);
    for (size_t k = D; k >= 1; k--) inv_fact[k - 1] = host::mont_mul(inv_fact[k], host::from_u64(uint64_t(k)));
    for (size_t x = 0; x <= D; x++) {
        out[x] = host::mont_mul(inv_fact[x], inv_fact[D - x]);
        if ((D - x) & 1) out[x] = host::neg(out[x]);
    }
    return out;
}

static std::vector<host::Fr64> extrapolation_weights(const SumcheckDesc &d, const uint8_t *coefficients,
                                                     size_t degree) {
    using host::Fr64;
    const int S = d.slot_count, D = int(degree);
    std::vector<Fr64> w(size_t(D + 1) * S, Fr64{{0, 0, 0, 0}});
    // inverse factorials 0..kMaxDegree
    std::vector<Fr64> fact(kMaxDegree + 1), inv_fact(kMaxDegree + 1);
    fact[0] = host::one();
    for (int k = 1; k <= kMaxDegree; k++) fact[k] = host::mont_mul(fact[k - 1], host::from_u64(uint64_t(k)));
    inv_fact[kMaxDegree] = host::inverse(fact[kMaxDegree]);
    for (int k = kMaxDegree; k >= 1; k--) inv_fact[k - 1] = host::mont_mul(inv_fact[k], host::from_u64(uint64_t(k)));
    for (int p = 0; p < d.product_count; p++) {
        const int m = d.offsets[p + 1] - d.offsets[p], base = d.slot_base[p];
        Fr64 c;
        if (!host::from_canonical(coefficients + 32 * size_t(p), c)) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
        for (int i = 0; i <= m; i++) {
            Fr64 den = host::mont_mul(inv_fact[i], inv_fact[m - i]);
            if ((m - i) & 1) den = host::neg(den);
            const Fr64 ci = host::mont_mul(c, den);
            for (int x = 0; x <= D; x++) {
                Fr64 v;
                if (x <= m) {
                    v = x == i ? c : Fr64{{0, 0, 0, 0}};
                } else {
                    v = ci;
                    for (int k = 0; k <= m; k++)
                        if (k != i) v = host::mont_mul(v, host::from_u64(uint64_t(x - k)));
                }
                w[size_t(x) * S + base + i] = v;
            }
        }
    }
    return w;
}

// Zero-check detection at state creation: the first factor whose table
// hp_cuda_v1_mle_build_eq_x_r built (its point rides with the buffer) and
// whose address occurs exactly once in every product.  Fills the state's
// eq fields and returns the host image of its device buffer (empty: no such
// factor, or a degree below 2, where the generic rounds stay).
static std::vector<host::Fr64> detect_eq_factor(HpCudaContext *ctx, HpCudaSumCheckProverState *s,
                                                const HpCudaDeviceAddress *factors, const uint8_t *coefficients,
                                                const size_t *product_offsets, const size_t *factor_indices) {
    using host::Fr64;
    const SumcheckDesc &d = s->desc;
    const size_t P = size_t(d.product_count), D = s->max_degree, nv = s->num_vars;
    if (D < 2 || P == 0) return {};
    for (int f = 0; f < d.factor_count; f++) {
        const auto &rec = ctx->buffers.at(factors[f]);
        if (rec.eq_point.size() != 4 * nv) continue;
        bool once = true;
        for (size_t p = 0; p < P && once; p++) {
            size_t c = 0;
            for (size_t i = product_offsets[p]; i < product_offsets[p + 1]; i++)
                c += factors[factor_indices[i]] == factors[f] ? 1 : 0;
            once = c == 1;
        }
        if (!once) continue;
        s->eq_factor = f;
        s->eq_r.resize(nv);
        for (size_t i = 0; i < nv; i++) std::memcpy(s->eq_r[i].v, &rec.eq_point[4 * i], 32);
        // 1 / (1 - r_i) for the claim's Q(0), by one batched inversion
        // (Montgomery's trick; a zero 1 - r_i is skipped and stays 0)
        {
            std::vector<Fr64> a(nv), pre(nv + 1);
            pre[0] = host::one();
            for (size_t i = 0; i < nv; i++) {
                a[i] = host::add(host::one(), host::neg(s->eq_r[i]));
                pre[i + 1] = host::is_zero(a[i]) ? pre[i] : host::mont_mul(pre[i], a[i]);
            }
            Fr64 inv = host::inverse(pre[nv]);
            s->eq_inv_a.assign(nv, Fr64{{0, 0, 0, 0}});
            for (size_t i = nv; i-- > 0;) {
                if (host::is_zero(a[i])) continue;
                s->eq_inv_a[i] = host::mont_mul(inv, pre[i]);
                inv = host::mont_mul(inv, a[i]);
            }
        }
        EqRoundDesc &ed = s->eq_desc;
        ed.product_count = int(P);
        ed.eq_factor = f;
        std::vector<Fr64> img(P + (D + 1) * D, Fr64{{0, 0, 0, 0}});
        const Fr64 one = host::one(), minus_one = host::neg(host::one());
        size_t n = 0;
        int max_rest = 0;
        for (size_t p = 0; p < P; p++) {
            ed.offsets[p] = uint16_t(n);
            for (size_t i = product_offsets[p]; i < product_offsets[p + 1]; i++)
                if (int(factor_indices[i]) != f) ed.indices[n++] = uint8_t(factor_indices[i]);
            max_rest = std::max(max_rest, int(n - ed.offsets[p]));
            Fr64 c;
            if (!host::from_canonical(coefficients + 32 * p, c)) fail(HP_CUDA_STATUS_INVALID_PARAMETERS);
            ed.coef_kind[p] = std::memcmp(&c, &one, sizeof c) == 0 ? 0 : std::memcmp(&c, &minus_one, sizeof c) == 0 ? 1 : 2;
            img[p] = c;
        }
        ed.offsets[P] = uint16_t(n);
        s->eq_max_rest = max_rest;
        // L[x][j] = prod_{m != j} (x - m) / (j - m) over the nodes m = 0..D-1,
        // 1 / prod_{m != j} (j - m) = (-1)^(D-1-j) / (j! (D-1-j)!): one inversion
        auto small = [](long long k) {
            return k >= 0 ? host::from_u64(uint64_t(k)) : host::neg(host::from_u64(uint64_t(-k)));
        };
        std::vector<Fr64> fact(D), inv_fact(D);
        fact[0] = one;
        for (size_t k = 1; k < D; k++) fact[k] = host::mont_mul(fact[k - 1], host::from_u64(uint64_t(k)));
        inv_fact[D - 1] = host::inverse(fact[D - 1]);
        for (size_t k = D - 1; k >= 1; k--) inv_fact[k - 1] = host::mont_mul(inv_fact[k], host::from_u64(uint64_t(k)));
        for (size_t j = 0; j < D; j++) {
            Fr64 inv_den = host::mont_mul(inv_fact[j], inv_fact[D - 1 - j]);
            if ((D - 1 - j) & 1) inv_den = host::neg(inv_den);
            for (size_t x = 0; x <= D; x++) {
                Fr64 num = inv_den;
                for (size_t m = 0; m < D; m++)
                    if (m != j) num = host::mont_mul(num, small((long long)x - (long long)m));
                img[P + x * D + j] = num;
            }
        }
        return img;
    }
    return {};
}

static void release_state(HpCudaContext *ctx, HpCudaSumCheckProverState *s) {
    for (void *p : s->inputs) {
        try { ctx->unref(p); } catch (...) {}
    }
    s->inputs.clear();
    if (s->fold_a) ctx->scratch_free(s->fold_a);
    if (s->fold_b) ctx->scratch_free(s->fold_b);
    if (s->weights) ctx->scratch_free(s->weights);
    if (s->partials) ctx->scratch_free(s->partials);
    if (s->eq_buf) ctx->scratch_free(s->eq_buf);
    s->fold_a = s->fold_b = s->weights = s->partials = s->eq_buf = nullptr;
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
            for (int p = 0; p < hp::kMaxProducts; p++) d.node0[p] = 0;
            for (int f = 0; f < hp::kMaxFactors; f++) d.writer[f] = hp::kNoWriter;
            for (size_t i = 0; i < index_count; i++) {
                d.indices[i] = uint8_t(factor_indices[i]);
                if (d.writer[factor_indices[i]] == hp::kNoWriter) d.writer[factor_indices[i]] = uint16_t(i);
            }
            d.slot_count = std::max(slots, 1);
            d.max_arity = max_arity;
            for (size_t f = 0; f < factor_count; f++) {
                hp::mle_ptr(ctx, factors[f], num_vars);
                ctx->ref(factors[f]);
                s->inputs.push_back(factors[f]);
            }
            std::vector<hp::host::Fr64> w = hp::extrapolation_weights(d, coefficients, max_degree);
            // rounds 2..: products of arity = degree lose their t = 0 slot; the
            // reduced matrix keeps rows 1..d of the remaining columns and takes
            // minus row 1 as row 0 (the claim is added to it)
            hp::SumcheckDesc &dr = s->desc_red;
            dr = d;
            int rslots = 0;
            for (size_t p = 0; p < product_count; p++) {
                const int m = int(product_offsets[p + 1] - product_offsets[p]);
                dr.node0[p] = uint8_t(size_t(m) == max_degree ? 1 : 0);
                dr.slot_base[p] = uint16_t(rslots);
                rslots += m + 1 - dr.node0[p];
            }
            dr.slot_count = std::max(rslots, 1);
            s->red_uniform = product_count > 0;
            for (size_t p = 0; p < product_count; p++) s->red_uniform = s->red_uniform && dr.node0[p] == 1;
            const size_t S = size_t(d.slot_count), SR = size_t(dr.slot_count), D = max_degree;
            std::vector<hp::host::Fr64> wr((D + 1) * SR, hp::host::Fr64{{0, 0, 0, 0}});
            for (size_t p = 0; p < product_count; p++) {
                const int m = int(product_offsets[p + 1] - product_offsets[p]);
                for (int t = dr.node0[p]; t <= m; t++)
                    for (size_t x = 1; x <= D; x++)
                        wr[x * SR + dr.slot_base[p] + size_t(t - dr.node0[p])] = w[x * S + d.slot_base[p] + size_t(t)];
            }
            if (D >= 1)
                for (size_t c = 0; c < SR; c++) wr[c] = hp::host::neg(wr[SR + c]);
            s->lag_den = hp::lagrange_denominators(D);
            s->weights_full = w.size();
            s->weights_red = wr.size();
            s->weights = ctx->scratch((w.size() + wr.size() + 4 + hp::kTileLimbFr) * sizeof(Fr));
            check_cuda(cudaMemsetAsync(s->weights, 0, 4 * sizeof(Fr), ctx->stream));
            check_cuda(cudaMemsetAsync(hp::state_tile_limbs(s), 0, hp::kTileLimbFr * sizeof(Fr), ctx->stream));
            check_cuda(cudaMemcpyAsync(static_cast<Fr *>(s->weights) + 4, w.data(), w.size() * sizeof(Fr),
                                       cudaMemcpyHostToDevice, ctx->stream));
            check_cuda(cudaMemcpyAsync(static_cast<Fr *>(s->weights) + 4 + w.size(), wr.data(),
                                       wr.size() * sizeof(Fr), cudaMemcpyHostToDevice, ctx->stream));
            s->partials_bytes = hp::partials_capacity(d, ctx->sm_count);
            s->partials = ctx->scratch(s->partials_bytes);
            std::vector<hp::host::Fr64> eq_host = hp::detect_eq_factor(ctx, s, factors, coefficients, product_offsets,
                                                                       factor_indices);
            if (!eq_host.empty()) {
                s->eq_buf = ctx->scratch(eq_host.size() * sizeof(Fr));
                check_cuda(cudaMemcpyAsync(s->eq_buf, eq_host.data(), eq_host.size() * sizeof(Fr),
                                           cudaMemcpyHostToDevice, ctx->stream));
            }
            ctx->sync();  // w and eq_host are pageable host vectors
            size_t a_len = hp::table_len(num_vars - 1);
            size_t b_len = num_vars >= 2 ? hp::table_len(num_vars - 2) : 1;
            size_t fcount = std::max(factor_count, size_t(1));
            s->fold_a = ctx->scratch(fcount * a_len * sizeof(Fr));
            s->fold_b = ctx->scratch(fcount * b_len * sizeof(Fr));
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

static size_t wide_max_pairs();
static size_t wide_min_pairs();
static size_t tiled_min_pairs();
static size_t tiled_blocks_per_sm();
static size_t eq_min_pairs();
static size_t env_size(const char *name, size_t dflt);
static bool product_pair_rounds();
static bool fused_fold_pp();
static size_t pp_min_pairs();
static bool big_slot_rounds();
static size_t big_blocks_per_sm();
static int separate_fold_arity();

// ---------------------------------------------------------------------------
// Round routes: which kernel runs a round, and its grid
// ---------------------------------------------------------------------------

// The shape facts a round's route depends on.
struct RoundShape {
    size_t pairs;
    bool fold;         // round > 1: the previous challenge is folded in
    bool regs;         // arity <= 8 and <= kMaxSlotsV2 slots (per-thread kernels)
    bool all_written;  // every factor is read by some product (fused folds store it)
    bool products;     // at least one product
    bool eq = false;   // a zero-check state (k_sumcheck_round_eq)
    int max_arity;
    int slots;
};

static RoundShape round_shape(const HpCudaSumCheckProverState *s) {
    const SumcheckDesc &d = s->desc;
    RoundShape sh;
    sh.pairs = table_len(s->num_vars - s->round - 1);
    sh.fold = s->round > 0;
    sh.regs = d.max_arity <= 8 && d.slot_count <= kMaxSlotsV2;
    sh.all_written = true;
    for (int f = 0; f < d.factor_count; f++) sh.all_written = sh.all_written && d.writer[f] != kNoWriter;
    sh.products = d.product_count > 0;
    sh.eq = s->eq_factor >= 0;
    sh.max_arity = d.max_arity;
    sh.slots = d.slot_count;
    return sh;
}

// Whether `route` can run a round of this shape.
static bool route_valid(const RoundShape &sh, const RoundRoute &rt) {
    switch (rt.kernel) {
        case kRouteOneBlock: return sh.regs && sh.pairs <= size_t(kSmallPairs);
        case kRoutePerPair: return sh.regs;
        case kRouteSlot: return sh.products;
        case kRouteSlotFused: return sh.products && sh.fold && sh.all_written;
        case kRoutePp: return sh.products && sh.max_arity <= 3 && sh.slots <= kMaxSlotsV2;
        case kRouteTiled: return sh.products && sh.regs;
        case kRouteEq: return sh.products && sh.eq;
        case kRoutePpFused: return sh.products && sh.max_arity <= 3 && sh.slots <= kMaxSlotsV2 && sh.fold &&
                                   sh.all_written;
        default: return false;
    }
}

// The built-in rules (sizes measured on GB300; the environment switches of
// the run-time table in the design notes override them).
static RoundRoute default_route(const RoundShape &sh) {
    const bool small = sh.regs && sh.pairs <= size_t(kSmallPairs);
    if (sh.products && sh.regs && tiled_min_pairs() > 0 && sh.pairs >= tiled_min_pairs())
        return RoundRoute{kRouteTiled, uint8_t(tiled_blocks_per_sm())};
    if (sh.products && sh.pairs >= pp_min_pairs() && sh.pairs > wide_max_pairs() && sh.max_arity <= 3 &&
        sh.slots <= kMaxSlotsV2 && product_pair_rounds())
        return RoundRoute{uint8_t(sh.fold && sh.all_written && fused_fold_pp() ? kRoutePpFused : kRoutePp),
                          uint8_t(kPpBlocksPerSm)};
    if (sh.products && !small) {
        if (sh.pairs > wide_max_pairs()) {
            if (big_slot_rounds() || !sh.regs) return RoundRoute{kRouteSlot, uint8_t(big_blocks_per_sm())};
        } else if (sh.pairs >= wide_min_pairs() || !sh.regs) {
            // the fused fold stores only factors some product reads; products
            // of arity >= separate_fold_arity() (HP_SEPARATE_FOLD_ARITY,
            // default 3) fold in a separate pass: one more launch, but each
            // item's chain loses the 2m products of re-folding its factors
            // (GB300, nv = 20: arity-4/5 middle rounds 56-60 -> 35-43 us)
            const bool separate = !sh.all_written || sh.max_arity >= separate_fold_arity();
            return RoundRoute{uint8_t(sh.fold && !separate ? kRouteSlotFused : kRouteSlot), 0};
        }
    }
    if (small) return RoundRoute{kRouteOneBlock, 0};
    return RoundRoute{kRoutePerPair, 0};
}

// The route of a round: the tuned entry for its shape when one exists and
// fits, else the built-in rules.
static RoundRoute chosen_route(const RoundShape &sh) {
    RoundRoute rt;
    if (sh.eq && sh.products && sh.pairs >= eq_min_pairs()) return RoundRoute{kRouteEq, 0};
    if (sumcheck_route_lookup(RoundKey{ceil_log2_size(sh.pairs), sh.max_arity, sh.slots, sh.fold ? 1 : 0}, rt) &&
        route_valid(sh, rt))
        return rt;
    return default_route(sh);
}

// k_sumcheck_fold of every table: dst_f[i] = src_f[2i] + r (src_f[2i+1] - src_f[2i]).
static void fold_all(HpCudaContext *ctx, const SumcheckDesc &d, const FrPtrList &src, const FrMutPtrList &dst,
                     size_t pairs, const Fr &r, cudaStream_t st) {
    int log_half = 0;
    while ((size_t(1) << log_half) < 2 * pairs) log_half++;
    const size_t total = size_t(d.factor_count) << log_half;
    const size_t sms = size_t(ctx->sm_count > 0 ? ctx->sm_count : 152);
    const unsigned fgrid = unsigned(std::max<size_t>(1, std::min<size_t>((total + 255) / 256, sms * 8)));
    k_sumcheck_fold<<<fgrid, 256, 0, st>>>(src, dst, d.factor_count, log_half, r);
    check_launch();
}

// Enqueues one round of state s on stream st along `rt`: fold with r (rounds
// > 1) and message into out_dev (degree + 1 canonical Fr, device).  Scratch
// is ordered on st.  Does not advance the state.
static void launch_round(HpCudaContext *ctx, HpCudaSumCheckProverState *s, const Fr &r, cudaStream_t st,
                         Fr *out_dev, const RoundShape &sh, const RoundRoute &rt) {
    // rounds after the first whose previous message was recorded take the
    // reduced layout and the claim (same message bytes, fewer slot products)
    host::Fr64 r64, claim64;
    std::memcpy(r64.v, r.v, 32);
    const bool pp_route = rt.kernel == kRoutePp || rt.kernel == kRoutePpFused;
    const bool red = (!pp_route || s->red_uniform) && round_claim(s, r64, claim64);
    const SumcheckDesc &d = red ? s->desc_red : s->desc;
    const Fr *wts = red ? state_weights_red(s) : state_weights(s);
    Fr claim = Fr::zero();
    if (red) std::memcpy(claim.v, claim64.v, 32);
    const bool fold = sh.fold;
    const int src_which = s->current;
    const int dst_which = fold ? (src_which == 1 ? 2 : 1) : src_which;
    const size_t pairs = sh.pairs;
    FrPtrList src{}, rd{};
    FrMutPtrList dst{};
    for (int f = 0; f < d.factor_count; f++) {
        src.p[f] = state_table(s, src_which, f);
        dst.p[f] = const_cast<Fr *>(state_table(s, dst_which, f));
        rd.p[f] = fold ? dst.p[f] : src.p[f];
    }
    const size_t sms = size_t(ctx->sm_count > 0 ? ctx->sm_count : 152);
    int tok = ctx->prof_begin("sumcheck_round", st);
    switch (rt.kernel) {
        case kRoutePp:
        case kRoutePpFused: {
            FrPtrList tables = src;
            bool fused_fold = fold && rt.kernel == kRoutePpFused;
            if (fold && !fused_fold) {
                fold_all(ctx, d, src, dst, pairs, r, st);
                tables = rd;
            }
            const size_t P = size_t(d.product_count);
            const size_t tiles = (pairs + kPpThreads - 1) / kPpThreads;
            const size_t target = sms * std::max<size_t>(1, rt.per_sm);
            const int bpp = int(std::max<size_t>(1, std::min(tiles, (target + P - 1) / P)));
            const unsigned grid = unsigned(P) * unsigned(bpp);
            Scratch spill;
            Fr *partials = round_partials(ctx, s, size_t(d.slot_count) * size_t(bpp) * sizeof(Fr), spill, st);
            const size_t smem = size_t(d.slot_count) * sizeof(Fr);
            auto launch = [&](auto kernel) {
                kernel<<<grid, kPpThreads, smem, st>>>(d, tables, dst, fused_fold, r, pairs, bpp, partials,
                                                       round_counter(s), wts, int(s->max_degree), out_dev, claim,
                                                       red);
            };
            if (red) {
                if (d.max_arity <= 2) launch(k_sumcheck_round_pp<2, 1>);
                else launch(k_sumcheck_round_pp<3, 1>);
            } else {
                if (d.max_arity <= 2) launch(k_sumcheck_round_pp<2, 0>);
                else launch(k_sumcheck_round_pp<3, 0>);
            }
            check_launch();
            break;
        }
        case kRouteSlot:
        case kRouteSlotFused: {
            const size_t tiles = (pairs + kWideThreads - 1) / kWideThreads;
            int bps = int(std::min(tiles, size_t(1) << 20));
            FrPtrList tables = src;
            bool fused_fold = fold && rt.kernel == kRouteSlotFused;
            if (fold && !fused_fold) {
                // fold every table first, then one pass over the folded tables
                fold_all(ctx, d, src, dst, pairs, r, st);
                tables = rd;
            }
            if (rt.per_sm > 0) {
                // about per_sm blocks per SM over all slots
                const size_t target = sms * rt.per_sm;
                bps = int(std::max<size_t>(1, std::min(tiles, (target + d.slot_count - 1) / d.slot_count)));
            }
            const unsigned grid = unsigned(d.slot_count) * unsigned(bps);
            Scratch spill;
            Fr *partials = round_partials(ctx, s, size_t(grid) * sizeof(Fr), spill, st);
            const size_t smem = size_t(d.slot_count) * sizeof(Fr);
            auto launch = [&](auto kernel) {
                if (smem > 32 * 1024)
                    check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
                kernel<<<grid, kWideThreads, smem, st>>>(d, tables, dst, fused_fold, r, pairs, bps, partials,
                                                         round_counter(s), wts, int(s->max_degree), out_dev, claim,
                                                         red);
            };
            if (d.max_arity <= 2) launch(k_sumcheck_round_wide<2>);
            else if (d.max_arity <= 4) launch(k_sumcheck_round_wide<4>);
            else if (d.max_arity <= 6) launch(k_sumcheck_round_wide<6>);
            else if (d.max_arity <= 8) launch(k_sumcheck_round_wide<8>);
            else launch(k_sumcheck_round_wide<0>);  // any arity, loop not unrolled
            check_launch();
            break;
        }
        case kRouteTiled: {
            int tile = 64;
            while (tile > 8 && tiled_smem(d.factor_count, tile, fold) > size_t(110) * 1024) tile >>= 1;
            const size_t smem = tiled_smem(d.factor_count, tile, fold);
            const size_t per_sm = std::max<size_t>(1, rt.per_sm);
            const unsigned grid =
                unsigned(std::max<size_t>(1, std::min(sms * per_sm, (pairs + size_t(tile) - 1) / size_t(tile))));
            FrPtrList tables = src;
            auto launch = [&](auto kernel) {
                check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
                kernel<<<grid, kTileThreads, smem, st>>>(d, tables, dst, fold, r, pairs, tile, wts,
                                                         int(s->max_degree), out_dev, claim, red,
                                                         state_tile_limbs(s), round_counter(s),
                                                         state_relay(s) + 2);
            };
            if (d.max_arity <= 2) launch(k_sumcheck_round_tiled<2>);
            else if (d.max_arity <= 4) launch(k_sumcheck_round_tiled<4>);
            else if (d.max_arity <= 6) launch(k_sumcheck_round_tiled<6>);
            else launch(k_sumcheck_round_tiled<8>);
            check_launch();
            break;
        }
        case kRouteEq: {
            FrPtrList tables = src;
            if (fold) {
                fold_all(ctx, d, src, dst, pairs, r, st);
                tables = rd;
            }
            const int D = int(s->max_degree);
            const host::Fr64 ri = s->eq_r[s->round];
            const host::Fr64 a64 = host::add(host::one(), host::neg(ri));  // 1 - r_i
            const host::Fr64 b64 = host::add(ri, host::neg(a64));          // 2 r_i - 1
            host::Fr64 u64{{0, 0, 0, 0}}, v64{{0, 0, 0, 0}};
            const bool use = red && !host::is_zero(a64);
            if (use) {
                const host::Fr64 &inv = s->eq_inv_a[s->round];
                u64 = host::mont_mul(claim64, inv);
                v64 = host::neg(host::mont_mul(ri, inv));
            }
            Fr a, b, u, v;
            std::memcpy(a.v, a64.v, 32);
            std::memcpy(b.v, b64.v, 32);
            std::memcpy(u.v, u64.v, 32);
            std::memcpy(v.v, v64.v, 32);
            const int node0 = use ? 1 : 0, nodes = D - node0;
            const size_t tiles = (pairs + kWideThreads - 1) / kWideThreads;
            const size_t target = sms * std::max<size_t>(1, env_size("HP_SUMCHECK_EQ_PER_SM", big_blocks_per_sm()));
            const int bpn = int(std::max<size_t>(1, std::min(tiles, (target + size_t(nodes) - 1) / size_t(nodes))));
            const unsigned grid = unsigned(nodes) * unsigned(bpn);
            Scratch spill;
            Fr *partials = round_partials(ctx, s, size_t(grid) * sizeof(Fr), spill, st);
            const Fr *coefs = static_cast<const Fr *>(s->eq_buf);
            const Fr *lag = coefs + s->desc.product_count;
            const int etok = ctx->prof_begin("sumcheck_round_eq", st);
            auto launch = [&](auto kernel) {
                kernel<<<grid, kWideThreads, 0, st>>>(s->eq_desc, tables, pairs, node0, nodes, bpn, coefs, partials,
                                                      round_counter(s), lag, D, a, b, u, v, out_dev);
            };
            if (s->eq_max_rest <= 2) launch(k_sumcheck_round_eq<2>);
            else if (s->eq_max_rest <= 4) launch(k_sumcheck_round_eq<4>);
            else if (s->eq_max_rest <= 6) launch(k_sumcheck_round_eq<6>);
            else if (s->eq_max_rest <= 8) launch(k_sumcheck_round_eq<8>);
            else launch(k_sumcheck_round_eq<0>);
            check_launch();
            ctx->prof_end(etok, st);
            break;
        }
        case kRouteOneBlock: {
            const size_t smem = size_t(d.slot_count) * (kSmallPairs + 1) * sizeof(Fr);
            auto launch = [&](auto kernel) {
                if (smem > 32 * 1024)
                    check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
                kernel<<<1, kSmallThreads, smem, st>>>(d, src, dst, rd, fold, r, int(pairs), wts,
                                                       int(s->max_degree), out_dev, claim, red);
            };
            if (d.max_arity <= 2) launch(k_sumcheck_round_small<2>);
            else if (d.max_arity <= 4) launch(k_sumcheck_round_small<4>);
            else if (d.max_arity <= 6) launch(k_sumcheck_round_small<6>);
            else launch(k_sumcheck_round_small<8>);
            check_launch();
            break;
        }
        case kRoutePerPair: {
            const unsigned grid = grid_for(ctx, pairs, kRoundThreads, HP_ROUND_BLOCKS_PER_SM);
            Scratch spill;
            Fr *partials = round_partials(ctx, s, size_t(grid) * d.slot_count * sizeof(Fr), spill, st);
            const size_t smem = size_t(d.slot_count) * kRoundThreads * sizeof(Fr);
            auto launch = [&](auto kernel) {
                // the kernel's own static shared memory counts against the same
                // 48 KiB default, so opt in well before the dynamic size reaches it
                if (smem > 32 * 1024)
                    check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
                kernel<<<grid, kRoundThreads, smem, st>>>(d, src, dst, rd, fold, r, pairs, partials,
                                                          round_counter(s), wts, int(s->max_degree), out_dev, claim,
                                                          red);
            };
            if (d.max_arity <= 2) launch(k_sumcheck_round_regs<2>);
            else if (d.max_arity <= 4) launch(k_sumcheck_round_regs<4>);
            else if (d.max_arity <= 6) launch(k_sumcheck_round_regs<6>);
            else launch(k_sumcheck_round_regs<8>);
            check_launch();
            break;
        }
        default: fail(HP_CUDA_STATUS_INVALID_STATE);
    }
    ctx->prof_end(tok, st);
}

// Enqueues one round of state s on stream st along its chosen route.
static void enqueue_round(HpCudaContext *ctx, HpCudaSumCheckProverState *s, const Fr &r, cudaStream_t st,
                          Fr *out_dev) {
    const RoundShape sh = round_shape(s);
    const RoundRoute rt = chosen_route(sh);
    if (!route_valid(sh, rt)) fail(HP_CUDA_STATUS_NOT_IMPLEMENTED);
    launch_round(ctx, s, r, st, out_dev, sh, rt);
}

// Rounds of wide_min_pairs() .. wide_max_pairs() pairs use the (slot, pair)
// kernel with the fold fused; HP_WIDE_MAX_PAIRS / HP_WIDE_MIN_PAIRS override
// the range (a maximum of 0 turns it off).
static size_t env_size(const char *name, size_t dflt) {
    const char *env = std::getenv(name);
    if (env == nullptr || *env == '\0') return dflt;
    return size_t(std::strtoull(env, nullptr, 10));
}
static size_t wide_max_pairs() {
    static const size_t v = env_size("HP_WIDE_MAX_PAIRS", size_t(1) << 13);
    return v;
}
static size_t wide_min_pairs() {
    static const size_t v = env_size("HP_WIDE_MIN_PAIRS", size_t(kSmallPairs) + 1);
    return v;
}
static int separate_fold_arity() {
    static const int v = int(env_size("HP_SEPARATE_FOLD_ARITY", 3));
    return v;
}
// Rounds of more than kSmallPairs pairs over products of arity <= 8 take the
// (product, pair) kernel; HP_SUMCHECK_PP=0 restores the (slot, pair) and
// per-pair kernels below for them.
static bool product_pair_rounds() {
    static const bool v = env_size("HP_SUMCHECK_PP", 1) != 0;
    return v;
}
// HP_SUMCHECK_PP_FOLD=1: the (product, pair) kernel folds its own factors
// (each factor re-folded once per product that reads it) instead of the
// separate fold pass.  Off by default: measured on GB300 at 2^19 pairs, the
// fused form took 225 us for round 2 against 82 + ~70 us for fold + round.
// Smallest round for the (product, pair) kernel (HP_SUMCHECK_PP_MIN_PAIRS):
// measured on GB300 (6 tables, 4 arity-2 products) it wins from 2^16 pairs on
// (2^17: 60 vs 66 us) and loses below (2^14: 43 vs 32 us).
static size_t pp_min_pairs() {
    static const size_t v = env_size("HP_SUMCHECK_PP_MIN_PAIRS", size_t(1) << 16);
    return v;
}
static bool fused_fold_pp() {
    static const bool v = env_size("HP_SUMCHECK_PP_FOLD", 0) != 0;
    return v;
}
// Rounds of at least HP_SUMCHECK_TILED pairs take the tiled kernel (0: none),
// with HP_SUMCHECK_TILED_PER_SM blocks per SM.
// Zero-check states take k_sumcheck_round_eq from rounds of this many pairs
// up (HP_SUMCHECK_EQ_MIN_PAIRS; HP_SUMCHECK_EQ=0: never).
static size_t eq_min_pairs() {
    const char *off = std::getenv("HP_SUMCHECK_EQ");
    if (off != nullptr && std::strcmp(off, "0") == 0) return SIZE_MAX;
    return std::max<size_t>(1, env_size("HP_SUMCHECK_EQ_MIN_PAIRS", size_t(1) << 13));
}

static size_t tiled_min_pairs() {
    static const size_t v = env_size("HP_SUMCHECK_TILED", 0);
    return v;
}
static size_t tiled_blocks_per_sm() {
    static const size_t v = std::max<size_t>(1, env_size("HP_SUMCHECK_TILED_PER_SM", 2));
    return v;
}
// Rounds above wide_max_pairs(): k_sumcheck_fold + the (slot, pair) kernel
// (HP_BIG_SLOTS=0: the per-pair shared-memory kernel instead), with about
// big_blocks_per_sm() blocks per SM in all (HP_BIG_BLOCKS_PER_SM).
static bool big_slot_rounds() {
    static const bool v = env_size("HP_BIG_SLOTS", 1) != 0;
    return v;
}
static size_t big_blocks_per_sm() {
    static const size_t v = std::max<size_t>(1, env_size("HP_BIG_BLOCKS_PER_SM", 16));
    return v;
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
            void *box_dev = nullptr;
            const uint8_t *box = ctx->mailbox(evaluation_count * sizeof(Fr), &box_dev);
            hp::enqueue_round(ctx, s, r, ctx->stream, static_cast<Fr *>(box_dev));
            ctx->sync();
            std::memcpy(out_evaluations, box, evaluation_count * sizeof(Fr));
            hp::record_message(s, s->round, out_evaluations);
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
            // the round kernels write their messages into the mapped mailbox
            void *box_dev = nullptr;
            const uint8_t *box = ctx->mailbox(total * sizeof(Fr), &box_dev);
            const int k = int(std::min<size_t>(count, HpCudaContext::kWorkers));
            ctx->fork(k);
            size_t off = 0;
            for (size_t i = 0; i < count; i++) {
                hp::enqueue_round(ctx, states[i], rs[i], ctx->workers[i % size_t(k)],
                                  static_cast<Fr *>(box_dev) + off);
                off += evaluation_counts[i];
            }
            ctx->join(k);
            ctx->sync();
            off = 0;
            for (size_t i = 0; i < count; i++) {
                std::memcpy(out_evaluations[i], box + off * sizeof(Fr), evaluation_counts[i] * sizeof(Fr));
                off += evaluation_counts[i];
                hp::record_message(states[i], states[i]->round, out_evaluations[i]);
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

namespace hp {

// Whether a kernel profiler is attached (Nsight Compute's injection sets
// these): the resident kernels exchange messages and challenges with the
// host while they run, which a profiled launch does not allow, so under a
// profiler they would wait until their bounded spins ran out; such runs take
// one launch per round instead.
static bool profiler_attached() {
    static const bool v = [] {
        for (const char *name : {"NV_COMPUTE_PROFILER_PERFWORKS_DIR", "NVIDIA_PROCESS_INJECTION_CRASH_REPORTING",
                                 "CUDA_INJECTION64_PATH"}) {
            const char *e = std::getenv(name);
            if (e != nullptr && *e != '\0') return true;
        }
        return false;
    }();
    return v;
}

// HP_SUMCHECK_TAIL=0: no resident tail block (every round a launch of its own).
static bool tail_enabled() {
    static const bool v = env_size("HP_SUMCHECK_TAIL", 1) != 0 && !profiler_attached();
    return v;
}

// Shared memory of the tail block for a first tail round of `pairs` pairs.
static size_t tail_smem(const SumcheckDesc &d, size_t pairs) {
    return (size_t(3 * d.factor_count + d.slot_count) * pairs + size_t(d.slot_count)) * sizeof(Fr);
}

// Pairs of the tail's first round for this state: the largest power of two
// <= kTailMaxPairs (or HP_SUMCHECK_TAIL_PAIRS) whose tables fit 200 KiB of
// shared memory; 0 when the shape takes no tail (products of arity > 8, more
// than kMaxSlotsV2 slots).
static size_t tail_pairs(const HpCudaSumCheckProverState *s) {
    static const size_t cap = std::min<size_t>(kTailMaxPairs, env_size("HP_SUMCHECK_TAIL_PAIRS", kTailMaxPairs));
    const SumcheckDesc &d = s->desc;
    if (!tail_enabled() || cap == 0 || d.product_count == 0 || d.max_arity > 8 || d.slot_count > kMaxSlotsV2)
        return 0;
    size_t p = size_t(1) << ceil_log2_size(cap);
    if (p > cap) p >>= 1;
    while (p > 1 && tail_smem(d, p) > size_t(200) * 1024) p >>= 1;
    return tail_smem(d, p) <= size_t(200) * 1024 ? p : 0;
}

// Rows of a resident-grid tile: the largest power of two <= 128 whose F x 2
// tile rows and the block's reduced sums fit 96 KiB of shared memory.
static int resident_tile(const SumcheckDesc &d) {
    int tile = 128;
    while (tile > 16 && (size_t(d.factor_count) * 2 * tile + kResThreads) * sizeof(Fr) > size_t(96) * 1024)
        tile >>= 1;
    return tile;
}

// First round (in pairs) of the cooperative resident grid for this state
// (HP_SUMCHECK_RESIDENT_PAIRS overrides the rule below; HP_SUMCHECK_RESIDENT=0:
// none); 0 when the shape takes none (products of arity > 8, more than
// kMaxSlotsV2 slots, no products).
static size_t resident_pairs(const HpCudaSumCheckProverState *s) {
    static const bool on = env_size("HP_SUMCHECK_RESIDENT", 1) != 0 && !profiler_attached();
    static const size_t first = env_size("HP_SUMCHECK_RESIDENT_PAIRS", 0);
    const SumcheckDesc &d = s->desc;
    if (!on || d.product_count == 0 || d.max_arity > 8 || d.slot_count > kMaxSlotsV2) return 0;
    if (first > 0) return first;
    // measured on GB300 (nv = 20): 6 tables in 4 arity-2 products (12 slots)
    // gain from 2^17 pairs on (0.935 ms per prove against 0.977 from 2^15);
    // the proof's wider shapes lose from 2^17 (47.09 against 46.85 ms)
    return d.max_arity <= 2 && d.slot_count <= 12 ? size_t(1) << 17 : size_t(1) << 15;
}


// Runs rounds k0.. of `s` in one resident launch -- the cooperative grid
// (`grid`) or the one-block tail -- with the Fiat-Shamir step of each round
// on this thread, writing messages and challenges like the per-round loop of
// hp_cuda_v1_sumcheck_prove_rounds; r_prev is the previous round's
// challenge (k0 > 0).
static void run_resident(HpCudaContext *ctx, HpCudaSumCheckProverState *s, size_t k0, const Fr &r_prev,
                         HpMerlinTranscript *transcript, uint8_t *out_messages, uint8_t *out_challenges,
                         bool grid) {
    // rounds k0 >= 1: the reduced layout, with the claim of round k0 from the
    // recorded message of round k0 - 1 and the host's claims after it
    const SumcheckDesc &d = s->desc_red;
    const size_t nv = s->num_vars, d1 = s->max_degree + 1;
    const int rounds = int(nv - k0);
    const size_t pairs0 = table_len(nv - k0 - 1);
    host::Fr64 r64, claim64;
    std::memcpy(r64.v, r_prev.v, 32);
    if (k0 == 0 || !round_claim(s, r64, claim64)) fail(HP_CUDA_STATUS_INVALID_STATE);
    Fr claim0;
    std::memcpy(claim0.v, claim64.v, 32);
    // handshake: 32-byte header, the challenges, the claims, the messages
    const size_t box_bytes = 32 + size_t(rounds) * sizeof(Fr) * (2 + d1);
    void *box_dev = nullptr;
    uint8_t *box = ctx->mailbox(box_bytes, &box_dev);
    uint32_t *hdr = reinterpret_cast<uint32_t *>(box);
    Fr *challenges = reinterpret_cast<Fr *>(box + 32);
    Fr *claims = challenges + rounds;
    const Fr *messages = claims + rounds;
    Handshake hs;
    hs.hdr = static_cast<uint32_t *>(box_dev);
    hs.challenges = reinterpret_cast<Fr *>(static_cast<uint8_t *>(box_dev) + 32);
    hs.claims = hs.challenges + rounds;
    hs.messages = hs.claims + rounds;
    volatile uint32_t *seq = &hdr[0];
    hdr[0] = hdr[1] = hdr[2] = 0;
    // where the per-round path would leave the tables: one buffer swap per
    // round after the first of the state
    HpCudaSumCheckProverState sim = HpCudaSumCheckProverState();
    sim.round = s->round;
    sim.current = s->current;
    for (int j = 0; j < rounds; j++) advance(&sim);
    int tok = ctx->prof_begin("sumcheck_round", ctx->stream);
    // the Fiat-Shamir loop runs on the context's responder thread, so the
    // launch below may block until the kernel ends
    std::atomic<bool> cancel{false};
    ctx->respond_start([&] {
        std::vector<uint8_t> msg(8 + 32 * d1, 0);
        for (int b = 0; b < 8; b++) msg[b] = uint8_t(uint64_t(d1) >> (8 * b));
        for (int j = 0; j < rounds; j++) {
            // the launch's message j: poll the mapped sequence number; the blocks
            // themselves give up after kTailSpinLimit polls, and a launch that
            // ends without the message is an error
            uint64_t polls = 0;
            const auto t0 = std::chrono::steady_clock::now();
            while (__atomic_load_n(seq, __ATOMIC_ACQUIRE) < uint32_t(j + 1)) {
                if (cancel.load(std::memory_order_relaxed)) fail(HP_CUDA_STATUS_INVALID_STATE);
                if ((++polls & 1023) == 0) {
                    const auto waited = std::chrono::steady_clock::now() - t0;
                    if (waited > std::chrono::seconds(60)) fail(HP_CUDA_STATUS_INVALID_STATE);
                    // a launch that ended without the message (checked only after
                    // 100 ms without one, so that no runtime call competes with a
                    // launch that serialised tools hold open)
                    if (waited > std::chrono::milliseconds(100)) {
                        const cudaError_t e = cudaStreamQuery(ctx->stream);
                        if (e != cudaErrorNotReady) {
                            if (__atomic_load_n(seq, __ATOMIC_ACQUIRE) >= uint32_t(j + 1)) break;
                            check_cuda(e);
                            fail(HP_CUDA_STATUS_INVALID_STATE);
                        }
                    }
                }
            }
            const uint8_t *m = reinterpret_cast<const uint8_t *>(messages + size_t(j) * d1);
            std::memcpy(msg.data() + 8, m, 32 * d1);
            std::memcpy(out_messages + 32 * d1 * (k0 + j), m, 32 * d1);
            merlin_append(transcript, "prover msg", msg.data(), msg.size());
            uint8_t wide[64], canon[32];
            merlin_challenge(transcript, "Internal round", wide, 64);
            const host::Fr64 c = host::from_wide64(wide);
            host::to_canonical(c, canon);
            merlin_append(transcript, "Internal round", canon, 32);
            std::memcpy(out_challenges + 32 * (k0 + j), canon, 32);
            if (j + 1 < rounds) {
                // the next round's claim: this message's polynomial at c
                std::vector<host::Fr64> mv(d1);
                for (size_t x = 0; x < d1; x++)
                    if (!host::from_canonical(m + 32 * x, mv[x])) fail(HP_CUDA_STATUS_INVALID_STATE);
                const host::Fr64 nc = message_at(mv, s->lag_den, c);
                std::memcpy(&claims[j + 1], nc.v, 32);
                std::memcpy(&challenges[j], c.v, 32);
                __atomic_store_n(&hdr[1], uint32_t(j + 1), __ATOMIC_RELEASE);
            }
        }
    });
    try {
        if (grid) {
            FoldBuffers fb;
            for (int f = 0; f < d.factor_count; f++) fb.inputs.p[f] = state_table(s, 0, f);
            fb.a = static_cast<Fr *>(s->fold_a);
            fb.b = static_cast<Fr *>(s->fold_b);
            fb.a_stride = nv >= 1 ? table_len(nv - 1) : 1;
            fb.b_stride = nv >= 2 ? table_len(nv - 2) : 1;
            int which0 = s->current;
            bool fold_first = k0 > 0;
            Fr r0 = r_prev;
            int tile = resident_tile(d);
            const Fr *w = state_weights_red(s);
            int degree = int(s->max_degree);
            uint64_t *limb_sums = static_cast<uint64_t *>(s->partials);  // 2 x 8 x kMaxSlotsV2 counters
            check_cuda(cudaMemsetAsync(limb_sums, 0, 2 * 8 * kMaxSlotsV2 * sizeof(uint64_t), ctx->stream));
            unsigned *counter = round_counter(s);
            uint32_t *relay = state_relay(s);
            size_t p0 = pairs0;
            int nrounds = rounds;
            const size_t smem = (size_t(d.factor_count) * 2 * tile + kResThreads) * sizeof(Fr);
            const size_t sms = size_t(ctx->sm_count > 0 ? ctx->sm_count : 152);
            auto launch = [&](auto kernel) {
                check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
                int per_sm = 0;
                check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kResThreads, smem));
                if (per_sm < 1) fail(HP_CUDA_STATUS_NOT_IMPLEMENTED);
                size_t blocks = sms * size_t(std::min(per_sm, 2));
                blocks = std::max<size_t>(1, std::min(blocks, (pairs0 + kResMinPairs - 1) / kResMinPairs));
                void *args[] = {const_cast<SumcheckDesc *>(&d), &fb, &which0, &fold_first, &r0, &p0, &nrounds,
                                &tile, &w, &degree, &claim0, &limb_sums, &counter, &relay, &hs};
                check_cuda(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(kernel), dim3(unsigned(blocks)),
                                                       dim3(kResThreads), args, smem, ctx->stream));
            };
            if (d.max_arity <= 2) launch(k_sumcheck_resident<2>);
            else if (d.max_arity <= 4) launch(k_sumcheck_resident<4>);
            else if (d.max_arity <= 6) launch(k_sumcheck_resident<6>);
            else launch(k_sumcheck_resident<8>);
        } else {
            FrPtrList src{};
            FrMutPtrList dst{};
            for (int f = 0; f < d.factor_count; f++) {
                src.p[f] = state_table(s, s->current, f);
                dst.p[f] = const_cast<Fr *>(state_table(s, sim.current, f));
            }
            const size_t smem = tail_smem(d, pairs0);
            auto launch = [&](auto kernel) {
                check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
                kernel<<<1, kTailThreads, smem, ctx->stream>>>(d, src, dst, k0 > 0, r_prev, int(pairs0), rounds,
                                                               state_weights_red(s), int(s->max_degree), claim0, hs);
            };
            if (d.max_arity <= 2) launch(k_sumcheck_tail<2>);
            else if (d.max_arity <= 4) launch(k_sumcheck_tail<4>);
            else if (d.max_arity <= 6) launch(k_sumcheck_tail<6>);
            else launch(k_sumcheck_tail<8>);
        }
        check_launch();
    } catch (...) {
        cancel.store(true);
        try {
            ctx->respond_wait();
        } catch (...) {
        }
        throw;
    }
    ctx->respond_wait();
    ctx->sync();
    ctx->prof_end(tok, ctx->stream);
    if (__atomic_load_n(&hdr[2], __ATOMIC_ACQUIRE)) fail(HP_CUDA_STATUS_INVALID_STATE);
    s->round = sim.round;
    s->current = sim.current;
}

}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_sumcheck_prove_rounds(HpCudaContext *ctx, HpCudaSumCheckProverState *s,
                                                         HpMerlinTranscript *transcript, size_t rounds,
                                                         uint8_t *out_messages, uint8_t *out_challenges) {
    return guard([&] {
        hp::require_ctx(ctx);
        require(s != nullptr && transcript != nullptr && out_messages != nullptr && out_challenges != nullptr);
        if (s->poisoned || s->round != 0) fail(HP_CUDA_STATUS_INVALID_STATE);
        require(rounds == s->num_vars);
        const size_t d1 = s->max_degree + 1;
        // each round's kernel writes its message into the mapped mailbox
        void *box_dev = nullptr;
        const uint8_t *box = ctx->mailbox(32 * d1, &box_dev);
        // "prover msg" payload: u64 LE element count, then the canonical elements
        std::vector<uint8_t> msg(8 + 32 * d1, 0);
        for (int b = 0; b < 8; b++) msg[b] = uint8_t(uint64_t(d1) >> (8 * b));
        Fr r = Fr::zero();
        const size_t resident = hp::resident_pairs(s);
        const size_t tail = resident ? 0 : hp::tail_pairs(s);
        for (size_t k = 0; k < rounds; k++) {
            const size_t pairs = hp::table_len(rounds - k - 1);
            if (k > 0 && ((resident > 0 && pairs <= resident) || (tail > 0 && pairs <= tail))) {
                // this and every later round in one resident launch (from the
                // second round on: the resident kernels take the reduced layout)
                try {
                    hp::run_resident(ctx, s, k, r, transcript, out_messages, out_challenges, resident > 0);
                } catch (const hp::Failure &f) {
                    if (f.kind == HP_CUDA_STATUS_INVALID_STATE) s->poisoned = true;
                    throw;
                }
                break;
            }
            try {
                hp::enqueue_round(ctx, s, r, ctx->stream, static_cast<Fr *>(box_dev));
                ctx->sync();
                hp::record_message(s, k, box);
                hp::advance(s);
            } catch (const hp::Failure &f) {
                if (f.kind == HP_CUDA_STATUS_INVALID_STATE) s->poisoned = true;
                throw;
            }
            std::memcpy(msg.data() + 8, box, 32 * d1);
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

// Sumcheck round autotuner: runs every round of `s` (a fresh state, which it
// consumes) once per candidate route -- each kernel family that can run the
// round, at a few grid sizes -- times each as the median of a few runs with
// CUDA events on the context stream, checks that every candidate's message
// equals the built-in rule's, and stores the fastest route for the round's
// key (ceil log2 pairs, largest arity, slot count) in the process-wide
// tuning table; then runs the round along it and advances.  Challenges are
// fixed small values (the route does not depend on them).
namespace hp {
namespace {

const RoundRoute kRouteCandidates[] = {
    {kRouteOneBlock, 0}, {kRoutePerPair, 0}, {kRouteSlot, 0},      {kRouteSlot, 4},  {kRouteSlot, 8},
    {kRouteSlot, 16},    {kRouteSlot, 32},   {kRouteSlotFused, 0}, {kRouteSlotFused, 16},
    {kRoutePp, 2},       {kRoutePp, 3},      {kRoutePp, 6},        {kRoutePpFused, 3},
    {kRouteTiled, 1},    {kRouteTiled, 2},
};

bool same_route(const RoundRoute &a, const RoundRoute &b) { return a.kernel == b.kernel && a.per_sm == b.per_sm; }

}  // namespace
}  // namespace hp

extern "C" HpCudaStatus hp_cuda_v1_sumcheck_autotune(HpCudaContext *ctx, HpCudaSumCheckProverState *s,
                                                     HpCudaRoundTuning *out, size_t capacity, size_t *out_count) {
    if (out_count) *out_count = 0;
    return guard([&] {
        using namespace hp;
        require_ctx(ctx);
        require(s != nullptr && out != nullptr && out_count != nullptr);
        if (s->poisoned || s->round != 0) fail(HP_CUDA_STATUS_INVALID_STATE);
        require(capacity >= s->num_vars);
        const size_t d1 = s->max_degree + 1;
        void *box_dev = nullptr;
        const uint8_t *box = ctx->mailbox(d1 * sizeof(Fr), &box_dev);
        Fr *msg_dev = static_cast<Fr *>(box_dev);
        cudaEvent_t a = nullptr, b = nullptr;
        check_cuda(cudaEventCreate(&a));
        check_cuda(cudaEventCreate(&b));
        struct Events {
            cudaEvent_t &a, &b;
            ~Events() {
                cudaEventDestroy(a);
                cudaEventDestroy(b);
            }
        } events{a, b};
        try {
            for (size_t k = 0; k < s->num_vars; k++) {
                uint8_t cb[32] = {0};
                cb[0] = uint8_t(k + 2);
                const Fr r = k == 0 ? Fr::zero() : host_scalar(cb);
                const RoundShape sh = round_shape(s);
                const RoundRoute dflt = default_route(sh);
                if (!route_valid(sh, dflt)) fail(HP_CUDA_STATUS_NOT_IMPLEMENTED);
                auto run_once = [&](const RoundRoute &rt) {
                    launch_round(ctx, s, r, ctx->stream, msg_dev, sh, rt);
                };
                auto timed = [&](const RoundRoute &rt) {
                    const int reps = sh.pairs >= (size_t(1) << 16) ? 5 : 9;
                    std::vector<float> ms;
                    for (int i = 0; i < reps; i++) {
                        check_cuda(cudaEventRecord(a, ctx->stream));
                        run_once(rt);
                        check_cuda(cudaEventRecord(b, ctx->stream));
                        check_cuda(cudaEventSynchronize(b));
                        float t = 0.f;
                        check_cuda(cudaEventElapsedTime(&t, a, b));
                        ms.push_back(t);
                    }
                    std::sort(ms.begin(), ms.end());
                    return double(ms[ms.size() / 2]) * 1e3;  // us
                };
                // the built-in rule's message is the one every candidate must give
                run_once(dflt);
                ctx->sync();
                std::vector<uint8_t> want(box, box + d1 * sizeof(Fr));
                const double dflt_us = timed(dflt);
                RoundRoute best = dflt;
                double best_us = dflt_us;
                for (const RoundRoute &cand : kRouteCandidates) {
                    if (same_route(cand, dflt) || !route_valid(sh, cand)) continue;
                    run_once(cand);
                    ctx->sync();
                    if (std::memcmp(box, want.data(), want.size()) != 0) fail(HP_CUDA_STATUS_INVALID_STATE);
                    const double us = timed(cand);
                    if (us < best_us * 0.98) {
                        best = cand;
                        best_us = us;
                    }
                }
                sumcheck_route_store(RoundKey{ceil_log2_size(sh.pairs), sh.max_arity, sh.slots, sh.fold ? 1 : 0},
                                     best, best_us);
                run_once(best);
                ctx->sync();
                record_message(s, k, box);
                advance(s);
                HpCudaRoundTuning &o = out[k];
                o.pairs = uint64_t(sh.pairs);
                o.kernel = best.kernel;
                o.blocks_per_sm = best.per_sm;
                o.default_kernel = dflt.kernel;
                o.default_blocks_per_sm = dflt.per_sm;
                o.default_us = dflt_us;
                o.tuned_us = best_us;
                *out_count = k + 1;
            }
        } catch (const Failure &f) {
            if (f.kind == HP_CUDA_STATUS_INVALID_STATE) s->poisoned = true;
            throw;
        }
    });
}

extern "C" HpCudaStatus hp_cuda_v1_sumcheck_route_query(size_t pairs, int32_t max_arity, int32_t slots,
                                                        int32_t fold, uint32_t *out2) {
    return guard([&] {
        using namespace hp;
        require(out2 != nullptr && pairs >= 1 && max_arity >= 1 && slots >= 1);
        RoundShape sh;
        sh.pairs = pairs;
        sh.fold = fold != 0;
        sh.regs = max_arity <= 8 && slots <= kMaxSlotsV2;
        sh.all_written = true;
        sh.products = true;
        sh.eq = false;  // the generic shape: zero-check states are recognised per state
        sh.max_arity = max_arity;
        sh.slots = slots;
        const RoundRoute rt = chosen_route(sh);
        out2[0] = rt.kernel;
        out2[1] = rt.per_sm;
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
