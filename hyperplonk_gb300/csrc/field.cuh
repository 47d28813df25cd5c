// field.cuh -- BLS12-381 Fr (8 x 32-bit limbs) and Fq (12 x 32-bit limbs)
// Montgomery arithmetic for sm_103a, register resident, carry chains in PTX.
//
// Storage on the device is Montgomery form with R = 2^256 (Fr) / 2^384 (Fq),
// little-endian 32-bit limbs, so one Fr element is 32 contiguous bytes and one
// Fq element 48.  This matches the reference's field semantics (arkworks
// ark-bls12-381 0.6.0 Fr/Fq, canonical packets backend/src/ascend910b3/
// encoding.rs:12-108); the limb layout is this library's own.
#pragma once
#include <cstdint>

namespace hp {

// ---------------------------------------------------------------------------
// PTX carry-chain primitives.  Each is one SASS integer instruction; they are
// asm volatile so the carry flag flows between consecutive calls unchanged.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t add_cc(uint32_t a, uint32_t b) {
    uint32_t r; asm volatile("add.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r;
}
__device__ __forceinline__ uint32_t addc_cc(uint32_t a, uint32_t b) {
    uint32_t r; asm volatile("addc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r;
}
__device__ __forceinline__ uint32_t addc(uint32_t a, uint32_t b) {
    uint32_t r; asm volatile("addc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r;
}
__device__ __forceinline__ uint32_t sub_cc(uint32_t a, uint32_t b) {
    uint32_t r; asm volatile("sub.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r;
}
__device__ __forceinline__ uint32_t subc_cc(uint32_t a, uint32_t b) {
    uint32_t r; asm volatile("subc.cc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r;
}
__device__ __forceinline__ uint32_t subc(uint32_t a, uint32_t b) {
    uint32_t r; asm volatile("subc.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b)); return r;
}

// ---------------------------------------------------------------------------
// Moduli.  P: modulus limbs, INV: -P^-1 mod 2^32, ONE: R mod P, R2: R^2 mod P.
// ---------------------------------------------------------------------------
struct FrParams {
    static constexpr int N = 8;
    static constexpr uint32_t INV = 0xffffffffu;
    static constexpr bool LAZY = false;  // 4r > 2^256: values kept in [0, r)
    __host__ __device__ __forceinline__ static uint32_t p(int i) {
        constexpr uint32_t P[8] = {0x00000001u, 0xffffffffu, 0xfffe5bfeu, 0x53bda402u,
                                   0x09a1d805u, 0x3339d808u, 0x299d7d48u, 0x73eda753u};
        return P[i];
    }
    __device__ __forceinline__ static uint32_t one(int i) {
        constexpr uint32_t R[8] = {0xfffffffeu, 0x00000001u, 0x00034802u, 0x5884b7fau,
                                   0xecbc4ff5u, 0x998c4fefu, 0xacc5056fu, 0x1824b159u};
        return R[i];
    }
    __device__ __forceinline__ static uint32_t r2(int i) {
        constexpr uint32_t R2[8] = {0xf3f29c6du, 0xc999e990u, 0x87925c23u, 0x2b6cedcbu,
                                    0x7254398fu, 0x05d31496u, 0x9f59ff11u, 0x0748d9d9u};
        return R2[i];
    }
};

// Fq values are kept in [0, 2p) between operations ("lazy" reduction): as
// 4p < 2^384 = R, a Montgomery product of two such values is already < 2p
// without its final subtraction; sums and differences reduce against 2p; a
// value is zero when it is 0 or p; from_mont returns the canonical value.
struct FqParams {
    static constexpr int N = 12;
    static constexpr uint32_t INV = 0xfffcfffdu;
    static constexpr bool LAZY = true;
    __device__ __forceinline__ static uint32_t p2(int i) {
        constexpr uint32_t P2[12] = {0xffff5556u, 0x73fdffffu, 0x62a7ffffu, 0x3d57fffdu,
                                     0xed61ec48u, 0xce61a541u, 0xe70a257eu, 0xc8ee9709u,
                                     0x869759aeu, 0x96374f6cu, 0x72ffcd34u, 0x340223d4u};
        return P2[i];
    }
    __host__ __device__ __forceinline__ static uint32_t p(int i) {
        constexpr uint32_t P[12] = {0xffffaaabu, 0xb9feffffu, 0xb153ffffu, 0x1eabfffeu,
                                    0xf6b0f624u, 0x6730d2a0u, 0xf38512bfu, 0x64774b84u,
                                    0x434bacd7u, 0x4b1ba7b6u, 0x397fe69au, 0x1a0111eau};
        return P[i];
    }
    __device__ __forceinline__ static uint32_t one(int i) {
        constexpr uint32_t R[12] = {0x0002fffdu, 0x76090000u, 0xc40c0002u, 0xebf4000bu,
                                    0x53c758bau, 0x5f489857u, 0x70525745u, 0x77ce5853u,
                                    0xa256ec6du, 0x5c071a97u, 0xfa80e493u, 0x15f65ec3u};
        return R[i];
    }
    __device__ __forceinline__ static uint32_t r2(int i) {
        constexpr uint32_t R2[12] = {0x1c341746u, 0xf4df1f34u, 0x09d104f1u, 0x0a76e6a6u,
                                     0x4c95b6d5u, 0x8de5476cu, 0x939d83c0u, 0x67eb88a9u,
                                     0xb519952du, 0x9a793e85u, 0x92cae3aau, 0x11988fe5u};
        return R2[i];
    }
};

template <class P>
struct Field {
    static constexpr int N = P::N;
    uint32_t v[N];

    __host__ __device__ __forceinline__ static Field zero() {
        Field r;
#pragma unroll
        for (int i = 0; i < N; i++) r.v[i] = 0;
        return r;
    }
    __device__ __forceinline__ static Field one() {
        Field r;
#pragma unroll
        for (int i = 0; i < N; i++) r.v[i] = P::one(i);
        return r;
    }
    __host__ __device__ __forceinline__ bool is_zero() const {
        uint32_t acc = 0, accp = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            acc |= v[i];
            accp |= v[i] ^ P::p(i);
        }
        return acc == 0 || (P::LAZY && accp == 0);
    }
    __device__ __forceinline__ bool operator==(const Field &o) const;
    __device__ __forceinline__ bool operator!=(const Field &o) const { return !(*this == o); }
};

using Fr = Field<FrParams>;
using Fq = Field<FqParams>;

// r = a - p if a >= p (a < 2p assumed, with `hi` the carry-out limb)
template <class P>
__device__ __forceinline__ void reduce_once(Field<P> &r, uint32_t hi) {
    constexpr int N = P::N;
    uint32_t t[N];
    t[0] = sub_cc(r.v[0], P::p(0));
#pragma unroll
    for (int i = 1; i < N; i++) t[i] = subc_cc(r.v[i], P::p(i));
    uint32_t borrow = subc(hi, 0);  // 0xffffffff if r < p (and no carry), else 0
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = borrow ? r.v[i] : t[i];
}

// r = a - 2p if a >= 2p (lazy Fq: a < 4p < 2^384, no carry-out limb)
template <class P>
__device__ __forceinline__ void reduce_2p(Field<P> &r) {
    constexpr int N = P::N;
    uint32_t t[N];
    t[0] = sub_cc(r.v[0], P::p2(0));
#pragma unroll
    for (int i = 1; i < N; i++) t[i] = subc_cc(r.v[i], P::p2(i));
    uint32_t borrow = subc(0, 0);
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = borrow ? r.v[i] : t[i];
}

template <class P>
__device__ __forceinline__ Field<P> operator+(const Field<P> &a, const Field<P> &b) {
    constexpr int N = P::N;
    Field<P> r;
    r.v[0] = add_cc(a.v[0], b.v[0]);
#pragma unroll
    for (int i = 1; i < N; i++) r.v[i] = addc_cc(a.v[i], b.v[i]);
    uint32_t hi = addc(0, 0);
    if constexpr (P::LAZY) {
        (void)hi;
        reduce_2p<P>(r);
    } else {
        reduce_once<P>(r, hi);
    }
    return r;
}

template <class P>
__device__ __forceinline__ Field<P> operator-(const Field<P> &a, const Field<P> &b) {
    constexpr int N = P::N;
    Field<P> r;
    r.v[0] = sub_cc(a.v[0], b.v[0]);
#pragma unroll
    for (int i = 1; i < N; i++) r.v[i] = subc_cc(a.v[i], b.v[i]);
    uint32_t borrow = subc(0, 0);  // 0xffffffff on borrow
    uint32_t t[N], m[N];
#pragma unroll
    for (int i = 0; i < N; i++) {
        if constexpr (P::LAZY) m[i] = P::p2(i) & borrow;
        else m[i] = P::p(i) & borrow;
    }
    t[0] = add_cc(r.v[0], m[0]);
#pragma unroll
    for (int i = 1; i < N - 1; i++) t[i] = addc_cc(r.v[i], m[i]);
    t[N - 1] = addc(r.v[N - 1], m[N - 1]);
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = t[i];
    return r;
}

template <class P>
__device__ __forceinline__ Field<P> neg(const Field<P> &a) {
    return Field<P>::zero() - a;
}

template <class P>
__device__ __forceinline__ Field<P> dbl(const Field<P> &a) {
    return a + a;
}

// CIOS Montgomery multiplication with 32x32 -> 64-bit multiply-adds: each
// partial product a_j * b_i + t_j + carry fits 64 bits, so one wide multiply
// and one 64-bit add replace separate low-half and high-half multiply-add
// chains (mad.lo.cc / madc.hi.cc); the high half of a 32x32 product costs
// two multiply issues on this GPU, the wide form fewer (probe on GB300, 12
// limbs: 20.7 G/s vs 19.9 G/s for the low/high form out of line, 25.3 G/s
// inlined with two products interleaved; 8 limbs: 63 vs 45 G/s).
template <class P>
__device__ __forceinline__ Field<P> mont_mul_wide(const Field<P> &a, const Field<P> &b) {
    constexpr int N = P::N;
    uint32_t t[N + 2];
#pragma unroll
    for (int i = 0; i < N + 2; i++) t[i] = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t bi = b.v[i];
        uint32_t carry = 0;
#pragma unroll
        for (int j = 0; j < N; j++) {
            const uint64_t d = uint64_t(a.v[j]) * bi + (uint64_t(t[j]) + carry);
            t[j] = uint32_t(d);
            carry = uint32_t(d >> 32);
        }
        uint64_t top = uint64_t(t[N]) + carry;
        t[N] = uint32_t(top);
        t[N + 1] = uint32_t(top >> 32);
        // t += m * p with t[0] becoming 0, shifted down one limb on the fly
        const uint32_t m = t[0] * P::INV;
        uint64_t d = uint64_t(m) * P::p(0) + t[0];
        carry = uint32_t(d >> 32);
#pragma unroll
        for (int j = 1; j < N; j++) {
            d = uint64_t(m) * P::p(j) + (uint64_t(t[j]) + carry);
            t[j - 1] = uint32_t(d);
            carry = uint32_t(d >> 32);
        }
        top = uint64_t(t[N]) + carry;
        t[N - 1] = uint32_t(top);
        t[N] = t[N + 1] + uint32_t(top >> 32);
        t[N + 1] = 0;
    }
    Field<P> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = t[i];
    if constexpr (!P::LAZY) reduce_once<P>(r, t[N]);  // lazy: already < 2p
    return r;
}

// Montgomery squaring, separated operand scanning: the 2N-limb square from
// the N(N-1)/2 cross products (doubled by one shift) plus the N diagonal
// squares -- (N^2 + N)/2 wide products instead of N^2 -- then N rows of
// Montgomery reduction; the carry out of each row's top limb is held in c2
// and added one limb higher in the next row.
template <class P>
__device__ __forceinline__ Field<P> mont_sqr_wide(const Field<P> &a) {
    constexpr int N = P::N;
    uint32_t T[2 * N];
#pragma unroll
    for (int i = 0; i < 2 * N; i++) T[i] = 0;
#pragma unroll
    for (int i = 0; i < N - 1; i++) {
        uint32_t carry = 0;
#pragma unroll
        for (int j = i + 1; j < N; j++) {
            const uint64_t d = uint64_t(a.v[i]) * a.v[j] + (uint64_t(T[i + j]) + carry);
            T[i + j] = uint32_t(d);
            carry = uint32_t(d >> 32);
        }
        T[i + N] = carry;
    }
    // T = 2 T (cross products < 2^(64N - 1), so no bit is lost)
#pragma unroll
    for (int k = 2 * N - 1; k > 0; k--) T[k] = (T[k] << 1) | (T[k - 1] >> 31);
    T[0] <<= 1;
    // + diagonal squares a_i^2 at limb 2i
    {
        uint32_t dg[2 * N];
#pragma unroll
        for (int i = 0; i < N; i++) {
            const uint64_t d = uint64_t(a.v[i]) * a.v[i];
            dg[2 * i] = uint32_t(d);
            dg[2 * i + 1] = uint32_t(d >> 32);
        }
        T[0] = add_cc(T[0], dg[0]);
#pragma unroll
        for (int k = 1; k < 2 * N; k++) T[k] = addc_cc(T[k], dg[k]);
    }
    uint32_t c2 = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t m = T[i] * P::INV;
        uint32_t carry = 0;
#pragma unroll
        for (int j = 0; j < N; j++) {
            const uint64_t d = uint64_t(m) * P::p(j) + (uint64_t(T[i + j]) + carry);
            T[i + j] = uint32_t(d);
            carry = uint32_t(d >> 32);
        }
        // T[i+N] += carry + c2 (c2: carries still owed to limb i+N)
        T[i + N] = add_cc(T[i + N], carry);
        uint32_t c = addc(0, 0);
        T[i + N] = add_cc(T[i + N], c2);
        c2 = addc(c, 0);
    }
    Field<P> r;
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = T[N + i];
    if constexpr (!P::LAZY) reduce_once<P>(r, c2);  // lazy: already < 2p
    return r;
}

// Karatsuba form of the 12-limb product, the library's out-of-line Fq
// product (HP_FQ_SCHOOLBOOK selects mont_mul_wide instead): three 6x6-limb
// schoolbook products (108 wide multiply-adds instead of 144) for the
// 24-limb a*b, then 12 rows of Montgomery reduction as in mont_sqr_wide
// (2^20 MSM on GB300: 8.50 ms vs 9.04 ms; a second Karatsuba level on the
// 6-limb halves measured slower, 8.77 ms).
template <int M>
__device__ __forceinline__ void school_wide(const uint32_t *a, const uint32_t *b, uint32_t *z) {
#pragma unroll
    for (int i = 0; i < 2 * M; i++) z[i] = 0;
#pragma unroll
    for (int i = 0; i < M; i++) {
        uint32_t carry = 0;
#pragma unroll
        for (int j = 0; j < M; j++) {
            const uint64_t d = uint64_t(a[j]) * b[i] + (uint64_t(z[i + j]) + carry);
            z[i + j] = uint32_t(d);
            carry = uint32_t(d >> 32);
        }
        z[i + M] = carry;
    }
}

__device__ __forceinline__ Field<FqParams> fq_mul_karatsuba(const Field<FqParams> &a, const Field<FqParams> &b) {
    uint32_t T[24], z0[12], z2[12], z1[14];
    school_wide<6>(a.v, b.v, z0);
    school_wide<6>(a.v + 6, b.v + 6, z2);
    // (a0 + a1)(b0 + b1) with the 193-bit sums split as s + c 2^192
    uint32_t sa[6], sb[6];
    sa[0] = add_cc(a.v[0], a.v[6]);
#pragma unroll
    for (int i = 1; i < 6; i++) sa[i] = addc_cc(a.v[i], a.v[i + 6]);
    const uint32_t ca = addc(0, 0);
    sb[0] = add_cc(b.v[0], b.v[6]);
#pragma unroll
    for (int i = 1; i < 6; i++) sb[i] = addc_cc(b.v[i], b.v[i + 6]);
    const uint32_t cb = addc(0, 0);
    school_wide<6>(sa, sb, z1);
    z1[12] = ca & cb;
    z1[13] = 0;
    uint32_t ma[6], mb[6];
#pragma unroll
    for (int i = 0; i < 6; i++) {
        ma[i] = sb[i] & (0u - ca);
        mb[i] = sa[i] & (0u - cb);
    }
    z1[6] = add_cc(z1[6], ma[0]);
#pragma unroll
    for (int i = 1; i < 6; i++) z1[6 + i] = addc_cc(z1[6 + i], ma[i]);
    z1[12] = addc_cc(z1[12], 0);
    z1[13] = addc(z1[13], 0);
    z1[6] = add_cc(z1[6], mb[0]);
#pragma unroll
    for (int i = 1; i < 6; i++) z1[6 + i] = addc_cc(z1[6 + i], mb[i]);
    z1[12] = addc_cc(z1[12], 0);
    z1[13] = addc(z1[13], 0);
    // middle = z1 - z0 - z2 (= a0 b1 + a1 b0 >= 0)
    z1[0] = sub_cc(z1[0], z0[0]);
#pragma unroll
    for (int i = 1; i < 12; i++) z1[i] = subc_cc(z1[i], z0[i]);
    z1[12] = subc_cc(z1[12], 0);
    z1[13] = subc(z1[13], 0);
    z1[0] = sub_cc(z1[0], z2[0]);
#pragma unroll
    for (int i = 1; i < 12; i++) z1[i] = subc_cc(z1[i], z2[i]);
    z1[12] = subc_cc(z1[12], 0);
    z1[13] = subc(z1[13], 0);
    // T = z0 + middle 2^192 + z2 2^384  (a b < p^2 < 2^768: no carry out of T[23])
#pragma unroll
    for (int i = 0; i < 12; i++) {
        T[i] = z0[i];
        T[12 + i] = z2[i];
    }
    T[6] = add_cc(T[6], z1[0]);
#pragma unroll
    for (int i = 1; i < 14; i++) T[6 + i] = addc_cc(T[6 + i], z1[i]);
#pragma unroll
    for (int i = 20; i < 24; i++) T[i] = addc_cc(T[i], 0);
    uint32_t c2 = 0;
#pragma unroll
    for (int i = 0; i < 12; i++) {
        const uint32_t m = T[i] * FqParams::INV;
        uint32_t carry = 0;
#pragma unroll
        for (int j = 0; j < 12; j++) {
            const uint64_t d = uint64_t(m) * FqParams::p(j) + (uint64_t(T[i + j]) + carry);
            T[i + j] = uint32_t(d);
            carry = uint32_t(d >> 32);
        }
        T[i + 12] = add_cc(T[i + 12], carry);
        const uint32_t c = addc(0, 0);
        T[i + 12] = add_cc(T[i + 12], c2);
        c2 = addc(c, 0);
    }
    Field<FqParams> r;
#pragma unroll
    for (int i = 0; i < 12; i++) r.v[i] = T[12 + i];
    (void)c2;  // lazy Fq: the result is < 2p < 2^382, c2 = 0
    return r;
}

struct FqPair;

// The 12-limb product is ~700 SASS instructions; inlined at every call site
// of a curve formula it overflows the instruction cache (ncu: instruction
// fetch stalls dominate the MSM bucket kernel), so Fq products go through an
// out-of-line copy per translation unit.  Arguments travel by value in
// registers.  The curve formulas name their independent products in pairs
// (mul2); building with HP_FQ_PAIR sends each pair through one out-of-line
// call whose two multiply chains interleave -- faster alone (probe: 23.0 vs
// 20.7 G/s) but slower in the bucket kernel, where the extra live registers
// spill (2^20 MSM 10.1-10.5 ms paired vs 9.2 ms single).
#ifndef HP_FQ_INLINE
static __device__ __noinline__ Field<FqParams> fq_mul_call(Field<FqParams> a, Field<FqParams> b) {
#ifndef HP_FQ_SCHOOLBOOK
    return fq_mul_karatsuba(a, b);
#else
    return mont_mul_wide<FqParams>(a, b);
#endif
}
#endif

template <class P>
__device__ __forceinline__ Field<P> operator*(const Field<P> &a, const Field<P> &b) {
    if constexpr (P::N == 12) {
#ifndef HP_FQ_INLINE
        return fq_mul_call(a, b);
#else
        return mont_mul_wide<P>(a, b);
#endif
    }
    // Fr (8 limbs) inlined: probe on GB300 63 G/s wide vs 45 G/s low/high CIOS
    return mont_mul_wide<P>(a, b);
}

struct FqPair {
    Field<FqParams> x, y;
};

#if !defined(HP_FQ_INLINE) && defined(HP_FQ_PAIR)
static __device__ __noinline__ FqPair fq_mul2_call(Field<FqParams> a, Field<FqParams> b, Field<FqParams> c,
                                                   Field<FqParams> d) {
    FqPair r;
    r.x = mont_mul_wide<FqParams>(a, b);
    r.y = mont_mul_wide<FqParams>(c, d);
    return r;
}
#endif

// (x, y) = (a * b, c * d): two independent Fq products in one call.
__device__ __forceinline__ void mul2(Field<FqParams> &x, Field<FqParams> &y, const Field<FqParams> &a,
                                     const Field<FqParams> &b, const Field<FqParams> &c,
                                     const Field<FqParams> &d) {
#if defined(HP_FQ_PAIR) && !defined(HP_FQ_INLINE)
    const FqPair r = fq_mul2_call(a, b, c, d);
    x = r.x;
    y = r.y;
#elif !defined(HP_FQ_INLINE)
    x = fq_mul_call(a, b);
    y = fq_mul_call(c, d);
#else
    x = mont_mul_wide<FqParams>(a, b);
    y = mont_mul_wide<FqParams>(c, d);
#endif
}

// Fq squaring: HP_FQ_SQR=0 multiplies (a * a), 1 calls an out-of-line
// squaring, 2 inlines it.
#ifndef HP_FQ_SQR
#define HP_FQ_SQR 0
#endif
#if HP_FQ_SQR == 1 && !defined(HP_FQ_INLINE)
static __device__ __noinline__ Field<FqParams> fq_sqr_call(Field<FqParams> a) {
    return mont_sqr_wide<FqParams>(a);
}
#endif

template <class P>
__device__ __forceinline__ Field<P> sqr(const Field<P> &a) {
    if constexpr (P::N == 12) {
#if HP_FQ_SQR == 1 && !defined(HP_FQ_INLINE)
        return fq_sqr_call(a);
#elif HP_FQ_SQR >= 1
        return mont_sqr_wide<P>(a);
#endif
    }
    return a * a;
}

// Montgomery form <-> canonical integer.
template <class P>
__device__ __forceinline__ Field<P> to_mont(const Field<P> &canonical) {
    Field<P> r2;
#pragma unroll
    for (int i = 0; i < P::N; i++) r2.v[i] = P::r2(i);
    return canonical * r2;
}
template <class P>
__device__ __forceinline__ Field<P> from_mont(const Field<P> &a) {
    Field<P> one = Field<P>::zero();
    one.v[0] = 1;
    Field<P> r = a * one;
    if constexpr (P::LAZY) reduce_once<P>(r, 0u);  // [0, 2p) -> canonical
    return r;
}

// The value in [0, p) (lazy Fq values may hold v + p).
template <class P>
__device__ __forceinline__ Field<P> canonical(const Field<P> &a) {
    Field<P> r = a;
    if constexpr (P::LAZY) reduce_once<P>(r, 0u);
    return r;
}

template <class P>
__device__ __forceinline__ bool Field<P>::operator==(const Field<P> &o) const {
    const Field<P> a = canonical(*this), b = canonical(o);
    uint32_t acc = 0;
#pragma unroll
    for (int i = 0; i < N; i++) acc |= a.v[i] ^ b.v[i];
    return acc == 0;
}

// True if the integer held in a is < p (canonical).
template <class P>
__device__ __forceinline__ bool is_canonical(const Field<P> &a) {
    constexpr int N = P::N;
    uint32_t t = sub_cc(a.v[0], P::p(0));
#pragma unroll
    for (int i = 1; i < N; i++) t = subc_cc(a.v[i], P::p(i));
    (void)t;
    uint32_t borrow = subc(0, 0);
    return borrow != 0;
}

// a^(p-2) by square-and-multiply over the modulus bits (p is odd, > 2).
// Modular inverse by the binary extended Euclidean algorithm (variable
// time; the method of arkworks' Fp::inverse, Guajardo, Kumar, Paar and Pelzl
// 2006, "Efficient software-implementation of finite fields with
// applications to cryptography", Algorithm 16).  It runs on the Montgomery
// representation A = aR: x1 = R^2, x2 = 0 keep x1 A = u R^2 and x2 A = v R^2
// (mod p) through every halving and subtraction, so when u (or v) reaches 1,
// x1 (or x2) = R^2 / (aR) = R / a, the Montgomery form of 1/a.  Each step is a
// few limb-wide shifts, adds and subtracts: a chain of about 2 log2 p short
// steps instead of the ~log2 p dependent multiplications of a^(p-2).  0 has no
// inverse and returns 0 (as a^(p-2) does).  The loops are bounded: there are
// at most log2 A + log2 p halvings and one subtraction more than halvings
// (each difference of two odd values is even), under 4 * 32N steps in all;
// the budget is 6 * 32N, and a budget that ran out would return 0 instead of
// spinning.
template <int N>
__device__ __forceinline__ bool limbs_is_one(const uint32_t *x) {
    uint32_t acc = x[0] ^ 1u;
#pragma unroll
    for (int i = 1; i < N; i++) acc |= x[i];
    return acc == 0;
}

// x = x / 2 mod p for x < p: (x + p) / 2 when x is odd (the sum's carry is
// the top bit of the shifted value)
template <class P>
__device__ __forceinline__ void limbs_half_mod(uint32_t *x) {
    constexpr int N = P::N;
    uint32_t top = 0;
    if (x[0] & 1u) {
        x[0] = add_cc(x[0], P::p(0));
#pragma unroll
        for (int i = 1; i < N; i++) x[i] = addc_cc(x[i], P::p(i));
        top = addc(0u, 0u);
    }
#pragma unroll
    for (int i = 0; i < N - 1; i++) x[i] = __funnelshift_r(x[i], x[i + 1], 1);
    x[N - 1] = (x[N - 1] >> 1) | (top << 31);
}

template <int N>
__device__ __forceinline__ void limbs_shr1(uint32_t *x) {
#pragma unroll
    for (int i = 0; i < N - 1; i++) x[i] = __funnelshift_r(x[i], x[i + 1], 1);
    x[N - 1] >>= 1;
}

// x -= y; returns the borrow (1 when y > x)
template <int N>
__device__ __forceinline__ uint32_t limbs_sub(uint32_t *x, const uint32_t *y) {
    x[0] = sub_cc(x[0], y[0]);
#pragma unroll
    for (int i = 1; i < N; i++) x[i] = subc_cc(x[i], y[i]);
    return subc(0u, 0u) & 1u;
}

// x = x - y mod p for x, y < p
template <class P>
__device__ __forceinline__ void limbs_sub_mod(uint32_t *x, const uint32_t *y) {
    constexpr int N = P::N;
    if (limbs_sub<N>(x, y)) {
        x[0] = add_cc(x[0], P::p(0));
#pragma unroll
        for (int i = 1; i < N - 1; i++) x[i] = addc_cc(x[i], P::p(i));
        x[N - 1] = addc(x[N - 1], P::p(N - 1));
    }
}

template <class P>
__device__ __noinline__ Field<P> inverse(const Field<P> &a) {
    constexpr int N = P::N;
    uint32_t u[N], v[N], x1[N], x2[N];
#pragma unroll
    for (int i = 0; i < N; i++) {
        u[i] = a.v[i];
        v[i] = P::p(i);
        x1[i] = P::r2(i);
        x2[i] = 0;
    }
    if (P::LAZY) {  // [0, 2p) -> [0, p)
        uint32_t t[N];
#pragma unroll
        for (int i = 0; i < N; i++) t[i] = u[i];
        if (!limbs_sub<N>(t, v)) {
#pragma unroll
            for (int i = 0; i < N; i++) u[i] = t[i];
        }
    }
    uint32_t nz = 0;
#pragma unroll
    for (int i = 0; i < N; i++) nz |= u[i];
    if (nz == 0) return Field<P>::zero();
    constexpr int kBits = 32 * N;
    int budget = 6 * kBits;
    while (!limbs_is_one<N>(u) && !limbs_is_one<N>(v) && budget > 0) {
        while ((u[0] & 1u) == 0 && budget > 0) {
            limbs_shr1<N>(u);
            limbs_half_mod<P>(x1);
            budget--;
        }
        while ((v[0] & 1u) == 0 && budget > 0) {
            limbs_shr1<N>(v);
            limbs_half_mod<P>(x2);
            budget--;
        }
        // u, v odd: the larger loses the smaller
        uint32_t t[N];
#pragma unroll
        for (int i = 0; i < N; i++) t[i] = u[i];
        if (!limbs_sub<N>(t, v)) {
#pragma unroll
            for (int i = 0; i < N; i++) u[i] = t[i];
            limbs_sub_mod<P>(x1, x2);
        } else {
            limbs_sub<N>(v, u);
            limbs_sub_mod<P>(x2, x1);
        }
        budget--;
    }
    Field<P> r;
    const bool u1 = limbs_is_one<N>(u), v1 = limbs_is_one<N>(v);
#pragma unroll
    for (int i = 0; i < N; i++) r.v[i] = u1 ? x1[i] : v1 ? x2[i] : 0u;
    return r;
}

// Small integer in Montgomery form.
template <class P>
__device__ __forceinline__ Field<P> from_u32(uint32_t x) {
    Field<P> t = Field<P>::zero();
    t.v[0] = x;
    return to_mont(t);
}

// ---------------------------------------------------------------------------
// Global-memory helpers (AoS, 16-byte vector accesses)
// ---------------------------------------------------------------------------
__device__ __forceinline__ Fr load_fr(const Fr *p) {
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
    uint4 a = q[0], b = q[1];
    Fr r;
    r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
    r.v[4] = b.x; r.v[5] = b.y; r.v[6] = b.z; r.v[7] = b.w;
    return r;
}
__device__ __forceinline__ void store_fr(Fr *p, const Fr &x) {
    uint4 *q = reinterpret_cast<uint4 *>(p);
    q[0] = make_uint4(x.v[0], x.v[1], x.v[2], x.v[3]);
    q[1] = make_uint4(x.v[4], x.v[5], x.v[6], x.v[7]);
}

// Unreduced sums of Fr Montgomery products: sum_i a_i b_i with each 512-bit
// product a_i * b_i added into a 17-limb accumulator (no overflow below 2^32
// products of values < r) and one Montgomery reduction at the end, as
// REDC(sum a_i b_i) = sum REDC(a_i b_i) mod r.  Each term costs the product
// half of a multiplication plus a carry chain instead of a full Montgomery
// product and a modular add; the reduction costs about 1.5 products, so it
// pays from about three terms on.
struct FrAcc {
    uint32_t w[17];
};

__device__ __forceinline__ void acc_zero(FrAcc &X) {
#pragma unroll
    for (int i = 0; i < 17; i++) X.w[i] = 0;
}

__device__ __forceinline__ void acc_mul_add(FrAcc &X, const Fr &a, const Fr &b) {
    uint32_t z[16];
    school_wide<8>(a.v, b.v, z);
    X.w[0] = add_cc(X.w[0], z[0]);
#pragma unroll
    for (int i = 1; i < 16; i++) X.w[i] = addc_cc(X.w[i], z[i]);
    X.w[16] = addc(X.w[16], 0);
}

// X += a * 2^256, whose REDC is a (products of arity 1)
__device__ __forceinline__ void acc_add_shifted(FrAcc &X, const Fr &a) {
    X.w[8] = add_cc(X.w[8], a.v[0]);
#pragma unroll
    for (int i = 1; i < 8; i++) X.w[8 + i] = addc_cc(X.w[8 + i], a.v[i]);
    X.w[16] = addc(X.w[16], 0);
}

// REDC(X) = X 2^-256 mod r, in [0, r): 8 Montgomery rows over the low 16
// limbs (result < 2^256 + r < 4r, so at most 3 subtractions of r), plus the
// share of limb 16, w 2^512 2^-256 = w 2^256 = to_mont(w).
static __device__ Fr acc_reduce(const FrAcc &X) {
    uint32_t t[17];
#pragma unroll
    for (int i = 0; i < 16; i++) t[i] = X.w[i];
    t[16] = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint32_t m = t[i] * FrParams::INV;
        uint32_t carry = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint64_t d = uint64_t(m) * FrParams::p(j) + (uint64_t(t[i + j]) + carry);
            t[i + j] = uint32_t(d);
            carry = uint32_t(d >> 32);
        }
#pragma unroll
        for (int j = i + 8; j < 17; j++) {
            const uint64_t d = uint64_t(t[j]) + carry;
            t[j] = uint32_t(d);
            carry = uint32_t(d >> 32);
        }
    }
    Fr r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = t[8 + i];
    uint32_t hi = t[16];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        uint32_t u[8];
        u[0] = sub_cc(r.v[0], FrParams::p(0));
#pragma unroll
        for (int i = 1; i < 8; i++) u[i] = subc_cc(r.v[i], FrParams::p(i));
        const uint32_t h2 = subc(hi, 0);
        const bool keep = h2 == 0xffffffffu;  // (hi, r) < p
#pragma unroll
        for (int i = 0; i < 8; i++) r.v[i] = keep ? r.v[i] : u[i];
        hi = keep ? hi : h2;
    }
    Fr w = Fr::zero();
    w.v[0] = X.w[16];
    return r + to_mont(w);
}


}  // namespace hp
