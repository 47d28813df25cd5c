// host_field.h -- host-side Fr Montgomery helpers for argument marshalling.
//
// The ABI carries canonical little-endian Fr (reference bridge.h:5-6); device
// tables hold Montgomery form with R = 2^256.  Scalars that ride in kernel
// parameters (coefficients, challenges, points) are converted here once per
// call.  The 4 x 64-bit little-endian limbs are bit-identical to the device's
// 8 x 32-bit limbs.  Pure C++ (unsigned __int128), builds on x86-64 and
// aarch64 alike.
#pragma once
#include <cstdint>
#include <cstring>

namespace hp {
namespace host {

struct Fr64 {
    uint64_t v[4];
};

static const uint64_t kFrP[4] = {0xffffffff00000001ULL, 0x53bda402fffe5bfeULL,
                                 0x3339d80809a1d805ULL, 0x73eda753299d7d48ULL};
static const uint64_t kFrR2[4] = {0xc999e990f3f29c6dULL, 0x2b6cedcb87925c23ULL,
                                  0x05d314967254398fULL, 0x0748d9d99f59ff11ULL};
static const uint64_t kFrOne[4] = {0x1fffffffeULL, 0x5884b7fa00034802ULL,
                                   0x998c4fefecbc4ff5ULL, 0x1824b159acc5056fULL};
static const uint64_t kFrR3[4] = {0xc62c1807439b73afULL, 0x1b3e0d188cf06990ULL,
                                  0x73d13c71c7b5f418ULL, 0x6e2a5bb9c8db33e9ULL};
static const uint64_t kFrInv = 0xfffffffeffffffffULL;

inline bool geq_p(const uint64_t *a) {
    for (int i = 3; i >= 0; i--) {
        if (a[i] != kFrP[i]) return a[i] > kFrP[i];
    }
    return true;
}

inline void sub_p(uint64_t *a) {
    unsigned __int128 borrow = 0;
    for (int i = 0; i < 4; i++) {
        unsigned __int128 d = (unsigned __int128)a[i] - kFrP[i] - borrow;
        a[i] = (uint64_t)d;
        borrow = (d >> 64) & 1;
    }
}

inline Fr64 mont_mul(const Fr64 &a, const Fr64 &b) {
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; i++) {
        unsigned __int128 c = 0;
        for (int j = 0; j < 4; j++) {
            c += (unsigned __int128)a.v[j] * b.v[i] + t[j];
            t[j] = (uint64_t)c;
            c >>= 64;
        }
        c += t[4];
        t[4] = (uint64_t)c;
        t[5] = (uint64_t)(c >> 64);
        uint64_t m = t[0] * kFrInv;
        c = (unsigned __int128)m * kFrP[0] + t[0];
        c >>= 64;
        for (int j = 1; j < 4; j++) {
            c += (unsigned __int128)m * kFrP[j] + t[j];
            t[j - 1] = (uint64_t)c;
            c >>= 64;
        }
        c += t[4];
        t[3] = (uint64_t)c;
        t[4] = t[5] + (uint64_t)(c >> 64);
    }
    Fr64 r;
    std::memcpy(r.v, t, 32);
    if (t[4] || geq_p(r.v)) sub_p(r.v);
    return r;
}

// Canonical LE32 -> Montgomery.  False if the value is not < r.
inline bool from_canonical(const uint8_t *bytes, Fr64 &out) {
    Fr64 raw;
    std::memcpy(raw.v, bytes, 32);
    if (geq_p(raw.v)) return false;
    Fr64 r2;
    std::memcpy(r2.v, kFrR2, 32);
    out = mont_mul(raw, r2);
    return true;
}

inline void to_canonical(const Fr64 &mont, uint8_t *bytes) {
    Fr64 one = {{1, 0, 0, 0}};
    Fr64 r = mont_mul(mont, one);
    std::memcpy(bytes, r.v, 32);
}

inline bool is_zero(const Fr64 &a) { return (a.v[0] | a.v[1] | a.v[2] | a.v[3]) == 0; }

inline Fr64 add(const Fr64 &a, const Fr64 &b) {
    Fr64 r;
    unsigned __int128 c = 0;
    for (int i = 0; i < 4; i++) {
        c += (unsigned __int128)a.v[i] + b.v[i];
        r.v[i] = (uint64_t)c;
        c >>= 64;
    }
    if (c || geq_p(r.v)) sub_p(r.v);
    return r;
}

// Fr::from_le_bytes_mod_order of 64 bytes (ark-ff): (lo + hi * 2^256) mod r,
// returned in Montgomery form: mont(lo * R2) + mont(hi * R3).
inline Fr64 from_wide64(const uint8_t *bytes) {
    Fr64 lo, hi, r2, r3;
    std::memcpy(lo.v, bytes, 32);
    std::memcpy(hi.v, bytes + 32, 32);
    std::memcpy(r2.v, kFrR2, 32);
    std::memcpy(r3.v, kFrR3, 32);
    return add(mont_mul(lo, r2), mont_mul(hi, r3));
}

inline Fr64 one() {
    Fr64 r;
    std::memcpy(r.v, kFrOne, 32);
    return r;
}

inline Fr64 neg(const Fr64 &a) {
    if (is_zero(a)) return a;
    Fr64 r;
    unsigned __int128 borrow = 0;
    for (int i = 0; i < 4; i++) {
        unsigned __int128 d = (unsigned __int128)kFrP[i] - a.v[i] - borrow;
        r.v[i] = (uint64_t)d;
        borrow = (d >> 64) & 1;
    }
    return r;
}

// Montgomery form of the integer k (k < 2^64, so k < r).
inline Fr64 from_u64(uint64_t k) {
    Fr64 raw = {{k, 0, 0, 0}}, r2;
    std::memcpy(r2.v, kFrR2, 32);
    return mont_mul(raw, r2);
}

// a^(r-2) = a^-1 for a != 0 (Fermat), Montgomery in and out.
inline Fr64 inverse(const Fr64 &a) {
    uint64_t e[4] = {kFrP[0] - 2, kFrP[1], kFrP[2], kFrP[3]};
    Fr64 acc = one();
    for (int i = 3; i >= 0; i--)
        for (int b = 63; b >= 0; b--) {
            acc = mont_mul(acc, acc);
            if ((e[i] >> b) & 1) acc = mont_mul(acc, a);
        }
    return acc;
}

}  // namespace host
}  // namespace hp
