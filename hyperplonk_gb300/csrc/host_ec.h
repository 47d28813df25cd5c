// host_ec.h -- host-side G1 finishing of MSM partial sums.
//
// The device leaves each MSM as a handful of XYZZ partial sums whose final
// combination is a short sequential chain (a few dozen doublings/additions
// and one field inversion).  A sequential chain of dependent 381-bit
// multiplications has far lower latency on a host core than on one GPU
// thread, so that chain runs here: Horner over the partial sums, conversion
// to affine, canonical bytes.  Same XYZZ formulas as g1.cuh; 6 x 64-bit
// Montgomery limbs (R = 2^384), bit-identical storage with the device's
// 12 x 32-bit limbs.  Portable C++ (unsigned __int128), x86-64 and aarch64.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

namespace hp {
namespace host {

struct Fq64 {
    uint64_t v[6];
};

static const uint64_t kFqP[6] = {0xb9feffffffffaaabULL, 0x1eabfffeb153ffffULL, 0x6730d2a0f6b0f624ULL,
                                 0x64774b84f38512bfULL, 0x4b1ba7b6434bacd7ULL, 0x1a0111ea397fe69aULL};
static const uint64_t kFqOne[6] = {0x760900000002fffdULL, 0xebf4000bc40c0002ULL, 0x5f48985753c758baULL,
                                   0x77ce585370525745ULL, 0x5c071a97a256ec6dULL, 0x15f65ec3fa80e493ULL};
static const uint64_t kFqInv = 0x89f3fffcfffcfffdULL;

inline bool fq_geq_p(const uint64_t *a) {
    for (int i = 5; i >= 0; i--)
        if (a[i] != kFqP[i]) return a[i] > kFqP[i];
    return true;
}
inline void fq_sub_p(uint64_t *a) {
    unsigned __int128 borrow = 0;
    for (int i = 0; i < 6; i++) {
        unsigned __int128 d = (unsigned __int128)a[i] - kFqP[i] - borrow;
        a[i] = (uint64_t)d;
        borrow = (d >> 64) & 1;
    }
}
// [0, 2p) -> [0, p): device Fq values are kept below 2p between operations.
inline Fq64 fq_canonical(Fq64 a) {
    if (fq_geq_p(a.v)) fq_sub_p(a.v);
    return a;
}

inline Fq64 fq_add(const Fq64 &a, const Fq64 &b) {
    Fq64 r;
    unsigned __int128 c = 0;
    for (int i = 0; i < 6; i++) {
        c += (unsigned __int128)a.v[i] + b.v[i];
        r.v[i] = (uint64_t)c;
        c >>= 64;
    }
    if (c || fq_geq_p(r.v)) fq_sub_p(r.v);
    return r;
}
inline Fq64 fq_sub(const Fq64 &a, const Fq64 &b) {
    Fq64 r;
    unsigned __int128 borrow = 0;
    for (int i = 0; i < 6; i++) {
        unsigned __int128 d = (unsigned __int128)a.v[i] - b.v[i] - borrow;
        r.v[i] = (uint64_t)d;
        borrow = (d >> 64) & 1;
    }
    if (borrow) {
        unsigned __int128 c = 0;
        for (int i = 0; i < 6; i++) {
            c += (unsigned __int128)r.v[i] + kFqP[i];
            r.v[i] = (uint64_t)c;
            c >>= 64;
        }
    }
    return r;
}
inline Fq64 fq_mul(const Fq64 &a, const Fq64 &b) {
    uint64_t t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 6; i++) {
        unsigned __int128 c = 0;
        for (int j = 0; j < 6; j++) {
            c += (unsigned __int128)a.v[j] * b.v[i] + t[j];
            t[j] = (uint64_t)c;
            c >>= 64;
        }
        c += t[6];
        t[6] = (uint64_t)c;
        t[7] = (uint64_t)(c >> 64);
        uint64_t m = t[0] * kFqInv;
        c = (unsigned __int128)m * kFqP[0] + t[0];
        c >>= 64;
        for (int j = 1; j < 6; j++) {
            c += (unsigned __int128)m * kFqP[j] + t[j];
            t[j - 1] = (uint64_t)c;
            c >>= 64;
        }
        c += t[6];
        t[5] = (uint64_t)c;
        t[6] = t[7] + (uint64_t)(c >> 64);
    }
    Fq64 r;
    std::memcpy(r.v, t, 48);
    if (t[6] || fq_geq_p(r.v)) fq_sub_p(r.v);
    return r;
}
inline bool fq_is_zero(const Fq64 &a) {
    return (a.v[0] | a.v[1] | a.v[2] | a.v[3] | a.v[4] | a.v[5]) == 0;
}
inline Fq64 fq_one() {
    Fq64 r;
    std::memcpy(r.v, kFqOne, 48);
    return r;
}
inline Fq64 fq_inverse(const Fq64 &a) {  // a^(p-2)
    uint64_t e[6];
    std::memcpy(e, kFqP, 48);
    e[0] -= 2;  // low limb 0xb9feffffffffaaab: no borrow
    Fq64 acc = fq_one();
    for (int i = 5; i >= 0; i--)
        for (int bit = 63; bit >= 0; bit--) {
            acc = fq_mul(acc, acc);
            if ((e[i] >> bit) & 1) acc = fq_mul(acc, a);
        }
    return acc;
}
inline void fq_to_canonical(const Fq64 &a, uint8_t *out48) {
    Fq64 one = {{1, 0, 0, 0, 0, 0}};
    Fq64 r = fq_mul(a, one);
    std::memcpy(out48, r.v, 48);
}

struct Xyzz64 {
    Fq64 x, y, zz, zzz;
};

inline bool xyzz_is_inf(const Xyzz64 &p) { return fq_is_zero(p.zz); }

inline Xyzz64 xyzz_inf() {
    Xyzz64 r;
    r.x = fq_one();
    r.y = fq_one();
    std::memset(r.zz.v, 0, 48);
    std::memset(r.zzz.v, 0, 48);
    return r;
}

inline Xyzz64 xyzz_double(const Xyzz64 &p) {
    if (xyzz_is_inf(p)) return p;
    Fq64 u = fq_add(p.y, p.y), v = fq_mul(u, u), w = fq_mul(u, v), s = fq_mul(p.x, v);
    Fq64 xx = fq_mul(p.x, p.x), m = fq_add(fq_add(xx, xx), xx);
    Xyzz64 r;
    r.x = fq_sub(fq_mul(m, m), fq_add(s, s));
    r.y = fq_sub(fq_mul(m, fq_sub(s, r.x)), fq_mul(w, p.y));
    r.zz = fq_mul(v, p.zz);
    r.zzz = fq_mul(w, p.zzz);
    return r;
}

inline Xyzz64 xyzz_add(const Xyzz64 &p, const Xyzz64 &q) {
    if (xyzz_is_inf(p)) return q;
    if (xyzz_is_inf(q)) return p;
    Fq64 u1 = fq_mul(p.x, q.zz), u2 = fq_mul(q.x, p.zz);
    Fq64 s1 = fq_mul(p.y, q.zzz), s2 = fq_mul(q.y, p.zzz);
    Fq64 pp_ = fq_sub(u2, u1), rr = fq_sub(s2, s1);
    if (fq_is_zero(pp_)) {
        if (fq_is_zero(rr)) return xyzz_double(p);
        return xyzz_inf();
    }
    Fq64 pp = fq_mul(pp_, pp_), ppp = fq_mul(pp_, pp), qq = fq_mul(u1, pp);
    Xyzz64 r;
    r.x = fq_sub(fq_sub(fq_mul(rr, rr), ppp), fq_add(qq, qq));
    r.y = fq_sub(fq_mul(rr, fq_sub(qq, r.x)), fq_mul(s1, ppp));
    r.zz = fq_mul(fq_mul(p.zz, q.zz), pp);
    r.zzz = fq_mul(fq_mul(p.zzz, q.zzz), ppp);
    return r;
}

// XYZZ -> 97-byte G1 packet (tag, x LE48, y LE48).
inline void xyzz_to_packet(const Xyzz64 &p, uint8_t *out97) {
    std::memset(out97, 0, 97);
    if (xyzz_is_inf(p)) {
        out97[0] = 1;
        return;
    }
    // x = X / ZZ, y = Y / ZZZ with one inversion of ZZ * ZZZ
    Fq64 inv = fq_inverse(fq_mul(p.zz, p.zzz));
    Fq64 x = fq_mul(p.x, fq_mul(inv, p.zzz));
    Fq64 y = fq_mul(p.y, fq_mul(inv, p.zz));
    fq_to_canonical(x, out97 + 1);
    fq_to_canonical(y, out97 + 49);
}

// Many points to packets with one inversion (Montgomery's trick over the
// finite points' ZZ * ZZZ); equal to xyzz_to_packet point by point.
inline void xyzz_to_packets(const Xyzz64 *p, size_t n, uint8_t *out97) {
    std::vector<Fq64> prefix(n);
    Fq64 acc = fq_one();
    bool any = false;
    for (size_t i = 0; i < n; i++) {
        prefix[i] = acc;
        if (!xyzz_is_inf(p[i])) {
            acc = fq_mul(acc, fq_mul(p[i].zz, p[i].zzz));
            any = true;
        }
    }
    Fq64 inv = any ? fq_inverse(acc) : acc;
    for (size_t i = n; i-- > 0;) {
        uint8_t *o = out97 + 97 * i;
        std::memset(o, 0, 97);
        if (xyzz_is_inf(p[i])) {
            o[0] = 1;
            continue;
        }
        const Fq64 v = fq_mul(p[i].zz, p[i].zzz);
        const Fq64 vinv = fq_mul(inv, prefix[i]);  // (zz zzz)^-1
        inv = fq_mul(inv, v);
        fq_to_canonical(fq_mul(p[i].x, fq_mul(vinv, p[i].zzz)), o + 1);
        fq_to_canonical(fq_mul(p[i].y, fq_mul(vinv, p[i].zz)), o + 49);
    }
}

}  // namespace host
}  // namespace hp
