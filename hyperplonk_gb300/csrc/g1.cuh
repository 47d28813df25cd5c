// g1.cuh -- BLS12-381 G1 (y^2 = x^3 + 4 over Fq) on the device.
//
// Buckets use XYZZ coordinates (x = X/ZZ, y = Y/ZZZ, ZZ^3 = ZZZ^2; ZZ = 0 is
// the point at infinity): a mixed addition of an affine base costs 8M + 2S
// and needs no inversion.  Formulas: the public Explicit-Formulas Database,
// "xyzz" shape for short Weierstrass curves with a = 0 (madd-2008-s,
// add-2008-s, dbl-2008-s-1, mdbl-2008-s-1), with the exceptional cases
// (doubling through an addition, P + (-P), infinity) handled explicitly so
// every addition is complete.  The reference's own device curve code is
// backend/src/ascend910b3/native/g1.h (Jacobian, cuZK-derived formulas); the
// values produced are the same group elements.
#pragma once
#include "field.cuh"

namespace hp {

struct Affine {  // (0, 0) encodes infinity (not on the curve since 0 != 4)
    Fq x, y;
};

struct Xyzz {
    Fq x, y, zz, zzz;
};

__device__ __forceinline__ bool affine_is_inf(const Affine &p) { return p.x.is_zero() && p.y.is_zero(); }
__device__ __forceinline__ bool xyzz_is_inf(const Xyzz &p) { return p.zz.is_zero(); }

__device__ __forceinline__ Xyzz xyzz_inf() {
    Xyzz r;
    r.x = Fq::one();
    r.y = Fq::one();
    r.zz = Fq::zero();
    r.zzz = Fq::zero();
    return r;
}

__device__ __forceinline__ Xyzz xyzz_from_affine(const Affine &a) {
    if (affine_is_inf(a)) return xyzz_inf();
    Xyzz r;
    r.x = a.x;
    r.y = a.y;
    r.zz = Fq::one();
    r.zzz = Fq::one();
    return r;
}

// Independent products are issued in pairs (mul2), so the two multiply
// chains of each pair interleave.

// mdbl-2008-s-1: 2 * (x, y) for an affine input.
__device__ __forceinline__ Xyzz xyzz_double_affine(const Fq &x, const Fq &y) {
    Fq u = y + y;
    Fq v = sqr(u), xx = sqr(x), w, s, wy;
    mul2(w, s, u, v, x, v);
    Fq m = xx + xx + xx;
    Fq mm = sqr(m);
    wy = w * y;
    Xyzz r;
    r.x = mm - (s + s);
    r.y = m * (s - r.x) - wy;
    r.zz = v;
    r.zzz = w;
    return r;
}

// dbl-2008-s-1
__device__ __forceinline__ Xyzz xyzz_double(const Xyzz &p) {
    if (xyzz_is_inf(p)) return p;
    Fq u = p.y + p.y;
    Fq v = sqr(u), xx = sqr(p.x), w, s, t1, t2;
    mul2(w, s, u, v, p.x, v);
    Fq m = xx + xx + xx;
    Fq mm = sqr(m), zzz = w * p.zzz;
    Xyzz r;
    r.x = mm - (s + s);
    mul2(t1, t2, m, s - r.x, w, p.y);
    r.y = t1 - t2;
    r.zz = v * p.zz;
    r.zzz = zzz;
    return r;
}

// madd-2008-s: p + (x2, y2) with (x2, y2) finite affine.
__device__ __forceinline__ Xyzz xyzz_add_affine(const Xyzz &p, const Fq &x2, const Fq &y2) {
    if (xyzz_is_inf(p)) {
        Xyzz r;
        r.x = x2;
        r.y = y2;
        r.zz = Fq::one();
        r.zzz = Fq::one();
        return r;
    }
    Fq u2, s2;
    mul2(u2, s2, x2, p.zz, y2, p.zzz);
    Fq pp_ = u2 - p.x;
    Fq rr = s2 - p.y;
    if (pp_.is_zero()) {
        if (rr.is_zero()) return xyzz_double_affine(x2, y2);
        return xyzz_inf();
    }
    Fq pp = sqr(pp_), r2 = sqr(rr), ppp, q, t1, t2;
    mul2(ppp, q, pp_, pp, p.x, pp);
    Xyzz r;
    r.x = r2 - ppp - (q + q);
    mul2(r.zz, r.zzz, p.zz, pp, p.zzz, ppp);
    mul2(t1, t2, rr, q - r.x, p.y, ppp);
    r.y = t1 - t2;
    return r;
}

// add-2008-s: general XYZZ addition.
__device__ __forceinline__ Xyzz xyzz_add(const Xyzz &p, const Xyzz &q) {
    if (xyzz_is_inf(p)) return q;
    if (xyzz_is_inf(q)) return p;
    Fq u1, u2, s1, s2;
    mul2(u1, u2, p.x, q.zz, q.x, p.zz);
    mul2(s1, s2, p.y, q.zzz, q.y, p.zzz);
    Fq pp_ = u2 - u1;
    Fq rr = s2 - s1;
    if (pp_.is_zero()) {
        if (rr.is_zero()) return xyzz_double(p);
        return xyzz_inf();
    }
    Fq pp = sqr(pp_), r2 = sqr(rr), ppp, qq, zz, zzz, t1, t2;
    mul2(ppp, qq, pp_, pp, u1, pp);
    mul2(zz, zzz, p.zz, q.zz, p.zzz, q.zzz);
    Xyzz r;
    r.x = r2 - ppp - (qq + qq);
    mul2(r.zz, r.zzz, zz, pp, zzz, ppp);
    mul2(t1, t2, rr, qq - r.x, s1, ppp);
    r.y = t1 - t2;
    return r;
}

// ---- global memory access (16-byte vectors) ----
template <class F>
__device__ __forceinline__ void load_words(F &dst, const uint32_t *src) {
    const uint4 *q = reinterpret_cast<const uint4 *>(src);
#pragma unroll
    for (int i = 0; i < F::N / 4; i++) {
        uint4 v = q[i];
        dst.v[4 * i] = v.x;
        dst.v[4 * i + 1] = v.y;
        dst.v[4 * i + 2] = v.z;
        dst.v[4 * i + 3] = v.w;
    }
}
template <class F>
__device__ __forceinline__ void store_words(uint32_t *dst, const F &src) {
    uint4 *q = reinterpret_cast<uint4 *>(dst);
#pragma unroll
    for (int i = 0; i < F::N / 4; i++)
        q[i] = make_uint4(src.v[4 * i], src.v[4 * i + 1], src.v[4 * i + 2], src.v[4 * i + 3]);
}

__device__ __forceinline__ Affine load_affine(const Affine *p) {
    Affine a;
    const uint32_t *w = reinterpret_cast<const uint32_t *>(p);
    load_words(a.x, w);
    load_words(a.y, w + 12);
    return a;
}
__device__ __forceinline__ void store_affine(Affine *p, const Affine &a) {
    uint32_t *w = reinterpret_cast<uint32_t *>(p);
    store_words(w, a.x);
    store_words(w + 12, a.y);
}
__device__ __forceinline__ Xyzz load_xyzz(const Xyzz *p) {
    Xyzz a;
    const uint32_t *w = reinterpret_cast<const uint32_t *>(p);
    load_words(a.x, w);
    load_words(a.y, w + 12);
    load_words(a.zz, w + 24);
    load_words(a.zzz, w + 36);
    return a;
}
__device__ __forceinline__ void store_xyzz(Xyzz *p, const Xyzz &a) {
    uint32_t *w = reinterpret_cast<uint32_t *>(p);
    store_words(w, a.x);
    store_words(w + 12, a.y);
    store_words(w + 24, a.zz);
    store_words(w + 36, a.zzz);
}

}  // namespace hp
