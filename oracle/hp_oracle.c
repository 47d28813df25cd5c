/*
 * hp_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the HyperPlonk reference's CPU backend for the prover hot
 * path: BLS12-381 Fr/Fq arithmetic, G1 curve arithmetic, the variable-base MSM,
 * the MLE table operations, the sumcheck prover round, multilinear-KZG
 * commit/open, the testing SRS and the fixture RNG.  It is the parity checker
 * for the CUDA library and the timed CPU baseline; no product code links it.
 *
 * Reference files restated here (paths inside the krn1pnc/hyperplonk tree):
 *   backend/src/cpu/multilinear_polynomial.rs:32-253   MLE operations
 *   backend/src/cpu/sum_check.rs:35-217                sumcheck prover state
 *   backend/src/cpu/multilinear_kzg.rs:40-137          commit / open
 *   backend/src/common/eq.rs:15-95                     eq_eval / build_eq_x_r
 *   subroutines/src/pcs/multilinear_kzg/srs.rs:25-53,158-235   testing SRS
 * and the third-party arithmetic they call (pinned in Cargo.lock, not vendored):
 *   ark-ec 0.6.0 VariableBaseMSM::msm_unchecked  -> or_msm (value only)
 *   ark-poly 0.6.0 DenseMultilinearExtension::{fix_variables,evaluate}
 *   ark-ff 0.6.0 batch_inversion, from_le_bytes_mod_order
 *
 * Representation: 64-bit limbs, Montgomery form with R = 2^256 (Fr) and
 * R = 2^384 (Fq).  Every exported function takes canonical little-endian
 * bytes (Fr 32 B, Fq 48 B, affine G1 96 B = x || y with (0,0) = infinity).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------------ */
/* Multi-precision Montgomery arithmetic                                     */
/* ------------------------------------------------------------------------ */

typedef struct { uint64_t v[4]; } fr_t;
typedef struct { uint64_t v[6]; } fq_t;

static const uint64_t FR_P[4] = {0xffffffff00000001ULL, 0x53bda402fffe5bfeULL,
                                 0x3339d80809a1d805ULL, 0x73eda753299d7d48ULL};
static const uint64_t FR_R[4] = {0x1fffffffeULL, 0x5884b7fa00034802ULL,
                                 0x998c4fefecbc4ff5ULL, 0x1824b159acc5056fULL};
static const uint64_t FR_R2[4] = {0xc999e990f3f29c6dULL, 0x2b6cedcb87925c23ULL,
                                  0x05d314967254398fULL, 0x0748d9d99f59ff11ULL};
static const uint64_t FR_R3[4] = {0xc62c1807439b73afULL, 0x1b3e0d188cf06990ULL,
                                  0x73d13c71c7b5f418ULL, 0x6e2a5bb9c8db33e9ULL};
static const uint64_t FR_INV = 0xfffffffeffffffffULL;

static const uint64_t FQ_P[6] = {0xb9feffffffffaaabULL, 0x1eabfffeb153ffffULL,
                                 0x6730d2a0f6b0f624ULL, 0x64774b84f38512bfULL,
                                 0x4b1ba7b6434bacd7ULL, 0x1a0111ea397fe69aULL};
static const uint64_t FQ_R[6] = {0x760900000002fffdULL, 0xebf4000bc40c0002ULL,
                                 0x5f48985753c758baULL, 0x77ce585370525745ULL,
                                 0x5c071a97a256ec6dULL, 0x15f65ec3fa80e493ULL};
static const uint64_t FQ_R2[6] = {0xf4df1f341c341746ULL, 0x0a76e6a609d104f1ULL,
                                  0x8de5476c4c95b6d5ULL, 0x67eb88a9939d83c0ULL,
                                  0x9a793e85b519952dULL, 0x11988fe592cae3aaULL};
static const uint64_t FQ_INV = 0x89f3fffcfffcfffdULL;

static inline int mp_geq(const uint64_t *a, const uint64_t *b, int n) {
    for (int i = n - 1; i >= 0; i--) {
        if (a[i] != b[i]) return a[i] > b[i];
    }
    return 1;
}
static inline uint64_t mp_sub(uint64_t *r, const uint64_t *a, const uint64_t *b, int n) {
    uint64_t borrow = 0;
    for (int i = 0; i < n; i++) {
        u128 d = (u128)a[i] - b[i] - borrow;
        r[i] = (uint64_t)d;
        borrow = (uint64_t)(d >> 64) & 1;
    }
    return borrow;
}
static inline uint64_t mp_add(uint64_t *r, const uint64_t *a, const uint64_t *b, int n) {
    u128 c = 0;
    for (int i = 0; i < n; i++) {
        c += (u128)a[i] + b[i];
        r[i] = (uint64_t)c;
        c >>= 64;
    }
    return (uint64_t)c;
}
static inline int mp_is_zero(const uint64_t *a, int n) {
    uint64_t acc = 0;
    for (int i = 0; i < n; i++) acc |= a[i];
    return acc == 0;
}

/* CIOS Montgomery product, inputs may be any value < 2^(64n) as long as one of
 * them is < p (the result is then < 2p before the final subtraction). */
static inline void mp_mont_mul(uint64_t *res, const uint64_t *a, const uint64_t *b,
                               const uint64_t *p, uint64_t inv, int n) {
    uint64_t t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; i++) {
        u128 c = 0;
        for (int j = 0; j < n; j++) {
            c += (u128)a[j] * b[i] + t[j];
            t[j] = (uint64_t)c;
            c >>= 64;
        }
        c += t[n];
        t[n] = (uint64_t)c;
        t[n + 1] = (uint64_t)(c >> 64);
        uint64_t m = t[0] * inv;
        c = (u128)m * p[0] + t[0];
        c >>= 64;
        for (int j = 1; j < n; j++) {
            c += (u128)m * p[j] + t[j];
            t[j - 1] = (uint64_t)c;
            c >>= 64;
        }
        c += t[n];
        t[n - 1] = (uint64_t)c;
        t[n] = t[n + 1] + (uint64_t)(c >> 64);
    }
    if (t[n] || mp_geq(t, p, n)) mp_sub(t, t, p, n);
    memcpy(res, t, (size_t)n * 8);
}

#define FIELD_OPS(PFX, T, N, P, RONE, R2, INV)                                       \
    static inline void PFX##_add(T *r, const T *a, const T *b) {                     \
        uint64_t c = mp_add(r->v, a->v, b->v, N);                                    \
        if (c || mp_geq(r->v, P, N)) mp_sub(r->v, r->v, P, N);                        \
    }                                                                                \
    static inline void PFX##_sub(T *r, const T *a, const T *b) {                     \
        if (mp_sub(r->v, a->v, b->v, N)) mp_add(r->v, r->v, P, N);                   \
    }                                                                                \
    static inline void PFX##_neg(T *r, const T *a) {                                 \
        if (mp_is_zero(a->v, N)) { *r = *a; return; }                                 \
        mp_sub(r->v, P, a->v, N);                                                    \
    }                                                                                \
    static inline void PFX##_mul(T *r, const T *a, const T *b) {                     \
        mp_mont_mul(r->v, a->v, b->v, P, INV, N);                                    \
    }                                                                                \
    static inline int PFX##_is_zero(const T *a) { return mp_is_zero(a->v, N); }     \
    static inline int PFX##_eq(const T *a, const T *b) {                             \
        return memcmp(a->v, b->v, N * 8) == 0;                                       \
    }                                                                                \
    static inline void PFX##_one(T *r) { memcpy(r->v, RONE, N * 8); }                \
    static inline void PFX##_zero(T *r) { memset(r->v, 0, N * 8); }                  \
    static inline void PFX##_from_u64(T *r, uint64_t x) {                            \
        T t; memset(&t, 0, sizeof t); t.v[0] = x;                                    \
        mp_mont_mul(r->v, t.v, R2, P, INV, N);                                       \
    }                                                                                \
    /* canonical LE bytes -> Montgomery; returns 0 if not canonical */               \
    static inline int PFX##_from_bytes(T *r, const uint8_t *bytes) {                 \
        T t;                                                                         \
        memcpy(t.v, bytes, N * 8);                                                   \
        if (mp_geq(t.v, P, N)) { memset(r->v, 0, N * 8); return 0; }                 \
        mp_mont_mul(r->v, t.v, R2, P, INV, N);                                       \
        return 1;                                                                    \
    }                                                                                \
    static inline void PFX##_to_bytes(uint8_t *bytes, const T *a) {                  \
        T one, t; memset(&one, 0, sizeof one); one.v[0] = 1;                         \
        mp_mont_mul(t.v, a->v, one.v, P, INV, N);                                    \
        memcpy(bytes, t.v, N * 8);                                                   \
    }                                                                                \
    static void PFX##_pow(T *r, const T *a, const uint64_t *e) {                     \
        T acc; PFX##_one(&acc);                                                      \
        for (int i = N - 1; i >= 0; i--)                                             \
            for (int bit = 63; bit >= 0; bit--) {                                    \
                PFX##_mul(&acc, &acc, &acc);                                         \
                if ((e[i] >> bit) & 1) PFX##_mul(&acc, &acc, a);                     \
            }                                                                        \
        *r = acc;                                                                    \
    }                                                                                \
    static void PFX##_inv(T *r, const T *a) {                                        \
        uint64_t e[N]; memcpy(e, P, N * 8);                                          \
        e[0] -= 2; /* p is odd and > 2: no borrow */                                 \
        PFX##_pow(r, a, e);                                                          \
    }

FIELD_OPS(fr, fr_t, 4, FR_P, FR_R, FR_R2, FR_INV)
FIELD_OPS(fq, fq_t, 6, FQ_P, FQ_R, FQ_R2, FQ_INV)

/* Fr::from_le_bytes_mod_order for a 64-byte input (ark-ff 0.6.0): the value of
 * the little-endian integer modulo r.  lo + hi * 2^256 with R = 2^256 gives
 * mont(lo) = lo*R2*R^-1 and mont(hi*2^256) = hi*R3*R^-1. */
static void fr_from_wide64(fr_t *r, const uint8_t *bytes) {
    fr_t lo, hi, a, b;
    memcpy(lo.v, bytes, 32);
    memcpy(hi.v, bytes + 32, 32);
    mp_mont_mul(a.v, lo.v, FR_R2, FR_P, FR_INV, 4);
    mp_mont_mul(b.v, hi.v, FR_R3, FR_P, FR_INV, 4);
    fr_add(r, &a, &b);
}

/* Montgomery-trick batch inversion of nonzero values (ark-ff batch_inversion). */
static void fr_batch_inverse(fr_t *v, size_t n) {
    if (n == 0) return;
    fr_t *pref = (fr_t *)malloc(n * sizeof(fr_t));
    fr_t acc;
    fr_one(&acc);
    for (size_t i = 0; i < n; i++) {
        pref[i] = acc;
        fr_mul(&acc, &acc, &v[i]);
    }
    fr_t inv;
    fr_inv(&inv, &acc);
    for (size_t i = n; i-- > 0;) {
        fr_t t;
        fr_mul(&t, &inv, &pref[i]);
        fr_mul(&inv, &inv, &v[i]);
        v[i] = t;
    }
    free(pref);
}

/* ------------------------------------------------------------------------ */
/* Parallel-for helper (pthreads)                                            */
/* ------------------------------------------------------------------------ */

static int g_threads = 1;

int or_set_threads(int n) {
    if (n <= 0) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        n = c > 0 ? (int)c : 1;
    }
    g_threads = n;
    return g_threads;
}

typedef void (*range_fn)(void *ctx, size_t begin, size_t end, int worker);
typedef struct { range_fn fn; void *ctx; size_t begin, end; int worker; } range_job;

static void *range_thread(void *arg) {
    range_job *j = (range_job *)arg;
    j->fn(j->ctx, j->begin, j->end, j->worker);
    return NULL;
}

/* Runs fn over [0, n) split into at most g_threads contiguous chunks. */
static void parallel_for(size_t n, range_fn fn, void *ctx) {
    int t = g_threads;
    if ((size_t)t > n) t = (int)(n ? n : 1);
    if (t <= 1) {
        fn(ctx, 0, n, 0);
        return;
    }
    pthread_t th[256];
    range_job jobs[256];
    memset(jobs, 0, sizeof jobs);
    if (t > 256) t = 256;
    size_t chunk = (n + t - 1) / t;
    int launched = 0;
    for (int i = 0; i < t; i++) {
        size_t b = (size_t)i * chunk, e = b + chunk;
        if (b >= n) break;
        if (e > n) e = n;
        jobs[i] = (range_job){fn, ctx, b, e, i};
        if (i == 0) continue;
        pthread_create(&th[i], NULL, range_thread, &jobs[i]);
        launched = i;
    }
    fn(ctx, jobs[0].begin, jobs[0].end, 0);
    for (int i = 1; i <= launched; i++) pthread_join(th[i], NULL);
}

/* ------------------------------------------------------------------------ */
/* G1: y^2 = x^3 + 4 over Fq                                                 */
/* ------------------------------------------------------------------------ */

typedef struct { fq_t x, y; int inf; } g1a_t;
typedef struct { fq_t x, y, z; } g1j_t; /* z == 0 <=> infinity */

static inline void g1j_set_inf(g1j_t *p) {
    fq_one(&p->x);
    fq_one(&p->y);
    fq_zero(&p->z);
}
static inline int g1j_is_inf(const g1j_t *p) { return fq_is_zero(&p->z); }

/* dbl-2009-l (a = 0) */
static void g1j_double(g1j_t *r, const g1j_t *p) {
    if (g1j_is_inf(p)) { *r = *p; return; }
    fq_t A, B, C, D, E, F, t;
    fq_mul(&A, &p->x, &p->x);
    fq_mul(&B, &p->y, &p->y);
    fq_mul(&C, &B, &B);
    fq_add(&t, &p->x, &B);
    fq_mul(&t, &t, &t);
    fq_sub(&t, &t, &A);
    fq_sub(&t, &t, &C);
    fq_add(&D, &t, &t);
    fq_add(&E, &A, &A);
    fq_add(&E, &E, &A);
    fq_mul(&F, &E, &E);
    fq_t z3;
    fq_mul(&z3, &p->y, &p->z);
    fq_add(&r->z, &z3, &z3);
    fq_t x3;
    fq_sub(&x3, &F, &D);
    fq_sub(&x3, &x3, &D);
    fq_t y3, c8;
    fq_sub(&y3, &D, &x3);
    fq_mul(&y3, &E, &y3);
    fq_add(&c8, &C, &C);
    fq_add(&c8, &c8, &c8);
    fq_add(&c8, &c8, &c8);
    fq_sub(&r->y, &y3, &c8);
    r->x = x3;
}

/* madd-2007-bl with the exceptional cases handled explicitly */
static void g1j_add_affine(g1j_t *r, const g1j_t *p, const g1a_t *q) {
    if (q->inf) { *r = *p; return; }
    if (g1j_is_inf(p)) {
        r->x = q->x;
        r->y = q->y;
        fq_one(&r->z);
        return;
    }
    fq_t Z1Z1, U2, S2, H, rr, HH, I, J, V, t;
    fq_mul(&Z1Z1, &p->z, &p->z);
    fq_mul(&U2, &q->x, &Z1Z1);
    fq_mul(&S2, &q->y, &p->z);
    fq_mul(&S2, &S2, &Z1Z1);
    fq_sub(&H, &U2, &p->x);
    fq_sub(&rr, &S2, &p->y);
    if (fq_is_zero(&H)) {
        if (fq_is_zero(&rr)) { g1j_double(r, p); return; }
        g1j_set_inf(r);
        return;
    }
    fq_mul(&HH, &H, &H);
    fq_add(&I, &HH, &HH);
    fq_add(&I, &I, &I);
    fq_mul(&J, &H, &I);
    fq_add(&rr, &rr, &rr);
    fq_mul(&V, &p->x, &I);
    fq_t x3, y3, z3;
    fq_mul(&x3, &rr, &rr);
    fq_sub(&x3, &x3, &J);
    fq_sub(&x3, &x3, &V);
    fq_sub(&x3, &x3, &V);
    fq_sub(&t, &V, &x3);
    fq_mul(&y3, &rr, &t);
    fq_mul(&t, &p->y, &J);
    fq_add(&t, &t, &t);
    fq_sub(&y3, &y3, &t);
    fq_add(&z3, &p->z, &H);
    fq_mul(&z3, &z3, &z3);
    fq_sub(&z3, &z3, &Z1Z1);
    fq_sub(&z3, &z3, &HH);
    r->x = x3;
    r->y = y3;
    r->z = z3;
}

/* add-2007-bl with exceptional cases */
static void g1j_add(g1j_t *r, const g1j_t *p, const g1j_t *q) {
    if (g1j_is_inf(p)) { *r = *q; return; }
    if (g1j_is_inf(q)) { *r = *p; return; }
    fq_t Z1Z1, Z2Z2, U1, U2, S1, S2, H, rr, I, J, V, t;
    fq_mul(&Z1Z1, &p->z, &p->z);
    fq_mul(&Z2Z2, &q->z, &q->z);
    fq_mul(&U1, &p->x, &Z2Z2);
    fq_mul(&U2, &q->x, &Z1Z1);
    fq_mul(&S1, &p->y, &q->z);
    fq_mul(&S1, &S1, &Z2Z2);
    fq_mul(&S2, &q->y, &p->z);
    fq_mul(&S2, &S2, &Z1Z1);
    fq_sub(&H, &U2, &U1);
    fq_sub(&rr, &S2, &S1);
    if (fq_is_zero(&H)) {
        if (fq_is_zero(&rr)) { g1j_double(r, p); return; }
        g1j_set_inf(r);
        return;
    }
    fq_add(&I, &H, &H);
    fq_mul(&I, &I, &I);
    fq_mul(&J, &H, &I);
    fq_add(&rr, &rr, &rr);
    fq_mul(&V, &U1, &I);
    fq_t x3, y3, z3;
    fq_mul(&x3, &rr, &rr);
    fq_sub(&x3, &x3, &J);
    fq_sub(&x3, &x3, &V);
    fq_sub(&x3, &x3, &V);
    fq_sub(&t, &V, &x3);
    fq_mul(&y3, &rr, &t);
    fq_mul(&t, &S1, &J);
    fq_add(&t, &t, &t);
    fq_sub(&y3, &y3, &t);
    fq_add(&z3, &p->z, &q->z);
    fq_mul(&z3, &z3, &z3);
    fq_sub(&z3, &z3, &Z1Z1);
    fq_sub(&z3, &z3, &Z2Z2);
    fq_mul(&z3, &z3, &H);
    r->x = x3;
    r->y = y3;
    r->z = z3;
}

static void g1j_to_affine(g1a_t *r, const g1j_t *p) {
    if (g1j_is_inf(p)) {
        memset(r, 0, sizeof *r);
        r->inf = 1;
        return;
    }
    fq_t zi, zi2, zi3;
    fq_inv(&zi, &p->z);
    fq_mul(&zi2, &zi, &zi);
    fq_mul(&zi3, &zi2, &zi);
    fq_mul(&r->x, &p->x, &zi2);
    fq_mul(&r->y, &p->y, &zi3);
    r->inf = 0;
}

/* Batch normalisation (one inversion for all finite points). */
static void g1j_batch_to_affine(g1a_t *out, const g1j_t *in, size_t n) {
    fq_t *pref = (fq_t *)malloc((n + 1) * sizeof(fq_t));
    fq_t acc;
    fq_one(&acc);
    for (size_t i = 0; i < n; i++) {
        pref[i] = acc;
        if (!g1j_is_inf(&in[i])) fq_mul(&acc, &acc, &in[i].z);
    }
    fq_t inv;
    if (!fq_is_zero(&acc)) fq_inv(&inv, &acc);
    for (size_t i = n; i-- > 0;) {
        if (g1j_is_inf(&in[i])) {
            memset(&out[i], 0, sizeof out[i]);
            out[i].inf = 1;
            continue;
        }
        fq_t zi, zi2, zi3;
        fq_mul(&zi, &inv, &pref[i]);
        fq_mul(&inv, &inv, &in[i].z);
        fq_mul(&zi2, &zi, &zi);
        fq_mul(&zi3, &zi2, &zi);
        fq_mul(&out[i].x, &in[i].x, &zi2);
        fq_mul(&out[i].y, &in[i].y, &zi3);
        out[i].inf = 0;
    }
    free(pref);
}

/* 96-byte canonical affine: x LE48 || y LE48, all-zero = infinity. */
static int g1a_from_bytes(g1a_t *r, const uint8_t *b) {
    int zero = 1;
    for (int i = 0; i < 96; i++) zero &= b[i] == 0;
    if (zero) {
        memset(r, 0, sizeof *r);
        r->inf = 1;
        return 1;
    }
    r->inf = 0;
    return fq_from_bytes(&r->x, b) && fq_from_bytes(&r->y, b + 48);
}
static void g1a_to_bytes(uint8_t *b, const g1a_t *p) {
    if (p->inf) {
        memset(b, 0, 96);
        return;
    }
    fq_to_bytes(b, &p->x);
    fq_to_bytes(b + 48, &p->y);
}

static void g1a_to_jac(g1j_t *r, const g1a_t *a) {
    if (a->inf) { g1j_set_inf(r); return; }
    r->x = a->x;
    r->y = a->y;
    fq_one(&r->z);
}

/* Scalar multiplication by a canonical 256-bit integer (4 limbs). */
static void g1j_mul_limbs(g1j_t *r, const g1j_t *p, const uint64_t *k, int limbs) {
    g1j_t acc;
    g1j_set_inf(&acc);
    for (int i = limbs - 1; i >= 0; i--)
        for (int bit = 63; bit >= 0; bit--) {
            g1j_double(&acc, &acc);
            if ((k[i] >> bit) & 1) g1j_add(&acc, &acc, p);
        }
    *r = acc;
}

/* ---- exported element-wise helpers (for golden-vector pinning) ---------- */

/* op: 0 add, 1 sub, 2 mul, 3 neg, 4 square, 5 inverse (0 -> 0).
 * field: 0 = Fr, 1 = Fq.  Returns the index+1 of the first non-canonical
 * input, 0 on success. */
size_t or_field_op(int field, int op, const uint8_t *a, const uint8_t *b, uint8_t *out,
                   size_t n) {
    for (size_t i = 0; i < n; i++) {
        if (field == 0) {
            fr_t x, y, z;
            if (!fr_from_bytes(&x, a + 32 * i)) return i + 1;
            if (op <= 2 && !fr_from_bytes(&y, b + 32 * i)) return i + 1;
            switch (op) {
                case 0: fr_add(&z, &x, &y); break;
                case 1: fr_sub(&z, &x, &y); break;
                case 2: fr_mul(&z, &x, &y); break;
                case 3: fr_neg(&z, &x); break;
                case 4: fr_mul(&z, &x, &x); break;
                default:
                    if (fr_is_zero(&x)) fr_zero(&z); else fr_inv(&z, &x);
            }
            fr_to_bytes(out + 32 * i, &z);
        } else {
            fq_t x, y, z;
            if (!fq_from_bytes(&x, a + 48 * i)) return i + 1;
            if (op <= 2 && !fq_from_bytes(&y, b + 48 * i)) return i + 1;
            switch (op) {
                case 0: fq_add(&z, &x, &y); break;
                case 1: fq_sub(&z, &x, &y); break;
                case 2: fq_mul(&z, &x, &y); break;
                case 3: fq_neg(&z, &x); break;
                case 4: fq_mul(&z, &x, &x); break;
                default:
                    if (fq_is_zero(&x)) fq_zero(&z); else fq_inv(&z, &x);
            }
            fq_to_bytes(out + 48 * i, &z);
        }
    }
    return 0;
}

/* Fr from 64-byte little-endian integers, reduced mod r. */
void or_fr_from_wide(const uint8_t *wide, uint8_t *out, size_t n) {
    for (size_t i = 0; i < n; i++) {
        fr_t x;
        fr_from_wide64(&x, wide + 64 * i);
        fr_to_bytes(out + 32 * i, &x);
    }
}

/* op: 0 add(a,b), 1 double(a), 2 neg(a), 3 mul(a, u64 k[i]).  Affine in/out. */
size_t or_g1_op(int op, const uint8_t *a, const uint8_t *b, const uint64_t *k, uint8_t *out,
                size_t n) {
    for (size_t i = 0; i < n; i++) {
        g1a_t pa, pb, res;
        g1j_t ja, jr;
        if (!g1a_from_bytes(&pa, a + 96 * i)) return i + 1;
        g1a_to_jac(&ja, &pa);
        switch (op) {
            case 0:
                if (!g1a_from_bytes(&pb, b + 96 * i)) return i + 1;
                g1j_add_affine(&jr, &ja, &pb);
                break;
            case 1: g1j_double(&jr, &ja); break;
            case 2:
                jr = ja;
                fq_neg(&jr.y, &ja.y);
                break;
            default: {
                uint64_t kk[1] = {k[i]};
                g1j_mul_limbs(&jr, &ja, kk, 1);
            }
        }
        g1j_to_affine(&res, &jr);
        g1a_to_bytes(out + 96 * i, &res);
    }
    return 0;
}

/* On-curve check for canonical affine points: returns 1 on curve (or infinity). */
int or_g1_on_curve(const uint8_t *a) {
    g1a_t p;
    if (!g1a_from_bytes(&p, a)) return 0;
    if (p.inf) return 1;
    fq_t l, r, four;
    fq_mul(&l, &p.y, &p.y);
    fq_mul(&r, &p.x, &p.x);
    fq_mul(&r, &r, &p.x);
    fq_from_u64(&four, 4);
    fq_add(&r, &r, &four);
    return fq_eq(&l, &r);
}

/* ------------------------------------------------------------------------ */
/* Variable-base MSM (value of ark-ec VariableBaseMSM::msm_unchecked)        */
/* ------------------------------------------------------------------------ */

typedef struct {
    const g1a_t *bases;
    const fr_t *scalars; /* canonical (non-Montgomery) limbs */
    size_t n;
    int c;
    g1j_t *window_sums;
} msm_ctx;

static void msm_windows(void *vctx, size_t wb, size_t we, int worker) {
    (void)worker;
    msm_ctx *m = (msm_ctx *)vctx;
    size_t nb = ((size_t)1 << m->c) - 1;
    g1j_t *buckets = (g1j_t *)malloc(nb * sizeof(g1j_t));
    for (size_t w = wb; w < we; w++) {
        for (size_t b = 0; b < nb; b++) g1j_set_inf(&buckets[b]);
        unsigned shift = (unsigned)(w * m->c);
        for (size_t i = 0; i < m->n; i++) {
            const uint64_t *s = m->scalars[i].v;
            unsigned limb = shift >> 6, off = shift & 63;
            uint64_t d = s[limb] >> off;
            if (off + m->c > 64 && limb + 1 < 4) d |= s[limb + 1] << (64 - off);
            d &= ((uint64_t)1 << m->c) - 1;
            if (d) g1j_add_affine(&buckets[d - 1], &buckets[d - 1], &m->bases[i]);
        }
        g1j_t run, acc;
        g1j_set_inf(&run);
        g1j_set_inf(&acc);
        for (size_t b = nb; b-- > 0;) {
            g1j_add(&run, &run, &buckets[b]);
            g1j_add(&acc, &acc, &run);
        }
        m->window_sums[w] = acc;
    }
    free(buckets);
}

static void msm_core(g1j_t *out, const g1a_t *bases, const fr_t *canon, size_t n) {
    int c = 3;
    if (n >= 32) {
        int lg = 0;
        while (((size_t)1 << (lg + 1)) <= n) lg++;
        c = lg * 69 / 100 + 2;
    }
    if (c > 16) c = 16;
    size_t windows = (255 + c - 1) / c;
    msm_ctx m = {bases, canon, n, c, (g1j_t *)malloc(windows * sizeof(g1j_t))};
    parallel_for(windows, msm_windows, &m);
    g1j_t total;
    g1j_set_inf(&total);
    for (size_t w = windows; w-- > 0;) {
        for (int k = 0; k < c; k++) g1j_double(&total, &total);
        g1j_add(&total, &total, &m.window_sums[w]);
    }
    free(m.window_sums);
    *out = total;
}

static fr_t *fr_canonical_copy(const fr_t *mont, size_t n) {
    fr_t *c = (fr_t *)malloc((n ? n : 1) * sizeof(fr_t));
    fr_t one;
    memset(&one, 0, sizeof one);
    one.v[0] = 1;
    for (size_t i = 0; i < n; i++) mp_mont_mul(c[i].v, mont[i].v, one.v, FR_P, FR_INV, 4);
    return c;
}

/* bases96: n canonical affine points; scalars32: n canonical Fr. */
int or_msm(const uint8_t *bases96, const uint8_t *scalars32, size_t n, uint8_t *out96) {
    g1a_t *bases = (g1a_t *)malloc((n ? n : 1) * sizeof(g1a_t));
    fr_t *canon = (fr_t *)malloc((n ? n : 1) * sizeof(fr_t));
    for (size_t i = 0; i < n; i++) {
        if (!g1a_from_bytes(&bases[i], bases96 + 96 * i)) { free(bases); free(canon); return 1; }
        memcpy(canon[i].v, scalars32 + 32 * i, 32);
        if (mp_geq(canon[i].v, FR_P, 4)) { free(bases); free(canon); return 1; }
    }
    g1j_t r;
    msm_core(&r, bases, canon, n);
    g1a_t a;
    g1j_to_affine(&a, &r);
    g1a_to_bytes(out96, &a);
    free(bases);
    free(canon);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* MLE operations (backend/src/cpu/multilinear_polynomial.rs)                */
/* ------------------------------------------------------------------------ */

static fr_t *load_fr_table(const uint8_t *bytes, size_t n, int *ok) {
    fr_t *t = (fr_t *)malloc((n ? n : 1) * sizeof(fr_t));
    *ok = 1;
    for (size_t i = 0; i < n; i++)
        if (!fr_from_bytes(&t[i], bytes + 32 * i)) *ok = 0;
    return t;
}
static void store_fr_table(uint8_t *bytes, const fr_t *t, size_t n) {
    for (size_t i = 0; i < n; i++) fr_to_bytes(bytes + 32 * i, &t[i]);
}

/* ark-poly fix_variables with a one-element partial point, in place:
 * f[b] = f[2b] + r * (f[2b+1] - f[2b]) for b < half. */
static void fix_low_variable(fr_t *f, size_t half, const fr_t *r) {
    for (size_t b = 0; b < half; b++) {
        fr_t d;
        fr_sub(&d, &f[2 * b + 1], &f[2 * b]);
        fr_mul(&d, &d, r);
        fr_add(&f[b], &f[2 * b], &d);
    }
}

/* linear_combination (multilinear_polynomial.rs:50-82): zero coefficients are
 * skipped, result keeps nv. */
int or_mle_linear_combination(size_t nv, const uint8_t *const *polys, const uint8_t *coefs,
                              size_t k, uint8_t *out) {
    size_t n = (size_t)1 << nv;
    fr_t *acc = (fr_t *)calloc(n, sizeof(fr_t));
    for (size_t j = 0; j < k; j++) {
        fr_t c;
        if (!fr_from_bytes(&c, coefs + 32 * j)) { free(acc); return 1; }
        if (fr_is_zero(&c)) continue;
        for (size_t i = 0; i < n; i++) {
            fr_t v;
            if (!fr_from_bytes(&v, polys[j] + 32 * i)) { free(acc); return 1; }
            fr_mul(&v, &v, &c);
            fr_add(&acc[i], &acc[i], &v);
        }
    }
    store_fr_table(out, acc, n);
    free(acc);
    return 0;
}

/* evaluate_mle (multilinear_polynomial.rs:84-100 -> ark-poly evaluate):
 * fix the low variable with point[0], then point[1], ... */
int or_mle_evaluate(const uint8_t *poly, size_t nv, const uint8_t *point, uint8_t *out) {
    size_t n = (size_t)1 << nv;
    int ok;
    fr_t *f = load_fr_table(poly, n, &ok);
    if (!ok) { free(f); return 1; }
    for (size_t i = 0; i < nv; i++) {
        fr_t r;
        if (!fr_from_bytes(&r, point + 32 * i)) { free(f); return 1; }
        fix_low_variable(f, n >> (i + 1), &r);
    }
    fr_to_bytes(out, &f[0]);
    free(f);
    return 0;
}

/* build_eq_x_r (common/eq.rs:38-95): r[0] <-> bit 0 of the table index.  The
 * recursion builds the table for r[1..] and then splits each entry b into
 * (b - r0*b, r0*b). */
int or_mle_build_eq_x_r(const uint8_t *r_bytes, size_t nv, uint8_t *out) {
    if (nv == 0) return 1;
    size_t n = (size_t)1 << nv;
    fr_t *buf = (fr_t *)malloc(n * sizeof(fr_t));
    fr_t *tmp = (fr_t *)malloc(n * sizeof(fr_t));
    fr_t r;
    if (!fr_from_bytes(&r, r_bytes + 32 * (nv - 1))) { free(buf); free(tmp); return 1; }
    fr_t one;
    fr_one(&one);
    fr_sub(&buf[0], &one, &r);
    buf[1] = r;
    size_t len = 2;
    for (size_t k = nv - 1; k-- > 0;) {
        if (!fr_from_bytes(&r, r_bytes + 32 * k)) { free(buf); free(tmp); return 1; }
        for (size_t i = 0; i < 2 * len; i++) {
            fr_t bi = buf[i >> 1], t;
            fr_mul(&t, &r, &bi);
            if (i & 1) tmp[i] = t; else fr_sub(&tmp[i], &bi, &t);
        }
        fr_t *sw = buf; buf = tmp; tmp = sw;
        len *= 2;
    }
    store_fr_table(out, buf, n);
    free(buf);
    free(tmp);
    return 0;
}

/* eq_eval (common/eq.rs:15-29) */
int or_eq_eval(const uint8_t *x, const uint8_t *y, size_t n, uint8_t *out) {
    fr_t res, one;
    fr_one(&res);
    fr_one(&one);
    for (size_t i = 0; i < n; i++) {
        fr_t xi, yi, t, u;
        if (!fr_from_bytes(&xi, x + 32 * i) || !fr_from_bytes(&yi, y + 32 * i)) return 1;
        fr_mul(&t, &xi, &yi);
        fr_add(&u, &t, &t);
        fr_sub(&u, &u, &xi);
        fr_sub(&u, &u, &yi);
        fr_add(&u, &u, &one);
        fr_mul(&res, &res, &u);
    }
    fr_to_bytes(out, &res);
    return 0;
}

/* compute_frac_poly (multilinear_polynomial.rs:110-140).  Returns 2 on a zero
 * denominator (checked before inversion), 1 on malformed input. */
int or_mle_frac(size_t nv, const uint8_t *const *nums, const uint8_t *const *dens, size_t k,
                uint8_t *out) {
    size_t n = (size_t)1 << nv;
    if (k == 0) return 1;
    int ok;
    int ok2;
    fr_t *num = load_fr_table(nums[0], n, &ok);
    fr_t *den = load_fr_table(dens[0], n, &ok2);
    ok &= ok2;
    for (size_t j = 1; j < k; j++) {
        for (size_t i = 0; i < n; i++) {
            fr_t v;
            ok &= fr_from_bytes(&v, nums[j] + 32 * i);
            fr_mul(&num[i], &num[i], &v);
            ok &= fr_from_bytes(&v, dens[j] + 32 * i);
            fr_mul(&den[i], &den[i], &v);
        }
    }
    if (!ok) { free(num); free(den); return 1; }
    for (size_t i = 0; i < n; i++)
        if (fr_is_zero(&den[i])) { free(num); free(den); return 2; }
    fr_batch_inverse(den, n);
    for (size_t i = 0; i < n; i++) fr_mul(&num[i], &num[i], &den[i]);
    store_fr_table(out, num, n);
    free(num);
    free(den);
    return 0;
}

/* compute_product_poly (multilinear_polynomial.rs:142-181) */
int or_mle_product_poly(const uint8_t *frac, size_t nv, uint8_t *out) {
    if (nv == 0) return 1;
    size_t n = (size_t)1 << nv;
    int ok;
    fr_t *f = load_fr_table(frac, n, &ok);
    fr_t *e = (fr_t *)malloc(n * sizeof(fr_t));
    size_t len = 0;
    for (size_t i = 0; i < n; i += 2) fr_mul(&e[len++], &f[i], &f[i + 1]);
    for (size_t c = 0; c + 2 <= n - 2; c += 2) {
        fr_mul(&e[len], &e[c], &e[c + 1]);
        len++;
    }
    fr_zero(&e[len++]);
    store_fr_table(out, e, n);
    free(f);
    free(e);
    return 0;
}

/* compute_nums_and_denoms (multilinear_polynomial.rs:183-217) */
int or_mle_nums_denoms(size_t nv, const uint8_t *beta_b, const uint8_t *gamma_b,
                       const uint8_t *const *fxs, const uint8_t *const *gxs,
                       const uint8_t *const *perms, size_t k, uint8_t *const *out_nums,
                       uint8_t *const *out_dens) {
    size_t n = (size_t)1 << nv;
    fr_t beta, gamma;
    if (!fr_from_bytes(&beta, beta_b) || !fr_from_bytes(&gamma, gamma_b)) return 1;
    for (size_t col = 0; col < k; col++) {
        fr_t id, base;
        fr_from_u64(&base, (uint64_t)(col * n));
        fr_mul(&id, &beta, &base);
        for (size_t i = 0; i < n; i++) {
            fr_t f, g, p, a, b;
            if (!fr_from_bytes(&f, fxs[col] + 32 * i) || !fr_from_bytes(&g, gxs[col] + 32 * i) ||
                !fr_from_bytes(&p, perms[col] + 32 * i))
                return 1;
            fr_add(&a, &f, &id);
            fr_add(&a, &a, &gamma);
            fr_mul(&b, &beta, &p);
            fr_add(&b, &g, &b);
            fr_add(&b, &b, &gamma);
            fr_to_bytes(out_nums[col] + 32 * i, &a);
            fr_to_bytes(out_dens[col] + 32 * i, &b);
            fr_add(&id, &id, &beta);
        }
    }
    return 0;
}

/* compute_product_factors (multilinear_polynomial.rs:219-253) */
int or_mle_product_factors(const uint8_t *frac, const uint8_t *prod, size_t nv, uint8_t *p1,
                           uint8_t *p2) {
    if (nv == 0) return 1;
    size_t n = (size_t)1 << nv, half = n / 2;
    for (size_t i = 0; i < half; i++) {
        memcpy(p1 + 32 * i, frac + 64 * i, 32);
        memcpy(p2 + 32 * i, frac + 64 * i + 32, 32);
        memcpy(p1 + 32 * (half + i), prod + 64 * i, 32);
        memcpy(p2 + 32 * (half + i), prod + 64 * i + 32, 32);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* SumCheck prover state (backend/src/cpu/sum_check.rs:35-217)               */
/* ------------------------------------------------------------------------ */

typedef struct {
    size_t round, nv, max_degree, factor_count, product_count;
    fr_t **tables;          /* factor tables, folded in place */
    fr_t *coefs;            /* product coefficients */
    size_t *offsets;        /* product_count + 1 */
    size_t *indices;
    /* barycentric weights: for degree m in 1..max_degree-1, m+1 weights */
    fr_t **weights;
} or_sumcheck;

/* barycentric_weights (sum_check.rs:183-200) for points 0..m */
static void barycentric_weights(fr_t *w, size_t m) {
    for (size_t j = 0; j <= m; j++) {
        fr_t acc, pj, pi, d;
        fr_one(&acc);
        fr_from_u64(&pj, j);
        for (size_t i = 0; i <= m; i++) {
            if (i == j) continue;
            fr_from_u64(&pi, i);
            fr_sub(&d, &pj, &pi);
            fr_mul(&acc, &acc, &d);
        }
        w[j] = acc;
    }
    fr_batch_inverse(w, m + 1);
}

/* extrapolate (sum_check.rs:202-217) from evaluations at 0..m to `at` */
static void extrapolate(fr_t *out, const fr_t *weights, const fr_t *evals, size_t m,
                        const fr_t *at) {
    fr_t *coeffs = (fr_t *)malloc((m + 1) * sizeof(fr_t));
    for (size_t i = 0; i <= m; i++) {
        fr_t pi;
        fr_from_u64(&pi, i);
        fr_sub(&coeffs[i], at, &pi);
    }
    fr_batch_inverse(coeffs, m + 1);
    fr_t sum, res;
    fr_zero(&sum);
    fr_zero(&res);
    for (size_t i = 0; i <= m; i++) {
        fr_mul(&coeffs[i], &coeffs[i], &weights[i]);
        fr_add(&sum, &sum, &coeffs[i]);
    }
    fr_t sum_inv;
    if (fr_is_zero(&sum)) fr_zero(&sum_inv); else fr_inv(&sum_inv, &sum);
    for (size_t i = 0; i <= m; i++) {
        fr_t t;
        fr_mul(&t, &coeffs[i], &evals[i]);
        fr_add(&res, &res, &t);
    }
    fr_mul(out, &res, &sum_inv);
    free(coeffs);
}

void or_sumcheck_destroy(or_sumcheck *s) {
    if (!s) return;
    for (size_t i = 0; i < s->factor_count; i++) free(s->tables[i]);
    free(s->tables);
    free(s->coefs);
    free(s->offsets);
    free(s->indices);
    if (s->weights) {
        for (size_t m = 1; m < s->max_degree; m++) free(s->weights[m]);
        free(s->weights);
    }
    free(s);
}

/* Returns NULL on invalid parameters (nv == 0 or max_degree == 0, malformed
 * product description). */
or_sumcheck *or_sumcheck_create(size_t nv, size_t max_degree, const uint8_t *const *factors,
                                size_t factor_count, const uint8_t *coefs,
                                const size_t *offsets, size_t product_count,
                                const size_t *indices, size_t index_count) {
    if (nv == 0 || max_degree == 0 || offsets[0] != 0 || offsets[product_count] != index_count)
        return NULL;
    for (size_t p = 0; p < product_count; p++) {
        size_t m = offsets[p + 1] - offsets[p];
        if (offsets[p + 1] < offsets[p] || m == 0 || m > max_degree) return NULL;
    }
    for (size_t i = 0; i < index_count; i++)
        if (indices[i] >= factor_count) return NULL;
    or_sumcheck *s = (or_sumcheck *)calloc(1, sizeof(or_sumcheck));
    s->nv = nv;
    s->max_degree = max_degree;
    s->factor_count = factor_count;
    s->product_count = product_count;
    size_t n = (size_t)1 << nv;
    s->tables = (fr_t **)calloc(factor_count ? factor_count : 1, sizeof(fr_t *));
    for (size_t f = 0; f < factor_count; f++) {
        int ok;
        s->tables[f] = load_fr_table(factors[f], n, &ok);
        if (!ok) { or_sumcheck_destroy(s); return NULL; }
    }
    s->coefs = (fr_t *)malloc((product_count ? product_count : 1) * sizeof(fr_t));
    for (size_t p = 0; p < product_count; p++)
        if (!fr_from_bytes(&s->coefs[p], coefs + 32 * p)) { or_sumcheck_destroy(s); return NULL; }
    s->offsets = (size_t *)malloc((product_count + 1) * sizeof(size_t));
    memcpy(s->offsets, offsets, (product_count + 1) * sizeof(size_t));
    s->indices = (size_t *)malloc((index_count ? index_count : 1) * sizeof(size_t));
    if (index_count) memcpy(s->indices, indices, index_count * sizeof(size_t));
    s->weights = (fr_t **)calloc(max_degree + 1, sizeof(fr_t *));
    for (size_t m = 1; m < max_degree; m++) {
        s->weights[m] = (fr_t *)malloc((m + 1) * sizeof(fr_t));
        barycentric_weights(s->weights[m], m);
    }
    return s;
}

typedef struct {
    or_sumcheck *s;
    const size_t *idx;
    size_t m;
    fr_t *partials; /* per worker (m + 1) sums */
} msg_ctx;

static void msg_range(void *vctx, size_t b0, size_t b1, int worker) {
    msg_ctx *c = (msg_ctx *)vctx;
    size_t m = c->m;
    fr_t *acc = c->partials + (size_t)worker * (m + 1);
    fr_t eval[64], step[64];
    for (size_t b = b0; b < b1; b++) {
        for (size_t j = 0; j < m; j++) {
            const fr_t *t = c->s->tables[c->idx[j]];
            eval[j] = t[2 * b];
            fr_sub(&step[j], &t[2 * b + 1], &t[2 * b]);
        }
        fr_t prod;
        prod = eval[0];
        for (size_t j = 1; j < m; j++) fr_mul(&prod, &prod, &eval[j]);
        fr_add(&acc[0], &acc[0], &prod);
        for (size_t k = 1; k <= m; k++) {
            for (size_t j = 0; j < m; j++) fr_add(&eval[j], &eval[j], &step[j]);
            prod = eval[0];
            for (size_t j = 1; j < m; j++) fr_mul(&prod, &prod, &eval[j]);
            fr_add(&acc[k], &acc[k], &prod);
        }
    }
}

typedef struct { or_sumcheck *s; fr_t r; size_t half; } fold_ctx;
static void fold_range(void *vctx, size_t f0, size_t f1, int worker) {
    (void)worker;
    fold_ctx *c = (fold_ctx *)vctx;
    for (size_t f = f0; f < f1; f++) fix_low_variable(c->s->tables[f], c->half, &c->r);
}

/* prove_round_and_update_state (sum_check.rs:74-180).  Returns 0 ok,
 * 2 invalid state (ordering / exhaustion), 1 malformed challenge. */
int or_sumcheck_round(or_sumcheck *s, const uint8_t *challenge, uint8_t *out) {
    if (s->round >= s->nv) return 2;
    if (challenge) {
        if (s->round == 0) return 2;
        fold_ctx fc;
        if (!fr_from_bytes(&fc.r, challenge)) return 1;
        fc.s = s;
        fc.half = (size_t)1 << (s->nv - s->round);
        parallel_for(s->factor_count, fold_range, &fc);
    } else if (s->round > 0) {
        return 2;
    }
    s->round++;
    size_t d = s->max_degree;
    fr_t *sum = (fr_t *)calloc(d + 1, sizeof(fr_t));
    size_t pairs = (size_t)1 << (s->nv - s->round);
    for (size_t p = 0; p < s->product_count; p++) {
        size_t m = s->offsets[p + 1] - s->offsets[p];
        int workers = g_threads > 0 ? g_threads : 1;
        msg_ctx mc = {s, s->indices + s->offsets[p], m,
                      (fr_t *)calloc((size_t)workers * (m + 1), sizeof(fr_t))};
        parallel_for(pairs, msg_range, &mc);
        fr_t *ps = (fr_t *)calloc(m + 1, sizeof(fr_t));
        for (int w = 0; w < workers; w++)
            for (size_t k = 0; k <= m; k++) fr_add(&ps[k], &ps[k], &mc.partials[w * (m + 1) + k]);
        for (size_t k = 0; k <= m; k++) fr_mul(&ps[k], &ps[k], &s->coefs[p]);
        for (size_t k = 0; k <= m; k++) fr_add(&sum[k], &sum[k], &ps[k]);
        for (size_t i = 0; i + m < d; i++) {
            fr_t at, e;
            fr_from_u64(&at, (uint64_t)(m + 1 + i));
            extrapolate(&e, s->weights[m], ps, m, &at);
            fr_add(&sum[m + 1 + i], &sum[m + 1 + i], &e);
        }
        free(ps);
        free(mc.partials);
    }
    store_fr_table(out, sum, d + 1);
    free(sum);
    return 0;
}

/* Final folded evaluations: fix the last variable with r_nv on a copy and
 * return each factor's single value (factor order).  Equals evaluate_mle of
 * each factor at the full challenge point.  State must have run all rounds. */
int or_sumcheck_final(or_sumcheck *s, const uint8_t *challenge, uint8_t *out) {
    if (s->round != s->nv) return 2;
    fr_t r;
    if (!fr_from_bytes(&r, challenge)) return 1;
    for (size_t f = 0; f < s->factor_count; f++) {
        fr_t *t = s->tables[f], d, v;
        fr_sub(&d, &t[1], &t[0]);
        fr_mul(&d, &d, &r);
        fr_add(&v, &t[0], &d);
        fr_to_bytes(out + 32 * f, &v);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Multilinear KZG (backend/src/cpu/multilinear_kzg.rs:40-137)               */
/* ------------------------------------------------------------------------ */

/* commit: MSM of the polynomial against layer (pp_nv - nv), given directly. */
int or_kzg_commit(const uint8_t *layer96, const uint8_t *evals, size_t nv, uint8_t *out96) {
    return or_msm(layer96, evals, (size_t)1 << nv, out96);
}

/* open: layers96[i] is layer (pp_nv - nv + 1 + i) for i < nv, of size
 * 2^(nv-1-i).  Writes nv affine quotient commitments and the evaluation. */
int or_kzg_open(const uint8_t *const *layers96, const uint8_t *poly, size_t nv,
                const uint8_t *point, uint8_t *out_q96, uint8_t *out_eval) {
    size_t n = (size_t)1 << nv;
    int ok;
    fr_t *f = load_fr_table(poly, n, &ok);
    if (!ok) { free(f); return 1; }
    if (nv == 0) {
        fr_to_bytes(out_eval, &f[0]);
        free(f);
        return 0;
    }
    fr_t *q = (fr_t *)malloc((n / 2) * sizeof(fr_t));
    for (size_t i = 0; i < nv; i++) {
        fr_t z;
        if (!fr_from_bytes(&z, point + 32 * i)) { free(f); free(q); return 1; }
        size_t cur = n >> (i + 1);
        for (size_t b = 0; b < cur; b++) {
            fr_t low = f[2 * b], t;
            fr_sub(&q[b], &f[2 * b + 1], &low);
            fr_mul(&t, &q[b], &z);
            fr_add(&f[b], &low, &t);
        }
        g1a_t *bases = (g1a_t *)malloc(cur * sizeof(g1a_t));
        for (size_t b = 0; b < cur; b++) g1a_from_bytes(&bases[b], layers96[i] + 96 * b);
        fr_t *canon = fr_canonical_copy(q, cur);
        g1j_t r;
        msm_core(&r, bases, canon, cur);
        g1a_t a;
        g1j_to_affine(&a, &r);
        g1a_to_bytes(out_q96 + 96 * i, &a);
        free(bases);
        free(canon);
    }
    fr_to_bytes(out_eval, &f[0]);
    free(f);
    free(q);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Fixture RNG: ChaCha20 block function (RFC 8439) keyed by a 64-bit seed.   */
/* Fr element i of a stream is from_le_bytes_mod_order of keystream block i. */
/* Block index i: counter = low 32 bits, nonce word 0 = high 32 bits.        */
/* ------------------------------------------------------------------------ */

#define ROTL32(v, n) (((v) << (n)) | ((v) >> (32 - (n))))
#define QR(a, b, c, d)                    \
    a += b; d ^= a; d = ROTL32(d, 16);    \
    c += d; b ^= c; b = ROTL32(b, 12);    \
    a += b; d ^= a; d = ROTL32(d, 8);     \
    c += d; b ^= c; b = ROTL32(b, 7);

static void chacha20_block(uint64_t seed, uint64_t index, uint8_t out[64]) {
    uint32_t s[16] = {0x61707865, 0x3320646e, 0x79622d32, 0x6b206574,
                      (uint32_t)seed, (uint32_t)(seed >> 32), 0, 0, 0, 0, 0, 0,
                      (uint32_t)index, (uint32_t)(index >> 32), 0, 0};
    uint32_t x[16];
    memcpy(x, s, sizeof x);
    for (int i = 0; i < 10; i++) {
        QR(x[0], x[4], x[8], x[12]);
        QR(x[1], x[5], x[9], x[13]);
        QR(x[2], x[6], x[10], x[14]);
        QR(x[3], x[7], x[11], x[15]);
        QR(x[0], x[5], x[10], x[15]);
        QR(x[1], x[6], x[11], x[12]);
        QR(x[2], x[7], x[8], x[13]);
        QR(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; i++) {
        uint32_t v = x[i] + s[i];
        out[4 * i] = (uint8_t)v;
        out[4 * i + 1] = (uint8_t)(v >> 8);
        out[4 * i + 2] = (uint8_t)(v >> 16);
        out[4 * i + 3] = (uint8_t)(v >> 24);
    }
}

void or_chacha20_block(uint64_t seed, uint64_t index, uint8_t *out64) {
    chacha20_block(seed, index, out64);
}

typedef struct { uint64_t seed, first; uint8_t *out; } rng_ctx;
static void rng_range(void *vctx, size_t b, size_t e, int worker) {
    (void)worker;
    rng_ctx *c = (rng_ctx *)vctx;
    uint8_t blk[64];
    for (size_t i = b; i < e; i++) {
        fr_t x;
        chacha20_block(c->seed, c->first + i, blk);
        fr_from_wide64(&x, blk);
        fr_to_bytes(c->out + 32 * i, &x);
    }
}

/* n canonical Fr from stream `seed`, blocks [first, first + n). */
void or_random_fr(uint64_t seed, uint64_t first, size_t n, uint8_t *out) {
    rng_ctx c = {seed, first, out};
    parallel_for(n, rng_range, &c);
}

/* ------------------------------------------------------------------------ */
/* Vanilla-plonk fixture (the full-prove workload), restated independently  */
/* of the product's generator.  Gate of hyperplonk/src/custom_gate.rs:86-96  */
/* (q_L w1 + q_R w2 + q_O w3 + q_M w1 w2 + q_C = 0, selectors [q_L, q_R,     */
/* q_O, q_M, q_C]); q_L, q_R, q_M, q_C = stream `seed` elements [k n,        */
/* (k+1) n) for k = 0..3, w1 = elements [4n, 5n), q_O = -1 and w3 solves the */
/* gate.  w1 and w2 come from stream `witness_seed` (= `seed` for the       */
/* circuit's own witness; another value gives another satisfying witness).  */
/*  - plain (wired = 0): w2 = elements [5n, 6n) and the identity permutation */
/*    over the 3 witness columns (label of cell (column k, row i) = k n + i,  */
/*    backend/src/common/permutation.rs:12-15);                              */
/*  - wired (wired = 1): w2[i] = w1[pi(i)] with pi(i) = (A i + B) mod n, A  */
/*    odd (a bijection of Z_n), B = seed * C1 + 1; every w2 cell i and w1   */
/*    cell pi(i) are swapped by the permutation (a 2-cycle: the copy         */
/*    constraint w2[i] = w1[pi(i)] holds), w3 cells stay fixed.  The         */
/*    product check then sees random fractions instead of ones.              */
/* ------------------------------------------------------------------------ */

#define WIRE_A 0x9E3779B97F4A7C15ULL
#define WIRE_C1 0xD1B54A32D192ED03ULL

typedef struct {
    uint64_t seed, witness_seed;
    size_t n;
    int wired;
    uint8_t *sel, *wit, *perm;
} fixture_ctx;

static size_t wire_of(uint64_t seed, size_t n, size_t i) {
    return (size_t)((WIRE_A * (uint64_t)i + seed * WIRE_C1 + 1) & (uint64_t)(n - 1));
}

static void stream_fr(uint64_t seed, uint64_t index, fr_t *out) {
    uint8_t blk[64];
    chacha20_block(seed, index, blk);
    fr_from_wide64(out, blk); /* Montgomery form */
}

static void put_label(uint8_t *dst, uint64_t label) {
    memset(dst, 0, 32);
    for (int b = 0; b < 8; b++) dst[b] = (uint8_t)(label >> (8 * b));
}

static void fixture_range(void *vctx, size_t b, size_t e, int worker) {
    (void)worker;
    fixture_ctx *c = (fixture_ctx *)vctx;
    const size_t n = c->n;
    fr_t minus_one, zero;
    fr_zero(&zero);
    fr_one(&minus_one);
    fr_sub(&minus_one, &zero, &minus_one);
    for (size_t i = b; i < e; i++) {
        fr_t ql, qr, qm, qc, w1, w2, w3, t;
        stream_fr(c->seed, i, &ql);
        stream_fr(c->seed, n + i, &qr);
        stream_fr(c->seed, 2 * n + i, &qm);
        stream_fr(c->seed, 3 * n + i, &qc);
        stream_fr(c->witness_seed, 4 * n + i, &w1);
        size_t pi = c->wired ? wire_of(c->seed, n, i) : i;
        stream_fr(c->witness_seed, c->wired ? 4 * n + pi : 5 * n + i, &w2);
        fr_mul(&w3, &ql, &w1);
        fr_mul(&t, &qr, &w2);
        fr_add(&w3, &w3, &t);
        fr_mul(&t, &qm, &w1);
        fr_mul(&t, &t, &w2);
        fr_add(&w3, &w3, &t);
        fr_add(&w3, &w3, &qc);
        const fr_t *sel[5] = {&ql, &qr, &minus_one, &qm, &qc};
        const fr_t *wit[3] = {&w1, &w2, &w3};
        for (int k = 0; k < 5; k++) fr_to_bytes(c->sel + 32 * ((size_t)k * n + i), sel[k]);
        for (int k = 0; k < 3; k++) fr_to_bytes(c->wit + 32 * ((size_t)k * n + i), wit[k]);
        if (c->wired) {
            put_label(c->perm + 32 * pi, (uint64_t)n + i);       /* w1 cell pi(i) -> w2 cell i */
            put_label(c->perm + 32 * (n + i), (uint64_t)pi);     /* w2 cell i -> w1 cell pi(i) */
        } else {
            put_label(c->perm + 32 * i, (uint64_t)i);
            put_label(c->perm + 32 * (n + i), (uint64_t)n + i);
        }
        put_label(c->perm + 32 * (2 * n + i), 2 * (uint64_t)n + i);
    }
}

/* Writes 5 selector tables (sel: 5 * 2^nv Fr), 3 witness tables and 3
 * permutation tables, canonical LE32, table-major.  Returns 1 for nv > 28. */
int or_fixture_vanilla_plonk(uint64_t seed, uint64_t witness_seed, size_t nv, int wired, uint8_t *sel, uint8_t *wit,
                             uint8_t *perm) {
    if (nv > 28) return 1;
    fixture_ctx c = {seed, witness_seed, (size_t)1 << nv, wired != 0, sel, wit, perm};
    parallel_for(c.n, fixture_range, &c);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Testing SRS (subroutines/src/pcs/multilinear_kzg/srs.rs:158-235)          */
/* g = s*G1 and t[0..nv) from the fixture stream `seed` (t_i = block i,      */
/* s = block nv).  Layer i (i < nv) = g * eq(t[i..], x) over 2^(nv-i) x with */
/* t[i] <-> bit 0; layer nv = [g].  Output: the layers back to back, 96 B   */
/* canonical affine each (2^(nv+1) - 1 + 1 points).                          */
/* ------------------------------------------------------------------------ */

typedef struct {
    const g1a_t *table; /* 32 windows x 256 entries of (d * 2^(8w)) * g */
    const fr_t *scalars; /* Montgomery */
    g1j_t *out;
} fixed_ctx;

static void fixed_range(void *vctx, size_t b, size_t e, int worker) {
    (void)worker;
    fixed_ctx *c = (fixed_ctx *)vctx;
    fr_t one;
    memset(&one, 0, sizeof one);
    one.v[0] = 1;
    for (size_t i = b; i < e; i++) {
        fr_t k;
        mp_mont_mul(k.v, c->scalars[i].v, one.v, FR_P, FR_INV, 4);
        g1j_t acc;
        g1j_set_inf(&acc);
        for (int w = 0; w < 32; w++) {
            unsigned d = (unsigned)((k.v[w / 8] >> (8 * (w % 8))) & 0xff);
            if (d) g1j_add_affine(&acc, &acc, &c->table[w * 256 + d]);
        }
        c->out[i] = acc;
    }
}

typedef struct { const g1j_t *in; g1a_t *out; size_t chunk; } norm_ctx;
static void norm_range(void *vctx, size_t b, size_t e, int worker) {
    (void)worker;
    norm_ctx *c = (norm_ctx *)vctx;
    for (size_t blk = b; blk < e; blk++) {
        size_t s = blk * c->chunk;
        g1j_batch_to_affine(c->out + s, c->in + s, c->chunk);
    }
}

/* Fixed-base multiplication of g by n Montgomery scalars -> affine. */
static void fixed_base_batch(const g1a_t *g, const fr_t *scalars, size_t n, g1a_t *out) {
    g1a_t *table = (g1a_t *)malloc(32 * 256 * sizeof(g1a_t));
    g1j_t *jt = (g1j_t *)malloc(32 * 256 * sizeof(g1j_t));
    g1j_t base;
    g1a_to_jac(&base, g);
    for (int w = 0; w < 32; w++) {
        g1j_set_inf(&jt[w * 256]);
        for (int d = 1; d < 256; d++) g1j_add(&jt[w * 256 + d], &jt[w * 256 + d - 1], &base);
        for (int k = 0; k < 8; k++) g1j_double(&base, &base);
    }
    g1j_batch_to_affine(table, jt, 32 * 256);
    free(jt);
    g1j_t *proj = (g1j_t *)malloc((n ? n : 1) * sizeof(g1j_t));
    fixed_ctx fc = {table, scalars, proj};
    parallel_for(n, fixed_range, &fc);
    size_t chunk = 1024;
    size_t full = n / chunk;
    norm_ctx nc = {proj, out, chunk};
    parallel_for(full, norm_range, &nc);
    if (n % chunk) g1j_batch_to_affine(out + full * chunk, proj + full * chunk, n % chunk);
    free(proj);
    free(table);
}

static const uint8_t G1_GEN_X[48] = {
    0xbb, 0xc6, 0x22, 0xdb, 0x0a, 0xf0, 0x3a, 0xfb, 0xef, 0x1a, 0x7a, 0xf9, 0x3f, 0xe8, 0x55, 0x6c,
    0x58, 0xac, 0x1b, 0x17, 0x3f, 0x3a, 0x4e, 0xa1, 0x05, 0xb9, 0x74, 0x97, 0x4f, 0x8c, 0x68, 0xc3,
    0x0f, 0xac, 0xa9, 0x4f, 0x8c, 0x63, 0x95, 0x26, 0x94, 0xd7, 0x97, 0x31, 0xa7, 0xd3, 0xf1, 0x17};
static const uint8_t G1_GEN_Y[48] = {
    0xe1, 0xe7, 0xc5, 0x46, 0x29, 0x23, 0xaa, 0x0c, 0xe4, 0x8a, 0x88, 0xa2, 0x44, 0xc7, 0x3c, 0xd0,
    0xed, 0xb3, 0x04, 0x2c, 0xcb, 0x18, 0xdb, 0x00, 0xf6, 0x0a, 0xd0, 0xd5, 0x95, 0xe0, 0xf5, 0xfc,
    0xe4, 0x8a, 0x1d, 0x74, 0xed, 0x30, 0x9e, 0xa0, 0xf1, 0xa0, 0xaa, 0xe3, 0x81, 0xf4, 0xb3, 0x08};

void or_g1_generator(uint8_t *out96) {
    memcpy(out96, G1_GEN_X, 48);
    memcpy(out96 + 48, G1_GEN_Y, 48);
}

int or_srs_gen(size_t nv, uint64_t seed, uint8_t *out) {
    if (nv == 0 || nv > 28) return 1;
    fr_t *t = (fr_t *)malloc((nv + 1) * sizeof(fr_t));
    uint8_t blk[64];
    for (size_t i = 0; i <= nv; i++) {
        chacha20_block(seed, i, blk);
        fr_from_wide64(&t[i], blk);
    }
    /* g = s * G1 generator */
    g1a_t gen, g;
    {
        uint8_t gb[96];
        or_g1_generator(gb);
        g1a_from_bytes(&gen, gb);
    }
    fr_t sc;
    mp_mont_mul(sc.v, t[nv].v, (const uint64_t[4]){1, 0, 0, 0}, FR_P, FR_INV, 4);
    g1j_t gj, gs;
    g1a_to_jac(&gj, &gen);
    g1j_mul_limbs(&gs, &gj, sc.v, 4);
    g1j_to_affine(&g, &gs);

    size_t total = ((size_t)1 << (nv + 1)) - 2; /* points in layers 0..nv-1 */
    fr_t *scal = (fr_t *)malloc(total * sizeof(fr_t));
    size_t off = 0;
    uint8_t *rb = (uint8_t *)malloc(32 * nv);
    for (size_t i = 0; i < nv; i++) fr_to_bytes(rb + 32 * i, &t[i]);
    for (size_t i = 0; i < nv; i++) {
        size_t sz = (size_t)1 << (nv - i);
        uint8_t *eqb = (uint8_t *)malloc(32 * sz);
        or_mle_build_eq_x_r(rb + 32 * i, nv - i, eqb);
        for (size_t x = 0; x < sz; x++) fr_from_bytes(&scal[off + x], eqb + 32 * x);
        free(eqb);
        off += sz;
    }
    g1a_t *pts = (g1a_t *)malloc(total * sizeof(g1a_t));
    fixed_base_batch(&g, scal, total, pts);
    for (size_t i = 0; i < total; i++) g1a_to_bytes(out + 96 * i, &pts[i]);
    g1a_to_bytes(out + 96 * total, &g);
    free(pts);
    free(scal);
    free(rb);
    free(t);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* BLS12-381 pairing -- for the verifier only (multilinear_kzg/mod.rs:169-221,
 * hyperplonk/src/snark.rs verify).  Textbook forms, written for clarity:
 *   Fq2  = Fq[u]/(u^2 + 1)
 *   Fq6  = Fq2[v]/(v^3 - xi), xi = 1 + u
 *   Fq12 = Fq6[w]/(w^2 - v)
 *   G2   = r-torsion of E': y^2 = x^3 + 4 xi over Fq2, mapped into E(Fq12)
 *          by (x, y) -> (x w^-2, y w^-3) (w^6 = xi)
 *   e(P, Q) = f_{|z|, Q}(P)^((p^12 - 1) / r), conjugated as z < 0, with the
 *   optimal-ate loop parameter |z| = 0xd201000000010000 and affine line
 *   functions in Fq12 (vertical lines dropped: they vanish under the final
 *   exponentiation).
 * The final exponent and the G2 cofactor are large integers computed by the
 * caller from p, r and z and passed in as little-endian 64-bit limbs.       */
/* ------------------------------------------------------------------------ */

typedef struct { fq_t c0, c1; } fq2_t;
typedef struct { fq2_t c0, c1, c2; } fq6_t;
typedef struct { fq6_t c0, c1; } fq12_t;

static void fq2_add(fq2_t *r, const fq2_t *a, const fq2_t *b) {
    fq_add(&r->c0, &a->c0, &b->c0);
    fq_add(&r->c1, &a->c1, &b->c1);
}
static void fq2_sub(fq2_t *r, const fq2_t *a, const fq2_t *b) {
    fq_sub(&r->c0, &a->c0, &b->c0);
    fq_sub(&r->c1, &a->c1, &b->c1);
}
static void fq2_neg(fq2_t *r, const fq2_t *a) {
    fq_neg(&r->c0, &a->c0);
    fq_neg(&r->c1, &a->c1);
}
static void fq2_mul(fq2_t *r, const fq2_t *a, const fq2_t *b) {
    fq_t t0, t1, t2, t3;
    fq_mul(&t0, &a->c0, &b->c0);
    fq_mul(&t1, &a->c1, &b->c1);
    fq_mul(&t2, &a->c0, &b->c1);
    fq_mul(&t3, &a->c1, &b->c0);
    fq_sub(&r->c0, &t0, &t1);
    fq_add(&r->c1, &t2, &t3);
}
static void fq2_mul_xi(fq2_t *r, const fq2_t *a) { /* (c0 + c1 u)(1 + u) */
    fq_t t0, t1;
    fq_sub(&t0, &a->c0, &a->c1);
    fq_add(&t1, &a->c0, &a->c1);
    r->c0 = t0;
    r->c1 = t1;
}
static void fq2_inv(fq2_t *r, const fq2_t *a) { /* (c0 - c1 u) / (c0^2 + c1^2) */
    fq_t n, t, ninv;
    fq_mul(&n, &a->c0, &a->c0);
    fq_mul(&t, &a->c1, &a->c1);
    fq_add(&n, &n, &t);
    fq_inv(&ninv, &n);
    fq_mul(&r->c0, &a->c0, &ninv);
    fq_mul(&t, &a->c1, &ninv);
    fq_neg(&r->c1, &t);
}
static int fq2_is_zero(const fq2_t *a) { return fq_is_zero(&a->c0) && fq_is_zero(&a->c1); }
static int fq2_eq(const fq2_t *a, const fq2_t *b) { return fq_eq(&a->c0, &b->c0) && fq_eq(&a->c1, &b->c1); }
static void fq2_zero(fq2_t *r) { fq_zero(&r->c0); fq_zero(&r->c1); }
static void fq2_one(fq2_t *r) { fq_one(&r->c0); fq_zero(&r->c1); }

static void fq6_add(fq6_t *r, const fq6_t *a, const fq6_t *b) {
    fq2_add(&r->c0, &a->c0, &b->c0);
    fq2_add(&r->c1, &a->c1, &b->c1);
    fq2_add(&r->c2, &a->c2, &b->c2);
}
static void fq6_sub(fq6_t *r, const fq6_t *a, const fq6_t *b) {
    fq2_sub(&r->c0, &a->c0, &b->c0);
    fq2_sub(&r->c1, &a->c1, &b->c1);
    fq2_sub(&r->c2, &a->c2, &b->c2);
}
static void fq6_neg(fq6_t *r, const fq6_t *a) {
    fq2_neg(&r->c0, &a->c0);
    fq2_neg(&r->c1, &a->c1);
    fq2_neg(&r->c2, &a->c2);
}
static void fq6_mul(fq6_t *r, const fq6_t *a, const fq6_t *b) {
    fq2_t a0b0, a1b1, a2b2, a0b1, a1b0, a0b2, a2b0, a1b2, a2b1, t;
    fq2_mul(&a0b0, &a->c0, &b->c0);
    fq2_mul(&a1b1, &a->c1, &b->c1);
    fq2_mul(&a2b2, &a->c2, &b->c2);
    fq2_mul(&a0b1, &a->c0, &b->c1);
    fq2_mul(&a1b0, &a->c1, &b->c0);
    fq2_mul(&a0b2, &a->c0, &b->c2);
    fq2_mul(&a2b0, &a->c2, &b->c0);
    fq2_mul(&a1b2, &a->c1, &b->c2);
    fq2_mul(&a2b1, &a->c2, &b->c1);
    fq6_t o;
    fq2_add(&t, &a1b2, &a2b1); /* c0 = a0b0 + xi (a1b2 + a2b1) */
    fq2_mul_xi(&t, &t);
    fq2_add(&o.c0, &a0b0, &t);
    fq2_mul_xi(&t, &a2b2); /* c1 = a0b1 + a1b0 + xi a2b2 */
    fq2_add(&o.c1, &a0b1, &a1b0);
    fq2_add(&o.c1, &o.c1, &t);
    fq2_add(&o.c2, &a0b2, &a1b1); /* c2 = a0b2 + a1b1 + a2b0 */
    fq2_add(&o.c2, &o.c2, &a2b0);
    *r = o;
}
static void fq6_mul_v(fq6_t *r, const fq6_t *a) { /* (c0, c1, c2) v = (xi c2, c0, c1) */
    fq6_t o;
    fq2_mul_xi(&o.c0, &a->c2);
    o.c1 = a->c0;
    o.c2 = a->c1;
    *r = o;
}
static void fq6_inv(fq6_t *r, const fq6_t *a) {
    /* (A + B v + C v^2) / N, A = a0^2 - xi a1 a2, B = xi a2^2 - a0 a1,
     * C = a1^2 - a0 a2, N = a0 A + xi (a2 B + a1 C) */
    fq2_t A, B, C, t, n, ninv;
    fq2_mul(&A, &a->c0, &a->c0);
    fq2_mul(&t, &a->c1, &a->c2);
    fq2_mul_xi(&t, &t);
    fq2_sub(&A, &A, &t);
    fq2_mul(&B, &a->c2, &a->c2);
    fq2_mul_xi(&B, &B);
    fq2_mul(&t, &a->c0, &a->c1);
    fq2_sub(&B, &B, &t);
    fq2_mul(&C, &a->c1, &a->c1);
    fq2_mul(&t, &a->c0, &a->c2);
    fq2_sub(&C, &C, &t);
    fq2_mul(&n, &a->c2, &B);
    fq2_mul(&t, &a->c1, &C);
    fq2_add(&n, &n, &t);
    fq2_mul_xi(&n, &n);
    fq2_mul(&t, &a->c0, &A);
    fq2_add(&n, &n, &t);
    fq2_inv(&ninv, &n);
    fq2_mul(&r->c0, &A, &ninv);
    fq2_mul(&r->c1, &B, &ninv);
    fq2_mul(&r->c2, &C, &ninv);
}
static void fq6_zero(fq6_t *r) { fq2_zero(&r->c0); fq2_zero(&r->c1); fq2_zero(&r->c2); }
static void fq6_one(fq6_t *r) { fq2_one(&r->c0); fq2_zero(&r->c1); fq2_zero(&r->c2); }
static int fq6_eq(const fq6_t *a, const fq6_t *b) {
    return fq2_eq(&a->c0, &b->c0) && fq2_eq(&a->c1, &b->c1) && fq2_eq(&a->c2, &b->c2);
}

static void fq12_add(fq12_t *r, const fq12_t *a, const fq12_t *b) {
    fq6_add(&r->c0, &a->c0, &b->c0);
    fq6_add(&r->c1, &a->c1, &b->c1);
}
static void fq12_sub(fq12_t *r, const fq12_t *a, const fq12_t *b) {
    fq6_sub(&r->c0, &a->c0, &b->c0);
    fq6_sub(&r->c1, &a->c1, &b->c1);
}
static void fq12_mul(fq12_t *r, const fq12_t *a, const fq12_t *b) {
    /* (a0 + a1 w)(b0 + b1 w) = a0 b0 + v a1 b1 + (a0 b1 + a1 b0) w */
    fq6_t t0, t1, t2, t3;
    fq6_mul(&t0, &a->c0, &b->c0);
    fq6_mul(&t1, &a->c1, &b->c1);
    fq6_mul(&t2, &a->c0, &b->c1);
    fq6_mul(&t3, &a->c1, &b->c0);
    fq6_mul_v(&t1, &t1);
    fq6_add(&r->c0, &t0, &t1);
    fq6_add(&r->c1, &t2, &t3);
}
static void fq12_inv(fq12_t *r, const fq12_t *a) { /* (a0 - a1 w) / (a0^2 - v a1^2) */
    fq6_t n, t, ninv;
    fq6_mul(&n, &a->c0, &a->c0);
    fq6_mul(&t, &a->c1, &a->c1);
    fq6_mul_v(&t, &t);
    fq6_sub(&n, &n, &t);
    fq6_inv(&ninv, &n);
    fq6_mul(&r->c0, &a->c0, &ninv);
    fq6_mul(&t, &a->c1, &ninv);
    fq6_neg(&r->c1, &t);
}
static void fq12_conj(fq12_t *r, const fq12_t *a) { r->c0 = a->c0; fq6_neg(&r->c1, &a->c1); }
static void fq12_one(fq12_t *r) { fq6_one(&r->c0); fq6_zero(&r->c1); }
static int fq12_eq(const fq12_t *a, const fq12_t *b) { return fq6_eq(&a->c0, &b->c0) && fq6_eq(&a->c1, &b->c1); }
static void fq12_from_fq2(fq12_t *r, const fq2_t *a) {
    fq6_zero(&r->c0);
    fq6_zero(&r->c1);
    r->c0.c0 = *a;
}
static void fq12_from_fq(fq12_t *r, const fq_t *a) {
    fq2_t t;
    t.c0 = *a;
    fq_zero(&t.c1);
    fq12_from_fq2(r, &t);
}
static void fq12_pow(fq12_t *r, const fq12_t *a, const uint64_t *e, size_t limbs) {
    fq12_t acc;
    fq12_one(&acc);
    int started = 0;
    for (size_t i = limbs; i-- > 0;)
        for (int bit = 63; bit >= 0; bit--) {
            if (started) fq12_mul(&acc, &acc, &acc);
            if ((e[i] >> bit) & 1) {
                fq12_mul(&acc, &acc, a);
                started = 1;
            }
        }
    *r = acc;
}

/* sqrt in Fq (p = 3 mod 4): a^((p+1)/4); returns 1 iff a is a square */
static int fq_sqrt(fq_t *r, const fq_t *a) {
    uint64_t e[6];
    memcpy(e, FQ_P, sizeof e);
    e[0] += 1; /* p + 1: p's low limb ends in ...aaab, no carry */
    for (int i = 0; i < 6; i++) e[i] = (e[i] >> 2) | (i < 5 ? e[i + 1] << 62 : 0);
    fq_t s, chk;
    fq_pow(&s, a, e);
    fq_mul(&chk, &s, &s);
    if (!fq_eq(&chk, a)) return 0;
    *r = s;
    return 1;
}

/* sqrt in Fq2 by the norm method; returns 1 iff a is a square */
static int fq2_sqrt(fq2_t *r, const fq2_t *a) {
    if (fq2_is_zero(a)) {
        fq2_zero(r);
        return 1;
    }
    fq_t two, half;
    fq_from_u64(&two, 2);
    fq_inv(&half, &two);
    fq2_t cand;
    if (fq_is_zero(&a->c1)) {
        fq_t s, n;
        if (fq_sqrt(&s, &a->c0)) {
            cand.c0 = s;
            fq_zero(&cand.c1);
        } else {
            fq_neg(&n, &a->c0);
            if (!fq_sqrt(&s, &n)) return 0;
            fq_zero(&cand.c0);
            cand.c1 = s; /* (s u)^2 = -s^2 */
        }
    } else {
        fq_t alpha, t, gamma, delta, x0, x1, d;
        fq_mul(&alpha, &a->c0, &a->c0);
        fq_mul(&t, &a->c1, &a->c1);
        fq_add(&alpha, &alpha, &t);
        if (!fq_sqrt(&gamma, &alpha)) return 0;
        fq_add(&delta, &a->c0, &gamma);
        fq_mul(&delta, &delta, &half);
        if (!fq_sqrt(&x0, &delta)) {
            fq_sub(&delta, &a->c0, &gamma);
            fq_mul(&delta, &delta, &half);
            if (!fq_sqrt(&x0, &delta)) return 0;
        }
        fq_add(&d, &x0, &x0);
        fq_inv(&d, &d);
        fq_mul(&x1, &a->c1, &d);
        cand.c0 = x0;
        cand.c1 = x1;
    }
    fq2_t chk;
    fq2_mul(&chk, &cand, &cand);
    if (!fq2_eq(&chk, a)) return 0;
    *r = cand;
    return 1;
}

typedef struct { fq2_t x, y; int inf; } g2a_t;

static void g2_b(fq2_t *b) { /* 4 xi = 4 + 4u */
    fq_from_u64(&b->c0, 4);
    fq_from_u64(&b->c1, 4);
}
static int g2_on_curve(const g2a_t *p) {
    if (p->inf) return 1;
    fq2_t l, r, b;
    fq2_mul(&l, &p->y, &p->y);
    fq2_mul(&r, &p->x, &p->x);
    fq2_mul(&r, &r, &p->x);
    g2_b(&b);
    fq2_add(&r, &r, &b);
    return fq2_eq(&l, &r);
}
static void g2_double(g2a_t *r, const g2a_t *p) {
    if (p->inf || fq2_is_zero(&p->y)) {
        memset(r, 0, sizeof *r);
        r->inf = 1;
        return;
    }
    fq2_t lam, t, d, x3, y3;
    fq2_mul(&t, &p->x, &p->x);
    fq2_add(&lam, &t, &t);
    fq2_add(&lam, &lam, &t);
    fq2_add(&d, &p->y, &p->y);
    fq2_inv(&d, &d);
    fq2_mul(&lam, &lam, &d);
    fq2_mul(&x3, &lam, &lam);
    fq2_sub(&x3, &x3, &p->x);
    fq2_sub(&x3, &x3, &p->x);
    fq2_sub(&t, &p->x, &x3);
    fq2_mul(&y3, &lam, &t);
    fq2_sub(&y3, &y3, &p->y);
    r->x = x3;
    r->y = y3;
    r->inf = 0;
}
static void g2_add(g2a_t *r, const g2a_t *p, const g2a_t *q) {
    if (p->inf) { *r = *q; return; }
    if (q->inf) { *r = *p; return; }
    if (fq2_eq(&p->x, &q->x)) {
        if (fq2_eq(&p->y, &q->y)) g2_double(r, p);
        else { memset(r, 0, sizeof *r); r->inf = 1; }
        return;
    }
    fq2_t lam, t, d, x3, y3;
    fq2_sub(&lam, &q->y, &p->y);
    fq2_sub(&d, &q->x, &p->x);
    fq2_inv(&d, &d);
    fq2_mul(&lam, &lam, &d);
    fq2_mul(&x3, &lam, &lam);
    fq2_sub(&x3, &x3, &p->x);
    fq2_sub(&x3, &x3, &q->x);
    fq2_sub(&t, &p->x, &x3);
    fq2_mul(&y3, &lam, &t);
    fq2_sub(&y3, &y3, &p->y);
    r->x = x3;
    r->y = y3;
    r->inf = 0;
}
static void g2_mul(g2a_t *r, const g2a_t *p, const uint64_t *k, size_t limbs) {
    g2a_t acc;
    memset(&acc, 0, sizeof acc);
    acc.inf = 1;
    for (size_t i = limbs; i-- > 0;)
        for (int bit = 63; bit >= 0; bit--) {
            g2_double(&acc, &acc);
            if ((k[i] >> bit) & 1) g2_add(&acc, &acc, p);
        }
    *r = acc;
}
static int g2_from_bytes(g2a_t *r, const uint8_t *b) {
    int zero = 1;
    for (int i = 0; i < 192; i++) zero &= b[i] == 0;
    memset(r, 0, sizeof *r);
    if (zero) {
        r->inf = 1;
        return 1;
    }
    return fq_from_bytes(&r->x.c0, b) && fq_from_bytes(&r->x.c1, b + 48) && fq_from_bytes(&r->y.c0, b + 96) &&
           fq_from_bytes(&r->y.c1, b + 144) && g2_on_curve(r);
}
static void g2_to_bytes(uint8_t *b, const g2a_t *p) {
    if (p->inf) {
        memset(b, 0, 192);
        return;
    }
    fq_to_bytes(b, &p->x.c0);
    fq_to_bytes(b + 48, &p->x.c1);
    fq_to_bytes(b + 96, &p->y.c0);
    fq_to_bytes(b + 144, &p->y.c1);
}

/* f_{|z|, Q}(P) with Q untwisted into E(Fq12), conjugated for z < 0 */
static void miller_loop(fq12_t *out, const g1a_t *P, const g2a_t *Q) {
    const uint64_t z = 0xd201000000010000ULL;
    fq12_t w, wi, wi2, wi3, qx, qy, px, py, tx, ty, f;
    fq6_zero(&w.c0);
    fq6_one(&w.c1);
    fq12_inv(&wi, &w);
    fq12_mul(&wi2, &wi, &wi);
    fq12_mul(&wi3, &wi2, &wi);
    fq12_from_fq2(&qx, &Q->x);
    fq12_mul(&qx, &qx, &wi2);
    fq12_from_fq2(&qy, &Q->y);
    fq12_mul(&qy, &qy, &wi3);
    fq12_from_fq(&px, &P->x);
    fq12_from_fq(&py, &P->y);
    tx = qx;
    ty = qy;
    fq12_one(&f);
    for (int bit = 62; bit >= 0; bit--) {
        fq12_t lam, num, den, l, t, nx, ny;
        /* tangent at T */
        fq12_mul(&t, &tx, &tx);
        fq12_add(&num, &t, &t);
        fq12_add(&num, &num, &t);
        fq12_add(&den, &ty, &ty);
        fq12_inv(&den, &den);
        fq12_mul(&lam, &num, &den);
        fq12_sub(&t, &px, &tx);
        fq12_mul(&t, &lam, &t);
        fq12_sub(&l, &py, &ty);
        fq12_sub(&l, &l, &t);
        fq12_mul(&f, &f, &f);
        fq12_mul(&f, &f, &l);
        fq12_mul(&nx, &lam, &lam);
        fq12_sub(&nx, &nx, &tx);
        fq12_sub(&nx, &nx, &tx);
        fq12_sub(&t, &tx, &nx);
        fq12_mul(&ny, &lam, &t);
        fq12_sub(&ny, &ny, &ty);
        tx = nx;
        ty = ny;
        if ((z >> bit) & 1) {
            /* chord through T and Q */
            fq12_sub(&num, &qy, &ty);
            fq12_sub(&den, &qx, &tx);
            fq12_inv(&den, &den);
            fq12_mul(&lam, &num, &den);
            fq12_sub(&t, &px, &tx);
            fq12_mul(&t, &lam, &t);
            fq12_sub(&l, &py, &ty);
            fq12_sub(&l, &l, &t);
            fq12_mul(&f, &f, &l);
            fq12_mul(&nx, &lam, &lam);
            fq12_sub(&nx, &nx, &tx);
            fq12_sub(&nx, &nx, &qx);
            fq12_sub(&t, &tx, &nx);
            fq12_mul(&ny, &lam, &t);
            fq12_sub(&ny, &ny, &ty);
            tx = nx;
            ty = ny;
        }
    }
    fq12_conj(out, &f);
}

/* The fixed G2 point: the first x = (k, 1), k = 1, 2, ..., with x^3 + 4 xi a
 * square, times the cofactor (#E'(Fq2) / r, given as limbs). */
int or_g2_derive(const uint64_t *cofactor, size_t limbs, uint8_t *out192) {
    for (uint64_t k = 1; k < 1000; k++) {
        g2a_t p, q;
        fq2_t rhs, b;
        memset(&p, 0, sizeof p);
        fq_from_u64(&p.x.c0, k);
        fq_from_u64(&p.x.c1, 1);
        fq2_mul(&rhs, &p.x, &p.x);
        fq2_mul(&rhs, &rhs, &p.x);
        g2_b(&b);
        fq2_add(&rhs, &rhs, &b);
        if (!fq2_sqrt(&p.y, &rhs)) continue;
        g2_mul(&q, &p, cofactor, limbs);
        if (q.inf) continue;
        g2_to_bytes(out192, &q);
        return 0;
    }
    return 1;
}

/* op 0: a + b; 1: -a; 2: k * a (k: canonical Fr, 32 bytes LE); 3: on-curve
 * check of a (returns 0 on curve).  Nonzero return: malformed input. */
int or_g2_op(int op, const uint8_t *a, const uint8_t *b, const uint8_t *k32, uint8_t *out192) {
    g2a_t pa, pb, res;
    if (!g2_from_bytes(&pa, a)) return 1;
    switch (op) {
        case 0:
            if (!g2_from_bytes(&pb, b)) return 1;
            g2_add(&res, &pa, &pb);
            break;
        case 1:
            res = pa;
            if (!pa.inf) fq2_neg(&res.y, &pa.y);
            break;
        case 2: {
            uint64_t k[4];
            memcpy(k, k32, 32);
            g2_mul(&res, &pa, k, 4);
            break;
        }
        case 3:
            return 0;
        default:
            return 1;
    }
    g2_to_bytes(out192, &res);
    return 0;
}

/* prod_i e(P_i, Q_i) == 1 ?  1: yes, 0: no, -1: malformed point.  `fexp` is
 * (p^12 - 1) / r as little-endian limbs. */
int or_pairing_product_is_one(const uint8_t *g1s96, const uint8_t *g2s192, size_t n, const uint64_t *fexp,
                              size_t limbs) {
    fq12_t acc, one;
    fq12_one(&acc);
    for (size_t i = 0; i < n; i++) {
        g1a_t p;
        g2a_t q;
        if (!g1a_from_bytes(&p, g1s96 + 96 * i) || !g2_from_bytes(&q, g2s192 + 192 * i)) return -1;
        if (p.inf || q.inf) continue;
        fq12_t f;
        miller_loop(&f, &p, &q);
        fq12_mul(&acc, &acc, &f);
    }
    fq12_pow(&acc, &acc, fexp, limbs);
    fq12_one(&one);
    return fq12_eq(&acc, &one) ? 1 : 0;
}
