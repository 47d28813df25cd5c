/* hp_oracle.h -- TEST INFRASTRUCTURE ONLY: C declarations of the oracle
 * library (hp_oracle.c, built into oracle/_build/libhp_oracle.so), for the C++
 * parity tests.  Every function takes canonical little-endian bytes (Fr 32 B,
 * affine G1 96 B = x || y with (0, 0) = infinity); tables are 2^nv Fr.
 * Return codes: 0 ok, 1 malformed input, 2 invalid state / zero denominator
 * where noted in hp_oracle.c. */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_sumcheck or_sumcheck;

int or_set_threads(int n);
int or_msm(const uint8_t *bases96, const uint8_t *scalars32, size_t n, uint8_t *out96);
int or_mle_linear_combination(size_t nv, const uint8_t *const *polys, const uint8_t *coefs, size_t k,
                              uint8_t *out);
int or_mle_evaluate(const uint8_t *poly, size_t nv, const uint8_t *point, uint8_t *out);
int or_mle_build_eq_x_r(const uint8_t *r_bytes, size_t nv, uint8_t *out);
int or_eq_eval(const uint8_t *x, const uint8_t *y, size_t n, uint8_t *out);
int or_mle_frac(size_t nv, const uint8_t *const *nums, const uint8_t *const *dens, size_t k, uint8_t *out);
int or_mle_product_poly(const uint8_t *frac, size_t nv, uint8_t *out);
int or_mle_nums_denoms(size_t nv, const uint8_t *beta, const uint8_t *gamma, const uint8_t *const *fxs,
                       const uint8_t *const *gxs, const uint8_t *const *perms, size_t k, uint8_t *const *out_nums,
                       uint8_t *const *out_dens);
int or_mle_product_factors(const uint8_t *frac, const uint8_t *prod, size_t nv, uint8_t *p1, uint8_t *p2);
or_sumcheck *or_sumcheck_create(size_t nv, size_t max_degree, const uint8_t *const *factors, size_t factor_count,
                                const uint8_t *coefs, const size_t *offsets, size_t product_count,
                                const size_t *indices, size_t index_count);
int or_sumcheck_round(or_sumcheck *s, const uint8_t *challenge, uint8_t *out);
int or_sumcheck_final(or_sumcheck *s, const uint8_t *challenge, uint8_t *out);
void or_sumcheck_destroy(or_sumcheck *s);
int or_kzg_commit(const uint8_t *layer96, const uint8_t *evals, size_t nv, uint8_t *out96);
int or_kzg_open(const uint8_t *const *layers96, const uint8_t *poly, size_t nv, const uint8_t *point,
                uint8_t *out_q96, uint8_t *out_eval);
void or_random_fr(uint64_t seed, uint64_t first, size_t n, uint8_t *out);
int or_srs_gen(size_t nv, uint64_t seed, uint8_t *out);
int or_fixture_vanilla_plonk(uint64_t seed, uint64_t witness_seed, size_t nv, int wired, uint8_t *sel, uint8_t *wit,
                             uint8_t *perm);
void or_g1_generator(uint8_t *out96);

#ifdef __cplusplus
}
#endif
