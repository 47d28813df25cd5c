/*
 * hp_cuda.h -- C ABI of the GB300 (sm_103a) HyperPlonk prover backend.
 *
 * Drop-in counterpart of the reference's Ascend bridge
 * (backend/src/ascend910b3/native/bridge.h:43-62, bound from Rust in
 * backend/src/ascend910b3/ffi.rs:34-173).  Every `hp_cuda_v1_*` entry below
 * replaces the `hp_ascend910b3_v1_*` entry of the same suffix with the same
 * argument order, meaning and error behaviour:
 *
 *  - Host packets, not device layouts: Fr is canonical little-endian 32 bytes;
 *    G1 is 97 bytes = tag (0 finite, 1 infinity with zero coordinates) then x
 *    and y as canonical little-endian 48-byte Fq.
 *  - Host buffers are borrowed only until return.  Zero-count arrays may be
 *    null, except product_offsets which always holds product_count + 1 entries
 *    starting at 0.
 *  - On success host outputs are completely written; device outputs (MLE
 *    addresses) are unique, immutable and owned by the caller until retired.
 *  - On failure partial resources are released and every resource output slot
 *    is nulled.  No C++ exception crosses this ABI.
 *  - A context is driven by one host thread and owns one CUDA stream; all
 *    device work of the context is ordered on that stream.
 *  - buffer_retire releases the caller's ownership; storage is returned to the
 *    stream-ordered pool only after all work already queued on the context's
 *    stream that uses it, and only when no prover state or parameter object
 *    still references it.
 *  - Zero denominators (including 0/0) are InvalidParameters.
 *  - Sumcheck: the first round requires a null challenge, later rounds a
 *    non-null one; misuse or exhaustion returns InvalidState without
 *    advancing the state.  An execution failure poisons the state; later
 *    rounds return InvalidState.
 *
 * Status: kind 0 success, 1 InvalidParameters, 2 InvalidState, 3
 * NotImplemented (bridge.h:29-34); native_code carries the CUDA error code of
 * a failed runtime call, or 0.
 *
 * Device layout (not part of the ABI contract): MLE tables are Montgomery Fr
 * (R = 2^256), eight little-endian 32-bit limbs, 32 bytes per entry,
 * low-bit-first evaluation order; SRS layers are affine Montgomery Fq points,
 * 96 bytes each.
 */
#ifndef HP_CUDA_H
#define HP_CUDA_H

#include <stddef.h>
#include <stdint.h>

#define HP_CUDA_STATUS_SUCCESS 0
#define HP_CUDA_STATUS_INVALID_PARAMETERS 1
#define HP_CUDA_STATUS_INVALID_STATE 2
#define HP_CUDA_STATUS_NOT_IMPLEMENTED 3

typedef struct HpCudaStatus {
    int32_t kind;
    int32_t native_code;
} HpCudaStatus;

typedef struct HpCudaContext HpCudaContext;
typedef struct HpCudaMultilinearKzgPreparedProverParam HpCudaMultilinearKzgPreparedProverParam;
typedef struct HpCudaSumCheckProverState HpCudaSumCheckProverState;
typedef void *HpCudaDeviceAddress;

#ifdef __cplusplus
extern "C" {
#endif

/* ---- context and buffers (bridge.h:43-45) ------------------------------ */

/* Replaces hp_ascend910b3_v1_context_create (bridge.h:43). */
HpCudaStatus hp_cuda_v1_context_create(int32_t device_id, HpCudaContext **out);
/* Replaces hp_ascend910b3_v1_context_destroy (bridge.h:44): drains the stream,
 * frees every buffer the context still holds. */
HpCudaStatus hp_cuda_v1_context_destroy(HpCudaContext *ctx);
/* Replaces hp_ascend910b3_v1_buffer_retire (bridge.h:45). */
HpCudaStatus hp_cuda_v1_buffer_retire(HpCudaContext *ctx, HpCudaDeviceAddress address);

/* ---- MLE tables (bridge.h:46-53; traits backend/src/multilinear_polynomial.rs:33-121) */

/* Replaces hp_ascend910b3_v1_mle_upload (bridge.h:46): evaluation_count must be
 * 2^num_vars canonical Fr. */
HpCudaStatus hp_cuda_v1_mle_upload(HpCudaContext *ctx, size_t num_vars, const uint8_t *evaluations,
                                   size_t evaluation_count, HpCudaDeviceAddress *out);
/* `count` tables of 2^num_vars canonical Fr uploaded in one call: the same
 * result as `count` hp_cuda_v1_mle_upload calls (bridge.h:46), with each
 * table's copy and conversion on its own worker stream (copies side by side)
 * and one validation synchronisation.  A non-canonical element in any table fails the whole
 * call (InvalidParameters) and leaves every out slot null.  No counterpart in
 * the reference, whose uploads are one table per call. */
HpCudaStatus hp_cuda_v1_mle_upload_many(HpCudaContext *ctx, size_t num_vars, const uint8_t *const *evaluations,
                                        size_t count, size_t evaluation_count, HpCudaDeviceAddress *out);
/* Replaces hp_ascend910b3_v1_mle_linear_combination (bridge.h:47). */
HpCudaStatus hp_cuda_v1_mle_linear_combination(HpCudaContext *ctx, size_t num_vars,
                                               const HpCudaDeviceAddress *polynomials,
                                               const uint8_t *coefficients, size_t count,
                                               HpCudaDeviceAddress *out);
/* Replaces hp_ascend910b3_v1_mle_evaluate (bridge.h:48). */
HpCudaStatus hp_cuda_v1_mle_evaluate(HpCudaContext *ctx, HpCudaDeviceAddress polynomial,
                                     size_t num_vars, const uint8_t *point,
                                     uint8_t *out_evaluation);
/* Replaces hp_ascend910b3_v1_mle_build_eq_x_r (bridge.h:49). */
HpCudaStatus hp_cuda_v1_mle_build_eq_x_r(HpCudaContext *ctx, const uint8_t *r, size_t num_vars,
                                         HpCudaDeviceAddress *out);
/* Replaces hp_ascend910b3_v1_mle_compute_frac_poly (bridge.h:50). */
HpCudaStatus hp_cuda_v1_mle_compute_frac_poly(HpCudaContext *ctx, size_t num_vars,
                                              const HpCudaDeviceAddress *numerators,
                                              const HpCudaDeviceAddress *denominators,
                                              size_t count, HpCudaDeviceAddress *out);
/* Replaces hp_ascend910b3_v1_mle_compute_product_poly (bridge.h:51). */
HpCudaStatus hp_cuda_v1_mle_compute_product_poly(HpCudaContext *ctx, HpCudaDeviceAddress frac,
                                                 size_t num_vars, HpCudaDeviceAddress *out);
/* Replaces hp_ascend910b3_v1_mle_compute_nums_and_denoms (bridge.h:52). */
HpCudaStatus hp_cuda_v1_mle_compute_nums_and_denoms(
    HpCudaContext *ctx, size_t num_vars, const uint8_t *beta, const uint8_t *gamma,
    const HpCudaDeviceAddress *fxs, const HpCudaDeviceAddress *gxs,
    const HpCudaDeviceAddress *permutations, size_t count, HpCudaDeviceAddress *out_numerators,
    HpCudaDeviceAddress *out_denominators);
/* Replaces hp_ascend910b3_v1_mle_compute_product_factors (bridge.h:53). */
HpCudaStatus hp_cuda_v1_mle_compute_product_factors(HpCudaContext *ctx, HpCudaDeviceAddress frac,
                                                    HpCudaDeviceAddress product, size_t num_vars,
                                                    HpCudaDeviceAddress *out_p1,
                                                    HpCudaDeviceAddress *out_p2);

/* ---- multilinear KZG (bridge.h:54-59; trait backend/src/multilinear_kzg.rs:20-55) */

/* Replaces hp_ascend910b3_v1_multilinear_kzg_params_create (bridge.h:54). */
HpCudaStatus hp_cuda_v1_multilinear_kzg_params_create(
    HpCudaContext *ctx, size_t num_vars, HpCudaMultilinearKzgPreparedProverParam **out);
/* Replaces hp_ascend910b3_v1_multilinear_kzg_params_upload_layer (bridge.h:55):
 * layer_index in 0..=num_vars carries 2^(num_vars - layer_index) 97-byte points. */
HpCudaStatus hp_cuda_v1_multilinear_kzg_params_upload_layer(
    HpCudaContext *ctx, HpCudaMultilinearKzgPreparedProverParam *params, size_t layer_index,
    const uint8_t *points, size_t point_count);
/* Replaces hp_ascend910b3_v1_multilinear_kzg_params_destroy (bridge.h:56). */
HpCudaStatus hp_cuda_v1_multilinear_kzg_params_destroy(
    HpCudaContext *ctx, HpCudaMultilinearKzgPreparedProverParam *params);
/* Replaces hp_ascend910b3_v1_multilinear_kzg_commit (bridge.h:57). */
HpCudaStatus hp_cuda_v1_multilinear_kzg_commit(
    HpCudaContext *ctx, const HpCudaMultilinearKzgPreparedProverParam *params,
    HpCudaDeviceAddress polynomial, size_t num_vars, uint8_t *out_commitment);
/* Replaces hp_ascend910b3_v1_multilinear_kzg_multi_commit (bridge.h:58). */
HpCudaStatus hp_cuda_v1_multilinear_kzg_multi_commit(
    HpCudaContext *ctx, const HpCudaMultilinearKzgPreparedProverParam *params,
    const HpCudaDeviceAddress *polynomials, const size_t *num_vars, size_t count,
    uint8_t *out_commitments);
/* Replaces hp_ascend910b3_v1_multilinear_kzg_open (bridge.h:59). */
HpCudaStatus hp_cuda_v1_multilinear_kzg_open(
    HpCudaContext *ctx, const HpCudaMultilinearKzgPreparedProverParam *params,
    HpCudaDeviceAddress polynomial, size_t num_vars, const uint8_t *point,
    uint8_t *out_quotients, uint8_t *out_evaluation);

/* ---- sumcheck prover (bridge.h:60-62; trait backend/src/sum_check.rs:17-38) */

/* Replaces hp_ascend910b3_v1_sumcheck_prover_state_create (bridge.h:60).
 * Zero-check states: when some factor is a table that
 * hp_cuda_v1_mle_build_eq_x_r returned (eq(x, r); tables are immutable, and
 * the context keeps r with the buffer) and its address occurs exactly once in
 * every product, the state's large rounds evaluate the polynomial without
 * that factor at max_degree nodes and multiply by eq's linear factor in the
 * current variable (the same messages; HP_SUMCHECK_EQ=0 turns it off). */
HpCudaStatus hp_cuda_v1_sumcheck_prover_state_create(
    HpCudaContext *ctx, size_t num_vars, size_t max_degree, const HpCudaDeviceAddress *factors,
    size_t factor_count, const uint8_t *coefficients, const size_t *product_offsets,
    size_t product_count, const size_t *factor_indices, size_t index_count,
    HpCudaSumCheckProverState **out);
/* Replaces hp_ascend910b3_v1_sumcheck_prover_state_round (bridge.h:61). */
HpCudaStatus hp_cuda_v1_sumcheck_prover_state_round(HpCudaContext *ctx,
                                                    HpCudaSumCheckProverState *state,
                                                    const uint8_t *challenge_or_null,
                                                    uint8_t *out_evaluations,
                                                    size_t evaluation_count);
/* Replaces hp_ascend910b3_v1_sumcheck_prover_state_destroy (bridge.h:62). */
HpCudaStatus hp_cuda_v1_sumcheck_prover_state_destroy(HpCudaContext *ctx,
                                                      HpCudaSumCheckProverState *state);

/* ---- additions of this backend ----------------------------------------- */

/* Final folded evaluations of every distinct factor after the last round:
 * fixes the last variable with `challenge` (r_nv) and writes factor_count
 * canonical Fr in the factor order given at create.  Equal to evaluate_mle of
 * each factor at the full challenge point (the reference obtains them through
 * evaluate_mle, backend/src/cpu/multilinear_polynomial.rs:84-100).  Requires
 * all num_vars rounds to have run; does not advance the state. */
HpCudaStatus hp_cuda_v1_sumcheck_prover_state_final_evaluations(
    HpCudaContext *ctx, HpCudaSumCheckProverState *state, const uint8_t *challenge,
    uint8_t *out_evaluations, size_t factor_count);

/* Copy a resident MLE back as canonical Fr (2^num_vars * 32 bytes).  The
 * reference exposes no such call (its tests re-evaluate instead); this one
 * lets callers and tests check tables byte for byte. */
HpCudaStatus hp_cuda_v1_mle_download(HpCudaContext *ctx, HpCudaDeviceAddress polynomial,
                                     size_t num_vars, uint8_t *out_evaluations,
                                     size_t evaluation_count);

/* One variable-base MSM sum_i scalars[i] * bases[i] over G1 from host
 * buffers: `count` 97-byte base packets and `count` canonical Fr, any count
 * (0 gives the point at infinity).  Counterpart of the reference's internal
 * run_msm (backend/src/ascend910b3/native/msm.h:13-16), which its bridge does
 * not export; commit/open use the prepared-layer path instead. */
HpCudaStatus hp_cuda_v1_msm(HpCudaContext *ctx, const uint8_t *bases, const uint8_t *scalars,
                            size_t count, uint8_t *out_point);

/* Batched execution (no counterpart in the reference's bridge; its
 * multi_commit, bridge_kzg.cpp:517-579, runs MSMs one after another).
 *
 * batch_msm: MSM i = sum_j s_i[j] * B[j] where s_i is the resident MLE
 * scalars[i] (2^num_vars[i] entries) and B the first 2^num_vars[i] bases of
 * prepared layer `layer_index` (prefix semantics).  A prefix shorter than the
 * layer is prepared once (its own window width and precomputed windows) and
 * cached in the parameter object.  All MSMs of the call overlap on the device;
 * writes count 97-byte packets in input order.
 *
 * batch_sumcheck_round: one round of each of `count` distinct prover states
 * (challenge_or_null per state, same rules as sumcheck_prover_state_round),
 * overlapped on the device with one synchronisation; out_evaluations[i] gets
 * evaluation_counts[i] canonical Fr.  A misuse of any state leaves every
 * state unchanged. */
HpCudaStatus hp_cuda_v1_batch_msm(HpCudaContext *ctx, HpCudaMultilinearKzgPreparedProverParam *params,
                                  size_t layer_index, const HpCudaDeviceAddress *scalars, const size_t *num_vars,
                                  size_t count, uint8_t *out_points);
HpCudaStatus hp_cuda_v1_batch_sumcheck_round(HpCudaContext *ctx, HpCudaSumCheckProverState *const *states,
                                             const uint8_t *const *challenges_or_null,
                                             uint8_t *const *out_evaluations, const size_t *evaluation_counts,
                                             size_t count);

/* Asynchronous upload of `count` tables of 2^num_vars canonical Fr, for
 * witness ingress that overlaps the context's computation (no counterpart in
 * the reference, whose upload returns after its copy).  The copies from
 * `evaluations` (pinned host memory, so the copies run asynchronously) and
 * the conversions run on the context's ingress stream; the call returns at
 * once with the device addresses.  Every later entry of this context that
 * reads one of these tables first makes the context stream wait for its
 * upload on the device (no host synchronisation), so a proof queued now
 * reads the uploaded values; entries that take raw device pointers
 * (mle_evaluate_noalloc) do not wait.  The host buffers are borrowed until
 * upload_wait returns for the tables.  upload_wait blocks until the uploads
 * of `tables` are complete and checks their encoding: a non-canonical
 * element is InvalidParameters, and then every table of that upload call is
 * released (its addresses become invalid); results computed from such tables
 * before the wait are unspecified.  At most 256 upload calls may be pending
 * (not yet waited for, with live tables) per context; beyond that
 * upload_async is InvalidState. */
HpCudaStatus hp_cuda_v1_mle_upload_async(HpCudaContext *ctx, size_t num_vars, const uint8_t *const *evaluations,
                                         size_t count, size_t evaluation_count, HpCudaDeviceAddress *out_addresses);
HpCudaStatus hp_cuda_v1_mle_upload_wait(HpCudaContext *ctx, const HpCudaDeviceAddress *tables, size_t count);

/* Evaluations of `count` resident MLEs, polynomial k at the point of
 * num_vars[k] canonical Fr starting at points + 32 * (num_vars[0] + ... +
 * num_vars[k-1]); writes count canonical Fr.  Each value equals
 * hp_cuda_v1_mle_evaluate of the same arguments; all share one
 * synchronisation.  No counterpart in the reference (its PcsAccumulator
 * evaluates one polynomial per call, hyperplonk/src/utils.rs:58). */
HpCudaStatus hp_cuda_v1_mle_evaluate_many(HpCudaContext *ctx, size_t count, const HpCudaDeviceAddress *polynomials,
                                          const size_t *num_vars, const uint8_t *points,
                                          uint8_t *out_evaluations);
/* Evaluation of a resident MLE that allocates no device memory.  No
 * counterpart in the reference.  For callers that cannot call cudaMalloc:
 * hosts that own all device memory through their own pre-reserved arena.
 * `table` is a device pointer, on the current device, to 2^num_vars Fr in
 * this library's layout (for example an address returned by
 * hp_cuda_v1_mle_upload); a host pointer or another device's memory is
 * InvalidParameters.  `point` holds
 * num_vars canonical Fr; the canonical result goes to out_evaluation (32
 * bytes, host).  Work runs on `stream` (a cudaStream_t; null = the legacy
 * default stream) of the current device, which the call synchronises.
 * Intermediate values live in one fixed device array of ~513 KiB that every
 * GPU loading this library holds until exit; num_vars above 24 returns
 * InvalidParameters.  All calls on a device share that array: calls that
 * overlap on the GPU race, so order them (one stream).  The first call on a
 * device looks up the array's address; make it before any stream capture. */
HpCudaStatus hp_cuda_v1_mle_evaluate_noalloc(const void *table, size_t num_vars, const uint8_t *point,
                                             uint8_t *out_evaluation, void *stream);

/* Synthetic workloads (no counterpart in the reference's bridge; the
 * reference builds its fixtures with arkworks' StdRng in Rust:
 * hyperplonk/examples/full_prove_bench.rs, subroutines/examples/sumcheck_bench.rs).
 *
 * fixture_random_fr: `count` canonical Fr of stream `seed`, elements
 * [first, first + count); element i = Fr::from_le_bytes_mod_order of ChaCha20
 * (RFC 8439) keystream block i, key words 0-1 = seed, counter = low 32 bits
 * of i, first nonce word = high 32 bits.  Host-only: needs no context.
 *
 * srs_generate: the testing SRS of subroutines/src/pcs/multilinear_kzg/
 * srs.rs:158-235 with this stream in place of StdRng: t_i = element i
 * (i < num_vars), s = element num_vars, g = s * G1; layer i < num_vars is
 * g * eq(t[i..], x) (t_i <-> bit 0), layer num_vars is [g].  Writes all
 * layers back to back as 97-byte packets, point_count = 2^(num_vars+1) - 1.
 * Computed on the device (fixed-base comb). */
HpCudaStatus hp_cuda_v1_fixture_random_fr(uint64_t seed, uint64_t first, size_t count, uint8_t *out);
/* Vanilla-plonk circuit of 2^num_vars gates for the full-prove workload:
 * q_L, q_R, q_M, q_C, w1, w2 are elements [k*N, (k+1)*N), k = 0..5, of stream
 * `seed`; q_O = -1; w3 = q_L w1 + q_R w2 + q_M w1 w2 + q_C, so the repo's gate
 * q_L w1 + q_R w2 + q_O w3 + q_M w1 w2 + q_C = 0 (hyperplonk/src/custom_gate.rs:86-96)
 * holds on every row.  Writes selectors [q_L, q_R, q_O, q_M, q_C] (5 tables),
 * witnesses [w1, w2, w3] (3 tables) and the identity permutation
 * (column * 2^num_vars + row, hyperplonk/src/snark.rs:69-76) as canonical Fr
 * tables back to back.  Host-only. */
HpCudaStatus hp_cuda_v1_fixture_vanilla_plonk(uint64_t seed, size_t num_vars, uint8_t *selectors,
                                              uint8_t *witnesses, uint8_t *permutation);
/* The same circuit with copy constraints that are not the identity (the
 * reference's non-identity-permutation end-to-end test,
 * hyperplonk/src/snark.rs:1008, on this fixture): w2[i] = w1[wire(i)] with
 * wire(i) = (0x9E3779B97F4A7C15 * i + seed * 0xD1B54A32D192ED03 + 1) mod N (a
 * bijection: the multiplier is odd), w3 solving the gate, and the
 * permutation swapping w2 cell i (label N + i) with w1 cell wire(i) (label
 * wire(i)); w3 cells keep their labels.  Selectors as above.  num_vars >= 1.
 * Host-only. */
HpCudaStatus hp_cuda_v1_fixture_vanilla_plonk_wired(uint64_t seed, size_t num_vars, uint8_t *selectors,
                                                    uint8_t *witnesses, uint8_t *permutation);
/* Another satisfying witness of the same circuit (serving workload: one
 * circuit per num_vars, independent witnesses per request): selectors from
 * stream `circuit_seed` as above, w1 and w2 from elements [4N, 5N) and
 * [5N, 6N) of stream `witness_seed`, w3 solving the gate.  Writes the 3
 * witness tables; equals the witnesses above when the seeds are equal.
 * No counterpart in the reference.  Host-only. */
HpCudaStatus hp_cuda_v1_fixture_vanilla_plonk_witness(uint64_t circuit_seed, uint64_t witness_seed,
                                                      size_t num_vars, uint8_t *witnesses);
/* Host Fiat-Shamir transcript used by the protocol drivers (Merlin 1.0 over
 * STROBE-128 / Keccak-f[1600]; the reference wraps merlin 3.0.0,
 * transcript/src/lib.rs:40-131).  Host-only, no device work. */
typedef struct HpMerlinTranscript HpMerlinTranscript;
HpCudaStatus hp_host_v1_merlin_new(const uint8_t *label, size_t label_len, HpMerlinTranscript **out);
HpCudaStatus hp_host_v1_merlin_append(HpMerlinTranscript *t, const uint8_t *label, size_t label_len,
                                      const uint8_t *msg, size_t msg_len);
HpCudaStatus hp_host_v1_merlin_challenge(HpMerlinTranscript *t, const uint8_t *label, size_t label_len,
                                         uint8_t *out, size_t out_len);
HpCudaStatus hp_host_v1_merlin_clone(const HpMerlinTranscript *t, HpMerlinTranscript **out);
HpCudaStatus hp_host_v1_merlin_free(HpMerlinTranscript *t);
HpCudaStatus hp_host_v1_keccak_f1600(uint8_t *state200);
/* All `rounds` (= num_vars) rounds of a fresh sumcheck state, with the
 * Fiat-Shamir step of subroutines/src/poly_iop/sum_check/mod.rs:147-155 done
 * here instead of by the caller: round k's message (max_degree+1 canonical
 * Fr) is appended to `transcript` under "prover msg" as a serialized
 * Vec<Fr> (u64 LE length, 32-byte LE elements), the challenge is 64 bytes
 * under "Internal round" reduced mod r and appended back under the same
 * label, and it folds the next round.  Writes the messages
 * (rounds * (max_degree+1) * 32 bytes) and the challenges (rounds * 32).
 * Afterwards the state is where the last per-round call would leave it
 * (final_evaluations takes the last challenge).  InvalidState unless the
 * state is at round 0; an execution failure poisons the state.  The middle
 * and last rounds (from the first of <= 2^15 or 2^17 pairs, by shape) run in
 * one resident cooperative launch that exchanges messages and challenges
 * with this call through the context's mapped mailbox; the host side of that
 * exchange runs on a thread the context creates on first use (joined by
 * hp_cuda_v1_context_destroy).  While a kernel profiler is attached every
 * round is a launch of its own.  No counterpart in the reference (its caller drives the
 * rounds one at a time through the transcript). */
HpCudaStatus hp_cuda_v1_sumcheck_prove_rounds(HpCudaContext *ctx, HpCudaSumCheckProverState *state,
                                              HpMerlinTranscript *transcript, size_t rounds,
                                              uint8_t *out_messages, uint8_t *out_challenges);
HpCudaStatus hp_cuda_v1_srs_generate(HpCudaContext *ctx, size_t num_vars, uint64_t seed,
                                     uint8_t *out_packets, size_t point_count);

/* Kernel timing (off by default; no counterpart in the reference, which
 * profiles offline with msprof).  While enabled, named device phases are
 * bracketed by CUDA events on the context stream; profile_read returns the
 * accumulated milliseconds and launch count of one name ("msm",
 * "msm_accumulate", "sumcheck_round", ...).  Enabling or disabling resets the
 * totals. */
HpCudaStatus hp_cuda_v1_context_profile(HpCudaContext *ctx, int32_t enable);
HpCudaStatus hp_cuda_v1_context_profile_read(HpCudaContext *ctx, const char *kernel, double *total_ms,
                                             uint64_t *launches);
/* Number of kernels this library has launched in the process so far. */
HpCudaStatus hp_cuda_v1_kernel_launch_count(uint64_t *out);
/* Device memory of the context's stream-ordered pool (no counterpart in the
 * reference; a serving host uses it to budget HBM per request from measured
 * use): out3 = bytes in use now, the high-water mark of bytes in use since
 * the last reset, bytes the pool holds from the device.  reset_high != 0
 * resets the high-water mark to the current use after reading. */
HpCudaStatus hp_cuda_v1_context_memory(HpCudaContext *ctx, int32_t reset_high, uint64_t *out3);

/* The context's CUDA stream (a cudaStream_t), so a caller can order its own
 * work or timing events with the backend's. */
HpCudaStatus hp_cuda_v1_context_stream(HpCudaContext *ctx, void **out_stream);

/* MSM autotuner (no counterpart in the reference, whose MSM geometry is fixed
 * in backend/src/ascend910b3/native/msm*.cpp).  The MSM's window width,
 * reduction segment length and accumulation chunk length come from a
 * process-wide tuning table, else from a size rule; the table holds measured
 * entries keyed by ceil(log2 points) for an MSM run alone (mode 0) and by
 * ceil(log2 records) for a launch shared by many MSMs (mode 1).  Tuning never
 * changes a result: every candidate's point is checked against the size
 * rule's (InvalidState on a mismatch, table unchanged).
 *
 * msm_autotune: mode 0 measures an MSM of 2^num_vars[i] points (the first
 * bases of params' layer 0) for each i, records the fastest geometry, then
 * re-prepares params' layers accordingly (window tables rebuilt where the
 * width changed) and drops its cached prefix layers; out gets count entries.
 * Mode 1 measures one shared launch over all count sizes (<= 64, prefix
 * layers of layer 0 as batch_msm builds them) and records its chunk length;
 * out gets one entry.  InvalidState when layer 0 is not uploaded or a
 * geometry override (HP_MSM_WINDOW_BITS, HP_MSM_SEG, HP_ACC_CHUNK) is set in
 * the environment.  Takes seconds per size (median device time of several
 * runs per candidate).
 *
 * msm_tuning_query: the geometry a new layer of `size` points (mode 0:
 * out3 = window bits, segment, chunk) or a shared launch of `size` records
 * (mode 1: out3 = 0, 0, chunk) would use now; needs no device.
 * msm_tuning_save / msm_tuning_load: the table as a text file; load merges
 * its entries and, when `device` is non-null, rejects a file measured on
 * another device name (InvalidParameters).  At the first lookup the table
 * takes the library's built-in entries measured on an NVIDIA GB300 (when the
 * current device has that name), then the file named by the environment
 * variable HP_CUDA_MSM_TUNING over them; HP_CUDA_MSM_TUNING=off keeps it
 * empty.  msm_tuning_clear: empties the table (the size rules apply again). */
typedef struct HpCudaMsmTuning {
    uint64_t size;        /* points (mode 0) or records of the launch (mode 1) */
    uint32_t mode;        /* 0 alone, 1 shared launch */
    uint32_t window_bits; /* mode 0 */
    uint32_t segment;     /* mode 0 */
    uint32_t chunk;
    double model_ms;      /* median device time with the size rule's geometry */
    double tuned_ms;      /* median device time with the chosen geometry */
} HpCudaMsmTuning;
HpCudaStatus hp_cuda_v1_msm_autotune(HpCudaContext *ctx, HpCudaMultilinearKzgPreparedProverParam *params,
                                     const size_t *num_vars, size_t count, int32_t mode, HpCudaMsmTuning *out);
HpCudaStatus hp_cuda_v1_msm_tuning_query(int32_t mode, size_t size, uint32_t *out3);
HpCudaStatus hp_cuda_v1_msm_tuning_save(const char *path);
HpCudaStatus hp_cuda_v1_msm_tuning_load(const char *path, const char *device);
HpCudaStatus hp_cuda_v1_msm_tuning_clear(void);

/* Sumcheck round autotuner (no counterpart in the reference, which fixes its
 * kernel geometry by plan).  A round can run on several kernel families --
 * one block (<= 64 pairs), one pair per thread, (slot, pair) items with a
 * separate or a fused fold, (product, pair) items with a separate or a fused
 * fold -- each with its own grid (blocks per SM).  sumcheck_autotune runs
 * every round of `state` (a fresh prover state, which it consumes: destroy
 * it afterwards) once per candidate, times each as the median of a few runs,
 * checks that every candidate's round message equals the built-in rule's
 * (InvalidState otherwise, the state poisoned), stores the fastest route for
 * the round's key -- ceil(log2 pairs), largest product arity, slot count,
 * whether the round folds the previous challenge (every round but the first) --
 * in the process-wide tuning table (saved and loaded with the MSM entries by
 * msm_tuning_save / _load; msm_tuning_clear empties it), and writes one
 * record per round (capacity >= num_vars).  Later rounds of any state with
 * the same key take the stored route.  sumcheck_route_query: the route
 * (out2 = kernel, blocks per SM) a round of `pairs` pairs of that shape
 * (fold != 0: a round after the first) would take now (kernel codes: 1 one block, 2 one pair per thread, 3
 * (slot, pair), 4 (slot, pair) with fused fold, 5 (product, pair), 6
 * (product, pair) with fused fold, 7 shared-memory tiles staged by bulk
 * copies, 8 (node, pair) items of the polynomial without its eq factor:
 * zero-check states only, recognised per state, so never the answer here). */
typedef struct HpCudaRoundTuning {
    uint64_t pairs;
    uint32_t kernel, blocks_per_sm;
    uint32_t default_kernel, default_blocks_per_sm;
    double default_us; /* median device time of the built-in rule's route */
    double tuned_us;   /* median device time of the chosen route */
} HpCudaRoundTuning;
HpCudaStatus hp_cuda_v1_sumcheck_autotune(HpCudaContext *ctx, HpCudaSumCheckProverState *state,
                                          HpCudaRoundTuning *out, size_t capacity, size_t *out_count);
HpCudaStatus hp_cuda_v1_sumcheck_route_query(size_t pairs, int32_t max_arity, int32_t slots, int32_t fold,
                                             uint32_t *out2);

/* Runtime audit and failure injection (test support; no counterpart in the
 * reference's bridge -- its native tests wrap the runtime's copy, sync and
 * allocation calls at link time, backend/src/ascend910b3/native/
 * CMakeLists.txt:106-116 with tests/runtime_audit.h, and the library does
 * the same to itself).
 *
 * debug_runtime_counters: process-wide counts of the CUDA runtime calls the
 * library has made since load, by kind; copies are split by direction with
 * their bytes.  Read them before and after a call and compare.  Needs no
 * device.
 *
 * debug_inject_failure: what = HP_CUDA_INJECT_POOL_ALLOCATION makes the
 * nth stream-ordered pool allocation from now fail with
 * cudaErrorMemoryAllocation (nothing is allocated); HP_CUDA_INJECT_SYNCHRONIZE
 * makes the nth stream / event synchronisation from now complete and then
 * report cudaErrorLaunchFailure, which the caller sees as an execution
 * failure (InvalidState) while the device and the context stay usable;
 * HP_CUDA_INJECT_NONE disarms both.  nth = 0 disarms that kind.  The
 * environment variable HP_CUDA_FAIL_ALLOC_AT=n arms the allocation failure
 * when the library loads.  Process wide; for tests only. */
typedef struct HpCudaRuntimeCounters {
    uint64_t device_allocs;    /* cudaMalloc */
    uint64_t host_allocs;      /* cudaHostAlloc, cudaMallocHost */
    uint64_t pool_allocs;      /* cudaMallocFromPoolAsync, cudaMallocAsync */
    uint64_t pool_alloc_bytes;
    uint64_t frees;            /* cudaFree, cudaFreeHost, cudaFreeAsync */
    uint64_t h2d_copies, h2d_bytes;
    uint64_t d2h_copies, d2h_bytes;
    uint64_t d2d_copies, d2d_bytes;
    uint64_t other_copies, other_bytes;
    uint64_t memsets;
    uint64_t syncs;            /* stream, event and device synchronisations */
    uint64_t injected_failures;
} HpCudaRuntimeCounters;
#define HP_CUDA_INJECT_NONE 0
#define HP_CUDA_INJECT_POOL_ALLOCATION 1
#define HP_CUDA_INJECT_SYNCHRONIZE 2
HpCudaStatus hp_cuda_v1_debug_runtime_counters(HpCudaRuntimeCounters *out);
HpCudaStatus hp_cuda_v1_debug_inject_failure(int32_t what, uint64_t nth);

#ifdef __cplusplus
}
#endif

#endif /* HP_CUDA_H */
