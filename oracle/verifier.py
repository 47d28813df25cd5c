"""TEST INFRASTRUCTURE ONLY -- the HyperPlonk verifier, host side.

Restates the reference's verifier so that tests can check that proofs from
either backend are accepted and that altered proofs are rejected:
- SumCheck verify:      subroutines/src/poly_iop/sum_check/mod.rs:171-218,
                        sum_check/verifier.rs (round loop, subclaim,
                        interpolate_uni_poly)
- ZeroCheck verify:     subroutines/src/poly_iop/zero_check/mod.rs:94-124
- ProductCheck verify:  subroutines/src/poly_iop/prod_check/mod.rs:217-247
- PermutationCheck:     subroutines/src/poly_iop/perm_check/mod.rs:160-178
- KZG verify:           subroutines/src/pcs/multilinear_kzg/mod.rs:169-221
- batch verify:         subroutines/src/pcs/multilinear_kzg/batching.rs:195-300
- HyperPlonk verify:    hyperplonk/src/snark.rs:343-640, utils.rs:229-290
                        (eval_f, eval_perm_gate), structs.rs:73-90
                        (eval_id_oracle), snark.rs:26-35 (gen_eval_point)

The transcript is the oracle's pure-Python Merlin (transcript_ref), the
pairing and G2 arithmetic are pairing.py's; byte encodings of transcript
messages are the ones the prover uses (hyperplonk_gb300.serialize).
Verification failures return False (a rejected proof); malformed shapes
raise VerifyError.
"""
from __future__ import annotations

import oracle  # oracle/oracle.py
import pairing
import transcript_ref

from hyperplonk_gb300 import serialize as ser

R = oracle.R


class VerifyError(Exception):
    pass


def _inv(x: int) -> int:
    return pow(x % R, R - 2, R)


def ceil_log2(k: int) -> int:
    """ark_std::log2: bits to index k items (0 for k <= 1)."""
    return 0 if k <= 1 else (k - 1).bit_length()


def eq_eval(x, y) -> int:
    """common/eq.rs:15-29: prod (x_i y_i + (1 - x_i)(1 - y_i))."""
    if len(x) != len(y):
        raise VerifyError("x and y have different length")
    res = 1
    for a, b in zip(x, y):
        res = res * ((2 * a * b - a - b + 1) % R) % R
    return res


def eq_weights(t) -> list:
    """eq(t, <i>) for i < 2^len(t), t[0] <-> bit 0 (batch_weights)."""
    out = [1]
    for ti in t:
        out = [v * (1 - ti) % R for v in out] + [v * ti % R for v in out]
    return out


def mle_evaluate(table, point) -> int:
    """Evaluation of the MLE of `table` at `point`, point[0] <-> bit 0."""
    f = [v % R for v in table]
    for r in point:
        f = [(f[2 * b] + r * (f[2 * b + 1] - f[2 * b])) % R for b in range(len(f) // 2)]
    if len(f) != 1:
        raise VerifyError("point length does not match the table")
    return f[0]


def interpolate_uni_poly(evals, x: int) -> int:
    """The degree-d polynomial through (i, evals[i]), i = 0..d, at x."""
    d = len(evals) - 1
    x %= R
    if x <= d:
        return evals[x] % R
    # Lagrange at integer nodes: l_i(x) = prod_{j != i} (x - j) / (i - j)
    total = 0
    full = 1
    for j in range(d + 1):
        full = full * (x - j) % R
    fact = [1] * (d + 1)
    for i in range(1, d + 1):
        fact[i] = fact[i - 1] * i % R
    for i in range(d + 1):
        denom = fact[i] * fact[d - i] % R
        if (d - i) & 1:
            denom = (R - denom) % R
        total += evals[i] * full * _inv((x - i) * denom)
    return total % R


# ---------------------------------------------------------------------------
# PolyIOP verifiers
# ---------------------------------------------------------------------------

def sumcheck_verify(claimed_sum: int, proof, max_degree: int, num_vars: int, transcript):
    """Returns (point, expected evaluation) or raises VerifyError."""
    if num_vars == 0 or max_degree == 0:
        raise VerifyError("SumCheck requires positive variable count and degree")
    if len(proof.point) != num_vars or len(proof.proofs) != num_vars:
        raise VerifyError("incorrect SumCheck dimensions")
    if any(len(m) != max_degree + 1 for m in proof.proofs):
        raise VerifyError("incorrect number of evaluations")
    transcript.append_serializable_element(b"aux info", ser.aux_info(max_degree, num_vars))
    challenges = []
    for msg in proof.proofs:
        transcript.append_serializable_element(b"prover msg", ser.vec_fr(msg))
        challenges.append(transcript.get_and_append_challenge(b"Internal round"))
    expected = claimed_sum % R
    for msg, c in zip(proof.proofs, challenges):
        if (msg[0] + msg[1]) % R != expected:
            raise VerifyError("prover message is not consistent with the claim")
        expected = interpolate_uni_poly(msg, c)
    return challenges, expected


def zerocheck_verify(proof, max_degree: int, num_vars: int, transcript):
    r = transcript.get_and_append_challenge_vectors(b"0check r", num_vars)
    point, ev = sumcheck_verify(0, proof, max_degree + 1, num_vars, transcript)
    return point, ev * _inv(eq_eval(point, r)) % R


def prodcheck_verify(proof, max_degree: int, num_vars: int, transcript):
    transcript.append_serializable_element(b"frac(x)", ser.g1_compressed(proof.frac_comm))
    transcript.append_serializable_element(b"prod(x)", ser.g1_compressed(proof.prod_x_comm))
    alpha = transcript.get_and_append_challenge(b"alpha")
    point, expected = zerocheck_verify(proof.zero_check_proof, max_degree, num_vars, transcript)
    final_query = ([0] + [1] * (num_vars - 1), 1)
    return point, expected, final_query, alpha


def permcheck_verify(proof, max_degree: int, num_vars: int, transcript):
    beta = transcript.get_and_append_challenge(b"beta")
    gamma = transcript.get_and_append_challenge(b"gamma")
    point, expected, final_query, alpha = prodcheck_verify(proof, max_degree, num_vars, transcript)
    return point, expected, final_query, alpha, beta, gamma


# ---------------------------------------------------------------------------
# PCS
# ---------------------------------------------------------------------------

def _g1_mul(p, k: int):
    if p is None:
        return None
    return oracle.affine_to_point(oracle.msm(oracle.point_to_affine(p), (k % R).to_bytes(32, "little")))


def _g1_neg(p):
    return None if p is None else (p[0], (-p[1]) % pairing.P)


def _g1_sub(a, b):
    if b is None:
        return a
    nb = oracle.point_to_affine(_g1_neg(b))
    if a is None:
        return oracle.affine_to_point(nb)
    return oracle.affine_to_point(oracle.g1_op(0, oracle.point_to_affine(a), nb))


def kzg_verify(vp: dict, commitment, point, value: int, proofs) -> bool:
    """e(g v - C, h) * prod_i e(pi_i, h_mask_i - z_i h) == 1."""
    num_var = len(point)
    if num_var > vp["num_vars"]:
        raise VerifyError("point length exceeds the parameter limit")
    if len(proofs) != num_var:
        raise VerifyError("proof length does not match the point")
    ignored = vp["num_vars"] - num_var
    pairs = []
    for i in range(num_var):
        hz = pairing.g2_mul(vp["h"], point[i])
        pairs.append((proofs[i], pairing.g2_add(vp["h_mask"][ignored + i], pairing.g2_neg(hz))))
    pairs.append((_g1_sub(_g1_mul(vp["g"], value), commitment), vp["h"]))
    return pairing.pairing_product_is_one(pairs)


def batch_verify(vp: dict, commitments, points, batch_proof, transcript) -> bool:
    k = len(commitments)
    evals = batch_proof.f_i_eval_at_point_i
    if k == 0 or len(points) != k or len(evals) != k:
        raise VerifyError("batch commitments, points, and evaluations must have equal nonzero lengths")
    num_var = len(points[0])
    if num_var == 0 or any(len(p) != num_var for p in points):
        raise VerifyError("batch points must have the same positive dimension")
    for pt in points:
        transcript.append_serializable_element(b"eval_point", ser.vec_fr(pt))
    for e in evals:
        transcript.append_field_element(b"eval", e)
    t = transcript.get_and_append_challenge_vectors(b"t", ceil_log2(k))
    eq_t = eq_weights(t)
    total = sum(eq_t[i] * evals[i] for i in range(k)) % R
    a2, g_eval = sumcheck_verify(total, batch_proof.sum_check_proof, 2, num_var, transcript)
    scalars = [eq_eval(a2, points[i]) * eq_t[i] % R for i in range(k)]
    bases = b"".join(oracle.point_to_affine(c) for c in commitments)
    g_prime = oracle.affine_to_point(oracle.msm(bases, b"".join(s.to_bytes(32, "little") for s in scalars)))
    return kzg_verify(vp, g_prime, a2, g_eval, batch_proof.g_prime_proof)


# ---------------------------------------------------------------------------
# HyperPlonk
# ---------------------------------------------------------------------------

def gate_degree(gate) -> int:
    return max((1 if sel is not None else 0) + len(wits) for _, sel, wits in gate)


def eval_f(gate, selector_evals, witness_evals) -> int:
    res = 0
    for coeff, sel, wits in gate:
        v = coeff % R
        if sel is not None:
            v = v * selector_evals[sel] % R
        for w in wits:
            v = v * witness_evals[w] % R
        res += v
    return res % R


def eval_perm_gate(prod_evals, frac_evals, witness_perm_evals, id_evals, perm_evals, alpha, beta, gamma,
                   x1) -> int:
    p1 = frac_evals[1] + x1 * (prod_evals[1] - frac_evals[1])
    p2 = frac_evals[2] + x1 * (prod_evals[2] - frac_evals[2])
    f_prod = 1
    for w, i in zip(witness_perm_evals, id_evals):
        f_prod = f_prod * (w + beta * i + gamma) % R
    g_prod = 1
    for w, p in zip(witness_perm_evals, perm_evals):
        g_prod = g_prod * (w + beta * p + gamma) % R
    return (prod_evals[0] - p1 * p2 + alpha * (frac_evals[0] * g_prod - f_prod)) % R


def gen_eval_point(index: int, index_len: int, point) -> list:
    return list(point) + [(index >> j) & 1 for j in range(index_len)]


def eval_id_oracle(point) -> int:
    """sum_j 2^j point[j]: the MLE of the identity labels col * 2^nv + row."""
    res, base = 0, 1
    for v in point:
        res += base * v
        base *= 2
    return res % R


def hyperplonk_verify(vk, pub_input, proof) -> bool:
    """True iff the proof verifies; malformed shapes raise VerifyError."""
    transcript = transcript_ref.OracleIOPTranscript(b"hyperplonk")
    num_sel = 1 + max(sel for _, sel, _ in vk.gate if sel is not None)
    num_wit = 1 + max(max(w) for _, _, w in vk.gate if w)
    nv = vk.num_vars
    ell = ceil_log2(vk.num_pub_input)
    if len(pub_input) != vk.num_pub_input:
        raise VerifyError("public input length is not correct")
    if len(proof.witness_commits) != num_wit:
        raise VerifyError("incorrect witness commitment count")
    evals = proof.batch_openings.f_i_eval_at_point_i
    expected_num = 3 * num_wit + num_sel + 8
    if len(evals) != expected_num:
        raise VerifyError("incorrect opening evaluation count")
    prod_evals = evals[0:4]
    frac_evals = evals[4:7]
    perm_evals = evals[7:7 + num_wit]
    witness_perm_evals = evals[7 + num_wit:7 + 2 * num_wit]
    witness_gate_evals = evals[7 + 2 * num_wit:7 + 3 * num_wit]
    selector_evals = evals[7 + 3 * num_wit:7 + 3 * num_wit + num_sel]
    pi_eval = evals[expected_num - 1]

    # 1. gate zero-check
    for c in proof.witness_commits:
        transcript.append_serializable_element(b"w", ser.g1_compressed(c))
    try:
        zc_point, zc_expected = zerocheck_verify(proof.zero_check_proof, gate_degree(vk.gate), nv, transcript)
    except VerifyError:
        return False
    if eval_f(vk.gate, selector_evals, witness_gate_evals) != zc_expected:
        return False

    # 2. permutation check
    try:
        pc_point, pc_expected, final_query, alpha, beta, gamma = permcheck_verify(
            proof.perm_check_proof, num_wit + 1, nv, transcript)
    except VerifyError:
        return False
    if prod_evals[3] % R != final_query[1]:
        return False
    id_len = ceil_log2(num_wit)
    id_evals = [eval_id_oracle(gen_eval_point(i, id_len, pc_point)) for i in range(num_wit)]
    if eval_perm_gate(prod_evals, frac_evals, witness_perm_evals, id_evals, perm_evals, alpha, beta, gamma,
                      pc_point[-1]) != pc_expected:
        return False

    # 3. openings
    p0 = [0] + pc_point[:nv - 1]
    p1 = [1] + pc_point[:nv - 1]
    comms, points = [], []
    for pt in (pc_point, p0, p1, final_query[0]):
        comms.append(proof.perm_check_proof.prod_x_comm)
        points.append(pt)
    for pt in (pc_point, p0, p1):
        comms.append(proof.perm_check_proof.frac_comm)
        points.append(pt)
    for c in vk.perm_commitments:
        comms.append(c)
        points.append(pc_point)
    for c in proof.witness_commits:
        comms.append(c)
        points.append(pc_point)
    for c in proof.witness_commits:
        comms.append(c)
        points.append(zc_point)
    for c in vk.selector_commitments:
        comms.append(c)
        points.append(zc_point)
    r_pi = transcript.get_and_append_challenge_vectors(b"r_pi", ell)
    if mle_evaluate(pub_input, r_pi) != pi_eval % R:
        return False
    comms.append(proof.witness_commits[0])
    points.append(r_pi + [0] * (nv - ell))
    try:
        return batch_verify(vk.pcs_param, comms, points, proof.batch_openings, transcript)
    except VerifyError:
        return False
