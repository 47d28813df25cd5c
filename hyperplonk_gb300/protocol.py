"""Host protocol drivers above the backend traits: the PolyIOP provers and the
multilinear-KZG batch opening.

Restates the reference's prover-side logic, which calls only backend trait
methods and the transcript, so it runs unchanged over the GB300 backend
(`CudaBackend`) or any object with the same methods (the oracle's
`CpuBackend`):

- SumCheck prove:     subroutines/src/poly_iop/sum_check/mod.rs:130-169
- ZeroCheck prove:    subroutines/src/poly_iop/zero_check/mod.rs:70-92
- ProductCheck prove: subroutines/src/poly_iop/prod_check/mod.rs:150-212 and util.rs:24-65
- PermutationCheck:   subroutines/src/poly_iop/perm_check/mod.rs:105-158
- batch opening:      subroutines/src/pcs/multilinear_kzg/batching.rs:49-194

Values: Fr as ints, G1 as (x, y) / None, MLEs as backend handles.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

from . import serialize as ser
from .errors import InvalidParameters
from .virtual_polynomial import R_MODULUS, VirtualPolynomial

R = R_MODULUS


class PolyIOPError(Exception):
    """subroutines/src/poly_iop/errors.rs."""


@dataclass
class IOPProof:
    """poly_iop/structs.rs:16-27: the challenge point and the round messages."""
    point: list
    proofs: list  # list of lists of Fr (IOPProverMessage.evaluations)

    def to_bytes(self) -> bytes:
        return ser.vec_fr(self.point) + ser.usize(len(self.proofs)) + b"".join(ser.vec_fr(m) for m in self.proofs)


@dataclass
class ProductCheckProof:
    zero_check_proof: IOPProof
    prod_x_comm: object
    frac_comm: object

    def to_bytes(self) -> bytes:
        return (self.zero_check_proof.to_bytes() + ser.g1_compressed(self.prod_x_comm)
                + ser.g1_compressed(self.frac_comm))


@dataclass
class BatchProof:
    """batching.rs:21-29."""
    sum_check_proof: IOPProof
    f_i_eval_at_point_i: list
    g_prime_proof: list  # MultilinearKzgProof.proofs (G1 list)

    def to_bytes(self) -> bytes:
        return (self.sum_check_proof.to_bytes() + ser.vec_fr(self.f_i_eval_at_point_i)
                + ser.vec_g1(self.g_prime_proof))


# ---------------------------------------------------------------------------
# PolyIOP
# ---------------------------------------------------------------------------

def sumcheck_prove(backend, poly: VirtualPolynomial, transcript, final_evaluations: list | None = None) -> IOPProof:
    nv, d = poly.aux_info.num_variables, poly.aux_info.max_degree
    if nv == 0 or d == 0:
        raise PolyIOPError("SumCheck requires positive variable count and degree.")
    transcript.append_serializable_element(b"aux info", ser.aux_info(d, nv))
    state = backend.prover_init(poly)
    native = getattr(transcript, "native_merlin", lambda: None)()
    if native is not None and hasattr(backend, "prove_rounds"):
        # every round and its Fiat-Shamir step inside the library, one call
        msgs, point = backend.prove_rounds(state, native, nv)
        if final_evaluations is not None:
            final_evaluations.extend(backend.final_evaluations(state, point[-1]))
        return IOPProof(point, msgs)
    challenge = None
    msgs, point = [], []
    for _ in range(nv):
        msg = backend.prove_round_and_update_state(state, challenge)
        transcript.append_serializable_element(b"prover msg", ser.vec_fr(msg))
        msgs.append(msg)
        challenge = transcript.get_and_append_challenge(b"Internal round")
        point.append(challenge)
    if final_evaluations is not None:
        final_evaluations.extend(backend.final_evaluations(state, challenge))
    return IOPProof(point, msgs)


def batch_sumcheck_prove(backend, polys: list, transcripts: list, final_evaluations: list | None = None) -> list:
    """Independent sumcheck proofs of `polys` (uneven num_vars allowed), each
    under its own transcript, advanced in lockstep: round k of every instance
    still running goes to the device in one batch_prove_round call.  Each
    proof equals sumcheck_prove(backend, polys[i], transcripts[i]); with
    `final_evaluations` a list, one list of final factor values per instance
    is appended to it."""
    if len(polys) != len(transcripts):
        raise InvalidParameters("one transcript per polynomial")
    for p in polys:
        if p.aux_info.num_variables == 0 or p.aux_info.max_degree == 0:
            raise PolyIOPError("SumCheck requires positive variable count and degree.")
    for p, t in zip(polys, transcripts):
        t.append_serializable_element(b"aux info", ser.aux_info(p.aux_info.max_degree, p.aux_info.num_variables))
    states = [backend.prover_init(p) for p in polys]
    nvs = [p.aux_info.num_variables for p in polys]
    challenges = [None] * len(polys)
    msgs = [[] for _ in polys]
    points = [[] for _ in polys]
    batched = hasattr(backend, "batch_prove_round")
    for rnd in range(max(nvs, default=0)):
        live = [i for i, nv in enumerate(nvs) if rnd < nv]
        if batched:
            out = backend.batch_prove_round([states[i] for i in live], [challenges[i] for i in live])
        else:
            out = [backend.prove_round_and_update_state(states[i], challenges[i]) for i in live]
        for i, msg in zip(live, out):
            transcripts[i].append_serializable_element(b"prover msg", ser.vec_fr(msg))
            msgs[i].append(msg)
            challenges[i] = transcripts[i].get_and_append_challenge(b"Internal round")
            points[i].append(challenges[i])
    if final_evaluations is not None:
        for s, c in zip(states, challenges):
            final_evaluations.append(backend.final_evaluations(s, c))
    return [IOPProof(pt, m) for pt, m in zip(points, msgs)]


def zerocheck_prove(backend, poly: VirtualPolynomial, transcript) -> IOPProof:
    r = transcript.get_and_append_challenge_vectors(b"0check r", poly.aux_info.num_variables)
    eq = backend.build_eq_x_r(r)
    f_hat = poly.clone()
    f_hat.mul_by_mle(eq, 1)
    return sumcheck_prove(backend, f_hat, transcript)


def prodcheck_prove(backend, pcs_param, fxs, gxs, transcript):
    if not fxs:
        raise PolyIOPError("fxs is empty")
    if len(fxs) != len(gxs):
        raise PolyIOPError("fxs and gxs have different number of polynomials")
    nv = fxs[0].num_vars
    if any(p.num_vars != nv for p in list(fxs) + list(gxs)):
        raise PolyIOPError("fx and gx have different number of variables")
    frac = backend.compute_frac_poly(fxs, gxs)
    prod = backend.compute_product_poly(frac)
    # prod_check/mod.rs commits frac then prod; one multi_commit gives the
    # same two commitments and lets the two MSMs overlap
    frac_comm, prod_comm = backend.multi_commit(pcs_param, [frac, prod])
    transcript.append_serializable_element(b"frac(x)", ser.g1_compressed(frac_comm))
    transcript.append_serializable_element(b"prod(x)", ser.g1_compressed(prod_comm))
    alpha = transcript.get_and_append_challenge(b"alpha")
    p1, p2 = backend.compute_product_factors(frac, prod)
    # Q(x) = prod(x) - p1 p2 + alpha * frac * g1..gk - alpha * f1..fk (util.rs:24-65)
    q = VirtualPolynomial.new_from_mle(prod, 1)
    q.add_mle_list([p1, p2], R - 1)
    q.add_mle_list(list(gxs) + [frac], alpha)
    q.add_mle_list(list(fxs), (R - alpha) % R)
    zc = zerocheck_prove(backend, q, transcript)
    return ProductCheckProof(zc, prod_comm, frac_comm), prod, frac


def permcheck_prove(backend, pcs_param, fxs, gxs, perms, transcript):
    if not fxs:
        raise PolyIOPError("fxs is empty")
    if len(fxs) != len(gxs) or len(fxs) != len(perms):
        raise PolyIOPError("fxs, gxs and perms lengths differ")
    nv = fxs[0].num_vars
    if any(p.num_vars != nv for p in list(fxs) + list(gxs) + list(perms)):
        raise PolyIOPError("number of variables unmatched")
    beta = transcript.get_and_append_challenge(b"beta")
    gamma = transcript.get_and_append_challenge(b"gamma")
    nums, dens = backend.compute_nums_and_denoms(beta, gamma, fxs, gxs, perms)
    return prodcheck_prove(backend, pcs_param, nums, dens, transcript)


# ---------------------------------------------------------------------------
# PCS batch opening
# ---------------------------------------------------------------------------

class PhaseClock:
    """Adds the host wall time since the previous mark to phases[name]
    (seconds); a no-op when `phases` is None."""

    def __init__(self, phases: dict | None):
        self.phases = phases
        self.t = time.perf_counter()

    def __call__(self, name: str) -> None:
        if self.phases is None:
            return
        now = time.perf_counter()
        self.phases[name] = self.phases.get(name, 0.0) + now - self.t
        self.t = now

    def restart(self) -> None:
        self.t = time.perf_counter()


def ceil_log2(k: int) -> int:
    """ark_std::log2: number of bits to index k items (0 for k <= 1)."""
    return 0 if k <= 1 else (k - 1).bit_length()


def eq_eval(x, y) -> int:
    """common/eq.rs:15-29."""
    if len(x) != len(y):
        raise InvalidParameters("x and y have different length")
    res = 1
    for xi, yi in zip(x, y):
        xy = xi * yi % R
        res = res * ((xy + xy - xi - yi + 1) % R) % R
    return res


def eq_table(point) -> list:
    """build_eq_x_r_vec on the host (batch weights; point[0] <-> bit 0)."""
    if not point:
        return [1]
    n = len(point)
    out = [1] * (1 << n)
    for x in range(1 << n):
        v = 1
        for i in range(n):
            v = v * (point[i] if (x >> i) & 1 else (1 - point[i])) % R
        out[x] = v
    return out


def multi_open(backend, pcs_param, polynomials, points, evals, transcript, phases: dict | None = None) -> BatchProof:
    mark = PhaseClock(phases)
    k = len(polynomials)
    if k == 0 or len(points) != k or len(evals) != k:
        raise InvalidParameters("batch polynomials, points, and evaluations must have equal nonzero lengths")
    nv = polynomials[0].num_vars
    if nv == 0 or any(p.num_vars != nv for p in polynomials) or any(len(pt) != nv for pt in points):
        raise InvalidParameters("batch polynomials and points must have the same positive dimension")
    for pt in points:
        transcript.append_serializable_element(b"eval_point", ser.vec_fr(pt))
    for e in evals:
        transcript.append_field_element(b"eval", e)
    ell = ceil_log2(k)
    t = transcript.get_and_append_challenge_vectors(b"t", ell)
    eq_t = eq_table(t)
    # group by distinct point, first-occurrence order (batching.rs:98-116)
    order: dict = {}
    for pt in points:
        order.setdefault(tuple(pt), len(order))
    deduped = [list(p) for p, _ in sorted(order.items(), key=lambda kv: kv[1])]
    groups = [[] for _ in deduped]
    for i, pt in enumerate(points):
        groups[order[tuple(pt)]].append(i)
    merged = [backend.linear_combination([polynomials[i] for i in g], [eq_t[i] for i in g]) for g in groups]
    tilde_eqs = [backend.build_eq_x_r(pt) for pt in deduped]
    vp = VirtualPolynomial(nv)
    for g, e in zip(merged, tilde_eqs):
        vp.add_mle_list([g, e], 1)
    mark("batch_open.merge")
    proof = sumcheck_prove(backend, vp, transcript)
    mark("batch_open.sumcheck")
    a2 = proof.point
    coefs = [eq_eval(a2, pt) for pt in deduped]
    g_prime = backend.linear_combination(merged, coefs)
    g_prime_proof, _ = backend.open(pcs_param, g_prime, a2)
    mark("batch_open.pcs_open")
    return BatchProof(proof, list(evals), g_prime_proof)
