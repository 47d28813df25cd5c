"""HyperPlonk prover driver (hyperplonk/src/snark.rs:56-341, utils.rs:16-227)
over any backend with the reference's trait methods, and the vanilla-plonk
fixture of the full-prove workload.

The gate is the repo's vanilla gate (custom_gate.rs:86-96):
    q_L w1 + q_R w2 + q_O w3 + q_M w1 w2 + q_C = 0
with selectors ordered [q_L, q_R, q_O, q_M, q_C] and witnesses [w1, w2, w3].
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import serialize as ser
from .errors import InvalidParameters
from .protocol import (BatchProof, IOPProof, PhaseClock, ProductCheckProof, ceil_log2, multi_open, permcheck_prove,
                       zerocheck_prove)
from .transcript import IOPTranscript
from .virtual_polynomial import R_MODULUS, VirtualPolynomial

R = R_MODULUS

# (coefficient, selector index or None, witness indices) -- custom_gate.rs:86-96
VANILLA_GATE = [(1, 0, [0]), (1, 1, [1]), (1, 2, [2]), (1, 3, [0, 1]), (1, 4, [])]


@dataclass
class ProvingKey:
    """structs.rs:126-146."""
    num_vars: int
    num_pub_input: int
    gate: list
    pcs_param: object
    selector_oracles: list
    permutation_oracles: list
    selector_commitments: list = field(default_factory=list)
    permutation_commitments: list = field(default_factory=list)

    def verifying_key(self, pcs_verifier_param) -> "VerifyingKey":
        """The matching verifying key; `pcs_verifier_param` is the SRS's
        verifier half (g, h, h_mask), which the prover never needs."""
        return VerifyingKey(self.num_vars, self.num_pub_input, self.gate, pcs_verifier_param,
                            list(self.selector_commitments), list(self.permutation_commitments))


@dataclass
class VerifyingKey:
    """structs.rs:150-159: instance parameters, the PCS verifier parameter and
    the preprocessed commitments."""
    num_vars: int
    num_pub_input: int
    gate: list
    pcs_param: object
    selector_commitments: list
    perm_commitments: list


@dataclass
class HyperPlonkProof:
    """hyperplonk/src/structs.rs:21-38."""
    witness_commits: list
    batch_openings: BatchProof
    zero_check_proof: IOPProof
    perm_check_proof: ProductCheckProof

    def to_bytes(self) -> bytes:
        return (ser.vec_g1(self.witness_commits) + self.batch_openings.to_bytes()
                + self.zero_check_proof.to_bytes() + self.perm_check_proof.to_bytes())


def preprocess(backend, num_vars: int, num_pub_input: int, selectors: list, permutation: list,
               srs_layers: list, gate=VANILLA_GATE, commit: bool = True) -> ProvingKey:
    """snark.rs:56-105: prepare the trimmed SRS, upload the permutation and
    selector oracles and commit to them (permutations first, then selectors,
    one multi_commit each, as the reference does).  `srs_layers` are the
    num_vars + 1 layers of the trimmed prover parameters; selectors /
    permutation are table packets.  commit=False skips the commitments (a
    prover that never hands out a verifying key)."""
    pcs = backend.prepare_prover_param(num_vars, srs_layers)
    perms = [backend.mle_from_evaluations(num_vars, p) for p in permutation]
    sels = [backend.mle_from_evaluations(num_vars, s) for s in selectors]
    pk = ProvingKey(num_vars, num_pub_input, gate, pcs, sels, perms)
    if commit:
        pk.permutation_commitments = list(backend.multi_commit(pcs, perms))
        pk.selector_commitments = list(backend.multi_commit(pcs, sels))
    return pk


def build_f(gate, num_vars: int, selector_mles, witness_mles) -> VirtualPolynomial:
    """utils.rs:179-227."""
    res = VirtualPolynomial(num_vars)
    for coeff, sel, wits in gate:
        mles = ([selector_mles[sel]] if sel is not None else []) + [witness_mles[w] for w in wits]
        res.add_mle_list(mles, coeff % R)
    return res


class PcsAccumulator:
    """utils.rs:16-86: polynomials with their opening points and evaluations."""

    def __init__(self, num_var: int):
        self.num_var = num_var
        self.polynomials, self.points, self.evals = [], [], []

    def insert_poly_and_points(self, backend, poly, point) -> None:
        """The evaluation is due by multi_open (its only reader); backends with
        evaluate_many compute all of them there in one call."""
        assert poly.num_vars == self.num_var
        if not hasattr(backend, "evaluate_many"):
            self.evals.append(backend.evaluate_mle(poly, point))
        self.polynomials.append(poly)
        self.points.append(list(point))

    def evaluations(self, backend) -> list:
        if len(self.evals) < len(self.polynomials):
            self.evals = backend.evaluate_many(self.polynomials, self.points)
        return self.evals

    def multi_open(self, backend, pcs_param, transcript, phases: dict | None = None) -> BatchProof:
        evals = self.evaluations(backend)
        return multi_open(backend, pcs_param, self.polynomials, self.points, evals, transcript, phases)


def prove(backend, pk: ProvingKey, pub_input: list, witnesses: list, transcript_cls=IOPTranscript,
          witness_mles: list | None = None, phases: dict | None = None) -> HyperPlonkProof:
    """snark.rs:156-341.  `witnesses` are table packets (or already-resident
    MLEs passed as `witness_mles`); `pub_input` the public values.  When
    `phases` is a dict, the host wall time of each prover phase (seconds) is
    added to it; every phase ends on a host read of a device result, so the
    phases partition the proof."""
    mark = PhaseClock(phases)
    transcript = transcript_cls(b"hyperplonk")
    nv = pk.num_vars
    ell = ceil_log2(pk.num_pub_input)
    acc = PcsAccumulator(nv)
    # 1. witnesses
    if witness_mles is None:
        if hasattr(backend, "mle_from_evaluations_many"):  # one upload call, one validation sync
            witness_mles = backend.mle_from_evaluations_many(nv, witnesses)
        else:
            witness_mles = [backend.mle_from_evaluations(nv, w) for w in witnesses]
    commits = backend.multi_commit(pk.pcs_param, witness_mles)
    mark("witness_commit")
    for c in commits:
        transcript.append_serializable_element(b"w", ser.g1_compressed(c))
    # 2. gate zero-check
    fx = build_f(pk.gate, nv, pk.selector_oracles, witness_mles)
    zc = zerocheck_prove(backend, fx, transcript)
    mark("gate_zerocheck")
    # 3. permutation check
    pc, prod_x, frac = permcheck_prove(backend, pk.pcs_param, witness_mles, witness_mles,
                                       pk.permutation_oracles, transcript)
    mark("perm_check")
    pcp = pc.zero_check_proof.point
    p0 = [0] + pcp[:nv - 1]
    p1 = [1] + pcp[:nv - 1]
    final_q = [0] + [1] * (nv - 1)
    for pt in (pcp, p0, p1, final_q):
        acc.insert_poly_and_points(backend, prod_x, pt)
    for pt in (pcp, p0, p1):
        acc.insert_poly_and_points(backend, frac, pt)
    for perm in pk.permutation_oracles:
        acc.insert_poly_and_points(backend, perm, pcp)
    for w in witness_mles:
        acc.insert_poly_and_points(backend, w, pcp)
    for w in witness_mles:
        acc.insert_poly_and_points(backend, w, zc.point)
    for s in pk.selector_oracles:
        acc.insert_poly_and_points(backend, s, zc.point)
    r_pi = transcript.get_and_append_challenge_vectors(b"r_pi", ell)
    acc.insert_poly_and_points(backend, witness_mles[0], r_pi + [0] * (nv - ell))
    acc.evaluations(backend)
    mark("evaluations")
    batch = acc.multi_open(backend, pk.pcs_param, transcript, phases)
    mark.restart()
    return HyperPlonkProof(commits, batch, zc, pc)


# ---------------------------------------------------------------------------
# vanilla-plonk fixture (full-prove workload)
# ---------------------------------------------------------------------------

def vanilla_fixture(num_vars: int, seed: int, num_pub_input: int = 16, wired: bool = False):
    """Selectors [q_L, q_R, q_O, q_M, q_C] and witnesses [w1, w2, w3] as
    canonical table packets (uint8 arrays), the identity permutation over the
    three witness columns (labels column * 2^nv + row, common/permutation.rs
    and snark.rs:69-76), and the public inputs w1[0..num_pub_input].

    q_L, q_R, q_M, q_C, w1, w2 are uniform (fixture stream `seed`, elements
    [k*N, (k+1)*N) for k = 0..5), q_O = -1 and w3 = q_L w1 + q_R w2 + q_M w1 w2
    + q_C, so the repo's gate holds on every row.  With `wired`, the copy
    constraints are not the identity: w2[i] = w1[wire(i)] for a bijection
    wire of the rows, and the permutation swaps those cells
    (hp_cuda_v1_fixture_vanilla_plonk_wired).  Built by the host fixture
    generator of libhp_cuda.so."""
    from . import _native
    from .errors import check_status
    lib = _native.load()
    n = 1 << num_vars
    sel = np.empty((5, 32 * n), dtype=np.uint8)
    wit = np.empty((3, 32 * n), dtype=np.uint8)
    perm = np.empty((3, 32 * n), dtype=np.uint8)
    entry = lib.hp_cuda_v1_fixture_vanilla_plonk_wired if wired else lib.hp_cuda_v1_fixture_vanilla_plonk
    check_status(entry(
        ctypes.c_uint64(seed), num_vars, sel.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
        wit.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), perm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
        "fixture_vanilla_plonk")
    pub = [int.from_bytes(wit[0, 32 * i:32 * i + 32].tobytes(), "little") for i in range(min(num_pub_input, n))]
    return list(sel), list(wit), list(perm), pub


def vanilla_witness(num_vars: int, circuit_seed: int, witness_seed: int) -> list:
    """Witnesses [w1, w2, w3] of the vanilla_fixture(num_vars, circuit_seed)
    circuit with w1, w2 drawn from fixture stream `witness_seed` (elements
    [4N, 6N)) and w3 solving the gate; equal to that fixture's own witnesses
    when the seeds are equal."""
    from . import _native
    from .errors import check_status
    n = 1 << num_vars
    wit = np.empty((3, 32 * n), dtype=np.uint8)
    check_status(_native.load().hp_cuda_v1_fixture_vanilla_plonk_witness(
        ctypes.c_uint64(circuit_seed), ctypes.c_uint64(witness_seed), num_vars,
        wit.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))), "fixture_vanilla_plonk_witness")
    return list(wit)
