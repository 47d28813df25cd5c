"""GB300 results for the measured workloads at their stated sizes, compared
byte for byte with the oracle's (tests/golden/headline.json, written by
tests/golden/make_headline.py from the oracle alone: oracle/prover.py over
the C oracle and the oracle's Python transcript), plus the circuit whose copy
constraints are not the identity against the live oracle prover
(hyperplonk/src/snark.rs:1008, test_ascend_e2e_nonidentity_permutation_matches_cpu,
is the reference's test of that case).

The device-generated testing SRS is checked against the oracle's SRS digest
first, so a difference in the proof cannot hide an SRS difference."""
import base64
import hashlib
import json
import pathlib

import numpy as np
import pytest

from hyperplonk_gb300 import protocol, serialize as ser, snark, workloads
from hyperplonk_gb300.transcript import IOPTranscript

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((pathlib.Path(__file__).resolve().parent / "golden" / "headline.json").read_text())


def affine_digest(layers) -> str:
    """SHA-256 of 97-byte packets as 96-byte affine points (infinity -> zeros)."""
    h = hashlib.sha256()
    for layer in layers:
        a = np.frombuffer(bytes(layer), dtype=np.uint8).reshape(-1, 97)
        aff = a[:, 1:].copy()
        aff[a[:, 0] == 1] = 0
        h.update(aff.tobytes())
    return h.hexdigest()


def first_difference(a: bytes, b: bytes):
    for i, (x, y) in enumerate(zip(a, b)):
        if x != y:
            return i
    return None if len(a) == len(b) else min(len(a), len(b))


def test_commit_nv16_equals_oracle(gpu):
    g = GOLDEN["commit"]
    nv = g["num_vars"]
    layers = gpu.generate_srs(nv, g["srs_seed"])
    assert affine_digest(layers) == g["srs_sha256"]
    params = gpu.prepare_prover_param(nv, layers)
    mle = gpu.mle_from_evaluations(nv, workloads.fixture_fr(g["scalar_seed"], 1 << nv))
    assert ser.g1_compressed(gpu.commit(params, mle)).hex() == g["commitment"]


def test_sumcheck_nv20_equals_oracle(gpu):
    g = GOLDEN["sumcheck"]
    nv, seed = g["num_vars"], g["seed"]
    mles = [gpu.mle_from_evaluations(nv, t) for t in workloads.sumcheck_tables(nv, seed)]
    vp = workloads.sumcheck_polynomial(nv, mles, workloads.sumcheck_coefficients(seed))
    finals = []
    proof = protocol.sumcheck_prove(gpu, vp, IOPTranscript(workloads.SUMCHECK_LABEL), finals)
    hexs = lambda xs: [ser.fr(x).hex() for x in xs]  # noqa: E731
    for k, (got, want) in enumerate(zip(proof.proofs, g["messages"])):
        assert hexs(got) == want, f"round {k + 1}"
    assert len(proof.proofs) == nv
    assert hexs(proof.point) == g["point"]
    assert hexs(finals) == g["finals"]


def _prove_section(gpu, g, wired: bool) -> bytes:
    nv = g["num_vars"]
    layers = gpu.generate_srs(nv, g["srs_seed"])
    assert affine_digest(layers) == g["srs_sha256"]
    sel, wit, perm, pub = snark.vanilla_fixture(nv, g["seed"], wired=wired)
    pk = snark.preprocess(gpu, nv, min(16, 1 << nv), sel, perm, layers, commit=False)
    del layers
    got = snark.prove(gpu, pk, pub, wit).to_bytes()
    want = base64.b64decode(g["proof_b64"])
    assert hashlib.sha256(want).hexdigest() == g["proof_sha256"]
    assert got == want, f"first differing byte at {first_difference(got, want)} of {len(want)}"
    return got


def test_proof_nv20_equals_oracle(gpu):
    _prove_section(gpu, GOLDEN["prove"], wired=False)


def test_wired_proof_equals_oracle_and_verifies(gpu, oracle):
    """Copy constraints that are not the identity: frac and prod hold random
    fractions, so their commitments take the full MSM and real inversions."""
    import prover as oprover
    import pairing
    import verifier
    g = GOLDEN["wired"]
    got = _prove_section(gpu, g, wired=True)
    nv = g["num_vars"]
    # the live oracle prover agrees with the stored bytes
    assert oprover.prove_fixture(nv, g["seed"], srs_seed=g["srs_seed"], wired=True) == got
    # and the host verifier accepts the GB300 proof
    sel, wit, perm, pub = snark.vanilla_fixture(nv, g["seed"], wired=True)
    layers = gpu.generate_srs(nv, g["srs_seed"])
    pk = snark.preprocess(gpu, nv, min(16, 1 << nv), sel, perm, layers)
    proof = snark.prove(gpu, pk, pub, wit)
    assert proof.to_bytes() == got
    assert verifier.hyperplonk_verify(pk.verifying_key(pairing.srs_verifier_param(nv, g["srs_seed"])), pub, proof)


def test_wired_proof_nv20_equals_oracle(gpu):
    _prove_section(gpu, GOLDEN["wired20"], wired=True)


def test_batch_plan_equals_oracle(gpu):
    """The whole batch plan (64 MSMs of 2^12..2^22 points, 32 sumchecks of
    14..22 variables), batched, against per-instance oracle runs."""
    g = GOLDEN["batch"]
    nv_srs = g["srs_num_vars"]
    layers = gpu.generate_srs(nv_srs, g["srs_seed"])
    assert affine_digest(layers[:1]) == g["layer0_sha256"]
    params = gpu.prepare_prover_param(nv_srs, layers)
    del layers
    ks, nvs = workloads.batch_plan(g["seed"])
    assert (ks, nvs) == (g["msm_log_sizes"], g["sumcheck_num_vars"])
    wl = workloads.BatchWorkload(gpu, params, ks, nvs, seed=g["seed"])
    commits, sumchecks = wl.run_batched(IOPTranscript)
    for i, (c, want) in enumerate(zip(commits, g["commitments"])):
        assert ser.g1_compressed(c).hex() == want, f"MSM {i} (2^{ks[i]} points)"
    for i, ((proof, finals), want) in enumerate(zip(sumchecks, g["sumchecks"])):
        got = hashlib.sha256(proof.to_bytes() + ser.vec_fr(finals)).hexdigest()
        assert got == want, f"sumcheck {i} (nv {nvs[i]})"


def test_served_mix_equals_oracle(gpu):
    """Serving requests of 2^16..2^18 gates submitted together (2 lanes x 3
    slots, coalesced commitments and rounds): every served proof equals the
    oracle's proof of the same request."""
    from hyperplonk_gb300 import serve
    g = GOLDEN["serve"]
    nv_max = g["nv_max"]
    layers = gpu.generate_srs(nv_max, g["srs_seed"])
    srv = serve.ProofServer(0, nv_max=nv_max, lanes=2, slots_per_lane=3, srs_layers=layers)
    tickets = []
    for r in g["requests"]:
        nv = r["num_vars"]
        wit = snark.vanilla_witness(nv, g["circuit_seed"], r["witness_seed"])
        pub = [int.from_bytes(wit[0][32 * i:32 * i + 32].tobytes(), "little") for i in range(min(16, 1 << nv))]
        tickets.append(srv.submit(nv, wit, pub))
    served = [srv.wait(t, timeout=900) for t in tickets]
    srv.close()
    for r, proof in zip(g["requests"], served):
        assert hashlib.sha256(proof).hexdigest() == r["proof_sha256"], r
