"""The oracle's own prover (oracle/prover.py) and fixtures (hp_oracle.c
or_fixture_vanilla_plonk), on CPU:

- the oracle's fixtures equal the product's host fixture generator
  (hp_cuda_v1_fixture_vanilla_plonk / _wired / _witness) table for table;
- the circuit with non-identity copy constraints satisfies its gate and its
  copy constraints, and its permutation is a permutation of the labels;
- the oracle prover and the product's driver (hyperplonk_gb300.snark over the
  oracle's CpuBackend) give the same proof bytes: two drivers written
  separately agree;
- the host verifier accepts the non-identity circuit's proof and rejects a
  witness that breaks a copy constraint (the reference's
  test_ascend_rejects_bad_copy_constraints_and_witnesses, snark.rs:1058);
- the small sections of tests/golden/headline.json reproduce from the
  committed generator."""
import json
import pathlib

import pytest

from hyperplonk_gb300 import snark

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def op(oracle):
    import prover
    return prover


def ints(table) -> list:
    b = bytes(table)
    return [int.from_bytes(b[i:i + 32], "little") for i in range(0, len(b), 32)]


@pytest.mark.parametrize("nv,wired", [(1, False), (5, False), (9, False), (1, True), (5, True), (9, True)])
def test_oracle_fixture_equals_product_fixture(native_lib, op, nv, wired):
    sel, wit, perm, pub = snark.vanilla_fixture(nv, 2, wired=wired)
    osel, owit, operm, opub = op.vanilla_fixture(nv, 2, wired=wired)
    assert [bytes(t) for t in sel] == osel
    assert [bytes(t) for t in wit] == owit
    assert [bytes(t) for t in perm] == operm
    assert pub == opub


def test_oracle_request_witness_equals_product(native_lib, op):
    for ws in (4 << 32, (4 << 32) | 5):
        assert [bytes(t) for t in snark.vanilla_witness(7, 2, ws)] == op.vanilla_fixture(7, 2, witness_seed=ws)[1]


def test_wired_circuit_satisfies_gate_and_copy_constraints(op):
    nv = 6
    n = 1 << nv
    sel, wit, perm, _ = op.vanilla_fixture(nv, 2, wired=True)
    ql, qr, qo, qm, qc = (ints(s) for s in sel)
    w = [ints(t) for t in wit]
    sigma = [v for t in perm for v in ints(t)]
    assert sorted(sigma) == list(range(3 * n))
    assert sum(1 for i, s in enumerate(sigma) if s != i) >= n  # most w1/w2 cells move
    cells = w[0] + w[1] + w[2]
    assert all(cells[i] == cells[sigma[i]] for i in range(3 * n))
    for i in range(n):
        assert (ql[i] * w[0][i] + qr[i] * w[1][i] + qo[i] * w[2][i] + qm[i] * w[0][i] * w[1][i] + qc[i]) % R == 0


@pytest.mark.parametrize("nv,wired", [(4, False), (6, True)])
def test_oracle_prover_equals_product_driver_on_the_oracle(oracle, op, native_lib, nv, wired):
    import transcript_ref as tref
    cpu = oracle.CpuBackend()
    sel, wit, perm, pub = snark.vanilla_fixture(nv, 2, wired=wired)
    layers = oracle.srs_layers(nv, 30 + nv)
    pk = snark.preprocess(cpu, nv, min(16, 1 << nv), sel, perm, layers, commit=False)
    a = snark.prove(cpu, pk, pub, wit, transcript_cls=tref.OracleIOPTranscript).to_bytes()
    assert a == op.prove_fixture(nv, 2, wired=wired, srs_layers=layers)


def test_verifier_accepts_wired_proof_and_rejects_broken_copy(oracle, op, native_lib):
    import pairing
    import transcript_ref as tref
    import verifier
    nv, srs_seed = 5, 17
    cpu = oracle.CpuBackend()
    sel, wit, perm, pub = snark.vanilla_fixture(nv, 2, wired=True)
    pk = snark.preprocess(cpu, nv, 16, sel, perm, oracle.srs_layers(nv, srs_seed))
    vk = pk.verifying_key(pairing.srs_verifier_param(nv, srs_seed))
    proof = snark.prove(cpu, pk, pub, wit, transcript_cls=tref.OracleIOPTranscript)
    assert verifier.hyperplonk_verify(vk, pub, proof)
    # break the copy constraint of row 3 (w2[3] = w1[wire(3)]) but keep the gate:
    # w2[3] += 1 and w3[3] re-solved
    ql, qr, qo, qm, qc = (ints(s) for s in sel)
    w1, w2, w3 = (ints(t) for t in wit)
    i = 3
    w2[i] = (w2[i] + 1) % R
    w3[i] = (ql[i] * w1[i] + qr[i] * w2[i] + qm[i] * w1[i] * w2[i] + qc[i]) % R
    bad = [oracle.frs_bytes(t) for t in (w1, w2, w3)]
    broken = snark.prove(cpu, pk, pub, bad, transcript_cls=tref.OracleIOPTranscript)
    assert not verifier.hyperplonk_verify(vk, pub, broken)


@pytest.mark.parametrize("section", ["commit", "wired", "sumcheck"])
def test_golden_headline_sections_reproduce(oracle, section):
    sys_path_has = __import__("sys").path
    sys_path_has.insert(0, str(GOLDEN))
    import make_headline
    data = json.loads((GOLDEN / "headline.json").read_text())
    fresh = make_headline.SECTIONS[section]()
    stored = {k: v for k, v in data[section].items() if not k.startswith("oracle_")}
    assert fresh == stored
