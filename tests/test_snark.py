"""Full HyperPlonk prove (hyperplonk/src/snark.rs:156-341) of the
vanilla-plonk fixture: CPU checks of the fixture and of the driver over the
oracle, and the GPU parity test -- the serialized proof from the GB300 backend
(native transcript) must equal the oracle's (CPU backend, independent Python
transcript) byte for byte."""
import random

import pytest

from hyperplonk_gb300 import protocol, snark
from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def ints(table) -> list:
    b = bytes(table)
    return [int.from_bytes(b[i:i + 32], "little") for i in range(0, len(b), 32)]


def test_fixture_satisfies_the_gate(native_lib):
    nv = 6
    sel, wit, perm, pub = snark.vanilla_fixture(nv, 2)
    ql, qr, qo, qm, qc = (ints(s) for s in sel)
    w1, w2, w3 = (ints(w) for w in wit)
    for i in range(1 << nv):
        assert (ql[i] * w1[i] + qr[i] * w2[i] + qo[i] * w3[i] + qm[i] * w1[i] * w2[i] + qc[i]) % R == 0
    assert qo[0] == R - 1
    assert ints(perm[2])[5] == 2 * (1 << nv) + 5
    assert pub == w1[:16]


def test_request_witnesses_satisfy_the_same_circuit(native_lib):
    nv = 5
    sel, wit, _, _ = snark.vanilla_fixture(nv, 2)
    assert all((a == b).all() for a, b in zip(snark.vanilla_witness(nv, 2, 2), wit))
    ql, qr, qo, qm, qc = (ints(s) for s in sel)
    for seed in (4 << 32, (4 << 32) + 1):
        w1, w2, w3 = (ints(w) for w in snark.vanilla_witness(nv, 2, seed))
        assert w1 != ints(wit[0])
        for i in range(1 << nv):
            assert (ql[i] * w1[i] + qr[i] * w2[i] + qo[i] * w3[i] + qm[i] * w1[i] * w2[i] + qc[i]) % R == 0


def oracle_prove(oracle, nv, seed, num_pub=16):
    import transcript_ref as tref
    cpu = oracle.CpuBackend()
    sel, wit, perm, pub = snark.vanilla_fixture(nv, seed, num_pub)
    layers = oracle.srs_layers(nv, 100 + nv)
    pk = snark.preprocess(cpu, nv, min(num_pub, 1 << nv), sel, perm, layers)
    return snark.prove(cpu, pk, pub, wit, transcript_cls=tref.OracleIOPTranscript), (sel, wit, perm, pub, layers)


def test_oracle_prove_is_consistent(oracle, native_lib):
    proof, _ = oracle_prove(oracle, 4, 2)
    # the gate zero-check claims a zero sum: s_1(0) + s_1(1) = 0
    first = proof.zero_check_proof.proofs[0]
    assert (first[0] + first[1]) % R == 0
    assert len(proof.zero_check_proof.proofs) == 4
    assert len(proof.zero_check_proof.proofs[0]) == 5  # degree 3 gate x eq -> 4, +1
    # perm-check zero-check: also a zero sum
    pz = proof.perm_check_proof.zero_check_proof.proofs[0]
    assert (pz[0] + pz[1]) % R == 0
    assert len(proof.batch_openings.f_i_eval_at_point_i) == 22
    assert len(proof.to_bytes()) > 1000


@pytest.mark.gpu
@pytest.mark.parametrize("nv", [4, 7, 10])
def test_gpu_proof_bytes_equal_oracle(gpu, oracle, nv):
    from hyperplonk_gb300.transcript import IOPTranscript
    expect, (sel, wit, perm, pub, layers) = oracle_prove(oracle, nv, 2)
    pk = snark.preprocess(gpu, nv, min(16, 1 << nv), sel, perm, [oracle.affine_to_packets(l) for l in layers])
    got = snark.prove(gpu, pk, pub, wit, transcript_cls=IOPTranscript)
    assert got.witness_commits == expect.witness_commits
    assert got.zero_check_proof == expect.zero_check_proof
    assert got.perm_check_proof == expect.perm_check_proof
    assert got.batch_openings == expect.batch_openings
    assert got.to_bytes() == expect.to_bytes()


@pytest.mark.gpu
def test_sumcheck_prove_config2_shape(gpu, cpu, oracle):
    """PolyIOP SumCheck prove of 4 arity-2 products over 6 MLEs (degree 2),
    transcript 'Initializing SumCheck transcript', with final folded values."""
    import transcript_ref as tref
    from hyperplonk_gb300.transcript import IOPTranscript
    nv = 12
    tables = [oracle.random_fr(1, 1 << nv, first=j << nv) for j in range(6)]
    coefs = [int.from_bytes(oracle.random_fr(11, 4)[32 * i:32 * i + 32], "little") for i in range(4)]
    pairs = [(0, 1), (2, 3), (4, 5), (0, 3)]

    def run(be, tcls):
        m = [be.mle_from_evaluations(nv, t) for t in tables]
        vp = VirtualPolynomial(nv)
        for c, (a, b) in zip(coefs, pairs):
            vp.add_mle_list([m[a], m[b]], c)
        finals = []
        proof = protocol.sumcheck_prove(be, vp, tcls(b"Initializing SumCheck transcript"), final_evaluations=finals)
        return proof, finals

    pg, fg = run(gpu, IOPTranscript)
    pc, fc = run(cpu, tref.OracleIOPTranscript)
    assert pg == pc
    assert fg == fc
    assert fg == [cpu.evaluate_mle(cpu.mle_from_evaluations(nv, t), pg.point) for t in tables]
