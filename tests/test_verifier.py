"""The host verifier (oracle/verifier.py over oracle/pairing.py): the pairing
is bilinear and non-degenerate, KZG openings and whole HyperPlonk proofs from
both backends are accepted, and altered proofs are rejected.

Mirrors the reference's verifier tests: subroutines/src/pcs/multilinear_kzg/
mod.rs (single_commit_verify: a wrong value fails), batching.rs (batch
verify), hyperplonk/src/snark.rs (test_hyperplonk_e2e: prove then verify)."""
import copy

import pytest

from hyperplonk_gb300 import snark

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


@pytest.fixture(scope="module")
def pr(oracle):
    import pairing
    return pairing


@pytest.fixture(scope="module")
def ver(oracle):
    import verifier
    return verifier


def g1_mul(oracle, p, k):
    return oracle.affine_to_point(oracle.msm(oracle.point_to_affine(p), (k % R).to_bytes(32, "little")))


def g1_neg(pr, p):
    return (p[0], (-p[1]) % pr.P)


def test_g2_point_has_order_r(pr):
    h = pr.g2_base()
    assert h != pr.G2_INFINITY
    assert pr.g2_mul_unreduced(h, pr.R) == pr.G2_INFINITY
    assert pr.g2_mul_unreduced(h, pr.R - 1) == pr.g2_neg(h)
    assert pr.g2_add(h, pr.g2_neg(h)) == pr.G2_INFINITY


def test_pairing_bilinear_and_nondegenerate(oracle, pr):
    g = oracle.affine_to_point(oracle.g1_generator())
    h = pr.g2_base()
    a, b = 0x1234567890ABCDEF1234, R - 77
    assert not pr.pairing_product_is_one([(g, h)])
    # e(aG, H) = e(G, aH)
    assert pr.pairing_product_is_one([(g1_mul(oracle, g, a), h), (g1_neg(pr, g), pr.g2_mul(h, a))])
    # e(aG, bH) = e(abG, H), and not e((ab+1)G, H)
    lhs = (g1_mul(oracle, g, a), pr.g2_mul(h, b))
    assert pr.pairing_product_is_one([lhs, (g1_neg(pr, g1_mul(oracle, g, a * b)), h)])
    assert not pr.pairing_product_is_one([lhs, (g1_neg(pr, g1_mul(oracle, g, a * b + 1)), h)])
    # identity pairs are skipped
    assert pr.pairing_product_is_one([(None, h), (g, pr.G2_INFINITY)])


def test_kzg_open_verifies(oracle, cpu, pr, ver):
    nv = 5
    layers = oracle.srs_layers(nv, 9)
    vp = pr.srs_verifier_param(nv, 9)
    pp = cpu.prepare_prover_param(nv, layers)
    f = cpu.mle_from_evaluations(nv, oracle.random_fr(3, 1 << nv))
    point = [int.from_bytes(oracle.random_fr(4, nv)[32 * i:32 * i + 32], "little") for i in range(nv)]
    comm = cpu.commit(pp, f)
    proofs, value = cpu.open(pp, f, point)
    assert ver.kzg_verify(vp, comm, point, value, proofs)
    assert not ver.kzg_verify(vp, comm, point, (value + 1) % R, proofs)
    bad = list(proofs)
    bad[0] = g1_mul(oracle, bad[0], 2)
    assert not ver.kzg_verify(vp, comm, point, value, bad)
    # a commitment to another polynomial fails
    other = cpu.commit(pp, cpu.mle_from_evaluations(nv, oracle.random_fr(5, 1 << nv)))
    assert not ver.kzg_verify(vp, other, point, value, proofs)


def _oracle_keys(oracle, cpu, pr, nv, seed, srs_seed):
    import transcript_ref as tref
    sel, wit, perm, pub = snark.vanilla_fixture(nv, seed, 16)
    layers = oracle.srs_layers(nv, srs_seed)
    pk = snark.preprocess(cpu, nv, min(16, 1 << nv), sel, perm, layers)
    proof = snark.prove(cpu, pk, pub, wit, transcript_cls=tref.OracleIOPTranscript)
    return pk, pk.verifying_key(pr.srs_verifier_param(nv, srs_seed)), proof, (sel, wit, perm, pub, layers)


def test_oracle_proof_verifies_and_alterations_fail(oracle, cpu, pr, ver):
    pk, vk, proof, (_, _, _, pub, _) = _oracle_keys(oracle, cpu, pr, 4, 2, 104)
    assert len(vk.selector_commitments) == 5 and len(vk.perm_commitments) == 3
    assert ver.hyperplonk_verify(vk, pub, proof)

    def rejected(mutate, public=pub, key=vk):
        bad = copy.deepcopy(proof)
        mutate(bad)
        return not ver.hyperplonk_verify(key, public, bad)

    # an opened evaluation (perm-check claim), a round message of each
    # sumcheck, a quotient of the final opening (caught only by the pairing),
    # a witness commitment (changes every later challenge)
    assert rejected(lambda b: b.batch_openings.f_i_eval_at_point_i.__setitem__(
        5, (b.batch_openings.f_i_eval_at_point_i[5] + 1) % R))
    assert rejected(lambda b: b.zero_check_proof.proofs[1].__setitem__(2, (b.zero_check_proof.proofs[1][2] + 1) % R))
    assert rejected(lambda b: b.perm_check_proof.zero_check_proof.proofs[0].__setitem__(
        3, (b.perm_check_proof.zero_check_proof.proofs[0][3] + 1) % R))
    assert rejected(lambda b: b.batch_openings.sum_check_proof.proofs[2].__setitem__(
        0, (b.batch_openings.sum_check_proof.proofs[2][0] + 1) % R))
    assert rejected(lambda b: b.batch_openings.g_prime_proof.__setitem__(
        1, g1_mul(oracle, b.batch_openings.g_prime_proof[1], 3)))
    assert rejected(lambda b: b.witness_commits.__setitem__(2, g1_mul(oracle, b.witness_commits[2], 2)))
    # wrong public input; a verifying key with another selector commitment
    assert rejected(lambda b: None, public=[(pub[0] + 1) % R] + pub[1:])
    key = copy.deepcopy(vk)
    key.selector_commitments[3] = g1_mul(oracle, key.selector_commitments[3], 5)
    assert rejected(lambda b: None, key=key)
    with pytest.raises(ver.VerifyError):
        ver.hyperplonk_verify(vk, pub[:8], proof)


@pytest.mark.gpu
@pytest.mark.parametrize("nv", [5, 8])
def test_gpu_proof_verifies_and_keys_equal_oracle(gpu, oracle, cpu, pr, ver, nv):
    from hyperplonk_gb300.transcript import IOPTranscript
    pk_cpu, vk, _, (sel, wit, perm, pub, layers) = _oracle_keys(oracle, cpu, pr, nv, 3, 200 + nv)
    pk = snark.preprocess(gpu, nv, min(16, 1 << nv), sel, perm, [oracle.affine_to_packets(l) for l in layers])
    assert pk.selector_commitments == pk_cpu.selector_commitments
    assert pk.permutation_commitments == pk_cpu.permutation_commitments
    proof = snark.prove(gpu, pk, pub, wit, transcript_cls=IOPTranscript)
    assert ver.hyperplonk_verify(pk.verifying_key(vk.pcs_param), pub, proof)
    bad = copy.deepcopy(proof)
    bad.batch_openings.g_prime_proof[0] = g1_mul(oracle, bad.batch_openings.g_prime_proof[0], 2)
    assert not ver.hyperplonk_verify(vk, pub, bad)


@pytest.mark.gpu
def test_gpu_headline_proof_verifies(gpu, oracle, pr, ver):
    """The nv=20 proof of the default bench workload (vanilla fixture seed 2,
    device-generated testing SRS seed 0) is accepted."""
    nv = 20
    layers = gpu.generate_srs(nv, 0)
    assert oracle.affine_to_point(oracle.packets_to_affine(layers[nv])) == pr.srs_verifier_param(nv, 0)["g"]
    sel, wit, perm, pub = snark.vanilla_fixture(nv, 2)
    pk = snark.preprocess(gpu, nv, 16, sel, perm, layers)
    del layers
    proof = snark.prove(gpu, pk, pub, wit)
    vk = pk.verifying_key(pr.srs_verifier_param(nv, 0))
    assert ver.hyperplonk_verify(vk, pub, proof)
