"""Batched execution (the batch workload's shape, small): many MSMs over
prefixes of one SRS layer in one call, and many sumcheck instances advanced
one round per call -- every result must equal the per-instance oracle run."""
import random

import pytest

from hyperplonk_gb300 import protocol
from hyperplonk_gb300.errors import InvalidState
from hyperplonk_gb300.virtual_polynomial import VirtualPolynomial

pytestmark = pytest.mark.gpu

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def test_batch_msm_prefixes_match_oracle(gpu, oracle):
    nv_srs = 12
    layers = oracle.srs_layers(nv_srs, 41)
    pg = gpu.prepare_prover_param(nv_srs, [oracle.affine_to_packets(l) for l in layers])
    rng = random.Random(3)
    dims = [rng.randint(4, nv_srs) for _ in range(12)] + [nv_srs, 0]
    tables = [oracle.random_fr(200 + i, 1 << d) for i, d in enumerate(dims)]
    mles = [gpu.mle_from_evaluations(d, t) for d, t in zip(dims, tables)]
    got = gpu.batch_msm(pg, 0, mles)
    for d, t, g in zip(dims, tables, got):
        expect = oracle.affine_to_point(oracle.msm(layers[0][:96 * (1 << d)], t))
        assert g == expect, d
    # a second call reuses the cached prefix layers
    assert gpu.batch_msm(pg, 0, mles[:3]) == got[:3]


def test_batch_sumcheck_rounds_match_oracle(gpu, cpu, oracle):
    rng = random.Random(8)
    nvs = [rng.randint(3, 11) for _ in range(6)]
    vps_g, vps_c = [], []
    for i, nv in enumerate(nvs):
        tables = [oracle.random_fr(300 + i, 1 << nv, first=j << nv) for j in range(6)]
        gm = [gpu.mle_from_evaluations(nv, t) for t in tables]
        cm = [cpu.mle_from_evaluations(nv, t) for t in tables]
        vg, vc = VirtualPolynomial(nv), VirtualPolynomial(nv)
        for c, (a, b) in zip([5, 7, 11, 13], [(0, 1), (2, 3), (4, 5), (0, 3)]):
            vg.add_mle_list([gm[a], gm[b]], c)
            vc.add_mle_list([cm[a], cm[b]], c)
        vps_g.append(vg)
        vps_c.append(vc)
    sg = [gpu.prover_init(v) for v in vps_g]
    sc = [cpu.prover_init(v) for v in vps_c]
    ch = [None] * len(nvs)
    for rnd in range(max(nvs)):
        live = [i for i, nv in enumerate(nvs) if rnd < nv]
        msgs = gpu.batch_prove_round([sg[i] for i in live], [ch[i] for i in live])
        for i, m in zip(live, msgs):
            assert m == cpu.prove_round_and_update_state(sc[i], ch[i])
            ch[i] = rng.randrange(R)
    # misuse in a batch leaves every state unchanged
    with pytest.raises(InvalidState):
        gpu.batch_prove_round([sg[0]], [None])


def test_batch_workload_batched_equals_plain_and_oracle(gpu, cpu, oracle):
    """The batch plan's shape at small sizes (MSMs 2^4..2^10 on a nv=10 SRS,
    sumchecks of 3..8 variables): the batched run (one batch_msm call, rounds
    in lockstep) equals the plain one-at-a-time run and the oracle's
    per-instance results."""
    import transcript_ref as tref
    from hyperplonk_gb300 import workloads
    from hyperplonk_gb300.transcript import IOPTranscript
    nv_srs = 10
    layers = oracle.srs_layers(nv_srs, 5)
    pg = gpu.prepare_prover_param(nv_srs, [oracle.affine_to_packets(l) for l in layers])
    ks, nvs = workloads.batch_plan(3, msm_count=10, msm_k=(4, nv_srs), sumcheck_count=6, sumcheck_nv=(3, 8))
    wl = workloads.BatchWorkload(gpu, pg, ks, nvs)
    batched = wl.run_batched(IOPTranscript)
    plain = wl.run_plain(IOPTranscript)
    assert batched == plain
    commits, sumchecks = batched
    for k, s, got in zip(ks, workloads.batch_msm_scalars(ks), commits):
        assert got == oracle.affine_to_point(oracle.msm(layers[0][:96 * (1 << k)], s.tobytes()))
    ref = workloads.BatchWorkload(cpu, None, [], nvs)
    for i, (vp, (proof, finals)) in enumerate(zip(ref.polynomials(), sumchecks)):
        fc = []
        pc = protocol.sumcheck_prove(cpu, vp, tref.OracleIOPTranscript(workloads.SUMCHECK_LABEL), fc)
        assert (proof, finals) == (pc, fc), i
