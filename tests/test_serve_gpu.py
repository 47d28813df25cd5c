"""Prove server on the GPU: requests of several sizes submitted together
(several lanes, several proofs in flight per lane, coalesced commitments and
sumcheck rounds) give, for every request, the same proof bytes as the
request proven alone on the GPU and by the oracle."""
import pytest

from hyperplonk_gb300 import serve, snark

pytestmark = pytest.mark.gpu


def test_served_proofs_equal_alone_and_oracle(gpu, oracle):
    import transcript_ref as tref
    nv_max = 8
    layers = oracle.srs_layers(nv_max, 12)
    packets = [oracle.affine_to_packets(l) for l in layers]
    srv = serve.ProofServer(0, nv_max=nv_max, lanes=2, slots_per_lane=3, hbm_budget_bytes=1 << 34,
                            srs_layers=packets)
    reqs = [(nv, (4 << 32) | i) for i, nv in enumerate([5, 8, 6, 7, 5, 8, 6, 4])]
    tickets = []
    for nv, ws in reqs:
        wit = snark.vanilla_witness(nv, 2, ws)
        pub = [int.from_bytes(wit[0][32 * i:32 * i + 32].tobytes(), "little") for i in range(min(16, 1 << nv))]
        tickets.append((srv.submit(nv, wit, pub), nv, wit, pub))
    served = [srv.wait(t, timeout=600) for t, _, _, _ in tickets]
    srv.close()
    assert sum(l.coalesced_calls for l in srv.lanes) > sum(l.flushes for l in srv.lanes)  # calls were batched
    gparam = gpu.prepare_prover_param(nv_max, packets)
    cpu = oracle.CpuBackend()
    cparam = cpu.prepare_prover_param(nv_max, layers)
    for (t, nv, wit, pub), got in zip(tickets, served):
        sel, _, perm, _ = snark.vanilla_fixture(nv, 2)
        gpk = snark.ProvingKey(nv, min(16, 1 << nv), snark.VANILLA_GATE, gparam,
                               [gpu.mle_from_evaluations(nv, s) for s in sel],
                               [gpu.mle_from_evaluations(nv, p) for p in perm])
        assert snark.prove(gpu, gpk, pub, wit).to_bytes() == got, nv
        cpk = snark.ProvingKey(nv, min(16, 1 << nv), snark.VANILLA_GATE, cparam,
                               [cpu.mle_from_evaluations(nv, s) for s in sel],
                               [cpu.mle_from_evaluations(nv, p) for p in perm])
        assert snark.prove(cpu, cpk, pub, wit, transcript_cls=tref.OracleIOPTranscript).to_bytes() == got, nv


def test_server_rejects_oversized_and_reports_errors(gpu, oracle):
    nv_max = 4
    layers = [oracle.affine_to_packets(l) for l in oracle.srs_layers(nv_max, 13)]
    srv = serve.ProofServer(0, nv_max=nv_max, lanes=1, slots_per_lane=1, hbm_budget_bytes=1 << 30,
                            srs_layers=layers)
    from hyperplonk_gb300.errors import InvalidParameters
    with pytest.raises(InvalidParameters):
        srv.submit(5, [], [])
    wit = snark.vanilla_witness(3, 2, 7)
    bad = srv.submit(3, wit[:2] + [wit[2][:32 * 4]], [])  # a witness table of the wrong size
    with pytest.raises(InvalidParameters):
        srv.wait(bad, timeout=60)
    ok = srv.submit(3, wit, [int.from_bytes(wit[0][32 * i:32 * i + 32].tobytes(), "little") for i in range(8)])
    assert isinstance(srv.wait(ok, timeout=60), bytes)  # the lane recovered
    srv.close()


def test_admission_waits_for_the_memory_budget(gpu, oracle):
    """A budget that holds one proof's measured memory but not two: the second
    request waits in the queue until the first proof has finished, and both
    proofs equal the requests proven alone."""
    nv = 9
    layers = [oracle.affine_to_packets(l) for l in oracle.srs_layers(nv, 14)]
    srv = serve.ProofServer(0, nv_max=nv, lanes=1, slots_per_lane=2, hbm_budget_bytes=1 << 40, srs_layers=layers)
    srv.prepare([nv], measure=True)
    need = srv.measured[nv]
    assert need > 0
    srv.budget = need + need // 2
    reqs = []
    for i in range(2):
        wit = snark.vanilla_witness(nv, 2, (5 << 32) | i)
        pub = [int.from_bytes(wit[0][32 * j:32 * j + 32].tobytes(), "little") for j in range(16)]
        reqs.append((wit, pub))
    tickets = [srv.submit(nv, w, p) for w, p in reqs]
    proofs = [srv.wait(t, timeout=300) for t in tickets]
    srv.close()
    first, second = srv.ticket(tickets[0]), srv.ticket(tickets[1])
    assert second.admitted >= first.finished  # queued behind the budget, not the slots
    gparam = gpu.prepare_prover_param(nv, layers)
    sel, _, perm, _ = snark.vanilla_fixture(nv, 2)
    pk = snark.ProvingKey(nv, 16, snark.VANILLA_GATE, gparam, [gpu.mle_from_evaluations(nv, s) for s in sel],
                          [gpu.mle_from_evaluations(nv, p) for p in perm])
    for (wit, pub), got in zip(reqs, proofs):
        assert snark.prove(gpu, pk, pub, wit).to_bytes() == got
